// sm_103a kernels of the BUFF hot path.
//
// Layout: a warp owns 512 consecutive rows per step; lane L owns rows
// [16L, 16L+16) of that step, i.e. one 16-byte vector of every byte slice and
// 2r bytes of the packed tail.  Slices are streamed with 128-bit
// non-allocating loads; bitmap words are assembled from per-lane 16-bit masks
// with one shuffle.  Later slices and the tail are only touched by lanes that
// still have candidate rows (prefix equal to the target), so a filter reads
// slice 0 in full and only the 32-byte sectors of later slices that hold
// candidates.
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <type_traits>

#include "buff_device.cuh"

#include "buff_internal.h"

namespace buffk {

namespace {

using namespace dev;

std::atomic<uint64_t> g_launches{0};

// ---------------------------------------------------------------- encode

struct MinMax {
  long long lo, hi;
};

// Pass 1 of buff_simd256_encode (compress/buff_simd.rs:3139-3148): the
// column min over all rows and the max over rows >= from.  KEYS: on order
// keys of the raw values (pure bandwidth); otherwise on the quantized values
// (exact for every input, used when the key pass reports a non-finite or
// out-of-range extreme).
template <typename T, bool KEYS>
__global__ void __launch_bounds__(kThreads) k_encode_reduce(const T *__restrict__ x, uint32_t n,
                                                            uint32_t from, int pexp,
                                                            uint32_t dlen, MinMax *part) {
  using EL = Elem<T>;
  constexpr int E = EL::E;
  long long lo = LLONG_MAX, hi = LLONG_MIN;
  const uint32_t nv = n / E;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nth = gridDim.x * blockDim.x;
  const typename EL::V *xv = reinterpret_cast<const typename EL::V *>(x);
  for (uint32_t v0 = tid; v0 < nv; v0 += kU * nth) {
    typename EL::V raw[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t v = v0 + u * nth;
      if (v < nv) raw[u] = __ldcs(xv + v);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t v = v0 + u * nth;
      if (v >= nv) break;
      const uint32_t i0 = v * E;
#pragma unroll
      for (int j = 0; j < E; ++j) {
        const unsigned long long b = EL::bits(raw[u], j);
        const long long q = KEYS ? order_key(b) : fetch_bits(b, pexp, dlen);
        lo = q < lo ? q : lo;
        if (i0 + j >= from) hi = q > hi ? q : hi;
      }
    }
  }
  for (uint32_t i = nv * E + tid; i < n; i += nth) {  // ragged end
    const unsigned long long b = EL::one(x, i);
    const long long q = KEYS ? order_key(b) : fetch_bits(b, pexp, dlen);
    lo = q < lo ? q : lo;
    if (i >= from) hi = q > hi ? q : hi;
  }
  __shared__ long long s_lo[kThreads / 32], s_hi[kThreads / 32];
  lo = warp_min<long long>(lo);
  hi = warp_max_ll(hi);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    s_lo[w] = lo;
    s_hi[w] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < kThreads / 32; ++i) {
      lo = s_lo[i] < lo ? s_lo[i] : lo;
      hi = s_hi[i] > hi ? s_hi[i] : hi;
    }
    part[blockIdx.x].lo = lo;
    part[blockIdx.x].hi = hi;
  }
}

// Combines the per-block extremes, quantizes them (key mode: flags `ok`
// when both extremes are finite and their shift does not wrap, so that
// quantizing commutes with min/max), and finds brk = the first row i >= 1
// with x_i >= x_{i-1} (quantized) -- the end of the leading strictly
// decreasing run that the reference's `else if` max skips.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_encode_finalize(const T *__restrict__ x, uint32_t n,
                                                              int pexp, uint32_t dlen,
                                                              const MinMax *part, int nparts,
                                                              int keys, int find_brk,
                                                              EncStats *out) {
  using EL = Elem<T>;
  __shared__ long long s_lo[kThreads / 32], s_hi[kThreads / 32];
  __shared__ unsigned int s_brk;
  long long lo = LLONG_MAX, hi = LLONG_MIN;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) {
    lo = part[i].lo < lo ? part[i].lo : lo;
    hi = part[i].hi > hi ? part[i].hi : hi;
  }
  lo = warp_min<long long>(lo);
  hi = warp_max_ll(hi);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    s_lo[w] = lo;
    s_hi[w] = hi;
  }
  if (threadIdx.x == 0) s_brk = n;
  __syncthreads();
  // brk: scan the leading rows one block-width at a time
  if (find_brk) {
    for (uint32_t b0 = 1; b0 < n; b0 += blockDim.x) {
      const uint32_t i = b0 + threadIdx.x;
      if (i < n) {
        const long long q = fetch_bits(EL::one(x, i), pexp, dlen);
        const long long p = fetch_bits(EL::one(x, i - 1), pexp, dlen);
        if (q >= p) atomicMin(&s_brk, i);
      }
      __syncthreads();
      if (s_brk < n) break;
    }
  }
  if (threadIdx.x == 0) {
    for (int i = 1; i < kThreads / 32; ++i) {
      lo = s_lo[i] < lo ? s_lo[i] : lo;
      hi = s_hi[i] > hi ? s_hi[i] : hi;
    }
    EncStats st;
    st.ok = 1;
    if (keys) {
      const unsigned long long bl = key_bits(lo), bh = key_bits(hi);
      const int el = (int)((bl >> 52) & 0x7FFu) - 1023, eh = (int)((bh >> 52) & 0x7FFu) - 1023;
      const int lim = 63 - (int)dlen;
      st.ok = (el <= lim && eh <= lim) ? 1 : 0;  // finite (exp 1024 fails) and no wrap
      st.mn = fetch_bits(bl, pexp, dlen);
      st.mx1 = hi == LLONG_MIN ? LLONG_MIN : fetch_bits(bh, pexp, dlen);
    } else {
      st.mn = lo;
      st.mx1 = hi;
    }
    st.x0 = n > 0 ? fetch_bits(EL::one(x, 0), pexp, dlen) : 0;
    st.x1 = n > 1 ? fetch_bits(EL::one(x, 1), pexp, dlen) : 0;
    st.mx0 = n > 1 ? (st.x0 > st.mx1 ? st.x0 : st.mx1) : st.x0;
    st.brk = s_brk;
    *out = st;
  }
}

// Pass 2 of buff_simd256_encode (compress/buff_simd.rs:3181-3232): quantize,
// split each code MSB-first into k flipped bytes and an r-bit tail.  Lane L
// loads its part of the warp's 512 rows coalesced; the code is shifted to the
// top of a 64-bit word so that slice s is byte 7-s, the bytes of neighbouring
// rows are gathered with byte permutes into shared memory, and every lane
// then stores one 16-byte vector per slice and packs the tail of its 16 rows
// into 2r bytes.
template <typename T, int K>
__global__ void __launch_bounds__(kThreads) k_encode_scatter(
    const T *__restrict__ x, uint32_t n, int pexp, uint32_t dlen, long long base, uint32_t fl,
    uint32_t r, uint8_t *__restrict__ slices, size_t stride, uint8_t *__restrict__ tail,
    uint8_t *__restrict__ lead, uint32_t nlead) {
  constexpr uint32_t k = K;
  using EL = Elem<T>;
  constexpr int E = EL::E;
  constexpr int LOADS = 16 / E;
  extern __shared__ uint8_t smem[];
  const uint32_t planes = k + (r ? 1u : 0u);
  const uint32_t lane = threadIdx.x & 31;
  uint8_t *ws = smem + (size_t)(threadIdx.x >> 5) * planes * kRowChunk;
  const uint32_t nchunks = (n + kRowChunk - 1) / kRowChunk;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const unsigned long long rmask = r ? ((1ull << r) - 1ull) : 0ull;
  const uint32_t up = 64u - fl;  // left shift that puts slice s at byte 7-s
  for (uint32_t ch = warp; ch < nchunks; ch += nwarps) {
    const uint32_t r0 = ch * kRowChunk;
    typename EL::V raw[LOADS];
#pragma unroll
    for (int m = 0; m < LOADS; ++m) {
      const uint32_t i0 = r0 + m * 32 * E + lane * E;
      if (i0 + E <= n) raw[m] = __ldcs(reinterpret_cast<const typename EL::V *>(x + i0));
    }
#pragma unroll
    for (int m = 0; m < LOADS; ++m) {
      const uint32_t off = m * 32 * E + lane * E;  // row offset within the chunk
      const uint32_t i0 = r0 + off;
      unsigned long long c[E];
#pragma unroll
      for (int j = 0; j < E; ++j) {
        unsigned long long b = 0;
        if (i0 + E <= n)
          b = EL::bits(raw[m], j);
        else if (i0 + j < n)
          b = EL::one(x, i0 + j);
        c[j] = (i0 + j < n) ? (unsigned long long)(fetch_bits(b, pexp, dlen) - base) : 0ull;
      }
      if constexpr (K > 0) {
        uint32_t hw[E], lw[E];
#pragma unroll
        for (int j = 0; j < E; ++j) {
          // up == 64 only for an all-zero buff-slice code width: every byte is 0
          const unsigned long long a = (up >= 64 ? 0ull : (c[j] << up)) ^ 0x8080808080808080ull;
          hw[j] = (uint32_t)(a >> 32);
          lw[j] = (uint32_t)a;
        }
#pragma unroll
        for (uint32_t sl = 0; sl < k; ++sl) {
          const bool in_hi = sl < 4;
          const uint32_t b = in_hi ? 3u - sl : 7u - sl;  // byte within the 32-bit half
          const uint32_t sel = b | ((4u + b) << 4);
          if (E == 2) {
            const uint32_t v = __byte_perm(in_hi ? hw[0] : lw[0], in_hi ? hw[1] : lw[1], sel);
            *reinterpret_cast<uint16_t *>(ws + sl * kRowChunk + off) = (uint16_t)v;
          } else {
            const uint32_t v01 = __byte_perm(in_hi ? hw[0] : lw[0], in_hi ? hw[1] : lw[1], sel);
            const uint32_t v23 = __byte_perm(in_hi ? hw[2 % E] : lw[2 % E],
                                             in_hi ? hw[3 % E] : lw[3 % E], sel);
            *reinterpret_cast<uint32_t *>(ws + sl * kRowChunk + off) =
                __byte_perm(v01, v23, 0x5410);
          }
        }
      }
      if (r) {
        uint32_t packed = 0;
#pragma unroll
        for (int j = 0; j < E; ++j) packed |= (uint32_t)(c[j] & rmask) << (8 * j);
        if (E == 2)
          *reinterpret_cast<uint16_t *>(ws + k * kRowChunk + off) = (uint16_t)packed;
        else
          *reinterpret_cast<uint32_t *>(ws + k * kRowChunk + off) = packed;
      }
    }
    __syncwarp();
#pragma unroll
    for (int sl = 0; sl < K; ++sl) {
      uint4 v = *reinterpret_cast<const uint4 *>(ws + sl * kRowChunk + lane * 16);
      // the first `nlead` slices go to `lead` (buff-major sparse columns)
      uint8_t *dst = (uint32_t)sl < nlead ? lead + sl * stride : slices + (sl - nlead) * stride;
      __stcs(reinterpret_cast<uint4 *>(dst + r0 + lane * 16), v);
    }
    if (r == 1) {  // one bit per row: gather bit 0 of 8 bytes with one multiply
      const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(ws + k * kRowChunk + lane * 16);
      const uint32_t lo8 = (uint32_t)((v.x * 0x0102040810204080ull) >> 56);
      const uint32_t hi8 = (uint32_t)((v.y * 0x0102040810204080ull) >> 56);
      *reinterpret_cast<uint16_t *>(tail + (size_t)2 * ((r0 >> 4) + lane)) =
          (uint16_t)(lo8 | (hi8 << 8));
    } else if (r) {
      uint4 v = *reinterpret_cast<const uint4 *>(ws + k * kRowChunk + lane * 16);
      const uint8_t *b = reinterpret_cast<const uint8_t *>(&v);
      unsigned long long lo = 0, hi = 0;
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const uint32_t p = i * r;
        const unsigned long long f = b[i];
        if (p >= 64)
          hi |= f << (p - 64);
        else {
          lo |= f << p;
          if (p + r > 64) hi |= f >> (64 - p);
        }
      }
      uint16_t *dst = reinterpret_cast<uint16_t *>(tail + (size_t)2 * r * ((r0 >> 4) + lane));
      for (uint32_t i = 0; i < r; ++i)
        dst[i] = (uint16_t)(i < 4 ? (lo >> (16 * i)) : (hi >> (16 * (i - 4))));
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------- filters

// buff_simd_range_filter / buff_simd_equal_filter (compress/buff_simd.rs:
// 3361-3733) and their fused `_with_slice` forms (:3736-4025).  For every
// 16-row vector: compare slice 0 to the target byte; while some rows still
// equal the target prefix, compare the next slice (gt |= eq & gt_j,
// eq &= eq_j), then the packed tail.  Rows >= full_rows stay clear, which
// reproduces the reference's 32-byte SIMD loop that never reaches the rows
// after the last full 32-row block.
// Candidate refinement of one 32-row block (rows whose prefix equals the
// target so far): the remaining slices, then the packed tail.  Kept out of
// line: it runs for few blocks and would otherwise inflate the streaming
// loop's registers.
__device__ __noinline__ void refine32(const uint8_t *__restrict__ slices, size_t stride,
                                      uint32_t k_used, unsigned long long tb,
                                      const uint8_t *__restrict__ tail, uint32_t r, uint32_t ttail,
                                      uint32_t row0, uint32_t &gt, uint32_t &eq) {
  for (uint32_t j = 1; j < k_used && eq; ++j) {
    const Bytes32 b = ld_cand32(slices + j * stride + row0);
    const ByteTarget t = make_target((uint32_t)(tb >> (8 * j)) & 0xFFu);
    uint32_t g[8], e[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) cmp4(b.w[q], t, g[q], e[q]);
    gt |= eq & gather32(g);
    eq &= gather32(e);
  }
  if (r && eq) {
    // 32 rows of r bits = 4r bytes at byte (row0 / 32) * 4r (4-byte aligned)
    const uint32_t *tp = reinterpret_cast<const uint32_t *>(tail + (size_t)(row0 >> 5) * 4 * r);
    uint32_t tw[8];
#pragma unroll
    for (int i = 0; i < 7; ++i) tw[i] = (uint32_t)i < r ? __ldg(tp + i) : 0u;
    tw[7] = 0;
    uint32_t gtt = 0, eqt = 0;
    for (uint32_t i = 0; i < 32; ++i) {
      if (!(eq >> i & 1u)) continue;
      const uint32_t bit = i * r, wi = bit >> 5, sh = bit & 31;
      const uint32_t f = __funnelshift_r(tw[wi], tw[wi + 1], sh) & ((1u << r) - 1u);
      gtt |= (uint32_t)(f > ttail) << i;
      eqt |= (uint32_t)(f == ttail) << i;
    }
    gt |= eq & gtt;
    eq &= eqt;
  }
}

// A queued block's refinement (the later slices, the tail), its row limit,
// its result word; returns the rows set.
template <bool IS_RANGE>
__device__ __forceinline__ uint32_t finish_filter_block(const FilterArgs &a, unsigned long long tb,
                                                        uint32_t blk, uint32_t gt, uint32_t eq) {
  const uint32_t row0 = blk * 32;
  refine32(a.slices, a.stride, a.k_used, tb, a.tail, a.r, a.ttail, row0, gt, eq);
  uint32_t res = IS_RANGE ? gt : eq;
  if (row0 + 32 > a.full_rows) {
    const uint32_t lim = a.full_rows > row0 ? a.full_rows - row0 : 0u;
    res &= lim >= 32 ? 0xFFFFFFFFu : ((1u << lim) - 1u);
  }
  __stcs(a.words + blk, res);
  return __popc(res);
}

// buff_simd_range_filter / buff_simd_equal_filter (compress/buff_simd.rs:
// 3361-3733) and their fused `_with_slice` forms (:3736-4025).  Lane L owns
// 32 consecutive rows -- one bitmap word -- per load: 32 bytes of slice 0 are
// compared to the target byte (per-byte SWAR on 32-bit words, MSB gather with
// one multiply per 8 rows); while some rows still equal the target prefix the
// next slice refines them (gt |= eq & gt_j, eq &= eq_j), then the packed tail.
// Rows >= full_rows stay clear, which reproduces the reference's 32-byte SIMD
// loop that never reaches the rows after the last full 32-row block.  TH is
// the top bit of the slice-0 target byte.  Blocks that still hold rows equal
// to the target after slice 0 go to a per-warp queue and are refined 32 at a
// time, one per lane, so the dependent loads of the later slices are waited
// on once per 32 such blocks instead of in every step that meets one.  A
// step's slice-0 loads are issued before the previous step is compared (two
// steps, 128 bytes per lane, in flight; 4 CTAs per SM at 64 registers).
template <bool IS_RANGE, bool TH>
__global__ void __launch_bounds__(kThreads, 4) k_filter(FilterArgs a) {
  constexpr int U = 2;  // 32-byte loads in flight per lane
  constexpr int kQ = 96;  // queue entries per warp (at most 31 + 2 * 32)
  __shared__ uint32_t s_q[kThreads / 32][3][kQ];
  const uint32_t lane = threadIdx.x & 31;
  uint32_t(*q)[kQ] = s_q[threadIdx.x >> 5];
  uint32_t qn = 0;  // warp-uniform queue length
  const uint32_t nwords = (a.n + 31) / 32;
  const uint32_t nblk = a.k_used ? (a.n + 31) / 32 : 0u;  // 32-row blocks with a slice byte
  const uint32_t nsteps = (nblk + U * 32 - 1) / (U * 32);
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long tb = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) tb |= (unsigned long long)a.tbyte[j] << (8 * j);
  const uint32_t t0 = (uint32_t)(tb & 0xFFu);
  const uint32_t lo0 = (t0 & 0x7Fu) * 0x01010101u, lo1 = ((t0 & 0x7Fu) + 1u) * 0x01010101u;
  const bool deep = a.k_used > 1 || a.r;
  uint32_t cnt = 0;
  // a step's slice-0 loads are issued before the previous step is compared
  Bytes32 nd[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const uint32_t blk = warp * (U * 32) + lane + u * 32;
    nd[u] = Bytes32{};
    if (warp < nsteps && blk < nblk) nd[u] = ld_stream32_pf(a.slices + (size_t)blk * 32);
  }
  for (uint32_t st = warp; st < nsteps; st += nwarps) {
    const uint32_t blk0 = st * (U * 32) + lane;
    Bytes32 d[U];
#pragma unroll
    for (int u = 0; u < U; ++u) d[u] = nd[u];
    if (st + nwarps < nsteps) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t blk = blk0 + nwarps * (U * 32) + u * 32;
        if (blk < nblk) nd[u] = ld_stream32_pf(a.slices + (size_t)blk * 32);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t blk = blk0 + u * 32;
      const bool live = blk < nblk;
      const uint32_t row0 = blk * 32;
      uint32_t m[8];
      uint32_t eor = 0;
#pragma unroll
      for (int qq = 0; qq < 8; ++qq) {
        m[qq] = eq4t<TH>(d[u].w[qq], lo0, lo1);
        eor |= m[qq];
      }
      uint32_t eq = eor ? gather32(m) : 0u;
      uint32_t gt = 0;
      if (IS_RANGE) {
#pragma unroll
        for (int qq = 0; qq < 8; ++qq) m[qq] = gt4t<TH>(d[u].w[qq], lo1);
        gt = gather32(m);
      }
      if (eq && !deep && a.tail_only_eq) eq = 0;
      const bool more = live && deep && eq != 0;
      const uint32_t qv = __ballot_sync(0xFFFFFFFFu, more);
      if (more) {
        const uint32_t at = qn + __popc(qv & ((1u << lane) - 1u));
        q[0][at] = blk;
        q[1][at] = gt;
        q[2][at] = eq;
      } else if (live) {
        uint32_t res = IS_RANGE ? gt : eq;
        if (row0 + 32 > a.full_rows) {
          const uint32_t lim = a.full_rows > row0 ? a.full_rows - row0 : 0u;
          res &= lim >= 32 ? 0xFFFFFFFFu : ((1u << lim) - 1u);
        }
        __stcs(a.words + blk, res);
        cnt += __popc(res);
      }
      qn += __popc(qv);
    }
    __syncwarp();
    while (qn >= 32) {  // refine 32 queued blocks, one per lane
      qn -= 32;
      const uint32_t blk = q[0][qn + lane];
      uint32_t gt = q[1][qn + lane], eq = q[2][qn + lane];
      __syncwarp();
      cnt += finish_filter_block<IS_RANGE>(a, tb, blk, gt, eq);
    }
  }
  if (lane < qn) {  // what is left in the queue
    const uint32_t blk = q[0][lane];
    uint32_t gt = q[1][lane], eq = q[2][lane];
    cnt += finish_filter_block<IS_RANGE>(a, tb, blk, gt, eq);
  }
  // fixed_len < 8: no slices, every row compared in full on its packed code
  if (!a.k_used) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    for (uint32_t wd = tid; wd < nwords; wd += gridDim.x * blockDim.x) {
      uint32_t gt = 0, eq = 0xFFFFFFFFu;
      if (a.r) {
        eq = 0;
        for (uint32_t i = 0; i < 32; ++i) {
          const unsigned long long bit = (unsigned long long)(wd * 32 + i) * a.r;
          const uint32_t b0 = __ldg(a.tail + (bit >> 3));
          const uint32_t b1 = ((bit & 7) + a.r > 8) ? __ldg(a.tail + (bit >> 3) + 1) : 0u;
          const uint32_t f = ((b0 | (b1 << 8)) >> (bit & 7)) & ((1u << a.r) - 1u);
          gt |= (uint32_t)(f > a.ttail) << i;
          eq |= (uint32_t)(f == a.ttail) << i;
        }
      }
      uint32_t res = IS_RANGE ? gt : eq;
      const uint32_t row0 = wd * 32;
      if (row0 + 32 > a.full_rows) {
        const uint32_t lim = a.full_rows > row0 ? a.full_rows - row0 : 0u;
        res &= lim >= 32 ? 0xFFFFFFFFu : ((1u << lim) - 1u);
      }
      a.words[wd] = res;
      cnt += __popc(res);
    }
  }
  if (a.count) {
    const unsigned long long c = warp_sum_ull(cnt);
    if (lane == 0 && c) atomicAdd(a.count, c);
  }
}

__global__ void k_fill_words(uint32_t *words, uint32_t n, uint32_t value,
                             unsigned long long *count) {
  const uint32_t nw = (n + 31) / 32;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += gridDim.x * blockDim.x) {
    uint32_t v = value;
    if (i == nw - 1 && (n & 31)) v &= (1u << (n & 31)) - 1u;
    words[i] = v;
  }
  if (count && blockIdx.x == 0 && threadIdx.x == 0) *count = value ? n : 0;
}

// Zeroes n u64 result words (counts, partial sums) ahead of the kernel that
// accumulates into them.  In a graph a kernel node keeps the chain on the
// SMs: a copy-engine memset node between two kernels costs about a
// microsecond of engine switching on each side.
__global__ void k_zero_u64(unsigned long long *p, uint32_t n, unsigned long long *q, uint32_t m) {
  // the accumulating kernel after it may start now (a programmatic dependent
  // launch that waits for this one before its first atomic)
  asm volatile("griddepcontrol.launch_dependents;");
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = 0;
  if (i < m) q[i] = 0;
}

// ---------------------------------------------------------------- sum

// byte_fixed_sum (compress/split_double.rs:2127-2208): the per-slice sums of
// the unflipped bytes and the sum of the packed tail fields, exact in u64.
// Each slice is streamed as one flat array of `stride` bytes (padding rows
// hold the flipped zero 0x80), and the tail as a flat bit stream of
// n * ts bits, so every load is a coalesced 16-byte vector.
__global__ void __launch_bounds__(kThreads) k_sum(const uint8_t *__restrict__ slices,
                                                  size_t stride, uint32_t ks,
                                                  const uint8_t *__restrict__ tail, uint32_t ts,
                                                  unsigned long long tail_bits,
                                                  unsigned long long *partials) {
  __shared__ unsigned long long s_acc[9];
  if (threadIdx.x < 9) s_acc[threadIdx.x] = 0;
  __syncthreads();
  sum_slices_tail(slices, stride, ks, tail, ts, tail_bits, blockIdx.x * blockDim.x + threadIdx.x,
                  gridDim.x * blockDim.x, s_acc);
  __syncthreads();
  if (threadIdx.x < ks && s_acc[threadIdx.x]) atomicAdd(&partials[threadIdx.x], s_acc[threadIdx.x]);
  if (threadIdx.x == 8 && ts && s_acc[8]) atomicAdd(&partials[ks], s_acc[8]);
}

// The query pair "range filter, then sum" in one pass (buff_range_filter_sum):
// k_sum's flat streaming of every slice, with slice 0 read as one 256-bit
// load per 32-row block -- the block's bitmap word -- so the byte sums and
// the per-byte SWAR compare with the target share the load.  Candidate
// blocks are refined through the later slices and the tail (refine32).
// Rows >= full_rows stay clear (the reference's 32-row SIMD loop).
template <bool TH>
__global__ void __launch_bounds__(kThreads) k_filter_sum(FilterArgs a, uint32_t ks, uint32_t ts,
                                                         unsigned long long tail_bits,
                                                         unsigned long long *partials) {
  constexpr int U = 2;  // 32-byte blocks in flight per thread
  __shared__ unsigned long long s_acc[9];
  if (threadIdx.x < 9) s_acc[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nth = gridDim.x * blockDim.x;
  const uint32_t nv = (uint32_t)(a.stride / 16);
  const uint32_t nblk = (uint32_t)(a.stride / 32);
  const uint32_t nwords = (a.n + 31) / 32;
  unsigned long long tb = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) tb |= (unsigned long long)a.tbyte[j] << (8 * j);
  const uint32_t t0 = (uint32_t)(tb & 0xFFu);
  const uint32_t lo0 = (t0 & 0x7Fu) * 0x01010101u, lo1 = ((t0 & 0x7Fu) + 1u) * 0x01010101u;
  const bool deep = a.k_used > 1 || a.r;
  uint32_t cnt = 0;
  {
    uint32_t acc = 0;
    for (uint32_t b0 = tid; b0 < nblk; b0 += U * nth) {
      Bytes32 d[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t blk = b0 + u * nth;
        if (blk < nblk) {
          d[u] = ld_stream32(a.slices + (size_t)blk * 32);
        } else {
#pragma unroll
          for (int q = 0; q < 8; ++q) d[u].w[q] = H;
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t blk = b0 + u * nth;
        uint32_t me[8], mg[8], eor = 0;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          acc = __dp4a(d[u].w[q] ^ H, 0x01010101u, acc);
          me[q] = eq4t<TH>(d[u].w[q], lo0, lo1);
          mg[q] = gt4t<TH>(d[u].w[q], lo1);
          eor |= me[q];
        }
        if (blk >= nwords) continue;  // padding blocks: summed (zero bytes), never filtered
        uint32_t eq = eor ? gather32(me) : 0u;
        uint32_t gt = gather32(mg);
        const uint32_t row0 = blk * 32;
        if (eq && deep)
          refine32(a.slices, a.stride, a.k_used, tb, a.tail, a.r, a.ttail, row0, gt, eq);
        if (row0 + 32 > a.full_rows) {
          const uint32_t lim = a.full_rows > row0 ? a.full_rows - row0 : 0u;
          gt &= lim >= 32 ? 0xFFFFFFFFu : ((1u << lim) - 1u);
        }
        __stcs(a.words + blk, gt);
        cnt += __popc(gt);
      }
    }
    const unsigned long long w = warp_sum_ull(acc);
    if (lane == 0 && w) atomicAdd(&s_acc[0], w);
  }
  for (uint32_t s = 1; s < ks; ++s) {
    const uint8_t *sl = a.slices + (size_t)s * a.stride;
    uint32_t acc = 0;
    for (uint32_t v0 = tid; v0 < nv; v0 += kU * nth) {
      uint4 d[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const uint32_t v = v0 + u * nth;
        d[u] = v < nv ? ld_stream(sl + (size_t)v * 16) : make_uint4(H, H, H, H);
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        acc = __dp4a(d[u].x ^ H, 0x01010101u, acc);
        acc = __dp4a(d[u].y ^ H, 0x01010101u, acc);
        acc = __dp4a(d[u].z ^ H, 0x01010101u, acc);
        acc = __dp4a(d[u].w ^ H, 0x01010101u, acc);
      }
    }
    const unsigned long long w = warp_sum_ull(acc);
    if (lane == 0 && w) atomicAdd(&s_acc[s], w);
  }
  if (ts) {
    const unsigned long long nbytes = (tail_bits + 7) / 8;
    const uint32_t ntv = (uint32_t)((nbytes + 15) / 16);
    unsigned long long acc = 0;
    const uint32_t c32 = 32 % ts;
    const uint32_t cstep = (uint32_t)(((unsigned long long)nth * 128) % ts);
    uint32_t pv = (uint32_t)(((unsigned long long)tid * 128) % ts);  // phase of word 0 of v
    for (uint32_t v = tid; v < ntv; v += nth) {
      uint4 d = *reinterpret_cast<const uint4 *>(a.tail + (size_t)v * 16);
      const uint32_t *w = reinterpret_cast<const uint32_t *>(&d);
      uint32_t ph = pv;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const unsigned long long b0 = (unsigned long long)v * 128 + 32 * q;
        uint32_t word = w[q];
        if (b0 >= tail_bits)
          word = 0;
        else if (b0 + 32 > tail_bits)
          word &= (1u << (uint32_t)(tail_bits - b0)) - 1u;
        acc += wpopc(word, ph, ts);
        ph += c32;
        if (ph >= ts) ph -= ts;
      }
      pv += cstep;
      if (pv >= ts) pv -= ts;
    }
    acc = warp_sum_ull(acc);
    if (lane == 0 && acc) atomicAdd(&s_acc[8], acc);
  }
  if (a.count) {
    const unsigned long long c = warp_sum_ull(cnt);
    if (lane == 0 && c) atomicAdd(a.count, c);
  }
  __syncthreads();
  if (threadIdx.x < ks && s_acc[threadIdx.x]) atomicAdd(&partials[threadIdx.x], s_acc[threadIdx.x]);
  if (threadIdx.x == 8 && ts && s_acc[8]) atomicAdd(&partials[ks], s_acc[8]);
}

// The same one-pass filter + sum with the slices interleaved: a lane takes
// one 32-row block at a time and loads that block's 32 bytes of every slice
// and its r tail words together, so the filter's compare work on slice 0 is
// spread over the whole stream instead of running while only slice 0 is read.
// KS = k (1..4) slices.  The tail sum is the weighted popcount of the block's
// r words (bits past n*r masked); candidate blocks are refined as in k_filter.
template <bool TH, int KS>
__global__ void __launch_bounds__(kThreads) k_filter_sum_il(FilterArgs a, uint32_t ts,
                                                            unsigned long long tail_bits,
                                                            unsigned long long *partials) {
  __shared__ unsigned long long s_acc[9];
  if (threadIdx.x < 9) s_acc[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nth = gridDim.x * blockDim.x;
  const uint32_t nblk = (uint32_t)(a.stride / 32);
  const uint32_t nwords = (a.n + 31) / 32;
  unsigned long long tb = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) tb |= (unsigned long long)a.tbyte[j] << (8 * j);
  const uint32_t t0 = (uint32_t)(tb & 0xFFu);
  const uint32_t lo0 = (t0 & 0x7Fu) * 0x01010101u, lo1 = ((t0 & 0x7Fu) + 1u) * 0x01010101u;
  const bool deep = a.k_used > 1 || a.r;
  const uint32_t c32 = ts ? 32 % ts : 0u;  // phase step of one tail word
  uint32_t acc[KS];
#pragma unroll
  for (int s = 0; s < KS; ++s) acc[s] = 0;
  unsigned long long tacc = 0;
  uint32_t cnt = 0;
  for (uint32_t blk = tid; blk < nblk; blk += nth) {
    Bytes32 d[KS];
#pragma unroll
    for (int s = 0; s < KS; ++s) d[s] = ld_stream32(a.slices + (size_t)s * a.stride + (size_t)blk * 32);
    uint32_t tw[7];
#pragma unroll
    for (int q = 0; q < 7; ++q)
      tw[q] = (q < (int)ts && blk < nwords)
                  ? __ldcs(reinterpret_cast<const uint32_t *>(a.tail) + (size_t)ts * blk + q)
                  : 0u;
#pragma unroll
    for (int s = 0; s < KS; ++s)
#pragma unroll
      for (int q = 0; q < 8; ++q) acc[s] = __dp4a(d[s].w[q] ^ H, 0x01010101u, acc[s]);
    uint32_t ph = 0;  // a block's tail starts at a stream bit that is a multiple of ts
#pragma unroll
    for (int q = 0; q < 7; ++q) {
      if (q < (int)ts) {
        const unsigned long long b0 = ((unsigned long long)ts * blk + q) * 32;
        uint32_t word = tw[q];
        if (b0 >= tail_bits)
          word = 0;
        else if (b0 + 32 > tail_bits)
          word &= (1u << (uint32_t)(tail_bits - b0)) - 1u;
        tacc += wpopc(word, ph, ts);
        ph += c32;
        if (ph >= ts) ph -= ts;
      }
    }
    if (blk >= nwords) continue;  // padding blocks: summed (zero bytes), never filtered
    uint32_t me[8], mg[8], eor = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      me[q] = eq4t<TH>(d[0].w[q], lo0, lo1);
      mg[q] = gt4t<TH>(d[0].w[q], lo1);
      eor |= me[q];
    }
    uint32_t eq = eor ? gather32(me) : 0u;
    uint32_t gt = gather32(mg);
    const uint32_t row0 = blk * 32;
    if (eq && deep) refine32(a.slices, a.stride, a.k_used, tb, a.tail, a.r, a.ttail, row0, gt, eq);
    if (row0 + 32 > a.full_rows) {
      const uint32_t lim = a.full_rows > row0 ? a.full_rows - row0 : 0u;
      gt &= lim >= 32 ? 0xFFFFFFFFu : ((1u << lim) - 1u);
    }
    __stcs(a.words + blk, gt);
    cnt += __popc(gt);
  }
  // the zeroed count and partials (the launch before this one, when this is
  // its programmatic dependent) are added to only from here on
  asm volatile("griddepcontrol.wait;" ::: "memory");
#pragma unroll
  for (int s = 0; s < KS; ++s) {
    const unsigned long long w = warp_sum_ull(acc[s]);
    if (lane == 0 && w) atomicAdd(&s_acc[s], w);
  }
  {
    const unsigned long long w = warp_sum_ull(tacc);
    if (lane == 0 && w) atomicAdd(&s_acc[8], w);
  }
  if (a.count) {
    const unsigned long long c = warp_sum_ull(cnt);
    if (lane == 0 && c) atomicAdd(a.count, c);
  }
  __syncthreads();
  if (threadIdx.x < KS && s_acc[threadIdx.x]) atomicAdd(&partials[threadIdx.x], s_acc[threadIdx.x]);
  if (threadIdx.x == 8 && ts && s_acc[8]) atomicAdd(&partials[KS], s_acc[8]);
}

// ---------------------------------------------------------------- max


// The full stored code of row i (slices MSB-first, then the tail field).
__device__ __forceinline__ unsigned long long code_at(const uint8_t *slices, size_t stride,
                                                      uint32_t k, const uint8_t *tail,
                                                      uint32_t r, uint32_t i) {
  unsigned long long c = 0;
  for (uint32_t s = 0; s < k; ++s) c = (c << 8) | (uint32_t)(__ldg(slices + s * stride + i) ^ 0x80u);
  if (r) {
    const unsigned long long bit = (unsigned long long)i * r;
    const uint32_t b0 = __ldg(tail + (bit >> 3));
    const uint32_t b1 = ((bit & 7) + r > 8) ? __ldg(tail + (bit >> 3) + 1) : 0u;
    c = (c << r) | (((b0 | (b1 << 8)) >> (bit & 7)) & ((1u << r) - 1u));
  }
  return c;
}


// byte_fixed_max (compress/split_double.rs:3919-4105): the maximum stored
// code.  Lanes own 32 rows per 256-bit load.  Each warp keeps the best code it
// has seen and, per step, first tests with per-byte SWAR whether any leading
// byte reaches the best's leading byte; only then does it find the step's
// largest leading byte and gather the remaining slices of those rows.
__global__ void __launch_bounds__(kThreads) k_max(const uint8_t *__restrict__ slices, size_t stride,
                                                  uint32_t k, const uint8_t *__restrict__ tail,
                                                  uint32_t r, uint32_t fl, uint32_t n,
                                                  unsigned long long *out) {
  constexpr int U = 2;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  if (k == 0) {  // packed codes only (fixed_len < 8)
    const uint32_t nvec = (n + 15) / 16;
    unsigned long long best = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nvec; v += gridDim.x * blockDim.x) {
      unsigned long long lo, hi;
      load_tail16(tail, v, r, lo, hi);
      for (uint32_t i = 0; i < 16 && v * 16 + i < n; ++i) {
        unsigned long long f = field16(lo, hi, i, r);
        best = f > best ? f : best;
      }
    }
    best = warp_max_ull(best);
    if (lane == 0 && n) atomicMax(out, best);
    return;
  }
  const uint32_t nblk = (n + 31) / 32;
  const uint32_t nsteps = (nblk + U * 32 - 1) / (U * 32);
  unsigned long long best = 0;
  bool have = false;
  uint32_t top = 0;  // leading byte of best
  // a step's loads are issued before the previous step is tested
  Bytes32 nd[U];
#pragma unroll
  for (int u = 0; u < U; ++u) {
    const uint32_t blk = warp * (U * 32) + lane + u * 32;
    nd[u] = Bytes32{};
    if (warp < nsteps && blk < nblk) nd[u] = ld_stream32_pf(slices + (size_t)blk * 32);
  }
  for (uint32_t st = warp; st < nsteps; st += nwarps) {
    const uint32_t blk0 = st * (U * 32) + lane;
    Bytes32 d[U];
#pragma unroll
    for (int u = 0; u < U; ++u) d[u] = nd[u];
    if (st + nwarps < nsteps) {
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const uint32_t blk = blk0 + nwarps * (U * 32) + u * 32;
        if (blk < nblk) nd[u] = ld_stream32_pf(slices + (size_t)blk * 32);
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t blk = blk0 + u * 32;
      if (blk < nblk) {
        const uint32_t row0 = blk * 32;
        if (row0 + 32 > n) {  // padding rows -> flipped zero
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const uint32_t lo = row0 + 4u * q;
            const uint32_t keep = n >= lo + 4 ? 0xFFFFFFFFu : (n <= lo ? 0u : ((1u << (8 * (n - lo))) - 1u));
            d[u].w[q] = (d[u].w[q] & keep) | (H & ~keep);
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) d[u].w[q] = H;
      }
    }
    // any leading byte >= top?  (a >= t: t_hi ? a_hi & a_lo>=t_lo : a_hi | a_lo>=t_lo)
    const uint32_t lo0 = (top & 0x7Fu) * 0x01010101u;
    const uint32_t th = (top & 0x80u) ? 0xFFFFFFFFu : 0u;
    uint32_t any = 0;
#pragma unroll
    for (int u = 0; u < U; ++u)
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        const uint32_t w = d[u].w[q];
        const uint32_t d0 = (w | H) - lo0;
        any |= ((th & ~w & d0) | (~th & (~w | d0))) & H;
      }
    if (have && !__any_sync(0xFFFFFFFFu, any != 0)) continue;
    uint32_t mb[U];
    uint32_t lm = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      uint32_t m = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) m = __vmaxu4(m, d[u].w[q] ^ H);
      m = __vmaxu4(m, m >> 16);
      m = __vmaxu4(m, m >> 8);
      mb[u] = m & 0xFFu;
      lm = mb[u] > lm ? mb[u] : lm;
    }
    const uint32_t wmb = __reduce_max_sync(0xFFFFFFFFu, lm);
    if (have && wmb < top) continue;
    unsigned long long m = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const uint32_t blk = blk0 + u * 32;
      if (blk < nblk && mb[u] == wmb) {
        uint32_t e[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) e[q] = eqbytes(d[u].w[q], (wmb ^ 0x80u) * 0x01010101u);
        const uint32_t cand = gather32(e);
        const unsigned long long c = max_in_block(slices, stride, k, tail, r, blk * 32, cand, wmb);
        m = c > m ? c : m;
      }
    }
    m = warp_max_ull(m);
    if (!have || m > best) best = m;
    have = true;
    // publish the warp's best and take the best any warp has published, so
    // that every warp's threshold rises with the column's running maximum
    unsigned long long g = 0;
    if (lane == 0) g = atomicMax(out, best);
    g = __shfl_sync(0xFFFFFFFFu, g, 0);
    if (g > best) best = g;
    top = (uint32_t)(best >> (fl - 8)) & 0xFFu;
  }
  if (lane == 0 && have) atomicMax(out, best);
}

// Rows whose stored code equals the maximum (the arg-max bitmap `res` of
// byte_fixed_max).
__global__ void __launch_bounds__(kThreads) k_argmax(const uint8_t *__restrict__ slices,
                                                     size_t stride, uint32_t k,
                                                     const uint8_t *__restrict__ tail, uint32_t r,
                                                     uint32_t fl, uint32_t n,
                                                     const unsigned long long *dmax,
                                                     uint32_t *words, unsigned long long *count) {
  const uint32_t nw = (n + 31) / 32;
  const unsigned long long M = *dmax;
  const uint32_t top = k ? (uint32_t)(M >> (fl - 8)) & 0xFFu : 0u;
  unsigned long long cnt = 0;
  for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nw; w += gridDim.x * blockDim.x) {
    uint32_t bits = 0;
    const uint32_t r0 = w * 32;
    for (uint32_t i = 0; i < 32 && r0 + i < n; ++i) {
      if (k && (uint32_t)(__ldg(slices + r0 + i) ^ 0x80u) != top) continue;
      if (code_at(slices, stride, k, tail, r, r0 + i) == M) bits |= 1u << i;
    }
    words[w] = bits;
    cnt += __popc(bits);
  }
  cnt = warp_sum_ull(cnt);
  if ((threadIdx.x & 31) == 0 && cnt && count) atomicAdd(count, cnt);
}

// ---------------------------------------------------------------- decode

// buff_simd256_decode (compress/buff_simd.rs:3252-3357) and the
// precision-limited decode (compress/split_double.rs:1612-1893).  KS leading
// slices and `ts` packed bits per row are rebuilt; the reference walks its
// slices as if the code were 8*KS+ts bits wide, so with the quirk kept
// (keep == ~0) the value is (base + X) / 2^dlen with X those bits *not*
// shifted back, and when ts != r the packed bits are read with a stride of ts.
// The INTENDED form passes all bits and a `keep` mask instead.
//
// Lane L produces rows 64m + 2L and 64m + 2L + 1 of each 512-row chunk, so the
// f64 results leave as coalesced 16-byte stores; the two slice bytes per row
// pair are 2-byte loads (64 contiguous bytes per warp), and the packed bits of
// a 64-row group (8*ts bytes) are loaded by the first 2*ts lanes and handed out
// with shuffles.
//
// N32: every value base + code of the column fits in 32 bits (checked on the
// host), so the code is built in 32 bits and converted with the exact 32-bit
// path.
template <int KS, bool N32 = false>
__global__ void __launch_bounds__(kThreads) k_decode(const uint8_t *__restrict__ slices,
                                                     size_t stride,
                                                     const uint8_t *__restrict__ tail,
                                                     uint32_t ts, uint32_t n, long long base,
                                                     int dlen, unsigned long long keep,
                                                     uint32_t rshift, double *__restrict__ out) {
  using CodeT = typename std::conditional<N32, uint32_t, unsigned long long>::type;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nchunks = (n + kRowChunk - 1) / kRowChunk;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const unsigned long long tmask = ts ? ((1ull << ts) - 1ull) : 0ull;
  for (uint32_t ch = warp; ch < nchunks; ch += nwarps) {
    const uint32_t r0 = ch * kRowChunk;
    uint32_t sb[8][KS > 0 ? KS : 1];
#pragma unroll
    for (int m = 0; m < 8; ++m)
#pragma unroll
      for (int s = 0; s < KS; ++s)
        sb[m][s] = __ldg(reinterpret_cast<const uint16_t *>(slices + s * stride + r0 + m * 64 +
                                                            2 * lane));
    uint32_t tw[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      tw[m] = 0;
      if (ts && lane < 2 * ts)
        tw[m] = __ldg(reinterpret_cast<const uint32_t *>(
                          tail + (size_t)8 * ts * (r0 / 64 + m)) + lane);
    }
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      CodeT c0 = 0, c1 = 0;
#pragma unroll
      for (int s = 0; s < KS; ++s) {
        c0 = (c0 << 8) | ((sb[m][s] & 0xFFu) ^ 0x80u);
        c1 = (c1 << 8) | (((sb[m][s] >> 8) & 0xFFu) ^ 0x80u);
      }
      if (ts) {
        const uint32_t bit = 2 * lane * ts, wi = bit >> 5;
        const uint32_t w0 = __shfl_sync(0xFFFFFFFFu, tw[m], wi);
        const uint32_t w1 = __shfl_sync(0xFFFFFFFFu, tw[m], (wi + 1) & 31);
        const uint32_t f = __funnelshift_r(w0, w1, bit & 31);
        c0 = (c0 << ts) | (f & tmask);
        c1 = (c1 << ts) | ((f >> ts) & tmask);
      }
      const uint32_t i0 = r0 + m * 64 + 2 * lane;
      c0 >>= rshift;
      c1 >>= rshift;
      double v0, v1;
      if (N32) {
        v0 = i32_to_f64_scaled((int)((uint32_t)base + (uint32_t)(c0 & (CodeT)keep)), dlen);
        v1 = i32_to_f64_scaled((int)((uint32_t)base + (uint32_t)(c1 & (CodeT)keep)), dlen);
      } else {
        v0 = i64_to_f64_scaled((long long)((unsigned long long)base + (c0 & keep)), dlen);
        v1 = i64_to_f64_scaled((long long)((unsigned long long)base + (c1 & keep)), dlen);
      }
      if (i0 + 2 <= n)
        __stcs(reinterpret_cast<double2 *>(out + i0), make_double2(v0, v1));
      else if (i0 < n)
        out[i0] = v0;
    }
  }
}

// The same decode for codes of at most 32 bits that carry tail bits (KS <= 3
// slices, 0 < ts, 8 KS + ts <= 32) into a 32-byte aligned output: lane L
// takes 4 consecutive rows per 128-row group, so each slice costs one 4-byte
// load per lane (128 bytes per warp request), a 4x4 byte transpose (six byte
// permutes) turns the slice words into the 4 rows' codes, one shuffle pair
// brings the 4 tail fields, and the 4 values leave in one 32-byte store.
// Measured on the 2^28-row walk column (fixed_len 25): full decode 0.536 ->
// 0.496 ms; for byte-aligned reads (ts = 0) and 16-byte aligned outputs it
// was no faster than k_decode, which keeps those.
template <int KS, bool N32>
__global__ void __launch_bounds__(kThreads) k_decode4(const uint8_t *__restrict__ slices,
                                                      size_t stride,
                                                      const uint8_t *__restrict__ tail,
                                                      uint32_t ts, uint32_t n, long long base,
                                                      int dlen, unsigned long long keep,
                                                      uint32_t rshift, double *__restrict__ out) {
  static_assert(KS >= 1 && KS <= 3, "k_decode4 builds codes of at most 3 slices + tail");
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nchunks = (n + kRowChunk - 1) / kRowChunk;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t tmask = ts ? ((1u << ts) - 1u) : 0u;
  const uint32_t keep32 = (uint32_t)keep;
  // unflip only the bytes that hold slices
  const uint32_t kx = 0x80808080u & ((1u << (8 * KS)) - 1u);
  for (uint32_t ch = warp; ch < nchunks; ch += nwarps) {
    const uint32_t r0 = ch * kRowChunk;
    uint32_t sw[4][KS];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int s = 0; s < KS; ++s)
        sw[m][s] = __ldg(reinterpret_cast<const uint32_t *>(slices + s * stride + r0 + m * 128 +
                                                            4 * lane));
    uint32_t tw[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      tw[m] = 0;
      // a 128-row group's ts-bit fields: 4 ts words at byte 16 ts * group
      if (ts && lane < 4 * ts)
        tw[m] = __ldg(reinterpret_cast<const uint32_t *>(
                          tail + (size_t)16 * ts * (r0 / 128 + m)) + lane);
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      // W[j] = the slice whose byte lands at significance j (slice KS-1-j)
      uint32_t W[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) W[j] = j < KS ? sw[m][KS - 1 - j] : 0u;
      const uint32_t t0 = __byte_perm(W[0], W[1], 0x5140), t1 = __byte_perm(W[0], W[1], 0x7362);
      const uint32_t t2 = __byte_perm(W[2], W[3], 0x5140), t3 = __byte_perm(W[2], W[3], 0x7362);
      uint32_t c[4] = {__byte_perm(t0, t2, 0x5410), __byte_perm(t0, t2, 0x7632),
                       __byte_perm(t1, t3, 0x5410), __byte_perm(t1, t3, 0x7632)};
      uint32_t f = 0;
      if (ts) {
        const uint32_t bit = 4 * lane * ts, wi = bit >> 5;
        const uint32_t w0 = __shfl_sync(0xFFFFFFFFu, tw[m], wi);
        const uint32_t w1 = __shfl_sync(0xFFFFFFFFu, tw[m], (wi + 1) & 31);
        f = __funnelshift_r(w0, w1, bit & 31);
      }
      double v[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        uint32_t code = c[i] ^ kx;
        if (ts) code = (code << ts) | ((f >> (i * ts)) & tmask);
        code = (code >> rshift) & keep32;
        if (N32)
          v[i] = i32_to_f64_scaled((int)((uint32_t)base + code), dlen);
        else
          v[i] = i64_to_f64_scaled((long long)((unsigned long long)base + code), dlen);
      }
      const uint32_t i0 = r0 + m * 128 + 4 * lane;
      double *o = out + i0;
      if (i0 + 4 <= n) {
        asm volatile("st.global.cs.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(o), "d"(v[0]), "d"(v[1]),
                     "d"(v[2]), "d"(v[3])
                     : "memory");
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (i0 + i < n) o[i] = v[i];
      }
    }
  }
}

// Resident CTAs per SM of a kernel, asked of the runtime once per (kernel,
// threads, shared memory) and kept: the occupancy query costs microseconds
// of host time, which a small column's launch would otherwise pay every call.
int grid_for(const void *fn, int threads, size_t smem, int device) {
  struct Entry {
    const void *fn;
    int threads;
    size_t smem;
    int per_sm;
  };
  static Entry table[256];
  static int used = 0;
  static std::mutex mu;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lk(mu);
    for (int i = 0; i < used; ++i)
      if (table[i].fn == fn && table[i].threads == threads && table[i].smem == smem) {
        per_sm = table[i].per_sm;
        break;
      }
  }
  if (!per_sm) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
    if (per_sm < 1) per_sm = 1;
    std::lock_guard<std::mutex> lk(mu);
    if (used < 256) table[used++] = Entry{fn, threads, smem, per_sm};
  }
  return per_sm * num_sms(device);
}

int cur_device() {
  int d = 0;
  cudaGetDevice(&d);
  return d;
}

}  // namespace

int num_sms(int device) {
  static std::atomic<int> cached[64];
  if (device < 0 || device >= 64) return 1;
  int c = cached[device].load(std::memory_order_relaxed);
  if (!c) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    c = v > 0 ? v : 1;
    cached[device].store(c, std::memory_order_relaxed);
  }
  return c;
}

void count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t launches() { return g_launches.load(std::memory_order_relaxed); }

template <typename T>
static cudaError_t reduce_impl(const T *x, uint32_t n, uint32_t from, int32_t pexp, uint32_t dlen,
                               int keys, int find_brk, EncStats *d_out, cudaStream_t s) {
  const int nb = 4 * num_sms(cur_device());
  MinMax *part = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&part), sizeof(MinMax) * nb, s);
  if (e != cudaSuccess) return e;
  if (keys)
    k_encode_reduce<T, true><<<nb, kThreads, 0, s>>>(x, n, from, pexp, dlen, part);
  else
    k_encode_reduce<T, false><<<nb, kThreads, 0, s>>>(x, n, from, pexp, dlen, part);
  k_encode_finalize<T><<<1, kThreads, 0, s>>>(x, n, pexp, dlen, part, nb, keys, find_brk, d_out);
  count_launch(2);
  e = cudaGetLastError();
  cudaFreeAsync(part, s);
  return e;
}

cudaError_t launch_encode_reduce_f64(const double *x, uint32_t n, uint32_t from, int32_t pexp,
                                     uint32_t dlen, int keys, int find_brk, EncStats *d_out,
                                     cudaStream_t s) {
  return reduce_impl<double>(x, n, from, pexp, dlen, keys, find_brk, d_out, s);
}
cudaError_t launch_encode_reduce_f32(const float *x, uint32_t n, uint32_t from, int32_t pexp,
                                     uint32_t dlen, int keys, int find_brk, EncStats *d_out,
                                     cudaStream_t s) {
  return reduce_impl<float>(x, n, from, pexp, dlen, keys, find_brk, d_out, s);
}

template <typename T, int K>
static cudaError_t scatter_k(const T *x, const buff_col *c, uint8_t *lead, uint32_t nlead,
                             cudaStream_t s) {
  const uint32_t planes = K + (c->r ? 1u : 0u);
  const size_t smem = (size_t)(kThreads / 32) * planes * kRowChunk;
  const void *fn = (const void *)k_encode_scatter<T, K>;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const uint32_t nchunks = (c->n + kRowChunk - 1) / kRowChunk;
  int grid = grid_for(fn, kThreads, smem, c->device);
  const int need = (int)((nchunks + (kThreads / 32) - 1) / (kThreads / 32));
  if (grid > need) grid = need;
  // a buff-slice column's last slice holds the low code bits left-aligned:
  // shifting by the unpadded width puts them at the top of that byte
  k_encode_scatter<T, K><<<grid, kThreads, smem, s>>>(x, c->n, c->precision_exp, c->dlen, c->base,
                                                      c->fixed_len - c->pad, c->r, c->slices,
                                                      c->stride, c->tail, lead, nlead);
  count_launch();
  return cudaGetLastError();
}

template <typename T>
static cudaError_t scatter_impl(const T *x, const buff_col *c, uint8_t *lead, uint32_t nlead,
                                cudaStream_t s) {
  if (c->n == 0 || (c->k == 0 && c->r == 0)) return cudaSuccess;
  switch (c->k) {
    case 0: return scatter_k<T, 0>(x, c, lead, nlead, s);
    case 1: return scatter_k<T, 1>(x, c, lead, nlead, s);
    case 2: return scatter_k<T, 2>(x, c, lead, nlead, s);
    case 3: return scatter_k<T, 3>(x, c, lead, nlead, s);
    case 4: return scatter_k<T, 4>(x, c, lead, nlead, s);
    case 5: return scatter_k<T, 5>(x, c, lead, nlead, s);
    case 6: return scatter_k<T, 6>(x, c, lead, nlead, s);
    case 7: return scatter_k<T, 7>(x, c, lead, nlead, s);
    case 8: return scatter_k<T, 8>(x, c, lead, nlead, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t launch_encode_scatter_f64(const double *x, const buff_col *c, cudaStream_t s,
                                      uint8_t *lead, uint32_t nlead) {
  return scatter_impl<double>(x, c, lead, nlead, s);
}
cudaError_t launch_encode_scatter_f32(const float *x, const buff_col *c, cudaStream_t s,
                                      uint8_t *lead, uint32_t nlead) {
  return scatter_impl<float>(x, c, lead, nlead, s);
}

cudaError_t launch_filter(const FilterArgs &a, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const bool th = a.tbyte[0] & 0x80u;
  void (*fn)(FilterArgs) = a.is_range ? (th ? k_filter<true, true> : k_filter<true, false>)
                                      : (th ? k_filter<false, true> : k_filter<false, false>);
  const uint32_t nsteps = ((a.n + 31) / 32 + 63) / 64;
  int grid = grid_for((const void *)fn, kThreads, 0, cur_device());
  const int need = (int)((nsteps + (kThreads / 32) - 1) / (kThreads / 32));
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  fn<<<grid, kThreads, 0, s>>>(a);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_fill_words(uint32_t *words, uint32_t n, uint32_t value,
                              unsigned long long *count, cudaStream_t s) {
  const uint32_t nw = (n + 31) / 32;
  int grid = (int)((nw + kThreads - 1) / kThreads);
  if (grid < 1) grid = 1;
  if (grid > 8 * num_sms(cur_device())) grid = 8 * num_sms(cur_device());
  k_fill_words<<<grid, kThreads, 0, s>>>(words, n, value, count);
  count_launch();
  return cudaGetLastError();
}

cudaError_t zero_u64(unsigned long long *p, uint32_t n, cudaStream_t s, unsigned long long *q,
                     uint32_t m) {
  if (!q) m = 0;
  const uint32_t big = n > m ? n : m;
  if (!big) return cudaSuccess;
  // issued from the host, one memset costs the caller less than a launch;
  // recorded into a graph, the kernel keeps the nodes on the SMs
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (!m && cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs == cudaStreamCaptureStatusNone)
    return cudaMemsetAsync(p, 0, sizeof(unsigned long long) * n, s);
  k_zero_u64<<<(big + 255) / 256, 256, 0, s>>>(p, n, q, m);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_sum(const buff_col *c, uint32_t k_used, uint32_t tail_bits,
                       unsigned long long *d_partials, cudaStream_t s) {
  if (c->n == 0) return cudaSuccess;
  int grid = grid_for((const void *)k_sum, kThreads, 0, c->device);
  const size_t nv = c->stride / 16;
  const int need = (int)((nv + kThreads - 1) / kThreads);
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  k_sum<<<grid, kThreads, 0, s>>>(c->slices, c->stride, k_used, c->tail, tail_bits,
                                  (unsigned long long)c->n * tail_bits, d_partials);
  count_launch();
  return cudaGetLastError();
}

template <bool TH, int KS>
cudaError_t launch_filter_sum_il(const FilterArgs &a, const buff_col *c,
                                 unsigned long long *d_partials, cudaStream_t s) {
  const void *fn = (const void *)k_filter_sum_il<TH, KS>;
  int grid = grid_for(fn, kThreads, 0, c->device);
  const size_t nblk = c->stride / 32;
  const int need = (int)((nblk + kThreads - 1) / kThreads);
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  // a programmatic dependent launch: the streaming starts while the zeroing
  // kernel before it runs; the kernel waits for it before adding to the
  // results (a plain launch when the stream's last operation is no kernel)
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(kThreads);
  cfg.stream = s;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  const cudaError_t e = cudaLaunchKernelEx(&cfg, k_filter_sum_il<TH, KS>, a, c->r,
                                           (unsigned long long)c->n * c->r, d_partials);
  count_launch();
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t launch_filter_sum(const FilterArgs &a, const buff_col *c,
                              unsigned long long *d_partials, cudaStream_t s) {
  if (c->n == 0) return cudaSuccess;
  const bool th = a.tbyte[0] & 0x80u;
  switch (c->k) {
    case 1: return th ? launch_filter_sum_il<true, 1>(a, c, d_partials, s)
                      : launch_filter_sum_il<false, 1>(a, c, d_partials, s);
    case 2: return th ? launch_filter_sum_il<true, 2>(a, c, d_partials, s)
                      : launch_filter_sum_il<false, 2>(a, c, d_partials, s);
    case 3: return th ? launch_filter_sum_il<true, 3>(a, c, d_partials, s)
                      : launch_filter_sum_il<false, 3>(a, c, d_partials, s);
    case 4: return th ? launch_filter_sum_il<true, 4>(a, c, d_partials, s)
                      : launch_filter_sum_il<false, 4>(a, c, d_partials, s);
    default: break;
  }
  const void *fn = th ? (const void *)k_filter_sum<true> : (const void *)k_filter_sum<false>;
  int grid = grid_for(fn, kThreads, 0, c->device);
  const size_t nv = c->stride / 16;
  const int need = (int)((nv + kThreads - 1) / kThreads);
  if (grid > need) grid = need;
  if (grid < 1) grid = 1;
  const unsigned long long tb = (unsigned long long)c->n * c->r;
  if (th)
    k_filter_sum<true><<<grid, kThreads, 0, s>>>(a, c->k, c->r, tb, d_partials);
  else
    k_filter_sum<false><<<grid, kThreads, 0, s>>>(a, c->k, c->r, tb, d_partials);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_max(const buff_col *c, unsigned long long *d_max, cudaStream_t s) {
  if (c->n == 0) return cudaSuccess;
  int grid = grid_for((const void *)k_max, kThreads, 0, c->device);
  const uint32_t nsteps = ((c->n + 31) / 32 + 63) / 64;
  const int need = (int)((nsteps + (kThreads / 32) - 1) / (kThreads / 32));
  if (grid > need) grid = need;
  k_max<<<grid, kThreads, 0, s>>>(c->slices, c->stride, c->k, c->tail, c->r, c->fixed_len, c->n,
                                  d_max);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_argmax(const buff_col *c, const unsigned long long *d_max, uint32_t *words,
                          unsigned long long *count, cudaStream_t s) {
  if (c->n == 0) return cudaSuccess;
  const uint32_t nw = (c->n + 31) / 32;
  int grid = (int)((nw + kThreads - 1) / kThreads);
  if (grid > 8 * num_sms(c->device)) grid = 8 * num_sms(c->device);
  k_argmax<<<grid, kThreads, 0, s>>>(c->slices, c->stride, c->k, c->tail, c->r, c->fixed_len,
                                     c->n, d_max, words, count);
  count_launch();
  return cudaGetLastError();
}

template <int KS>
static cudaError_t decode_ks(const buff_col *c, uint32_t ts, unsigned long long keep, double *out,
                             cudaStream_t s) {
  // the code is built in 32 bits (8 KS + ts <= 32) and every value base +
  // (code >> pad) fits in 32 bits
  const uint32_t bits = 8 * KS + ts;
  const long long maxc = bits >= 63 ? -1 : (long long)(((1ull << bits) - 1ull) >> c->pad);
  const bool n32 = bits <= 32 && c->base >= INT32_MIN && maxc >= 0 &&
                   c->base + maxc <= (long long)INT32_MAX;
  const uint32_t nchunks = (c->n + kRowChunk - 1) / kRowChunk;
  const int need = (int)((nchunks + (kThreads / 32) - 1) / (kThreads / 32));
  if (KS >= 1 && KS <= 3 && ts > 0 && bits <= 32 &&
      (reinterpret_cast<uintptr_t>(out) & 31u) == 0) {
    constexpr int K4 = KS >= 1 && KS <= 3 ? KS : 1;
    void (*f4)(const uint8_t *, size_t, const uint8_t *, uint32_t, uint32_t, long long, int,
               unsigned long long, uint32_t, double *) =
        n32 ? k_decode4<K4, true> : k_decode4<K4, false>;
    int grid = grid_for((const void *)f4, kThreads, 0, c->device);
    if (grid > need) grid = need;
    f4<<<grid, kThreads, 0, s>>>(c->slices, c->stride, c->tail, ts, c->n, c->base, (int)c->dlen,
                                 keep, c->pad, out);
    count_launch();
    return cudaGetLastError();
  }
  const void *fn = n32 ? (const void *)k_decode<KS, true> : (const void *)k_decode<KS, false>;
  int grid = grid_for(fn, kThreads, 0, c->device);
  if (grid > need) grid = need;
  if (n32)
    k_decode<KS, true><<<grid, kThreads, 0, s>>>(c->slices, c->stride, c->tail, ts, c->n, c->base,
                                                 (int)c->dlen, keep, c->pad, out);
  else
    k_decode<KS, false><<<grid, kThreads, 0, s>>>(c->slices, c->stride, c->tail, ts, c->n,
                                                  c->base, (int)c->dlen, keep, c->pad, out);
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_decode(const buff_col *c, uint32_t total, int intended_mask, double *out,
                          cudaStream_t s) {
  if (c->n == 0) return cudaSuccess;
  uint32_t ks, ts;
  unsigned long long keep = ~0ull;
  if (intended_mask) {
    ks = c->k;
    ts = c->r;
    const uint32_t drop = c->fixed_len - total;
    keep = drop >= 64 ? 0ull : (~0ull << drop);
  } else if (total < 8) {
    ks = 0;
    ts = total;  // packed reads straight after the header
  } else {
    ks = total / 8;
    ts = total % 8;
  }
  switch (ks) {
    case 0: return decode_ks<0>(c, ts, keep, out, s);
    case 1: return decode_ks<1>(c, ts, keep, out, s);
    case 2: return decode_ks<2>(c, ts, keep, out, s);
    case 3: return decode_ks<3>(c, ts, keep, out, s);
    case 4: return decode_ks<4>(c, ts, keep, out, s);
    case 5: return decode_ks<5>(c, ts, keep, out, s);
    case 6: return decode_ks<6>(c, ts, keep, out, s);
    case 7: return decode_ks<7>(c, ts, keep, out, s);
    case 8: return decode_ks<8>(c, ts, keep, out, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace buffk
