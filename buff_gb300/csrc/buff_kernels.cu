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

#include "buff_internal.h"

namespace buffk {

namespace {

std::atomic<uint64_t> g_launches{0};

constexpr uint32_t H = 0x80808080u;
constexpr int kThreads = 256;
constexpr int kU = 4;  // independent 16-byte loads a lane keeps in flight in streaming loops

__device__ __forceinline__ long long fetch_fixed(double v, int pexp, uint32_t dlen) {
  // PrecisionBound::fetch_fixed_aligned (methods/prec_double.rs:190-205):
  // IEEE bit manipulation; the shift amount wraps mod 64 like the reference's
  // release build.
  unsigned long long bdu = (unsigned long long)__double_as_longlong(v);
  int exp = (int)((bdu >> 52) & 0x7FFu) - 1023;
  if (exp < pexp) return 0;
  int sh = 63 - exp - (int)dlen;
  unsigned long long f = ((bdu << 11) | 0x8000000000000000ull) >> (sh & 63);
  if (bdu >> 63) f = ~(f - 1ull);
  return (long long)f;
}

__device__ __forceinline__ uint4 ld_stream(const uint8_t *p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

__device__ __forceinline__ uint4 ld_cand(const uint8_t *p) {
  return __ldg(reinterpret_cast<const uint4 *>(p));
}

// Per-slice compare constants for an unflipped target byte t.
struct ByteTarget {
  uint32_t lo1;  // (t & 0x7f) + 1 in every byte
  uint32_t lo0;  // (t & 0x7f) in every byte
  uint32_t th;   // all ones when t >= 0x80
};

__host__ __device__ __forceinline__ ByteTarget make_target(uint32_t t) {
  ByteTarget b;
  b.lo0 = (t & 0x7Fu) * 0x01010101u;
  b.lo1 = ((t & 0x7Fu) + 1u) * 0x01010101u;
  b.th = (t & 0x80u) ? 0xFFFFFFFFu : 0u;
  return b;
}

// SWAR compare of 4 flipped bytes w (a = w ^ 0x80 unflipped) against t.
// MSB of each byte of *gt is a > t, of *eq is a == t.  No borrow crosses a
// byte: (w|H) - lo1 and (w|H) - lo0 stay within [0, 255] per byte.
__device__ __forceinline__ void cmp4(uint32_t w, const ByteTarget &t, uint32_t &gt,
                                     uint32_t &eq) {
  uint32_t wh = w | H;
  uint32_t d1 = wh - t.lo1;  // MSB: a_lo > t_lo
  uint32_t d0 = wh - t.lo0;  // MSB: a_lo >= t_lo
  // a_hi = ~w_hi.  t_hi = 1: a > t iff a_hi & (a_lo > t_lo); t_hi = 0: a_hi | (a_lo > t_lo).
  gt = ((t.th & ~w & d1) | (~t.th & (~w | d1))) & H;
  eq = d0 & ~d1 & (w ^ t.th) & H;  // a_hi == t_hi  <=>  w_hi != t_hi
}

// Replaces the bytes of rows >= lim (0..16) in a 16-row vector by the flipped
// zero byte 0x80, so padding rows add nothing to sums or maxima.
__device__ __forceinline__ void clear_padding(uint4 &d, uint32_t lim) {
  uint32_t *w = reinterpret_cast<uint32_t *>(&d);
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint32_t lo = 4u * q;
    const uint32_t keep = lim >= lo + 4 ? 0xFFFFFFFFu : (lim <= lo ? 0u : ((1u << (8 * (lim - lo))) - 1u));
    w[q] = (w[q] & keep) | (H & ~keep);
  }
}

__device__ __forceinline__ uint32_t msb4(uint32_t m) {  // MSBs of 4 bytes -> 4 bits
  return (m * 0x00204081u) >> 28;
}

__device__ __forceinline__ void cmp16(const uint4 &d, const ByteTarget &t, uint32_t &gt,
                                      uint32_t &eq) {
  uint32_t g0, e0, g1, e1, g2, e2, g3, e3;
  cmp4(d.x, t, g0, e0);
  cmp4(d.y, t, g1, e1);
  cmp4(d.z, t, g2, e2);
  cmp4(d.w, t, g3, e3);
  gt = msb4(g0) | (msb4(g1) << 4) | (msb4(g2) << 8) | (msb4(g3) << 12);
  eq = msb4(e0) | (msb4(e1) << 4) | (msb4(e2) << 8) | (msb4(e3) << 12);
}

// The 16 r-bit tail fields of rows [16v, 16v+16): 2r bytes at byte 2r*v.
__device__ __forceinline__ void load_tail16(const uint8_t *tail, uint32_t v, uint32_t r,
                                            unsigned long long &lo, unsigned long long &hi) {
  const uint16_t *p = reinterpret_cast<const uint16_t *>(tail + (size_t)2 * r * v);
  lo = 0;
  hi = 0;
#pragma unroll
  for (uint32_t i = 0; i < 7; ++i) {
    if (i < r) {
      unsigned long long h = __ldg(p + i);
      if (i < 4)
        lo |= h << (16 * i);
      else
        hi |= h << (16 * (i - 4));
    }
  }
}

__device__ __forceinline__ uint32_t field16(unsigned long long lo, unsigned long long hi,
                                            uint32_t i, uint32_t r) {
  uint32_t p = i * r;
  unsigned long long v;
  if (p >= 64)
    v = hi >> (p - 64);
  else if (p + r > 64)
    v = (lo >> p) | (hi << (64 - p));
  else
    v = lo >> p;
  return (uint32_t)v & ((1u << r) - 1u);
}

template <typename T>
__device__ __forceinline__ long long warp_min(long long v) {
  for (int o = 16; o; o >>= 1) {
    long long x = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = x < v ? x : v;
  }
  return v;
}
__device__ __forceinline__ long long warp_max_ll(long long v) {
  for (int o = 16; o; o >>= 1) {
    long long x = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = x > v ? x : v;
  }
  return v;
}
__device__ __forceinline__ unsigned long long warp_max_ull(unsigned long long v) {
  for (int o = 16; o; o >>= 1) {
    unsigned long long x = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = x > v ? x : v;
  }
  return v;
}
__device__ __forceinline__ unsigned long long warp_min_ull(unsigned long long v) {
  for (int o = 16; o; o >>= 1) {
    unsigned long long x = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = x < v ? x : v;
  }
  return v;
}
__device__ __forceinline__ unsigned long long warp_sum_ull(unsigned long long v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  return v;
}

// ---------------------------------------------------------------- encode

template <typename T>
struct VecOf;
template <>
struct VecOf<double> {
  using V = double2;
  static constexpr int E = 2;
  __device__ static void get(const V &v, double *o) {
    o[0] = v.x;
    o[1] = v.y;
  }
};
template <>
struct VecOf<float> {
  using V = float4;
  static constexpr int E = 4;
  __device__ static void get(const V &v, double *o) {
    o[0] = v.x;
    o[1] = v.y;
    o[2] = v.z;
    o[3] = v.w;
  }
};

// Pass 1 of buff_simd256_encode (compress/buff_simd.rs:3139-3148): min over all
// rows, max over rows >= from, max over all rows, and the first row i >= 1
// with x_i >= x_{i-1}.  The reference's `else if` makes its max equal to the
// max over rows after the leading strictly decreasing run (each row of that
// run is a new minimum; afterwards every new minimum is below the running
// max), so the host finishes the reference max from these fields.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_encode_reduce(const T *__restrict__ x, uint32_t n,
                                                            uint32_t from, int pexp,
                                                            uint32_t dlen, EncStats *part) {
  using VO = VecOf<T>;
  constexpr int E = VO::E;
  long long mn = LLONG_MAX, mx1 = LLONG_MIN, mx0 = LLONG_MIN;
  unsigned long long brk = n;
  const uint32_t nv = n / E;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nth = gridDim.x * blockDim.x;
  const typename VO::V *xv = reinterpret_cast<const typename VO::V *>(x);
  for (uint32_t v0 = tid; v0 < nv; v0 += kU * nth) {
    typename VO::V raw[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t v = v0 + u * nth;
      if (v < nv) raw[u] = __ldcs(xv + v);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t v = v0 + u * nth;
      if (v >= nv) break;
      double e[E];
      VO::get(raw[u], e);
      const uint32_t i0 = v * E;
      long long prev = 0;
      if (i0 > 0) prev = fetch_fixed((double)__ldg(x + i0 - 1), pexp, dlen);
#pragma unroll
      for (int j = 0; j < E; ++j) {
        const long long q = fetch_fixed(e[j], pexp, dlen);
        const uint32_t i = i0 + j;
        mn = q < mn ? q : mn;
        mx0 = q > mx0 ? q : mx0;
        if (i >= from) mx1 = q > mx1 ? q : mx1;
        if (i > 0 && q >= prev && (unsigned long long)i < brk) brk = i;
        prev = q;
      }
    }
  }
  for (uint32_t i = nv * E + tid; i < n; i += nth) {  // ragged end
    long long q = fetch_fixed((double)x[i], pexp, dlen);
    mn = q < mn ? q : mn;
    mx0 = q > mx0 ? q : mx0;
    if (i >= from) mx1 = q > mx1 ? q : mx1;
    if (i > 0) {
      long long p = fetch_fixed((double)x[i - 1], pexp, dlen);
      if (q >= p && (unsigned long long)i < brk) brk = i;
    }
  }
  __shared__ long long s_mn[kThreads / 32], s_mx1[kThreads / 32], s_mx0[kThreads / 32];
  __shared__ unsigned long long s_brk[kThreads / 32];
  mn = warp_min<long long>(mn);
  mx1 = warp_max_ll(mx1);
  mx0 = warp_max_ll(mx0);
  brk = warp_min_ull(brk);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    s_mn[w] = mn;
    s_mx1[w] = mx1;
    s_mx0[w] = mx0;
    s_brk[w] = brk;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < kThreads / 32; ++i) {
      mn = s_mn[i] < mn ? s_mn[i] : mn;
      mx1 = s_mx1[i] > mx1 ? s_mx1[i] : mx1;
      mx0 = s_mx0[i] > mx0 ? s_mx0[i] : mx0;
      brk = s_brk[i] < brk ? s_brk[i] : brk;
    }
    EncStats s;
    s.mn = mn;
    s.mx1 = mx1;
    s.mx0 = mx0;
    s.brk = brk;
    s.x0 = 0;
    s.x1 = 0;
    part[blockIdx.x] = s;
  }
}

template <typename T>
__global__ void k_encode_finalize(const T *__restrict__ x, uint32_t n, int pexp, uint32_t dlen,
                                  const EncStats *part, int nparts, EncStats *out) {
  long long mn = LLONG_MAX, mx1 = LLONG_MIN, mx0 = LLONG_MIN;
  unsigned long long brk = n;
  for (int i = threadIdx.x; i < nparts; i += 32) {
    EncStats s = part[i];
    mn = s.mn < mn ? s.mn : mn;
    mx1 = s.mx1 > mx1 ? s.mx1 : mx1;
    mx0 = s.mx0 > mx0 ? s.mx0 : mx0;
    brk = s.brk < brk ? s.brk : brk;
  }
  mn = warp_min<long long>(mn);
  mx1 = warp_max_ll(mx1);
  mx0 = warp_max_ll(mx0);
  brk = warp_min_ull(brk);
  if (threadIdx.x == 0) {
    EncStats s;
    s.mn = mn;
    s.mx1 = mx1;
    s.mx0 = mx0;
    s.brk = brk;
    s.x0 = n > 0 ? fetch_fixed((double)x[0], pexp, dlen) : 0;
    s.x1 = n > 1 ? fetch_fixed((double)x[1], pexp, dlen) : 0;
    *out = s;
  }
}

// Pass 2 of buff_simd256_encode (compress/buff_simd.rs:3181-3232): quantize,
// split each code MSB-first into k flipped bytes and an r-bit tail.  Lane L
// loads its part of the warp's 512 rows coalesced, the bytes are transposed
// through shared memory so that every lane stores one 16-byte vector per
// slice, and the tail of 16 rows is packed into 2r bytes.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_encode_scatter(
    const T *__restrict__ x, uint32_t n, int pexp, uint32_t dlen, long long base, uint32_t fl,
    uint32_t k, uint32_t r, uint8_t *__restrict__ slices, size_t stride,
    uint8_t *__restrict__ tail) {
  using VO = VecOf<T>;
  constexpr int E = VO::E;
  constexpr int LOADS = 16 / E;
  extern __shared__ uint8_t smem[];
  const uint32_t planes = k + (r ? 1u : 0u);
  const uint32_t lane = threadIdx.x & 31;
  uint8_t *ws = smem + (size_t)(threadIdx.x >> 5) * planes * kRowChunk;
  const uint32_t nchunks = (n + kRowChunk - 1) / kRowChunk;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const unsigned long long rmask = r ? ((1ull << r) - 1ull) : 0ull;
  for (uint32_t ch = warp; ch < nchunks; ch += nwarps) {
    const uint32_t r0 = ch * kRowChunk;
#pragma unroll
    for (int m = 0; m < LOADS; ++m) {
      const uint32_t off = m * 32 * E + lane * E;  // row offset within the chunk
      const uint32_t i0 = r0 + off;
      double e[E];
      if (i0 + E <= n && (i0 % E) == 0) {
        VO::get(__ldcs(reinterpret_cast<const typename VO::V *>(x + i0)), e);
      } else {
#pragma unroll
        for (int j = 0; j < E; ++j) e[j] = (i0 + j < n) ? (double)x[i0 + j] : 0.0;
      }
      unsigned long long c[E];
#pragma unroll
      for (int j = 0; j < E; ++j)
        c[j] = (i0 + j < n) ? (unsigned long long)(fetch_fixed(e[j], pexp, dlen) - base) : 0ull;
      for (uint32_t s = 0; s < k; ++s) {
        const uint32_t sh = fl - 8u * (s + 1u);
        uint32_t packed = 0;
#pragma unroll
        for (int j = 0; j < E; ++j) packed |= (uint32_t)(((uint8_t)(c[j] >> sh)) ^ 0x80u) << (8 * j);
        if (E == 2)
          *reinterpret_cast<uint16_t *>(ws + s * kRowChunk + off) = (uint16_t)packed;
        else
          *reinterpret_cast<uint32_t *>(ws + s * kRowChunk + off) = packed;
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
    for (uint32_t s = 0; s < k; ++s) {
      uint4 v = *reinterpret_cast<const uint4 *>(ws + s * kRowChunk + lane * 16);
      __stcs(reinterpret_cast<uint4 *>(slices + s * stride + r0 + lane * 16), v);
    }
    if (r) {
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
// Candidate refinement of one 16-row vector (rows whose prefix equals the
// target so far): the remaining slices, then the packed tail.  Kept out of
// line: it runs for few vectors and would otherwise inflate the streaming
// loop's registers.
__device__ __noinline__ void refine_candidates(const uint8_t *__restrict__ slices, size_t stride,
                                               uint32_t k_used, unsigned long long tb,
                                               const uint8_t *__restrict__ tail, uint32_t r,
                                               uint32_t ttail, uint32_t row0, uint32_t &gt,
                                               uint32_t &eq) {
  for (uint32_t j = 1; j < k_used && eq; ++j) {
    uint32_t gj, ej;
    cmp16(ld_cand(slices + j * stride + row0), make_target((uint32_t)(tb >> (8 * j)) & 0xFFu), gj,
          ej);
    gt |= eq & gj;
    eq &= ej;
  }
  if (r && eq) {
    unsigned long long lo, hi;
    load_tail16(tail, row0 >> 4, r, lo, hi);
    uint32_t gtt = 0, eqt = 0;
    for (uint32_t i = 0; i < 16; ++i) {
      const uint32_t f = field16(lo, hi, i, r);
      gtt |= (uint32_t)(f > ttail) << i;
      eqt |= (uint32_t)(f == ttail) << i;
    }
    gt |= eq & gtt;
    eq &= eqt;
  }
}

template <bool IS_RANGE>
__global__ void __launch_bounds__(kThreads) k_filter(FilterArgs a) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nwords = (a.n + 31) / 32;
  const uint32_t step_rows = kU * kRowChunk;
  const uint32_t nsteps = (a.n + step_rows - 1) / step_rows;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long tb = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j) tb |= (unsigned long long)a.tbyte[j] << (8 * j);
  const ByteTarget tg0 = make_target((uint32_t)(tb & 0xFFu));
  unsigned long long cnt = 0;
  for (uint32_t st = warp; st < nsteps; st += nwarps) {
    const uint32_t base = st * step_rows;
    uint4 d[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t row0 = base + u * kRowChunk + lane * 16;
      if (a.k_used && row0 < a.n)
        d[u] = ld_stream(a.slices + row0);
      else
        d[u] = make_uint4(0, 0, 0, 0);
    }
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t row0 = base + u * kRowChunk + lane * 16;
      uint32_t res = 0;
      if (row0 < a.n) {
        uint32_t gt = 0, eq;
        if (a.k_used) {
          uint32_t g0 = 0, e0, g1 = 0, e1, g2 = 0, e2, g3 = 0, e3;
          cmp4(d[u].x, tg0, g0, e0);
          cmp4(d[u].y, tg0, g1, e1);
          cmp4(d[u].z, tg0, g2, e2);
          cmp4(d[u].w, tg0, g3, e3);
          if (IS_RANGE) gt = msb4(g0) | (msb4(g1) << 4) | (msb4(g2) << 8) | (msb4(g3) << 12);
          eq = (e0 | e1 | e2 | e3) ? (msb4(e0) | (msb4(e1) << 4) | (msb4(e2) << 8) | (msb4(e3) << 12)) : 0u;
        } else {
          eq = 0xFFFFu;
        }
        if (eq && (a.k_used > 1 || a.r)) {
          refine_candidates(a.slices, a.stride, a.k_used, tb, a.tail, a.r, a.ttail, row0, gt, eq);
        } else if (a.tail_only_eq && !a.r) {
          eq = 0;
        }
        res = IS_RANGE ? gt : eq;
        const uint32_t lim = a.full_rows > row0 ? a.full_rows - row0 : 0u;
        if (lim < 16) res &= (1u << lim) - 1u;
      }
      const uint32_t hi16 = __shfl_down_sync(0xFFFFFFFFu, res, 1);
      if (!(lane & 1)) {
        const uint32_t word = (base + u * kRowChunk) / 32 + (lane >> 1);
        if (word < nwords) {
          const uint32_t wv = (res & 0xFFFFu) | (hi16 << 16);
          __stcs(a.words + word, wv);
          cnt += __popc(wv);
        }
      }
    }
  }
  if (a.count) {
    cnt = warp_sum_ull(cnt);
    if (lane == 0 && cnt) atomicAdd(a.count, cnt);
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

// ---------------------------------------------------------------- sum

// Weighted popcount of one 32-bit word of a packed stream of `ts`-bit fields
// whose first bit sits at stream bit `bit0`: sum over set bits b of
// 2^((bit0 + b) mod ts).  (The sum of all fields of a stream only depends on
// each bit's position mod ts, not on row boundaries.)
__device__ __forceinline__ uint32_t wpopc(uint32_t w, uint32_t bit0, uint32_t ts) {
  if (ts == 1) return __popc(w);
  uint32_t pat = 0;  // bits 0, ts, 2ts, ...
  for (uint32_t j = 0; j < 32; j += ts) pat |= 1u << j;
  const uint32_t phase = bit0 % ts;
  uint32_t acc = 0;
  for (uint32_t p = 0; p < ts; ++p) {
    const uint32_t sh = (p + ts - phase) % ts;  // bits j with (phase + j) % ts == p
    acc += (uint32_t)__popc(w & (pat << sh)) << p;
  }
  return acc;
}

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
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nth = gridDim.x * blockDim.x;
  const uint32_t nv = (uint32_t)(stride / 16);
  for (uint32_t s = 0; s < ks; ++s) {
    const uint8_t *sl = slices + (size_t)s * stride;
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
    for (uint32_t v = tid; v < ntv; v += nth) {
      uint4 d = *reinterpret_cast<const uint4 *>(tail + (size_t)v * 16);
      const uint32_t *w = reinterpret_cast<const uint32_t *>(&d);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const unsigned long long b0 = (unsigned long long)v * 128 + 32 * q;
        uint32_t word = w[q];
        if (b0 >= tail_bits)
          word = 0;
        else if (b0 + 32 > tail_bits)
          word &= (1u << (uint32_t)(tail_bits - b0)) - 1u;
        acc += wpopc(word, (uint32_t)(b0 % ts), ts);
      }
    }
    acc = warp_sum_ull(acc);
    if (lane == 0 && acc) atomicAdd(&s_acc[8], acc);
  }
  __syncthreads();
  if (threadIdx.x < ks && s_acc[threadIdx.x]) atomicAdd(&partials[threadIdx.x], s_acc[threadIdx.x]);
  if (threadIdx.x == 8 && ts && s_acc[8]) atomicAdd(&partials[ks], s_acc[8]);
}

// ---------------------------------------------------------------- max

__device__ __forceinline__ uint32_t max_byte16(const uint4 &d) {
  uint32_t m = __vmaxu4(__vmaxu4(d.x ^ H, d.y ^ H), __vmaxu4(d.z ^ H, d.w ^ H));
  m = __vmaxu4(m, m >> 16);
  m = __vmaxu4(m, m >> 8);
  return m & 0xFFu;
}

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

// Largest full code among the rows of one 16-row vector whose leading byte is
// `top` (out of line for the same reason as refine_candidates).
__device__ __noinline__ unsigned long long max_in_vector(const uint8_t *__restrict__ slices,
                                                         size_t stride, uint32_t k,
                                                         const uint8_t *__restrict__ tail,
                                                         uint32_t r, uint32_t n, uint32_t row0,
                                                         uint4 d, uint32_t top) {
  const uint8_t *db = reinterpret_cast<const uint8_t *>(&d);
  unsigned long long m = 0;
  for (uint32_t i = 0; i < 16 && row0 + i < n; ++i)
    if ((uint32_t)(db[i] ^ 0x80u) == top) {
      const unsigned long long c = code_at(slices, stride, k, tail, r, row0 + i);
      m = c > m ? c : m;
    }
  return m;
}

// byte_fixed_max (compress/split_double.rs:3919-4105): the maximum stored
// code.  Each warp keeps the best code it has seen; only lanes holding the
// warp's largest leading byte, when that byte can still reach the warp's
// best, gather the remaining slices and the tail.
__global__ void __launch_bounds__(kThreads) k_max(const uint8_t *__restrict__ slices, size_t stride,
                                                  uint32_t k, const uint8_t *__restrict__ tail,
                                                  uint32_t r, uint32_t fl, uint32_t n,
                                                  unsigned long long *out) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long best = 0;
  bool have = false;
  if (k == 0) {  // packed codes only (fixed_len < 8)
    const uint32_t nvec = (n + 15) / 16;
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
  const uint32_t step_rows = kU * kRowChunk;
  const uint32_t nsteps = (n + step_rows - 1) / step_rows;
  for (uint32_t st = warp; st < nsteps; st += nwarps) {
    const uint32_t base = st * step_rows;
    uint4 d[kU];
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t row0 = base + u * kRowChunk + lane * 16;
      if (row0 < n) {
        d[u] = ld_stream(slices + row0);
        if (n - row0 < 16) clear_padding(d[u], n - row0);
      } else {
        d[u] = make_uint4(H, H, H, H);
      }
    }
    uint32_t mb[kU];
    uint32_t lm = 0;
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      mb[u] = max_byte16(d[u]);
      lm = mb[u] > lm ? mb[u] : lm;
    }
    const uint32_t wmb = __reduce_max_sync(0xFFFFFFFFu, lm);
    const uint32_t best_top = have ? (uint32_t)(best >> (fl - 8)) : 0u;
    if (have && wmb < best_top) continue;
    unsigned long long m = 0;
#pragma unroll
    for (int u = 0; u < kU; ++u) {
      const uint32_t row0 = base + u * kRowChunk + lane * 16;
      if (row0 < n && mb[u] == wmb) {
        const unsigned long long c = max_in_vector(slices, stride, k, tail, r, n, row0, d[u], wmb);
        m = c > m ? c : m;
      }
    }
    m = warp_max_ull(m);
    if (!have || m > best) best = m;
    have = true;
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
template <int KS>
__global__ void __launch_bounds__(kThreads) k_decode(const uint8_t *__restrict__ slices,
                                                     size_t stride,
                                                     const uint8_t *__restrict__ tail, uint32_t r,
                                                     uint32_t ts, uint32_t n, long long base,
                                                     double scl, unsigned long long keep,
                                                     double *__restrict__ out) {
  extern __shared__ double dsm[];
  const uint32_t lane = threadIdx.x & 31;
  double *ws = dsm + (size_t)(threadIdx.x >> 5) * kRowChunk;
  const uint32_t nchunks = (n + kRowChunk - 1) / kRowChunk;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t ch = warp; ch < nchunks; ch += nwarps) {
    const uint32_t row0 = ch * kRowChunk + lane * 16;
    unsigned long long c[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) c[i] = 0;
    if (row0 < n) {
      uint4 d[KS > 0 ? KS : 1];
#pragma unroll
      for (int s = 0; s < KS; ++s) d[s] = ld_stream(slices + s * stride + row0);
      unsigned long long lo = 0, hi = 0;
      if (ts && ts == r) load_tail16(tail, row0 >> 4, r, lo, hi);
#pragma unroll
      for (int s = 0; s < KS; ++s) {
        const uint32_t *w = reinterpret_cast<const uint32_t *>(&d[s]);
#pragma unroll
        for (int i = 0; i < 16; ++i)
          c[i] = (c[i] << 8) | (((w[i >> 2] >> (8 * (i & 3))) & 0xFFu) ^ 0x80u);
      }
      if (ts) {
        if (ts == r) {
#pragma unroll
          for (int i = 0; i < 16; ++i) c[i] = (c[i] << r) | field16(lo, hi, i, r);
        } else {  // the reference's stride-ts reads of the packed region
          for (int i = 0; i < 16; ++i) {
            const unsigned long long bit = (unsigned long long)(row0 + i) * ts;
            const uint32_t b0 = __ldg(tail + (bit >> 3));
            const uint32_t b1 = ((bit & 7) + ts > 8) ? __ldg(tail + (bit >> 3) + 1) : 0u;
            c[i] = (c[i] << ts) | (((b0 | (b1 << 8)) >> (bit & 7)) & ((1u << ts) - 1u));
          }
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const unsigned long long x = c[i] & keep;
      ws[lane * 16 + i] = (double)((long long)((unsigned long long)base + x)) * scl;
    }
    __syncwarp();
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const uint32_t off = m * 64 + lane * 2;
      const uint32_t i0 = ch * kRowChunk + off;
      double2 p = *reinterpret_cast<const double2 *>(ws + off);
      if (i0 + 2 <= n)
        __stcs(reinterpret_cast<double2 *>(out + i0), p);
      else if (i0 < n)
        out[i0] = p.x;
    }
    __syncwarp();
  }
}

int grid_for(const void *fn, int threads, size_t smem, int device) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem);
  if (per_sm < 1) per_sm = 1;
  return per_sm * num_sms(device);
}

int cur_device() {
  int d = 0;
  cudaGetDevice(&d);
  return d;
}

}  // namespace

int num_sms(int device) {
  static int cached[64] = {0};
  if (device < 0 || device >= 64) return 1;
  if (!cached[device]) {
    int v = 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
    cached[device] = v > 0 ? v : 1;
  }
  return cached[device];
}

void count_launch(uint64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
uint64_t launches() { return g_launches.load(std::memory_order_relaxed); }

template <typename T>
static cudaError_t encode_reduce_impl(const T *x, uint32_t n, uint32_t from, int32_t pexp,
                                      uint32_t dlen, EncStats *d_part, int nblocks,
                                      EncStats *d_out, cudaStream_t s) {
  k_encode_reduce<T><<<nblocks, kThreads, 0, s>>>(x, n, from, pexp, dlen, d_part);
  k_encode_finalize<T><<<1, 32, 0, s>>>(x, n, pexp, dlen, d_part, nblocks, d_out);
  count_launch(2);
  return cudaGetLastError();
}

cudaError_t launch_encode_reduce_f64(const double *x, uint32_t n, int32_t pexp, uint32_t dlen,
                                     EncStats *d_part, int nblocks, EncStats *d_out,
                                     cudaStream_t s) {
  return encode_reduce_impl<double>(x, n, 1, pexp, dlen, d_part, nblocks, d_out, s);
}
cudaError_t launch_encode_reduce_f32(const float *x, uint32_t n, int32_t pexp, uint32_t dlen,
                                     EncStats *d_part, int nblocks, EncStats *d_out,
                                     cudaStream_t s) {
  return encode_reduce_impl<float>(x, n, 1, pexp, dlen, d_part, nblocks, d_out, s);
}

int encode_reduce_blocks() { return 4 * num_sms(cur_device()); }

template <typename T>
static cudaError_t suffix_max_impl(const T *x, uint32_t n, uint32_t from, int32_t pexp,
                                   uint32_t dlen, long long *d_out, cudaStream_t s) {
  // Reuses the reduce with `from`: mx1 of the result is max over rows >= from.
  const int nb = 4 * num_sms(cur_device());
  EncStats *tmp = nullptr;
  cudaError_t e = cudaMallocAsync(&tmp, sizeof(EncStats) * (nb + 1), s);
  if (e != cudaSuccess) return e;
  k_encode_reduce<T><<<nb, kThreads, 0, s>>>(x, n, from, pexp, dlen, tmp);
  k_encode_finalize<T><<<1, 32, 0, s>>>(x, n, pexp, dlen, tmp, nb, tmp + nb);
  count_launch(2);
  e = cudaMemcpyAsync(d_out, &tmp[nb].mx1, sizeof(long long), cudaMemcpyDeviceToDevice, s);
  cudaFreeAsync(tmp, s);
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}
cudaError_t launch_suffix_max_f64(const double *x, uint32_t n, uint32_t from, int32_t pexp,
                                  uint32_t dlen, long long *d_out, cudaStream_t s) {
  return suffix_max_impl<double>(x, n, from, pexp, dlen, d_out, s);
}
cudaError_t launch_suffix_max_f32(const float *x, uint32_t n, uint32_t from, int32_t pexp,
                                  uint32_t dlen, long long *d_out, cudaStream_t s) {
  return suffix_max_impl<float>(x, n, from, pexp, dlen, d_out, s);
}

template <typename T>
static cudaError_t scatter_impl(const T *x, const buff_col *c, cudaStream_t s) {
  if (c->n == 0 || (c->k == 0 && c->r == 0)) return cudaSuccess;
  const uint32_t planes = c->k + (c->r ? 1u : 0u);
  const size_t smem = (size_t)(kThreads / 32) * planes * kRowChunk;
  const void *fn = (const void *)k_encode_scatter<T>;
  if (smem > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const uint32_t nchunks = (c->n + kRowChunk - 1) / kRowChunk;
  int grid = grid_for(fn, kThreads, smem, c->device);
  const int need = (int)((nchunks + (kThreads / 32) - 1) / (kThreads / 32));
  if (grid > need) grid = need;
  k_encode_scatter<T><<<grid, kThreads, smem, s>>>(x, c->n, c->precision_exp, c->dlen, c->base,
                                                   c->fixed_len, c->k, c->r, c->slices, c->stride,
                                                   c->tail);
  count_launch();
  return cudaGetLastError();
}
cudaError_t launch_encode_scatter_f64(const double *x, const buff_col *c, cudaStream_t s) {
  return scatter_impl<double>(x, c, s);
}
cudaError_t launch_encode_scatter_f32(const float *x, const buff_col *c, cudaStream_t s) {
  return scatter_impl<float>(x, c, s);
}

cudaError_t launch_filter(const FilterArgs &a, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const void *fn = a.is_range ? (const void *)k_filter<true> : (const void *)k_filter<false>;
  const uint32_t nsteps = (a.n + kU * kRowChunk - 1) / (kU * kRowChunk);
  int grid = grid_for(fn, kThreads, 0, cur_device());
  const int need = (int)((nsteps + (kThreads / 32) - 1) / (kThreads / 32));
  if (grid > need) grid = need;
  if (a.is_range)
    k_filter<true><<<grid, kThreads, 0, s>>>(a);
  else
    k_filter<false><<<grid, kThreads, 0, s>>>(a);
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

cudaError_t launch_max(const buff_col *c, unsigned long long *d_max, cudaStream_t s) {
  if (c->n == 0) return cudaSuccess;
  int grid = grid_for((const void *)k_max, kThreads, 0, c->device);
  const uint32_t nsteps = (c->n + kU * kRowChunk - 1) / (kU * kRowChunk);
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
  const size_t smem = (size_t)(kThreads / 32) * kRowChunk * sizeof(double);
  const void *fn = (const void *)k_decode<KS>;
  int grid = grid_for(fn, kThreads, smem, c->device);
  const uint32_t nchunks = (c->n + kRowChunk - 1) / kRowChunk;
  const int need = (int)((nchunks + (kThreads / 32) - 1) / (kThreads / 32));
  if (grid > need) grid = need;
  // 2^-dlen is exact; (base + X) * 2^-dlen equals the reference's division.
  double inv = 1.0;
  for (uint32_t i = 0; i < c->dlen; ++i) inv *= 0.5;
  k_decode<KS><<<grid, kThreads, smem, s>>>(c->slices, c->stride, c->tail, c->r, ts, c->n, c->base,
                                            inv, keep, out);
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
