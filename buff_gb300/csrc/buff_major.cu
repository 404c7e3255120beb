// The buff-major (outlier) layout on the GPU: encode, serialize/deserialize,
// filters, sum, max and decode (compress/buff_simd.rs:317-2861).
//
// Device form of a buff-major column: per sparse column c a major byte, the
// outlier-row bitmap (BitVec<u32> words), the number of outliers before every
// word (exclusive prefix) and the outlier bytes in row order; the dense
// slices are kept flipped like buff-simd slices so the shared compare code
// applies; the tail is the same packed r-bit stream.  Queries read one bitmap
// word per 32 rows for each sparse column (n/8 bytes instead of n), look up
// outlier bytes by rank, and touch dense slices only for 32-row blocks that
// still hold candidates.
//
// Results follow the reference bit for bit, including its behaviour on the
// second and later sparse columns: the range filter sets outliers above the
// target byte whether or not the row is still a candidate and drops the
// candidates when target and major byte are both 0; the max skips a column's
// major byte when no candidate is an outlier there and keeps the major byte
// when every candidate outlier is below it; the decode ORs the major byte
// shifted twice, and only into rows before the column's last outlier.
#include <cuda_runtime.h>
#include <limits.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <string.h>

#include <new>
#include <type_traits>
#include <vector>

#include "buff_device.cuh"
#include "buff_internal.h"
#include "buff_snappy.h"

namespace buffk {
namespace {

using namespace dev;

inline size_t rank_stride(const buff_col *c) { return c->nwp + 16; }

// ---------------------------------------------------------------- encode

// Outlier rows of one sparse column: bytes (flipped) that differ from the
// major byte; the bitmap word and its population per 32 rows.
__global__ void k_major_bits(const uint8_t *__restrict__ lead, uint32_t n, uint32_t major,
                             size_t nwp, uint32_t *__restrict__ bits, uint32_t *__restrict__ cnt) {
  const ByteTarget t = make_target(major);
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nwp;
       w += (size_t)gridDim.x * blockDim.x) {
    const uint32_t row0 = (uint32_t)(w * 32);
    uint32_t out = 0;
    if (row0 < n) {
      const uint4 a = __ldg(reinterpret_cast<const uint4 *>(lead + row0));
      const uint4 b = __ldg(reinterpret_cast<const uint4 *>(lead + row0 + 16));
      const uint32_t wv[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
      uint32_t e[8], g;
#pragma unroll
      for (int q = 0; q < 8; ++q) cmp4(wv[q], t, g, e[q]);
      out = ~gather32(e);
      if (n - row0 < 32) out &= (1u << (n - row0)) - 1u;
    }
    bits[w] = out;
    cnt[w] = __popc(out);
  }
}

// Exclusive prefix sums of `count` u32 values in place, the total at
// data[count]: per-block scan of 4096 values, a single-block scan of the
// block totals, then the block offsets added back.
constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4 * kScanThreads;

__global__ void __launch_bounds__(kScanThreads) k_scan_local(uint32_t *data, size_t count,
                                                              uint32_t *totals) {
  __shared__ uint32_t s_warp[32];
  const size_t base = (size_t)blockIdx.x * kScanItems + threadIdx.x * 4;
  uint32_t v[4];
#pragma unroll
  for (int i = 0; i < 4; ++i) v[i] = base + i < count ? data[base + i] : 0u;
  const uint32_t sum = v[0] + v[1] + v[2] + v[3];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t inc = sum;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
    if (lane >= o) inc += y;
  }
  if (lane == 31) s_warp[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    uint32_t t = s_warp[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, t, o);
      if (lane >= o) t += y;
    }
    s_warp[lane] = t;
  }
  __syncthreads();
  uint32_t run = inc - sum + (wid ? s_warp[wid - 1] : 0u);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    if (base + i < count) data[base + i] = run;
    run += v[i];
  }
  if (threadIdx.x == kScanThreads - 1) totals[blockIdx.x] = run;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_totals(uint32_t *totals, uint32_t nb,
                                                               uint32_t *grand) {
  __shared__ uint32_t s_warp[32];
  __shared__ uint32_t s_carry;
  if (threadIdx.x == 0) s_carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (uint32_t b0 = 0; b0 < nb; b0 += kScanThreads) {
    const uint32_t i = b0 + threadIdx.x;
    const uint32_t v = i < nb ? totals[i] : 0u;
    uint32_t inc = v;
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, inc, o);
      if (lane >= o) inc += y;
    }
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
      uint32_t t = s_warp[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, t, o);
        if (lane >= o) t += y;
      }
      s_warp[lane] = t;
    }
    __syncthreads();
    const uint32_t excl = s_carry + inc - v + (wid ? s_warp[wid - 1] : 0u);
    if (i < nb) totals[i] = excl;
    __syncthreads();
    if (threadIdx.x == kScanThreads - 1) s_carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) *grand = s_carry;
}

__global__ void k_scan_add(uint32_t *data, size_t count, const uint32_t *totals) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) data[i] += totals[i / kScanItems];
}

size_t scan_blocks(size_t count) { return (count + kScanItems - 1) / kScanItems; }

cudaError_t scan_exclusive(uint32_t *data, size_t count, uint32_t *tmp, cudaStream_t s) {
  const uint32_t nb = (uint32_t)((count + kScanItems - 1) / kScanItems);
  k_scan_local<<<nb, kScanThreads, 0, s>>>(data, count, tmp);
  k_scan_totals<<<1, kScanThreads, 0, s>>>(tmp, nb, data + count);
  k_scan_add<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(data, count, tmp);
  count_launch(3);
  return cudaGetLastError();
}

// Outlier bytes (unflipped) of one sparse column, compacted in row order.
__global__ void k_major_compact(const uint8_t *__restrict__ lead, const uint32_t *__restrict__ bits,
                                const uint32_t *__restrict__ rank, size_t nwp,
                                uint8_t *__restrict__ out) {
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nwp;
       w += (size_t)gridDim.x * blockDim.x) {
    uint32_t b = bits[w];
    uint32_t at = rank[w];
    while (b) {
      const uint32_t j = __ffs(b) - 1;
      b &= b - 1;
      out[at++] = lead[w * 32 + j] ^ 0x80u;
    }
  }
}

// 1 + the last outlier row of a sparse column (0 when it has none): each
// thread keeps its own maximum, one atomic per warp.
__global__ void k_major_last(const uint32_t *__restrict__ bits, size_t nwp, uint32_t *last) {
  uint32_t best = 0;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nwp;
       w += (size_t)gridDim.x * blockDim.x) {
    const uint32_t b = bits[w];
    if (b) best = max(best, (uint32_t)(w * 32) + (31 - __clz(b)) + 1);
  }
  best = __reduce_max_sync(0xFFFFFFFFu, best);
  if ((threadIdx.x & 31) == 0 && best) atomicMax(last, best);
}

// ---------------------------------------------------------------- filters

struct MajorArgs {
  uint32_t n, m, kd, r;
  size_t nwp, rs, stride;
  const uint32_t *obits, *orank;
  const uint8_t *obytes;
  unsigned long long oofs[8];
  uint8_t majors[8];
  uint8_t tbyte[8];  // target byte per full byte (sparse columns, then dense slices)
  uint32_t ttail;
  const uint8_t *slices, *tail;
  const uint32_t *cand;  // candidate rows (null: all rows)
  uint32_t *words;
  unsigned long long *count;
};

// buff_range_filter_majority (compress/buff_simd.rs:863-1277) and
// buff_equal_filter_majority (:1916-2292), one thread per 32 rows.
template <bool IS_RANGE>
__global__ void __launch_bounds__(kThreads) k_filter_major(MajorArgs a) {
  const size_t nwords = (a.n + 31) / 32;
  uint32_t cnt = 0;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nwords;
       w += (size_t)gridDim.x * blockDim.x) {
    const uint32_t row0 = (uint32_t)(w * 32);
    const uint32_t valid = a.n - row0 >= 32 ? 0xFFFFFFFFu : ((1u << (a.n - row0)) - 1u);
    uint32_t gt = 0, eq = valid;
    if (a.cand) eq &= a.cand[w];
    for (uint32_t c = 0; c < a.m; ++c) {
      const uint32_t B = a.obits[c * a.nwp + w];
      const uint32_t M = a.majors[c], T = a.tbyte[c];
      uint32_t ogt = 0, oeq = 0;
      if (B) {
        const uint8_t *ob = a.obytes + a.oofs[c] + a.orank[c * a.rs + w];
        uint32_t b = B;
        for (uint32_t k = 0; b; ++k) {
          const uint32_t j = __ffs(b) - 1;
          b &= b - 1;
          const uint32_t val = __ldg(ob + k);
          ogt |= (uint32_t)(val > T) << j;
          oeq |= (uint32_t)(val == T) << j;
        }
      }
      const uint32_t non = ~B & valid;
      if (!IS_RANGE) {
        eq &= oeq | (M == T ? non : 0u);
      } else if (c == 0) {
        gt = ogt | (M > T ? non : 0u);
        eq = oeq | (M == T ? non : 0u);
      } else if (T == 0 && M == 0) {
        gt |= eq & B;  // candidates that are outliers; the others are dropped
        eq = 0;
      } else {
        gt |= ogt;  // every outlier above the target byte, candidate or not
        if (T < M) gt |= eq & non;
        eq &= oeq | (T == M ? non : 0u);
      }
    }
    for (uint32_t j = 0; j < a.kd && eq; ++j) {  // dense slices, progressive
      const uint8_t *p = a.slices + j * a.stride + row0;
      const uint4 lo = __ldg(reinterpret_cast<const uint4 *>(p));
      const uint4 hi = __ldg(reinterpret_cast<const uint4 *>(p + 16));
      const uint32_t wv[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
      const ByteTarget t = make_target(a.tbyte[a.m + j]);
      uint32_t g[8], e[8];
#pragma unroll
      for (int q = 0; q < 8; ++q) cmp4(wv[q], t, g[q], e[q]);
      gt |= eq & gather32(g);
      eq &= gather32(e);
    }
    uint32_t res;
    if (a.r && eq) {
      const uint32_t *tp = reinterpret_cast<const uint32_t *>(a.tail + (size_t)(row0 >> 5) * 4 * a.r);
      uint32_t tw[8];
#pragma unroll
      for (int i = 0; i < 7; ++i) tw[i] = (uint32_t)i < a.r ? __ldg(tp + i) : 0u;
      tw[7] = 0;
      uint32_t gtt = 0, eqt = 0;
      for (uint32_t i = 0; i < 32; ++i) {
        if (!(eq >> i & 1u)) continue;
        const uint32_t bit = i * a.r, wi = bit >> 5;
        const uint32_t f = __funnelshift_r(tw[wi], tw[wi + 1], bit & 31) & ((1u << a.r) - 1u);
        gtt |= (uint32_t)(f > a.ttail) << i;
        eqt |= (uint32_t)(f == a.ttail) << i;
      }
      gt |= eq & gtt;
      eq &= eqt;
      res = IS_RANGE ? gt : eq;
    } else {
      // equality only sets rows in the tail step (:2235-2287)
      res = IS_RANGE ? gt : 0u;
    }
    a.words[w] = res;
    cnt += __popc(res);
  }
  if (a.count) {
    const unsigned long long c = warp_sum_ull(cnt);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(a.count, c);
  }
}

// The rest of one block's compare after its leading byte and first two dense
// bytes: the later dense slices (from slice index j0) while rows still equal
// the target prefix, then the packed tail.  Returns the block's bitmap word.
template <bool IS_RANGE>
__device__ __forceinline__ uint32_t finish_block(const MajorArgs &a, uint32_t row0, uint32_t j0,
                                                 uint32_t gt, uint32_t eq) {
  for (uint32_t j = j0; j < a.kd && eq; ++j) {
    const Bytes32 dj = ld_cand32(a.slices + j * a.stride + row0);
    const ByteTarget tj = make_target(a.tbyte[1 + j]);
    uint32_t g[8], e[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) cmp4(dj.w[q], tj, g[q], e[q]);
    gt |= eq & gather32(g);
    eq &= gather32(e);
  }
  if (a.r && eq) {
    const uint32_t *tp = reinterpret_cast<const uint32_t *>(a.tail + (size_t)(row0 >> 5) * 4 * a.r);
    uint32_t tw[8];
#pragma unroll
    for (int i = 0; i < 7; ++i) tw[i] = (uint32_t)i < a.r ? __ldg(tp + i) : 0u;
    tw[7] = 0;
    uint32_t gtt = 0, eqt = 0;
    for (uint32_t i = 0; i < 32; ++i) {
      if (!(eq >> i & 1u)) continue;
      const uint32_t bit = i * a.r, wi = bit >> 5;
      const uint32_t f = __funnelshift_r(tw[wi], tw[wi + 1], bit & 31) & ((1u << a.r) - 1u);
      gtt |= (uint32_t)(f > a.ttail) << i;
      eqt |= (uint32_t)(f == a.ttail) << i;
    }
    gt |= eq & gtt;
    eq &= eqt;
    return IS_RANGE ? gt : eq;
  }
  return IS_RANGE ? gt : 0u;  // equality only sets rows in the tail step
}

// The same filters for one sparse column whose major byte equals the
// target's leading byte -- a predicate inside the bulk of the values, where
// every non-outlier row stays a candidate for the dense slices.  Those rows
// stream like the plain filter (lane = 32 rows): the bitmap word, its
// outlier rank and 32 bytes of the first dense slice are loaded together,
// and the second dense slice with them while most lanes of the warp needed
// it in its previous step; outlier rows enter the compare with their own
// leading byte.  Blocks that still hold rows equal to the target after two
// dense bytes are queued per warp and refined 32 at a time, one per lane,
// so the later slices are compared with every lane busy instead of by the
// few lanes of each step that need them.  Results are those of
// k_filter_major.
template <bool IS_RANGE, bool TH1, bool TH2>
__global__ void __launch_bounds__(kThreads, 4) k_filter_major1(MajorArgs a) {
  constexpr int kQ = 64;  // queue entries per warp
  __shared__ uint32_t s_q[kThreads / 32][3][kQ];
  const uint32_t lane = threadIdx.x & 31;
  uint32_t(*q)[kQ] = s_q[threadIdx.x >> 5];
  const uint32_t nwords = (a.n + 31) / 32;
  const uint32_t T = a.tbyte[0];
  // per-byte compare constants of the first two dense target bytes, whose
  // top bits are the template arguments
  const uint32_t a0 = (a.tbyte[1] & 0x7Fu) * 0x01010101u, a1 = a0 + 0x01010101u;
  const uint32_t b0 = (a.tbyte[2] & 0x7Fu) * 0x01010101u, b1 = b0 + 0x01010101u;
  const uint8_t *ob0 = a.obytes + a.oofs[0];
  const uint8_t *s1 = a.slices + a.stride;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const bool two = a.kd >= 2;
  const bool deep = a.kd >= 3 || a.r;  // levels after the second dense byte
  bool pre = two;  // warp-uniform: load the second dense slice with the first
  uint32_t qn = 0;  // warp-uniform queue length
  uint32_t cnt = 0;
  const uint32_t step = nwarps * 32;
  // the loads of a lane's next block are issued before the compares of its
  // current one (two blocks in flight per lane)
  uint32_t nB = 0, nR = 0;
  Bytes32 nd0, nd1;
  bool npre = pre;
  {
    const uint32_t w = warp * 32 + lane;
    if (w < nwords) {
      nB = __ldg(a.obits + w);
      nR = __ldg(a.orank + w);
      nd0 = ld_stream32(a.slices + (size_t)w * 32);
      if (npre) nd1 = ld_stream32(s1 + (size_t)w * 32);
    }
  }
  for (uint32_t base = warp * 32; base < nwords; base += step) {
    const uint32_t w = base + lane;
    const bool live = w < nwords;
    const uint32_t B = nB, R = nR;
    const Bytes32 d0 = nd0;
    Bytes32 d1 = nd1;
    const bool dpre = npre;
    {
      const uint32_t wn = w + step;
      npre = pre;
      if (wn < nwords) {
        nB = __ldg(a.obits + wn);
        nR = __ldg(a.orank + wn);
        nd0 = ld_stream32(a.slices + (size_t)wn * 32);
        if (npre) nd1 = ld_stream32(s1 + (size_t)wn * 32);
      }
    }
    const uint32_t row0 = w * 32;
    const uint32_t valid =
        !live ? 0u : (a.n - row0 >= 32 ? 0xFFFFFFFFu : ((1u << (a.n - row0)) - 1u));
    uint32_t gt = 0, eq = ~B & valid;  // leading byte: major == target for non-outliers
    for (uint32_t b = B, k = 0; b; ++k) {
      const uint32_t j = __ffs(b) - 1;
      b &= b - 1;
      const uint32_t v = __ldg(ob0 + R + k);
      gt |= (uint32_t)(v > T) << j;
      eq |= (uint32_t)(v == T) << j;
    }
    gt &= valid;
    eq &= valid;
    uint32_t vote;
    if (dpre) {
      // both dense bytes at hand: their per-byte results are combined before
      // the one gather per result (row above the two target bytes: first
      // byte above, or equal and the second above; equal: both equal)
      uint32_t mg[8], me[8], eor = 0;
#pragma unroll
      for (int qq = 0; qq < 8; ++qq) {
        const uint32_t e0 = eq4t<TH1>(d0.w[qq], a0, a1), e1 = eq4t<TH2>(d1.w[qq], b0, b1);
        eor |= e0;
        me[qq] = e0 & e1;
        if (IS_RANGE) mg[qq] = gt4t<TH1>(d0.w[qq], a1) | (e0 & gt4t<TH2>(d1.w[qq], b1));
      }
      if (IS_RANGE) gt |= eq & gather32(mg);
      eq &= gather32(me);
      vote = __ballot_sync(0xFFFFFFFFu, live && eor != 0);
    } else {
      // the first dense byte, then the second for the lanes that still need it
      {
        uint32_t m[8];
#pragma unroll
        for (int qq = 0; qq < 8; ++qq) m[qq] = eq4t<TH1>(d0.w[qq], a0, a1);
        const uint32_t e = gather32(m);
        if (IS_RANGE) {
#pragma unroll
          for (int qq = 0; qq < 8; ++qq) m[qq] = gt4t<TH1>(d0.w[qq], a1);
          gt |= eq & gather32(m);
        }
        eq &= e;
      }
      const bool need1 = two && eq != 0;
      vote = __ballot_sync(0xFFFFFFFFu, need1);
      if (need1) {
        d1 = ld_cand32(s1 + row0);
        uint32_t m[8];
#pragma unroll
        for (int qq = 0; qq < 8; ++qq) m[qq] = eq4t<TH2>(d1.w[qq], b0, b1);
        const uint32_t e = gather32(m);
        if (IS_RANGE) {
#pragma unroll
          for (int qq = 0; qq < 8; ++qq) m[qq] = gt4t<TH2>(d1.w[qq], b1);
          gt |= eq & gather32(m);
        }
        eq &= e;
      }
    }
    pre = two && __popc(vote) >= 16;
    // blocks with rows still equal to the target go to the queue
    const bool more = live && deep && eq != 0;
    const uint32_t qv = __ballot_sync(0xFFFFFFFFu, more);
    if (more) {
      const uint32_t at = qn + __popc(qv & ((1u << lane) - 1u));
      q[0][at] = w;
      q[1][at] = gt;
      q[2][at] = eq;
    } else if (live) {
      const uint32_t res = IS_RANGE ? gt : ((a.r == 0 || !eq) ? 0u : eq);
      __stcs(a.words + w, res);
      cnt += __popc(res);
    }
    qn += __popc(qv);
    __syncwarp();
    if (qn >= 32) {  // refine 32 queued blocks, one per lane
      qn -= 32;
      const uint32_t qw = q[0][qn + lane], qg = q[1][qn + lane], qe = q[2][qn + lane];
      __syncwarp();
      const uint32_t res = finish_block<IS_RANGE>(a, qw * 32, two ? 2u : 1u, qg, qe);
      __stcs(a.words + qw, res);
      cnt += __popc(res);
    }
  }
  if (lane < qn) {  // what is left in the queue
    const uint32_t qw = q[0][lane];
    const uint32_t res = finish_block<IS_RANGE>(a, qw * 32, two ? 2u : 1u, q[1][lane], q[2][lane]);
    __stcs(a.words + qw, res);
    cnt += __popc(res);
  }
  if (a.count) {
    const unsigned long long c = warp_sum_ull(cnt);
    if (lane == 0 && c) atomicAdd(a.count, c);
  }
}

// The 32 R-bit tail fields of a 32-row block (R words, LSB-first) compared
// with `t`: four fields at a time spread into the bytes of a word (constant
// shifts), then per-byte SWAR -- field > t is the MSB of field + 127 - t,
// field == t the clear MSB of (field ^ t) + 127 (no byte carries: fields and
// t are below 128) -- and the MSBs gathered into row bitmaps.
template <int R>
__device__ __forceinline__ void tail_cmp32(const uint32_t *tw, uint32_t t, uint32_t &gtt,
                                           uint32_t &eqt) {
  constexpr uint32_t fm = (1u << R) - 1u;
  const uint32_t cg = (127u - t) * 0x01010101u, t4 = t * 0x01010101u;
  uint32_t mg[8], me[8];
#pragma unroll
  for (int g = 0; g < 8; ++g) {
    const int bit = 4 * g * R, wi = bit >> 5, sh = bit & 31;
    const uint32_t x = sh == 0 ? tw[wi] : __funnelshift_r(tw[wi], wi + 1 < R ? tw[wi + 1] : 0u, sh);
    const uint32_t y = (x & fm) | ((x << (8 - R)) & (fm << 8)) | ((x << (16 - 2 * R)) & (fm << 16)) |
                       ((x << (24 - 3 * R)) & (fm << 24));
    mg[g] = (y + cg) & H;
    me[g] = ~((y ^ t4) + 0x7F7F7F7Fu) & H;
  }
  gtt = gather32(mg);
  eqt = gather32(me);
}

// buff-major filters of a column with one sparse byte column and no dense
// slices (the RAPG-major layout of 8-bit values: the code is the byte, then
// R tail bits): thread = 32 rows -- the bitmap word, its outlier rank and
// the block's R tail words, loaded one block ahead; the block's outlier
// bytes (consecutive from its rank) come from three aligned words loaded
// together when it has at most 8 outliers, singly beyond; the tail fields
// of the rows still equal to the target are compared 4 at a time
// (tail_cmp32).  Results are those of k_filter_major.
template <bool IS_RANGE, int R>
__global__ void __launch_bounds__(kThreads) k_filter_major0(MajorArgs a) {
  const uint32_t nwords = (a.n + 31) / 32;
  const uint32_t M = a.majors[0], T = a.tbyte[0];
  const uint8_t *ob0 = a.obytes + a.oofs[0];
  uint32_t cnt = 0;
  const uint32_t step = gridDim.x * blockDim.x;
  // a thread's next block (bitmap word, rank, tail words) is loaded before
  // its current one is compared
  uint32_t nB = 0, nrk = 0, ntw[R > 0 ? R : 1];
  {
    const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
    if (w < nwords) {
      nB = __ldg(a.obits + w);
      nrk = __ldg(a.orank + w);
#pragma unroll
      for (int i = 0; i < R; ++i)
        ntw[i] = __ldg(reinterpret_cast<const uint32_t *>(a.tail + (size_t)w * 4 * R) + i);
    }
  }
  for (uint32_t w = blockIdx.x * blockDim.x + threadIdx.x; w < nwords; w += step) {
    const uint32_t row0 = w * 32;
    const uint32_t valid = a.n - row0 >= 32 ? 0xFFFFFFFFu : ((1u << (a.n - row0)) - 1u);
    const uint32_t B = nB, rk = nrk;
    uint32_t tw[R > 0 ? R : 1];
#pragma unroll
    for (int i = 0; i < R; ++i) tw[i] = ntw[i];
    if (w + step < nwords) {
      nB = __ldg(a.obits + w + step);
      nrk = __ldg(a.orank + w + step);
#pragma unroll
      for (int i = 0; i < R; ++i)
        ntw[i] = __ldg(reinterpret_cast<const uint32_t *>(a.tail + (size_t)(w + step) * 4 * R) + i);
    }
    uint32_t og = 0, oe = 0;
    if (B) {
      const uint32_t no = __popc(B);
      const uintptr_t p = reinterpret_cast<uintptr_t>(ob0 + rk);
      uint32_t w0 = 0, w1 = 0, w2 = 0;
      if (no <= 8) {  // bytes p .. p + 7 lie in the 3 aligned words from p & ~3
        const uint32_t *q = reinterpret_cast<const uint32_t *>(p & ~(uintptr_t)3);
        w0 = __ldg(q);
        w1 = __ldg(q + 1);
        w2 = __ldg(q + 2);
      }
      const uint32_t o8 = 8 * (uint32_t)(p & 3u);
      const uint32_t lo4 = __funnelshift_r(w0, w1, o8), hi4 = __funnelshift_r(w1, w2, o8);
      for (uint32_t b = B, k = 0; b; ++k) {
        const uint32_t j = __ffs(b) - 1;
        b &= b - 1;
        const uint32_t v = no > 8 ? (uint32_t)__ldg(ob0 + rk + k)
                                  : ((k < 4 ? lo4 : hi4) >> (8 * (k & 3))) & 0xFFu;
        og |= (uint32_t)(v > T) << j;
        oe |= (uint32_t)(v == T) << j;
      }
    }
    const uint32_t non = ~B & valid;
    uint32_t gt = IS_RANGE ? og | (M > T ? non : 0u) : 0u;
    uint32_t eq = (oe | (M == T ? non : 0u)) & valid;
    uint32_t res = IS_RANGE ? gt : 0u;  // equality only sets rows in the tail step
    if constexpr (R > 0) {
      if (eq) {
        uint32_t gtt, eqt;
        tail_cmp32<R>(tw, a.ttail, gtt, eqt);
        gt |= eq & gtt;
        eq &= eqt;
        res = IS_RANGE ? gt : eq;
      }
    }
    __stcs(a.words + w, res);
    cnt += __popc(res);
  }
  if (a.count) {
    const unsigned long long c = warp_sum_ull(cnt);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(a.count, c);
  }
}

template <bool IS_RANGE>
static void launch_filter_major0(const MajorArgs &a, int grid, cudaStream_t s) {
  switch (a.r) {
    case 0: k_filter_major0<IS_RANGE, 0><<<grid, kThreads, 0, s>>>(a); break;
    case 1: k_filter_major0<IS_RANGE, 1><<<grid, kThreads, 0, s>>>(a); break;
    case 2: k_filter_major0<IS_RANGE, 2><<<grid, kThreads, 0, s>>>(a); break;
    case 3: k_filter_major0<IS_RANGE, 3><<<grid, kThreads, 0, s>>>(a); break;
    case 4: k_filter_major0<IS_RANGE, 4><<<grid, kThreads, 0, s>>>(a); break;
    case 5: k_filter_major0<IS_RANGE, 5><<<grid, kThreads, 0, s>>>(a); break;
    case 6: k_filter_major0<IS_RANGE, 6><<<grid, kThreads, 0, s>>>(a); break;
    default: k_filter_major0<IS_RANGE, 7><<<grid, kThreads, 0, s>>>(a); break;
  }
}

// ---------------------------------------------------------------- sum / max helpers

// Sum of nbytes bytes from p (any alignment): the bytes before the first
// 16-byte boundary and after the last one singly, the rest as 16-byte
// vectors through dp4a.
__device__ __forceinline__ unsigned long long bytesum_thread(const uint8_t *__restrict__ p,
                                                             size_t nbytes, size_t tid,
                                                             size_t nth) {
  size_t head = (16 - (reinterpret_cast<uintptr_t>(p) & 15)) & 15;
  if (head > nbytes) head = nbytes;
  const size_t nvec = (nbytes - head) / 16;
  const uint8_t *body = p + head;
  unsigned long long acc = 0;
  uint32_t part = 0;
  for (size_t v = tid; v < nvec; v += nth) {
    const uint4 d = __ldg(reinterpret_cast<const uint4 *>(body + v * 16));
    part = __dp4a(d.x, 0x01010101u, part);
    part = __dp4a(d.y, 0x01010101u, part);
    part = __dp4a(d.z, 0x01010101u, part);
    part = __dp4a(d.w, 0x01010101u, part);
    if (part >= 0xF0000000u) {  // keep the 32-bit partial far from overflow
      acc += part;
      part = 0;
    }
  }
  acc += part;
  const size_t rest = head + nvec * 16;  // bytes before `rest` not in vectors: [0, head)
  if (tid < head) acc += p[tid];
  for (size_t i = rest + tid; i < nbytes; i += nth) acc += p[i];
  return acc;
}

__global__ void k_bytesum(const uint8_t *__restrict__ p, size_t nbytes, unsigned long long *out) {
  unsigned long long acc = bytesum_thread(p, nbytes, blockIdx.x * (size_t)blockDim.x + threadIdx.x,
                                          (size_t)gridDim.x * blockDim.x);
  acc = warp_sum_ull(acc);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

// The outlier bytes of each sparse column of a buff-major column.
struct SparseBytes {
  const uint8_t *p[8];
  uint32_t n[8];
  uint32_t m;
};

// buff_sum_majority's sums (buff_simd.rs:2294-2442) in one launch: the dense
// slices and the tail as k_sum does (into raw[8..]) and the outlier bytes of
// every sparse column (into raw[0..m)).  With `sum` set, the last block to
// finish -- a ticket in raw[23], taken after each block's sums are added and
// fenced -- combines them into the f64 sum (and the partials) as the host
// does; raw (24 u64) is zeroed beforehand.
__global__ void __launch_bounds__(kThreads) k_sum_major(const uint8_t *__restrict__ slices,
                                                        size_t stride, uint32_t kd,
                                                        const uint8_t *__restrict__ tail,
                                                        uint32_t ts, unsigned long long tail_bits,
                                                        SparseBytes sb, MajorSumArgs a,
                                                        unsigned long long *raw, double *sum,
                                                        unsigned long long *parts_out) {
  __shared__ unsigned long long s_acc[9], s_out[8];
  __shared__ bool s_last;
  if (threadIdx.x < 9) s_acc[threadIdx.x] = 0;
  if (threadIdx.x < 8) s_out[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
  const uint32_t nth = gridDim.x * blockDim.x;
  if (a.n) sum_slices_tail(slices, stride, kd, tail, ts, tail_bits, tid, nth, s_acc);
#pragma unroll
  for (uint32_t c = 0; c < 8; ++c) {  // unrolled: the parameter arrays stay out of local memory
    if (c >= sb.m || !sb.n[c]) continue;
    const unsigned long long v = warp_sum_ull(bytesum_thread(sb.p[c], sb.n[c], tid, nth));
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(&s_out[c], v);
  }
  __syncthreads();
  if (threadIdx.x < kd && s_acc[threadIdx.x]) atomicAdd(&raw[8 + threadIdx.x], s_acc[threadIdx.x]);
  if (threadIdx.x == 8 && ts && s_acc[8]) atomicAdd(&raw[8 + kd], s_acc[8]);
  if (threadIdx.x < sb.m && s_out[threadIdx.x]) atomicAdd(&raw[threadIdx.x], s_out[threadIdx.x]);
  if (!sum) return;
  if (threadIdx.x < 9) __threadfence();  // the threads that added to raw
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(&raw[23], 1ull) == gridDim.x - 1;
  __syncthreads();
  if (!s_last || threadIdx.x != 0) return;
  __threadfence();
  unsigned long long r[24], parts[9];
  for (int i = 0; i < 23; ++i) r[i] = __ldcg(raw + i);
  const uint32_t np = major_sum_parts(a, r, parts);
  *sum = major_sum_f64(a, parts);
  if (parts_out)
    for (uint32_t i = 0; i < np; ++i) parts_out[i] = parts[i];
}

// Largest outlier byte among rows set in `cand` (all outlier rows when cand is
// null) of sparse column c; any[0] |= 1 when there is such a row.
// The value of one row in a dense slice (flipped bytes; r == 0) or the
// packed tail (r bits).
__device__ __forceinline__ uint32_t field_at(const uint8_t *slice, const uint8_t *tail, uint32_t r,
                                             uint32_t row) {
  if (!r) return (uint32_t)(slice[row] ^ 0x80u);
  const unsigned long long bit = (unsigned long long)row * r;
  const uint32_t b0 = tail[bit >> 3];
  const uint32_t b1 = ((bit & 7) + r > 8) ? tail[(bit >> 3) + 1] : 0u;
  return ((b0 | (b1 << 8)) >> (bit & 7)) & ((1u << r) - 1u);
}

// The progressive max of buff_max_majority (buff_simd.rs:2444-2861) runs as
// a chain of candidate steps whose decisions never leave the device: each
// "max" kernel folds the largest byte among the candidate rows into
// st->best[step] (one atomic per warp), and the following "select" kernel
// reads it back, applies the reference's rule for that column, narrows the
// candidate bitmap and ORs the chosen byte into st->mx.
struct MaxState {
  uint32_t best[20];
  uint32_t flag[20];  // a sparse column's candidates include an outlier
  unsigned long long mx;
  unsigned long long count;
};

// Largest outlier byte among the candidate rows of a sparse column (all its
// outliers when cand is null).
__global__ void k_major_candmax(const uint32_t *__restrict__ bits, const uint32_t *__restrict__ rank,
                                const uint8_t *__restrict__ ob, const uint32_t *__restrict__ cand,
                                size_t nw, uint32_t *best, uint32_t *flag) {
  uint32_t bm = 0, any = 0;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nw;
       w += (size_t)gridDim.x * blockDim.x) {
    const uint32_t B = bits[w];
    const uint32_t sel = cand ? B & cand[w] : B;
    if (!sel) continue;
    any = 1;
    uint32_t b = B;
    for (uint32_t k = rank[w]; b; ++k) {
      const uint32_t j = __ffs(b) - 1;
      b &= b - 1;
      if (sel >> j & 1u) bm = max(bm, (uint32_t)ob[k]);
    }
  }
  bm = __reduce_max_sync(0xFFFFFFFFu, bm);
  any = __reduce_or_sync(0xFFFFFFFFu, any);
  if ((threadIdx.x & 31) == 0 && any) {
    atomicMax(best, bm);
    atomicOr(flag, 1u);
  }
}

// New candidate words for sparse column `col` (buff_simd.rs:2466-2557):
// first column: the outlier rows holding the largest outlier byte if it
// exceeds the major byte M, else every non-outlier row; later columns: if no
// candidate is an outlier, the candidates stay (minus outliers, i.e. all);
// if the largest candidate outlier byte exceeds M, those rows; else the
// candidates that are not outliers.  The chosen byte goes into *mx at `sh`.
__global__ void k_major_select(const uint32_t *__restrict__ bits, const uint32_t *__restrict__ rank,
                               const uint8_t *__restrict__ ob, uint32_t *cand, size_t nw,
                               uint32_t n, const uint32_t *best, const uint32_t *flag,
                               uint32_t M, uint32_t sh, int first, unsigned long long *mx) {
  const uint32_t bv = *best, fl = *flag;
  int mode;  // 0: ~B (valid rows); 1: rows of (B & cand) whose byte is bv; 2: cand & ~B
  unsigned long long add;
  if (first) {
    mode = (fl && bv > M) ? 1 : 0;
    add = (unsigned long long)(mode == 1 ? bv : M) << sh;
  } else if (!fl) {
    mode = 2;
    add = 0;
  } else {
    mode = bv > M ? 1 : 2;
    add = (unsigned long long)(bv > M ? bv : M) << sh;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && add) atomicOr(mx, add);
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nw;
       w += (size_t)gridDim.x * blockDim.x) {
    const uint32_t row0 = (uint32_t)(w * 32);
    const uint32_t valid = n - row0 >= 32 ? 0xFFFFFFFFu : ((1u << (n - row0)) - 1u);
    const uint32_t B = bits[w];
    uint32_t out;
    if (mode == 0) {
      out = ~B & valid;
    } else if (mode == 2) {
      out = cand[w] & ~B;
    } else {
      const uint32_t sel = B & cand[w];
      out = 0;
      uint32_t b = B;
      for (uint32_t k = rank[w]; b; ++k) {
        const uint32_t j = __ffs(b) - 1;
        b &= b - 1;
        if ((sel >> j & 1u) && ob[k] == bv) out |= 1u << j;
      }
    }
    cand[w] = out;
  }
}

// 0xFF in byte i of the result for each set bit i of the 4-bit x.
__device__ __forceinline__ uint32_t bytemask4(uint32_t x) {
  return ((x * 0x00204081u) & 0x01010101u) * 0xFFu;
}

// The 32 unflipped slice bytes of rows w*32 .. w*32+31 (one 32-byte block).
__device__ __forceinline__ void block_bytes(const uint8_t *slice, size_t w, uint32_t *u) {
  const uint4 lo = __ldg(reinterpret_cast<const uint4 *>(slice + w * 32));
  const uint4 hi = __ldg(reinterpret_cast<const uint4 *>(slice + w * 32 + 16));
  const uint32_t v[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
  for (int q = 0; q < 8; ++q) u[q] = v[q] ^ 0x80808080u;
}

// The 32 R-bit tail fields of rows w*32 .. w*32+31 (4R bytes at 4R*w).
template <int R>
__device__ __forceinline__ void block_fields(const uint8_t *tail, size_t w, uint32_t *f) {
  const uint32_t *p = reinterpret_cast<const uint32_t *>(tail + (size_t)4 * R * w);
  uint32_t tw[R];
#pragma unroll
  for (int i = 0; i < R; ++i) tw[i] = __ldg(p + i);
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int bit = i * R, wi = bit >> 5, sh = bit & 31;
    const uint32_t hi = (wi + 1 < R) ? tw[wi + 1] : 0u;
    f[i] = __funnelshift_r(tw[wi], hi, sh) & ((1u << R) - 1u);
  }
}

// Progressive max step over a dense slice (R == 0) or the R-bit tail: the
// largest value among the candidate rows, folded into *best.
template <int R>
__global__ void k_cand_max(const uint8_t *__restrict__ slice, const uint8_t *__restrict__ tail,
                           const uint32_t *__restrict__ cand, size_t nw, uint32_t *best) {
  uint32_t bm = 0;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nw;
       w += (size_t)gridDim.x * blockDim.x) {
    const uint32_t b = cand[w];
    if (!b) continue;
    if (R == 0) {
      uint32_t u[8], m = 0;
      block_bytes(slice, w, u);
#pragma unroll
      for (int q = 0; q < 8; ++q) m = __vmaxu4(m, u[q] & bytemask4((b >> (4 * q)) & 0xFu));
      m = __vmaxu4(m, m >> 16);
      m = __vmaxu4(m, m >> 8);
      bm = max(bm, m & 0xFFu);
    } else {
      uint32_t f[32];
      block_fields<R == 0 ? 1 : R>(tail, w, f);
#pragma unroll
      for (int i = 0; i < 32; ++i)
        if (b >> i & 1u) bm = max(bm, f[i]);
    }
  }
  bm = __reduce_max_sync(0xFFFFFFFFu, bm);
  if ((threadIdx.x & 31) == 0 && bm) atomicMax(best, bm);
}

// Keeps the candidate rows whose value equals *best and ORs *best << sh
// into *mx; count (may be null) receives the kept rows.
template <int R>
__global__ void k_cand_select(const uint8_t *__restrict__ slice, const uint8_t *__restrict__ tail,
                              uint32_t *cand, size_t nw, const uint32_t *best, uint32_t sh,
                              unsigned long long *mx, unsigned long long *count) {
  const uint32_t v = *best;
  if (blockIdx.x == 0 && threadIdx.x == 0 && v) atomicOr(mx, (unsigned long long)v << sh);
  unsigned long long c = 0;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nw;
       w += (size_t)gridDim.x * blockDim.x) {
    const uint32_t b = cand[w];
    uint32_t out = 0;
    if (b) {
      if (R == 0) {
        uint32_t u[8], e[8];
        block_bytes(slice, w, u);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const uint32_t x = u[q] ^ (v * 0x01010101u);  // zero bytes where equal
          e[q] = ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x) & 0x80808080u;
        }
        out = b & gather32(e);
      } else {
        uint32_t f[32];
        block_fields<R == 0 ? 1 : R>(tail, w, f);
#pragma unroll
        for (int i = 0; i < 32; ++i) out |= (uint32_t)(f[i] == v) << i;
        out &= b;
      }
      cand[w] = out;
    }
    c += __popc(out);
  }
  if (count) {
    c = warp_sum_ull(c);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
  }
}

__global__ void k_popc(const uint32_t *__restrict__ w, size_t nw, unsigned long long *out) {
  unsigned long long c = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nw;
       i += (size_t)gridDim.x * blockDim.x)
    c += __popc(w[i]);
  c = warp_sum_ull(c);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, c);
}

// ---------------------------------------------------------------- decode

struct DecodeMajorArgs {
  uint32_t n, m, kd, r, fl;
  size_t nwp, rs, stride;
  const uint32_t *obits, *orank;
  const uint8_t *obytes;
  unsigned long long oofs[8];
  uint8_t majors[8];
  uint32_t olast[8];
  const uint8_t *slices, *tail;
  long long base;
  int dlen;
  double *out;
};

// buff_decode_majority (compress/buff_simd.rs:633-861), one thread per row.
__global__ void __launch_bounds__(kThreads) k_decode_major(DecodeMajorArgs a) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < a.n;
       i += (size_t)gridDim.x * blockDim.x) {
    const size_t w = i >> 5;
    const uint32_t j = (uint32_t)(i & 31);
    unsigned long long v = 0;
    for (uint32_t c = 0; c < a.m; ++c) {
      const uint32_t sh = a.fl - 8 * (c + 1);
      const uint32_t B = a.obits[c * a.nwp + w];
      if (B >> j & 1u) {
        const uint32_t k = a.orank[c * a.rs + w] + __popc(B & ((1u << j) - 1u));
        const unsigned long long b = a.obytes[a.oofs[c] + k];
        v = c == 0 ? (b << sh) : (v | (b << sh));
      } else if (c == 0) {
        v = (unsigned long long)a.majors[0] << sh;
      } else if (i + 1 < a.olast[c]) {
        v |= (((unsigned long long)a.majors[c] << sh) << sh);
      }
    }
    for (uint32_t d = 0; d < a.kd; ++d) {
      const uint32_t sh = a.fl - 8 * (a.m + d + 1);
      v |= (unsigned long long)(a.slices[d * a.stride + i] ^ 0x80u) << sh;
    }
    if (a.r) v |= field_at(nullptr, a.tail, a.r, (uint32_t)i);
    a.out[i] = i64_to_f64_scaled((long long)((unsigned long long)a.base + v), a.dlen);
  }
}

// RAPG byte_residue_decode (compress/split_double.rs:1353-1610) and its
// precision-limited form (:1612-1893) over the top R bits of each code: the
// outlier bytes of the m sparse columns (zero elsewhere) and ks dense slices,
// each placed `remain` bits up as the reference's reader places them, then a
// ts-bit field of the packed tail; not shifted back when R < fixed_len.
struct RapgDecodeArgs {
  const uint32_t *obits, *orank;
  const uint8_t *obytes;
  uint64_t oofs[8];
  size_t nwp, rs, stride;
  const uint8_t *slices, *tail;
  uint32_t n, m, kd, ks, ts, R, skip;
  unsigned long long tbit0;
  unsigned long long sdef;  // sparse bits of a row that is an outlier in no column
  uint32_t smaj[8];         // a sparse column's byte on its non-outlier rows
  long long base;
  int dlen;
  double *out;
};

// Conversion forms of the fast decodes (k_rapg_decode_fast4's CV).
constexpr int kCvI32 = 0, kCvU53 = 1, kCvS53 = 2, kCvI64 = 3;

// `width`-bit field `row` of a stream packed LSB-first from bit `bit0`.
__device__ __forceinline__ uint32_t field_from(const uint8_t *p, unsigned long long bit0,
                                               uint32_t width, uint32_t row) {
  const unsigned long long bit = bit0 + (unsigned long long)row * width;
  const uint32_t b0 = p[bit >> 3];
  const uint32_t b1 = ((bit & 7) + width > 8) ? p[(bit >> 3) + 1] : 0u;
  return ((b0 | (b1 << 8)) >> (bit & 7)) & ((1u << width) - 1u);
}

// A thread takes 4 consecutive rows: one 32-bit load per dense slice, the
// 4 rows' bits of each sparse column from one bitmap word, two 16-byte
// stores (out 16-byte aligned).
__global__ void __launch_bounds__(kThreads) k_rapg_decode(RapgDecodeArgs a) {
  const uint32_t ngroups = (a.n + 3) / 4;
  for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < ngroups;
       g += gridDim.x * blockDim.x) {
    const uint32_t row0 = g * 4;
    const size_t w = row0 >> 5;
    const uint32_t j0 = row0 & 31;
    unsigned long long v[4] = {0, 0, 0, 0};
    uint32_t remain = a.R;
    for (uint32_t c = 0; c < a.m; ++c) {
      remain -= 8;
      const uint32_t B = __ldg(a.obits + c * a.nwp + w);
      const uint32_t nib = (B >> j0) & 0xFu;
      if (nib) {
        uint32_t k = __ldg(a.orank + c * a.rs + w) + __popc(B & ((1u << j0) - 1u));
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (nib >> i & 1u) v[i] |= (unsigned long long)a.obytes[a.oofs[c] + k++] << (remain & 63);
      }
    }
    for (uint32_t d = 0; d < a.ks; ++d) {
      remain -= 8;
      if (d < a.kd) {
        const uint32_t x =
            __ldg(reinterpret_cast<const uint32_t *>(a.slices + d * a.stride + row0)) ^ 0x80808080u;
#pragma unroll
        for (int i = 0; i < 4; ++i) v[i] |= (unsigned long long)((x >> (8 * i)) & 0xFFu) << (remain & 63);
      } else {  // past the dense slices the reader takes the bytes after them
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (row0 + i < a.n)
            v[i] |= (unsigned long long)a.tail[a.skip + (size_t)(d - a.kd) * a.n + row0 + i]
                    << (remain & 63);
      }
    }
    if (a.ts) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (row0 + i < a.n) v[i] |= field_from(a.tail, a.tbit0, a.ts, row0 + i);
    }
    double o[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
      o[i] = i64_to_f64_scaled((long long)((unsigned long long)a.base + v[i]), a.dlen);
    if (row0 + 4 <= a.n) {
      double2 *dst = reinterpret_cast<double2 *>(a.out + row0);
      __stcs(dst, make_double2(o[0], o[1]));
      __stcs(dst + 1, make_double2(o[2], o[3]));
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (row0 + i < a.n) a.out[row0 + i] = o[i];
    }
  }
}

// The common plans (every slice read lies in the dense region, tail fields
// from bit 0 with ts <= r): the code is the big-endian concatenation of the
// sparse bytes, KS dense bytes and ts tail bits.  This kernel writes every
// row with zero sparse bytes -- the value of every row that is an outlier in
// no sparse column -- and k_rapg_fixup rewrites the outlier rows.  Lane L
// produces rows 64m + 2L and 64m + 2L + 1 of each 512-row chunk (coalesced
// 16-byte stores); slice bytes are 2-byte loads; the ts-bit fields of a
// 64-row group (8*ts bytes) are loaded by the first 2*ts lanes and handed
// out with shuffles.
template <int KS, bool N32 = false>
__global__ void __launch_bounds__(kThreads) k_rapg_decode_fast(RapgDecodeArgs a) {
  using CodeT = typename std::conditional<N32, uint32_t, unsigned long long>::type;
  // the outlier fix-up (a programmatic dependent launch) may start once every
  // block of this pass runs; it waits for this pass before reading the values
  asm volatile("griddepcontrol.launch_dependents;");
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nchunks = (a.n + kRowChunk - 1) / kRowChunk;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t ts = a.ts;
  const unsigned long long tmask = ts ? ((1ull << ts) - 1ull) : 0ull;
  for (uint32_t ch = warp; ch < nchunks; ch += nwarps) {
    const uint32_t r0 = ch * kRowChunk;
    uint32_t sb[8][KS > 0 ? KS : 1];
#pragma unroll
    for (int m = 0; m < 8; ++m)
#pragma unroll
      for (int s = 0; s < KS; ++s)
        sb[m][s] = __ldg(reinterpret_cast<const uint16_t *>(a.slices + s * a.stride + r0 +
                                                            m * 64 + 2 * lane));
    uint32_t tw[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      tw[m] = 0;
      if (ts && lane < 2 * ts)
        tw[m] = __ldg(reinterpret_cast<const uint32_t *>(a.tail + (size_t)8 * ts * (r0 / 64 + m)) +
                      lane);
    }
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const uint32_t i0 = r0 + m * 64 + 2 * lane;
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
      c0 |= (CodeT)a.sdef;
      c1 |= (CodeT)a.sdef;
      double v0, v1;
      if (N32) {
        v0 = i32_to_f64_scaled((int)((uint32_t)a.base + (uint32_t)c0), a.dlen);
        v1 = i32_to_f64_scaled((int)((uint32_t)a.base + (uint32_t)c1), a.dlen);
      } else {
        v0 = i64_to_f64_scaled((long long)((unsigned long long)a.base + c0), a.dlen);
        v1 = i64_to_f64_scaled((long long)((unsigned long long)a.base + c1), a.dlen);
      }
      if (i0 + 2 <= a.n)
        __stcs(reinterpret_cast<double2 *>(a.out + i0), make_double2(v0, v1));
      else if (i0 < a.n)
        a.out[i0] = v0;
    }
  }
}

// The same plans for 1..4 dense slices: lane L takes 4 consecutive rows of
// each 128-row group -- one 4-byte load per dense slice, a 4x4 byte
// transpose into the 4 rows' dense bytes, the tail fields by one shuffle
// pair -- and the 4 values leave in one 32-byte store when the output is
// 32-byte aligned (ST32), else in two 16-byte stores.  Without SP1 every row
// is written with the default sparse bytes and a fix-up pass rewrites the
// outlier rows.  With SP1 (one sparse column) the outlier rows are decoded
// here: the chunk's 16 bitmap words and its first rank word are loaded one
// chunk ahead, a prefix count over the words gives each lane its first
// outlier's rank, and the chunk's outlier bytes (consecutive in the outlier
// byte array) arrive as one window of up to 32 aligned 4-byte words loaded
// with the slices -- no load of this chunk waits on another.  A chunk with
// more than 124 outliers reads its bytes one by one.  (A first merge, one
// dependent rank-and-byte load per outlier row, ran slower than the
// separate fix-up.)  A row's code is assembled as two 32-bit words (the
// sparse byte above KS dense bytes, the pair shifted left ts by one funnel
// shift, the tail field below) and converted by the form CV names:
// kCvI32 (every value in 32 bits), kCvU53 (every value in [1, 2^53)),
// kCvS53 (every |value| below 2^53) or kCvI64 (rounding conversion).
template <int KS, int CV, bool ST32, bool SP1>
__global__ void __launch_bounds__(kThreads) k_rapg_decode_fast4(RapgDecodeArgs a) {
  static_assert(KS >= 0 && KS <= 4, "k_rapg_decode_fast4 transposes at most 4 slices");
  static_assert(KS > 0 || SP1, "without dense slices the pass takes one sparse column");
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nchunks = (a.n + kRowChunk - 1) / kRowChunk;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t ts = a.ts;
  const uint32_t tmask = ts ? ((1u << ts) - 1u) : 0u;
  const uint32_t kx = KS == 4 ? 0x80808080u : (0x80808080u & ((1u << (8 * (KS & 3))) - 1u));
  const uint32_t sdef_hi = (uint32_t)(a.sdef >> 32), sdef_lo = (uint32_t)a.sdef;
  // SP1: the default sparse byte in every byte of a word; bitmap word
  // `lane` (< 16) of the chunk and the chunk's first rank
  const uint32_t spd4 = SP1 ? (uint32_t)(a.sdef >> (8 * KS + ts)) * 0x01010101u : 0u;
  const uint32_t nwords = (a.n + 31) / 32;
  const uint8_t *ob = a.obytes + a.oofs[0];
  uint32_t nW = 0, nR = 0;
  if (SP1 && warp < nchunks) {
    if (lane < 16 && warp * 16 + lane < nwords) nW = __ldg(a.obits + warp * 16 + lane);
    nR = __ldg(a.orank + warp * 16);
  }
  for (uint32_t ch = warp; ch < nchunks; ch += nwarps) {
    const uint32_t r0 = ch * kRowChunk;
    uint32_t Bw = 0, Rc = 0;
    if (SP1) {
      Bw = nW;
      Rc = nR;
      const uint32_t cn = ch + nwarps;
      if (cn < nchunks) {
        nW = lane < 16 && cn * 16 + lane < nwords ? __ldg(a.obits + cn * 16 + lane) : 0u;
        nR = __ldg(a.orank + cn * 16);
      }
    }
    uint32_t sw[4][KS > 0 ? KS : 1];
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int s = 0; s < KS; ++s)
        sw[m][s] = __ldg(reinterpret_cast<const uint32_t *>(a.slices + s * a.stride + r0 +
                                                            m * 128 + 4 * lane));
    uint32_t tw[4];
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      tw[m] = 0;
      // a 128-row group's ts-bit fields: 4 ts words at byte 16 ts * group
      if (ts && lane < 4 * ts)
        tw[m] = __ldg(reinterpret_cast<const uint32_t *>(a.tail + (size_t)16 * ts * (r0 / 128 + m)) +
                      lane);
    }
    // SP1: outliers before each lane's word within the chunk, the chunk's
    // count, and the window of its outlier bytes (from the aligned word
    // holding the first; the allocation extends 16 bytes past the last)
    uint32_t ex = 0, tot = 0, off = 0, win = 0;
    bool wide = false;
    if (SP1) {
      const uint32_t v = __popc(Bw);
      uint32_t x = v;
#pragma unroll
      for (int o = 1; o < 16; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (uint32_t)o) x += y;
      }
      ex = x - v;
      tot = __shfl_sync(0xFFFFFFFFu, x, 15);
      if (tot) {
        const uintptr_t p0 = reinterpret_cast<uintptr_t>(ob + Rc);
        off = (uint32_t)(p0 & 3u);
        const uint32_t nwin = (off + tot + 3) >> 2;
        wide = nwin > 32;
        if (!wide && lane < nwin) win = __ldg(reinterpret_cast<const uint32_t *>(p0 - off) + lane);
      }
    }
#pragma unroll
    for (int m = 0; m < 4; ++m) {
      const uint32_t row0 = r0 + m * 128 + 4 * lane;
      // SP1: the 4 rows' sparse bytes in one word (byte i = row i): the
      // default byte, or an outlier row's byte -- from the lane's 4 outlier
      // bits in this group and the 4 outlier bytes from its first outlier's
      // rank within the chunk
      uint32_t spw = spd4;
      if (SP1 && tot) {
        const uint32_t src = 4 * m + (lane >> 3), sh = 4 * (lane & 7);
        const uint32_t Wm = __shfl_sync(0xFFFFFFFFu, Bw, src);
        const uint32_t Em = __shfl_sync(0xFFFFFFFFu, ex, src);
        const uint32_t nib = (Wm >> sh) & 0xFu;
        const uint32_t k0 = Em + __popc(Wm & ((1u << sh) - 1u));
        uint32_t b4 = 0;
        if (!wide) {
          const uint32_t pos = off + k0;
          const uint32_t w0 = __shfl_sync(0xFFFFFFFFu, win, (pos >> 2) & 31);
          const uint32_t w1 = __shfl_sync(0xFFFFFFFFu, win, ((pos >> 2) + 1) & 31);
          b4 = __funnelshift_r(w0, w1, 8 * (pos & 3));
        } else {
          const uint32_t no = __popc(nib);
#pragma unroll
          for (uint32_t j = 0; j < 4; ++j)
            if (j < no) b4 |= (uint32_t)__ldg(ob + Rc + k0 + j) << (8 * j);
        }
        // row i takes byte popc(nib & (2^i - 1)): bit k < 3 of nib moved to
        // nibble k + 1 (the three shifted copies do not overlap), then each
        // nibble summed with those below it
        const uint32_t e = ((nib & 7u) * 0x490u) & 0x1110u;
        const uint32_t rows = __byte_perm(b4, 0u, e * 0x1111u);
        const uint32_t msk = expand4(nib);
        spw = (rows & msk) | (spd4 & ~msk);
      }
      uint32_t W[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) W[j] = j < KS ? sw[m][KS - 1 - j] : 0u;
      const uint32_t t0 = __byte_perm(W[0], W[1], 0x5140), t1 = __byte_perm(W[0], W[1], 0x7362);
      const uint32_t t2 = __byte_perm(W[2], W[3], 0x5140), t3 = __byte_perm(W[2], W[3], 0x7362);
      const uint32_t c[4] = {__byte_perm(t0, t2, 0x5410), __byte_perm(t0, t2, 0x7632),
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
        // (xhi:xlo) = sparse byte above the dense bytes; then << ts | field
        uint32_t xlo = c[i] ^ kx, xhi = 0;
        if (SP1) {
          const uint32_t sp = __byte_perm(spw, 0u, 0x4440 + i);
          if (KS == 4)
            xhi = sp;
          else
            xlo |= sp << (8 * (KS & 3));
        }
        uint32_t hi = __funnelshift_l(xlo, xhi, ts);
        uint32_t lo = (xlo << ts) | ((f >> (i * ts)) & tmask);
        if (!SP1) {
          hi |= sdef_hi;
          lo |= sdef_lo;
        }
        const unsigned long long A =
            (unsigned long long)a.base + (((unsigned long long)hi << 32) | lo);
        if (CV == kCvI32)
          v[i] = i32_to_f64_scaled((int)((uint32_t)a.base + lo), a.dlen);
        else if (CV == kCvU53)
          v[i] = u53w_to_f64_scaled((uint32_t)(A >> 32), (uint32_t)A, a.dlen);
        else if (CV == kCvS53)
          v[i] = s53_to_f64_scaled(A, a.dlen);
        else
          v[i] = i64_to_f64_scaled((long long)A, a.dlen);
      }
      double *o = a.out + row0;
      if (row0 + 4 <= a.n) {
        if (ST32) {
          asm volatile("st.global.cs.v4.f64 [%0], {%1, %2, %3, %4};" ::"l"(o), "d"(v[0]),
                       "d"(v[1]), "d"(v[2]), "d"(v[3])
                       : "memory");
        } else {
          __stcs(reinterpret_cast<double2 *>(o), make_double2(v[0], v[1]));
          __stcs(reinterpret_cast<double2 *>(o + 2), make_double2(v[2], v[3]));
        }
      } else {
#pragma unroll
        for (int i = 0; i < 4; ++i)
          if (row0 + i < a.n) o[i] = v[i];
      }
    }
  }
}

// Rows that are outliers in some sparse column, decoded in full after
// k_rapg_decode_fast wrote them with zero sparse bytes: one thread per
// 32-row bitmap word, the rows of the union of the columns' words.
__global__ void __launch_bounds__(kThreads) k_rapg_fixup(RapgDecodeArgs a) {
  const size_t nw = ((size_t)a.n + 31) / 32;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nw;
       w += (size_t)gridDim.x * blockDim.x) {
    // bitmap words and ranks of all sparse columns, loaded together
    uint32_t Bw[8], Rk[8], any = 0;
#pragma unroll
    for (uint32_t c = 0; c < 8; ++c) {
      Bw[c] = c < a.m ? __ldg(a.obits + c * a.nwp + w) : 0u;
      Rk[c] = c < a.m ? __ldg(a.orank + c * a.rs + w) : 0u;
      any |= Bw[c];
    }
    while (any) {
      const uint32_t j = __ffs(any) - 1;
      any &= any - 1;
      const uint32_t i = (uint32_t)(w * 32 + j);
      unsigned long long v = 0;
#pragma unroll
      for (uint32_t c = 0; c < 8; ++c) {
        if (c < a.m) {
          uint32_t b = a.smaj[c];
          if (Bw[c] >> j & 1u) b = a.obytes[a.oofs[c] + Rk[c] + __popc(Bw[c] & ((1u << j) - 1u))];
          v = (v << 8) | b;
        }
      }
      for (uint32_t d = 0; d < a.ks; ++d) v = (v << 8) | (a.slices[d * a.stride + i] ^ 0x80u);
      if (a.ts) v = (v << a.ts) | field_from(a.tail, 0, a.ts, i);
      a.out[i] = i64_to_f64_scaled((long long)((unsigned long long)a.base + v), a.dlen);
    }
  }
}

// The same fix-up when every value the fast pass wrote is exact (|base| +
// 2^R < 2^53): an outlier row's written value is read back as its integer
// code -- exact, since value * 2^dlen is an integer below 2^53 -- and only
// its sparse bytes are replaced, so the dense slices and the tail are not
// read again.  `low` = bits below the sparse bytes.
__global__ void __launch_bounds__(kThreads) k_rapg_fixup_patch(RapgDecodeArgs a, uint32_t low,
                                                               double scale) {
  const size_t nw = ((size_t)a.n + 31) / 32;
  const unsigned long long lowmask = (1ull << low) - 1ull;
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nw;
       w += (size_t)gridDim.x * blockDim.x) {
    uint32_t Bw[8], Rk[8], any = 0;
#pragma unroll
    for (uint32_t c = 0; c < 8; ++c) {
      Bw[c] = c < a.m ? __ldg(a.obits + c * a.nwp + w) : 0u;
      any |= Bw[c];
    }
    if (!any) continue;
#pragma unroll
    for (uint32_t c = 0; c < 8; ++c) Rk[c] = c < a.m ? __ldg(a.orank + c * a.rs + w) : 0u;
    while (any) {
      const uint32_t j = __ffs(any) - 1;
      any &= any - 1;
      const uint32_t i = (uint32_t)(w * 32 + j);
      unsigned long long sp = 0;
#pragma unroll
      for (uint32_t c = 0; c < 8; ++c) {
        if (c < a.m) {
          uint32_t b = a.smaj[c];
          if (Bw[c] >> j & 1u) b = a.obytes[a.oofs[c] + Rk[c] + __popc(Bw[c] & ((1u << j) - 1u))];
          sp = (sp << 8) | b;
        }
      }
      const long long whole = __double2ll_rn(a.out[i] * scale);  // base + written code
      const unsigned long long code =
          ((unsigned long long)(whole - a.base) & lowmask) | (sp << low);
      a.out[i] = i64_to_f64_scaled((long long)((unsigned long long)a.base + code), a.dlen);
    }
  }
}

// k_rapg_fixup_patch for one sparse column: a warp takes 32 bitmap words
// (1,024 rows) per step, the lanes' outlier ranks come from the step's first
// rank word plus a prefix count of the lanes before, and the next step's
// bitmap and rank words are loaded before this step's outlier bytes and
// written values are read -- one dependent load per step instead of three
// per word.
__global__ void __launch_bounds__(kThreads) k_rapg_fixup_patch1(RapgDecodeArgs a, uint32_t low,
                                                                double scale) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t step = ((gridDim.x * blockDim.x) >> 5) * 32;
  const uint32_t nwords = (a.n + 31) / 32;
  const unsigned long long lowmask = (1ull << low) - 1ull;
  const uint8_t *ob = a.obytes + a.oofs[0];
  uint32_t nB = 0, nR0 = 0;
  if (warp * 32 < nwords) nR0 = __ldg(a.orank + warp * 32);
  if (warp * 32 + lane < nwords) nB = __ldg(a.obits + warp * 32 + lane);
  // the written values are the dense pass's: wait for it (the bitmap and
  // rank loads above do not depend on it; a no-op when launched plainly)
  asm volatile("griddepcontrol.wait;" ::: "memory");
  for (uint32_t base = warp * 32; base < nwords; base += step) {
    const uint32_t w = base + lane;
    const uint32_t B = w < nwords ? nB : 0u, R0 = nR0;
    if (base + step < nwords) nR0 = __ldg(a.orank + base + step);
    if (w + step < nwords) nB = __ldg(a.obits + w + step);
    const uint32_t v = __popc(B);
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
      if (lane >= (uint32_t)o) x += y;
    }
    uint32_t k = R0 + x - v;  // rank of the lane's first outlier
    for (uint32_t b = B; b; b &= b - 1, ++k) {
      const uint32_t i = w * 32 + (__ffs(b) - 1);
      const unsigned long long sp = (unsigned long long)__ldg(ob + k);
      const long long whole = __double2ll_rn(a.out[i] * scale);  // base + written code
      const unsigned long long code =
          ((unsigned long long)(whole - a.base) & lowmask) | (sp << low);
      a.out[i] = i64_to_f64_scaled((long long)((unsigned long long)a.base + code), a.dlen);
    }
  }
}

__global__ void k_field_sum(const uint8_t *p, unsigned long long bit0, uint32_t width, uint32_t n,
                            unsigned long long *out) {
  unsigned long long acc = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    acc += field_from(p, bit0, width, i);
  acc = warp_sum_ull(acc);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

// The same sum for fields of 1..7 bits as a weighted popcount over the
// stream's 32-bit words (wpopc: stream bit q weighs 2^((q - bit0) mod width)),
// the words at both ends masked to [bit0, bit0 + nbits): one load per 32 bits
// instead of a field extraction per row.  The phase of a thread's next word
// advances by conditional subtraction, without a division in the loop.
__global__ void k_field_sum_words(const uint8_t *__restrict__ p, unsigned long long bit0,
                                  uint32_t width, unsigned long long nbits,
                                  unsigned long long *out) {
  const unsigned long long b_end = bit0 + nbits;
  const unsigned long long w0 = bit0 >> 5, w1 = (b_end + 31) >> 5, wfull = b_end >> 5;
  const unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  const unsigned long long nth = (unsigned long long)gridDim.x * blockDim.x;
  unsigned long long v = w0 + tid;
  long long d = (long long)(v * 32) - (long long)bit0;  // stream position of the word's bit 0
  int ph = (int)(d % (long long)width);
  if (ph < 0) ph += (int)width;
  const uint32_t step = (uint32_t)((nth * 32) % width);
  unsigned long long acc = 0;
  for (; v < w1; v += nth) {
    uint32_t word;
    if (v < wfull) {
      word = __ldg(reinterpret_cast<const uint32_t *>(p) + v);
    } else {  // the last, partial word: only the bytes holding stream bits
      word = 0;
      const unsigned long long nb = (b_end - v * 32 + 7) / 8;
      for (uint32_t k = 0; k < nb; ++k) word |= (uint32_t)__ldg(p + v * 4 + k) << (8 * k);
    }
    const unsigned long long lo = v * 32;
    if (lo < bit0) word &= ~0u << (uint32_t)(bit0 - lo);
    if (lo + 32 > b_end) word &= (1u << (uint32_t)(b_end - lo)) - 1u;
    acc += wpopc(word, (uint32_t)ph, width);
    ph += (int)step;
    if (ph >= (int)width) ph -= (int)width;
  }
  acc = warp_sum_ull(acc);
  if ((threadIdx.x & 31) == 0 && acc) atomicAdd(out, acc);
}

__global__ void k_xor80(uint8_t *p, size_t nbytes) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < nbytes;
       i += (size_t)gridDim.x * blockDim.x)
    p[i] ^= 0x80u;
}

__global__ void k_word_popc(const uint32_t *__restrict__ bits, size_t nw, uint32_t *cnt) {
  for (size_t w = blockIdx.x * (size_t)blockDim.x + threadIdx.x; w < nw;
       w += (size_t)gridDim.x * blockDim.x)
    cnt[w] = __popc(bits[w]);
}

int grid_of(size_t items, int threads) {
  size_t g = (items + threads - 1) / threads;
  int dev = 0;
  cudaGetDevice(&dev);
  const size_t cap = (size_t)8 * num_sms(dev);
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

}  // namespace

// Exclusive scan of `count` u32 in place; data[count] receives the total.
// tmp: exclusive_scan_tmp(count) u32 of device scratch.
size_t exclusive_scan_tmp(size_t count) { return scan_blocks(count) + 1; }
cudaError_t exclusive_scan(uint32_t *data, size_t count, uint32_t *tmp, cudaStream_t s) {
  return scan_exclusive(data, count, tmp, s);
}

// ================================================================ host side

cudaError_t flip_bytes(uint8_t *p, size_t nbytes, cudaStream_t s) {
  if (!nbytes) return cudaSuccess;
  k_xor80<<<grid_of(nbytes, 256), 256, 0, s>>>(p, nbytes);
  count_launch();
  return cudaGetLastError();
}

// Ranks and last-outlier rows of already loaded bitmaps (deserialize).
cudaError_t major_index(buff_col *c, cudaStream_t s) {
  cudaError_t e;
  const size_t rs = rank_stride(c);
  uint32_t *tmp = nullptr, *dlast = nullptr;
  const size_t nb = (c->nwp + kScanItems - 1) / kScanItems + 1;
  e = cudaMallocAsync(reinterpret_cast<void **>(&tmp), sizeof(uint32_t) * nb, s);
  if (e != cudaSuccess) return e;
  e = cudaMallocAsync(reinterpret_cast<void **>(&dlast), sizeof(uint32_t) * 8, s);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(dlast, 0, sizeof(uint32_t) * 8, s);
  for (uint32_t col = 0; col < c->m; ++col) {
    const uint32_t *bits = c->obits + col * c->nwp;
    uint32_t *rank = c->orank + col * rs;
    k_word_popc<<<grid_of(c->nwp, 256), 256, 0, s>>>(bits, c->nwp, rank);
    k_major_last<<<grid_of(c->nwp, 256), 256, 0, s>>>(bits, c->nwp, dlast + col);
    count_launch(2);
    if ((e = scan_exclusive(rank, c->nwp, tmp, s)) != cudaSuccess) return e;
  }
  uint32_t last[8];
  cudaMemcpyAsync(last, dlast, sizeof(uint32_t) * 8, cudaMemcpyDeviceToHost, s);
  e = cudaStreamSynchronize(s);
  for (uint32_t col = 0; col < c->m; ++col) c->olast[col] = last[col];
  cudaFreeAsync(tmp, s);
  cudaFreeAsync(dlast, s);
  return e != cudaSuccess ? e : cudaGetLastError();
}

cudaError_t major_build_sparse(buff_col *c, const uint8_t *lead, cudaStream_t s) {
  // bitmaps, ranks and compacted outlier bytes from the `m` leading slices
  cudaError_t e;
  const size_t rs = rank_stride(c);
  e = cudaMallocAsync(reinterpret_cast<void **>(&c->obits), sizeof(uint32_t) * c->m * c->nwp, s);
  if (e != cudaSuccess) return e;
  e = cudaMallocAsync(reinterpret_cast<void **>(&c->orank), sizeof(uint32_t) * c->m * rs, s);
  if (e != cudaSuccess) return e;
  uint32_t *tmp = nullptr, *dlast = nullptr;
  const size_t nb = (c->nwp + kScanItems - 1) / kScanItems + 1;
  e = cudaMallocAsync(reinterpret_cast<void **>(&tmp), sizeof(uint32_t) * nb, s);
  if (e != cudaSuccess) return e;
  e = cudaMallocAsync(reinterpret_cast<void **>(&dlast), sizeof(uint32_t) * 8, s);
  if (e != cudaSuccess) return e;
  cudaMemsetAsync(dlast, 0, sizeof(uint32_t) * 8, s);
  for (uint32_t col = 0; col < c->m; ++col) {
    uint32_t *bits = c->obits + col * c->nwp, *rank = c->orank + col * rs;
    k_major_bits<<<grid_of(c->nwp, 256), 256, 0, s>>>(lead + col * c->stride, c->n, c->majors[col],
                                                      c->nwp, bits, rank);
    k_major_last<<<grid_of(c->nwp, 256), 256, 0, s>>>(bits, c->nwp, dlast + col);
    count_launch(2);
    if ((e = scan_exclusive(rank, c->nwp, tmp, s)) != cudaSuccess) return e;
  }
  uint32_t totals[8], last[8];
  for (uint32_t col = 0; col < c->m; ++col)
    cudaMemcpyAsync(&totals[col], c->orank + col * rs + c->nwp, 4, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(last, dlast, sizeof(uint32_t) * 8, cudaMemcpyDeviceToHost, s);
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;
  uint64_t off = 0;
  for (uint32_t col = 0; col < c->m; ++col) {
    c->nout[col] = totals[col];
    c->olast[col] = last[col];
    c->oofs[col] = off;
    off += totals[col];
  }
  c->oofs[c->m] = off;
  e = cudaMallocAsync(reinterpret_cast<void **>(&c->obytes), off + 16, s);
  if (e != cudaSuccess) return e;
  for (uint32_t col = 0; col < c->m; ++col) {
    k_major_compact<<<grid_of(c->nwp, 256), 256, 0, s>>>(lead + col * c->stride,
                                                         c->obits + col * c->nwp,
                                                         c->orank + col * rs, c->nwp,
                                                         c->obytes + c->oofs[col]);
    count_launch();
  }
  cudaFreeAsync(tmp, s);
  cudaFreeAsync(dlast, s);
  return cudaGetLastError();
}

cudaError_t major_filter(const buff_col *c, int is_range, const uint8_t *tbyte, uint32_t ttail,
                         uint32_t *words, unsigned long long *count, cudaStream_t s,
                         const uint32_t *cand) {
  MajorArgs a;
  memset(&a, 0, sizeof(a));
  a.cand = cand;
  a.n = c->n;
  a.m = c->m;
  a.kd = c->k - c->m;
  a.r = c->r;
  a.nwp = c->nwp;
  a.rs = rank_stride(c);
  a.stride = c->stride;
  a.obits = c->obits;
  a.orank = c->orank;
  a.obytes = c->obytes;
  for (uint32_t i = 0; i < 8; ++i) {
    a.oofs[i] = c->oofs[i];
    a.majors[i] = c->majors[i];
    a.tbyte[i] = tbyte[i];
  }
  a.ttail = ttail;
  a.slices = c->slices;
  a.tail = c->tail;
  a.words = words;
  a.count = count;
  const size_t nw = (c->n + 31) / 32;
  if (c->m == 1 && !cand && a.kd >= 1 && c->majors[0] == tbyte[0]) {
    // one wave: 4 resident CTAs per SM (the kernel's launch bounds), fewer
    // when the column needs fewer warps
    int dev = 0;
    cudaGetDevice(&dev);
    const size_t need = (nw + kThreads - 1) / kThreads;
    const size_t cap = (size_t)4 * num_sms(dev);
    const int grid = (int)(need < cap ? (need ? need : 1) : cap);
    const int th = (a.tbyte[1] >> 7) | ((a.kd >= 2 ? a.tbyte[2] >> 7 : 0) << 1);
    void (*fn)(MajorArgs);
    if (is_range)
      fn = th == 0 ? k_filter_major1<true, false, false>
         : th == 1 ? k_filter_major1<true, true, false>
         : th == 2 ? k_filter_major1<true, false, true> : k_filter_major1<true, true, true>;
    else
      fn = th == 0 ? k_filter_major1<false, false, false>
         : th == 1 ? k_filter_major1<false, true, false>
         : th == 2 ? k_filter_major1<false, false, true> : k_filter_major1<false, true, true>;
    fn<<<grid, kThreads, 0, s>>>(a);
    count_launch();
    return cudaGetLastError();
  }
  const int grid = grid_of(nw, kThreads);
  if (c->m == 1 && !cand && a.kd == 0 && a.r <= 7) {
    if (is_range)
      launch_filter_major0<true>(a, grid, s);
    else
      launch_filter_major0<false>(a, grid, s);
  } else if (is_range) {
    k_filter_major<true><<<grid, kThreads, 0, s>>>(a);
  } else {
    k_filter_major<false><<<grid, kThreads, 0, s>>>(a);
  }
  count_launch();
  return cudaGetLastError();
}

// Exclusive prefix counts of set bits per word (rank[0..nw), total at
// rank[nw]); rank needs nw + 1 entries.
namespace {
}  // namespace

cudaError_t major_sums(const buff_col *c, const MajorSumArgs &a, unsigned long long *raw,
                       double *sum, unsigned long long *parts, cudaStream_t s) {
  cudaError_t e = zero_u64(raw, 24, s);
  if (e != cudaSuccess) return e;
  SparseBytes sb;
  memset(&sb, 0, sizeof(sb));
  sb.m = c->m;
  for (uint32_t col = 0; col < c->m; ++col) {
    sb.p[col] = c->obytes + c->oofs[col];
    sb.n[col] = c->nout[col];
  }
  static std::atomic<int> per_sm_cache{0};
  int per_sm = per_sm_cache.load(std::memory_order_relaxed);
  if (!per_sm) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sum_major, kThreads, 0);
    if (per_sm < 1) per_sm = 1;
    per_sm_cache.store(per_sm, std::memory_order_relaxed);
  }
  // enough threads for the larger of a slice's 16-byte vectors and the
  // outlier bytes, at most the resident grid
  size_t big = c->stride / 16;
  for (uint32_t col = 0; col < c->m; ++col) big = std::max(big, (size_t)c->nout[col] / 16 + 1);
  size_t grid = (big + kThreads - 1) / kThreads;
  const size_t cap = (size_t)per_sm * num_sms(c->device);
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  k_sum_major<<<(unsigned)grid, kThreads, 0, s>>>(c->slices, c->stride, c->k - c->m, c->tail, c->r,
                                                  (unsigned long long)c->n * c->r, sb, a, raw, sum,
                                                  parts);
  count_launch();
  return cudaGetLastError();
}

cudaError_t major_bytesum(const uint8_t *p, size_t nbytes, unsigned long long *out, cudaStream_t s) {
  k_bytesum<<<grid_of(nbytes / 16 + 1, 256), 256, 0, s>>>(p, nbytes, out);
  count_launch();
  return cudaGetLastError();
}

namespace {
// buff_max_majority (buff_simd.rs:2444-2861) of a column with one sparse
// byte column and rows outside it: its progressive max is then the largest
// full code, whose leading byte is a row's outlier byte or else the major
// byte M.  One pass finds it as k_max does: a lane owns 32 rows (one bitmap
// word, its outlier bytes reached through the warp's rank and a prefix count
// of the lanes before it); a step whose largest leading byte is below the
// running maximum's is skipped without touching the dense slices, otherwise
// the lanes holding that byte take the largest code among those rows
// (max_after_top over the dense slices and the tail), and the warp
// publishes its best into *out and raises its threshold from it.
__global__ void __launch_bounds__(kThreads) k_major1_max(const uint32_t *__restrict__ bits,
                                                         const uint32_t *__restrict__ rank,
                                                         const uint8_t *__restrict__ ob,
                                                         uint32_t M, uint32_t n,
                                                         const uint8_t *__restrict__ slices,
                                                         size_t stride, uint32_t kd,
                                                         const uint8_t *__restrict__ tail,
                                                         uint32_t r, uint32_t fl,
                                                         unsigned long long *out) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t nwords = (n + 31) / 32;
  const uint32_t step = nwarps * 32;
  unsigned long long best = 0;
  bool have = false;
  uint32_t top = 0;  // leading byte of best
  // the bitmap word and the warp's rank of the next step are loaded before
  // this step's outlier bytes are read
  uint32_t nB = 0, nR0 = 0;
  if (warp * 32 < nwords) nR0 = __ldg(rank + warp * 32);
  if (warp * 32 + lane < nwords) nB = __ldg(bits + warp * 32 + lane);
  for (uint32_t base = warp * 32; base < nwords; base += step) {
    const uint32_t w = base + lane;
    const bool live = w < nwords;
    const uint32_t B = live ? nB : 0u, R0 = nR0;
    if (base + step < nwords) nR0 = __ldg(rank + base + step);
    if (w + step < nwords) nB = __ldg(bits + w + step);
    const uint32_t row0 = w * 32;
    const uint32_t valid =
        !live ? 0u : (n - row0 >= 32 ? 0xFFFFFFFFu : ((1u << (n - row0)) - 1u));
    uint32_t R;
    {
      const uint32_t v = __popc(B);
      uint32_t x = v;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (uint32_t)o) x += y;
      }
      R = R0 + x - v;
    }
    const uint32_t non = ~B & valid;
    uint32_t L = non ? M : 0u;  // the lane's largest leading byte
    for (uint32_t b = B, k = 0; b; ++k, b &= b - 1) L = max(L, (uint32_t)__ldg(ob + R + k));
    const bool rows = valid != 0;
    const uint32_t wl = __reduce_max_sync(0xFFFFFFFFu, rows ? L : 0u);
    if (have && wl < top) continue;  // nothing in this step reaches the running maximum
    unsigned long long m = 0;
    if (rows && L == wl) {
      uint32_t cand = wl == M ? non : 0u;  // outlier bytes differ from M
      if (wl != M) {
        uint32_t b = B;
        for (uint32_t k = 0; b; ++k, b &= b - 1)
          if (__ldg(ob + R + k) == wl) cand |= b & (0u - b);
      }
      m = max_after_top(slices, stride, kd, tail, r, row0, cand, wl);
    }
    m = warp_max_ull(m);
    if (!have || m > best) best = m;
    have = true;
    unsigned long long g = 0;
    if (lane == 0) g = atomicMax(out, best);
    g = __shfl_sync(0xFFFFFFFFu, g, 0);
    if (g > best) best = g;
    top = (uint32_t)(best >> (fl - 8)) & 0xFFu;
  }
  if (lane == 0 && have) atomicMax(out, best);
}
}  // namespace

bool major1_max_applies(const buff_col *c) { return c->m == 1 && c->nout[0] < c->n; }

cudaError_t major1_max(const buff_col *c, unsigned long long *out, cudaStream_t s) {
  cudaError_t e = zero_u64(out, 1, s);
  if (e != cudaSuccess || !c->n) return e;
  static std::atomic<int> per_sm_cache{0};
  int per_sm = per_sm_cache.load(std::memory_order_relaxed);
  if (!per_sm) {
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_major1_max, kThreads, 0);
    if (per_sm < 1) per_sm = 1;
    per_sm_cache.store(per_sm, std::memory_order_relaxed);
  }
  const size_t steps = ((size_t)c->n + 1023) / 1024;  // one per warp at a time
  size_t grid = (steps + kThreads / 32 - 1) / (kThreads / 32);
  const size_t cap = (size_t)per_sm * num_sms(c->device);
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  k_major1_max<<<(unsigned)grid, kThreads, 0, s>>>(c->obits, c->orank, c->obytes + c->oofs[0],
                                                   c->majors[0], c->n, c->slices, c->stride,
                                                   c->k - 1, c->tail, c->r, c->fixed_len, out);
  count_launch();
  return cudaGetLastError();
}

// buff_max_majority's progressive max (buff_simd.rs:2444-2861) with every
// step's decision made on the device; one host synchronization at the end.
cudaError_t major_max(const buff_col *c, uint32_t *cand, void *state_dev, cudaStream_t s) {
  MaxState *st = static_cast<MaxState *>(state_dev);
  const size_t nw = ((size_t)c->n + 31) / 32;
  const uint32_t kd = c->k - c->m;
  const int g = grid_of(c->nwp, 256);
  static_assert(sizeof(MaxState) % 8 == 0, "MaxState is zeroed as u64 words");
  cudaError_t e =
      zero_u64(reinterpret_cast<unsigned long long *>(st), sizeof(MaxState) / 8, s);
  if (e != cudaSuccess) return e;
  uint32_t step = 0;
  for (uint32_t col = 0; col < c->m; ++col, ++step) {
    const uint32_t *bits = c->obits + col * c->nwp, *rank = c->orank + col * rank_stride(c);
    const uint8_t *ob = c->obytes + c->oofs[col];
    k_major_candmax<<<g, 256, 0, s>>>(bits, rank, ob, col == 0 ? nullptr : cand, c->nwp,
                                      st->best + step, st->flag + step);
    k_major_select<<<g, 256, 0, s>>>(bits, rank, ob, cand, c->nwp, c->n, st->best + step,
                                     st->flag + step, c->majors[col],
                                     c->fixed_len - 8 * (col + 1), col == 0 ? 1 : 0, &st->mx);
    count_launch(2);
  }
  const int gw = grid_of(nw, 256);
  for (uint32_t j = 0; j < kd; ++j, ++step) {  // dense slices (:2560-2612)
    const uint8_t *sl = c->slices + (size_t)j * c->stride;
    const uint32_t sh = c->fixed_len - 8 * (c->m + j + 1);
    k_cand_max<0><<<gw, 256, 0, s>>>(sl, nullptr, cand, nw, st->best + step);
    k_cand_select<0><<<gw, 256, 0, s>>>(sl, nullptr, cand, nw, st->best + step, sh, &st->mx,
                                        nullptr);
    count_launch(2);
  }
  if (c->r) {  // tail (:2613-2651): its candidates are the arg-max rows
    switch (c->r) {
#define TAIL_STEP(R)                                                                        \
  case R:                                                                                   \
    k_cand_max<R><<<gw, 256, 0, s>>>(nullptr, c->tail, cand, nw, st->best + step);          \
    k_cand_select<R><<<gw, 256, 0, s>>>(nullptr, c->tail, cand, nw, st->best + step, 0,     \
                                        &st->mx, &st->count);                               \
    break;
      TAIL_STEP(1) TAIL_STEP(2) TAIL_STEP(3) TAIL_STEP(4) TAIL_STEP(5) TAIL_STEP(6)
      TAIL_STEP(7)
#undef TAIL_STEP
      default: return cudaErrorInvalidValue;
    }
    count_launch(2);
  } else {
    // nwp is a multiple of 16 (the slice stride is a multiple of 512 rows)
    e = zero_u64(reinterpret_cast<unsigned long long *>(cand), c->nwp / 2, s);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

size_t major_max_state_bytes() { return sizeof(MaxState); }
size_t major_max_state_mx_offset() { return offsetof(MaxState, mx); }

cudaError_t popcount_words(const uint32_t *w, size_t nw, unsigned long long *out, cudaStream_t s) {
  k_popc<<<grid_of(nw, 256), 256, 0, s>>>(w, nw, out);
  count_launch();
  return cudaGetLastError();
}

cudaError_t field_sum(const uint8_t *p, uint64_t bit0, uint32_t width, uint32_t n,
                      unsigned long long *out, cudaStream_t s) {
  if (!n || !width) return cudaSuccess;
  if (width <= 7) {
    const unsigned long long nbits = (unsigned long long)n * width;
    const size_t words = (size_t)(((bit0 + nbits + 31) >> 5) - (bit0 >> 5));
    k_field_sum_words<<<grid_of(words, 256), 256, 0, s>>>(p, bit0, width, nbits, out);
  } else {
    k_field_sum<<<grid_of(n, 256), 256, 0, s>>>(p, bit0, width, n, out);
  }
  count_launch();
  return cudaGetLastError();
}

// The fast decode of a plan whose slice reads stay in the dense region and
// whose tail fields start at bit 0, then the outlier rows.
template <bool N32>
static void launch_fast_ks(const RapgDecodeArgs &a, int g, cudaStream_t s) {
  switch (a.ks) {
    case 0: k_rapg_decode_fast<0, N32><<<g, kThreads, 0, s>>>(a); break;
    case 1: k_rapg_decode_fast<1, N32><<<g, kThreads, 0, s>>>(a); break;
    case 2: k_rapg_decode_fast<2, N32><<<g, kThreads, 0, s>>>(a); break;
    case 3: k_rapg_decode_fast<3, N32><<<g, kThreads, 0, s>>>(a); break;
    case 4: k_rapg_decode_fast<4, N32><<<g, kThreads, 0, s>>>(a); break;
    case 5: k_rapg_decode_fast<5, N32><<<g, kThreads, 0, s>>>(a); break;
    case 6: k_rapg_decode_fast<6, N32><<<g, kThreads, 0, s>>>(a); break;
    case 7: k_rapg_decode_fast<7, N32><<<g, kThreads, 0, s>>>(a); break;
    default: k_rapg_decode_fast<8, N32><<<g, kThreads, 0, s>>>(a); break;
  }
}

template <int KS, int CV, bool SP1>
static void launch_fast4_cv(const RapgDecodeArgs &a, int g, cudaStream_t s) {
  if ((reinterpret_cast<uintptr_t>(a.out) & 31u) == 0)
    k_rapg_decode_fast4<KS, CV, true, SP1><<<g, kThreads, 0, s>>>(a);
  else
    k_rapg_decode_fast4<KS, CV, false, SP1><<<g, kThreads, 0, s>>>(a);
}

// The conversion form: every value in 32 bits; else every base + code in
// [1, 2^53) (unsigned, exact, no zero); else every |base + code| below 2^53
// (exact); else the rounding 64-bit form.  One sparse column: the outlier rows are
// decoded in the pass itself.
template <int KS, bool SP1>
static void launch_fast4_sp(const RapgDecodeArgs &a, bool n32, int g, cudaStream_t s) {
  const unsigned long long ab =
      a.base < 0 ? 0ull - (unsigned long long)a.base : (unsigned long long)a.base;
  const bool exact = a.R <= 52 && ab < (1ull << 53) - (1ull << a.R) && a.dlen <= 1000;
  if (n32)
    launch_fast4_cv<KS, kCvI32, SP1>(a, g, s);
  else if (exact && a.base >= 1)
    launch_fast4_cv<KS, kCvU53, SP1>(a, g, s);
  else if (exact)
    launch_fast4_cv<KS, kCvS53, SP1>(a, g, s);
  else
    launch_fast4_cv<KS, kCvI64, SP1>(a, g, s);
}
template <int KS>
static void launch_fast4(const RapgDecodeArgs &a, bool n32, int g, cudaStream_t s) {
  if (KS == 0 || a.m == 1)
    launch_fast4_sp<KS, true>(a, n32, g, s);
  else
    launch_fast4_sp<KS, KS == 0>(a, n32, g, s);
}

// The rows that are outliers in some sparse column, after a fast pass wrote
// every row with the default sparse bytes: patched in place while every value
// is exact (one sparse column: k_rapg_fixup_patch1, launched as a
// programmatic dependent of the pass), else rebuilt from the slices.
static void launch_fixup(const RapgDecodeArgs &a, cudaStream_t s) {
  const uint32_t low = 8 * a.ks + a.ts;
  const unsigned long long ab =
      a.base < 0 ? 0ull - (unsigned long long)a.base : (unsigned long long)a.base;
  const int gw = grid_of(((size_t)a.n + 31) / 32, kThreads);
  const bool patch =
      a.R <= 52 && low < 64 && ab < (1ull << 53) - (1ull << a.R) && a.dlen <= 1000;
  if (patch && a.m == 1) {
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3((unsigned)grid_of(((size_t)a.n + 1023) / 1024 * 32, kThreads));
    cfg.blockDim = dim3(kThreads);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, k_rapg_fixup_patch1, a, low, ldexp(1.0, a.dlen));
  } else if (patch) {
    k_rapg_fixup_patch<<<gw, kThreads, 0, s>>>(a, low, ldexp(1.0, a.dlen));
  } else {
    k_rapg_fixup<<<gw, kThreads, 0, s>>>(a);
  }
  count_launch();
}

static void launch_decode_fast(const RapgDecodeArgs &a, cudaStream_t s) {
  if ((a.ks >= 1 && a.ks <= 4) || (a.ks == 0 && a.m == 1)) {
    const int g = grid_of((size_t)(a.n + kRowChunk - 1) / kRowChunk * 32, kThreads);
    const long long maxc = a.R >= 63 ? -1 : (long long)((1ull << a.R) - 1ull);
    const bool n32 =
        a.R <= 32 && a.base >= INT32_MIN && maxc >= 0 && a.base + maxc <= (long long)INT32_MAX;
    switch (a.ks) {
      case 0: launch_fast4<0>(a, n32, g, s); break;
      case 1: launch_fast4<1>(a, n32, g, s); break;
      case 2: launch_fast4<2>(a, n32, g, s); break;
      case 3: launch_fast4<3>(a, n32, g, s); break;
      default: launch_fast4<4>(a, n32, g, s); break;
    }
    count_launch();
    if (a.m > 1) launch_fixup(a, s);
    return;
  }
  {
    const int g = grid_of((size_t)(a.n + kRowChunk - 1) / kRowChunk * 32, kThreads);
    // every value base + code (R bits) in 32 bits: the 32-bit build and conversion
    const long long maxc = a.R >= 63 ? -1 : (long long)((1ull << a.R) - 1ull);
    if (a.R <= 32 && a.base >= INT32_MIN && maxc >= 0 && a.base + maxc <= (long long)INT32_MAX)
      launch_fast_ks<true>(a, g, s);
    else
      launch_fast_ks<false>(a, g, s);
    count_launch();
    if (a.m) launch_fixup(a, s);
  }
}

cudaError_t rapg_decode(const buff_col *c, uint32_t R, uint32_t ks, uint32_t ts, uint64_t tbit0,
                        double *out, cudaStream_t s) {
  if (!c->n) return cudaSuccess;
  RapgDecodeArgs a;
  memset(&a, 0, sizeof(a));
  a.obits = c->obits;
  a.orank = c->orank;
  a.obytes = c->obytes;
  for (uint32_t i = 0; i < 8; ++i) a.oofs[i] = c->oofs[i];
  a.nwp = c->nwp;
  a.rs = rank_stride(c);
  a.stride = c->stride;
  a.slices = c->slices;
  a.tail = c->tail;
  a.n = c->n;
  a.m = c->m;
  a.kd = c->k - c->m;
  a.ks = ks;
  a.ts = ts;
  a.R = R;
  a.skip = c->rg_skip;
  a.tbit0 = tbit0;
  a.base = c->base;
  a.dlen = (int)c->dlen;
  a.out = out;
  if (ks <= a.kd && ks <= 8 && tbit0 == 0 && ts <= c->r) {
    launch_decode_fast(a, s);
  } else {
    k_rapg_decode<<<grid_of((c->n + 3) / 4, kThreads), kThreads, 0, s>>>(a);
    count_launch();
  }
  return cudaGetLastError();
}


cudaError_t major_decode(const buff_col *c, double *out, cudaStream_t s) {
  if (c->m == 1 && c->k - c->m <= 8) {
    // one sparse column: the code is (outlier byte or major) << (fl - 8),
    // then the dense bytes and the tail -- the RAPG fast decode with the
    // major byte as the default of non-outlier rows
    RapgDecodeArgs r;
    memset(&r, 0, sizeof(r));
    r.obits = c->obits;
    r.orank = c->orank;
    r.obytes = c->obytes;
    r.oofs[0] = c->oofs[0];
    r.nwp = c->nwp;
    r.rs = rank_stride(c);
    r.stride = c->stride;
    r.slices = c->slices;
    r.tail = c->tail;
    r.n = c->n;
    r.m = 1;
    r.kd = c->k - 1;
    r.ks = c->k - 1;
    r.ts = c->r;
    r.R = c->fixed_len;
    r.sdef = (unsigned long long)c->majors[0] << (c->fixed_len - 8);
    r.smaj[0] = c->majors[0];
    r.base = c->base;
    r.dlen = (int)c->dlen;
    r.out = out;
    launch_decode_fast(r, s);
    return cudaGetLastError();
  }
  DecodeMajorArgs a;
  memset(&a, 0, sizeof(a));
  a.n = c->n;
  a.m = c->m;
  a.kd = c->k - c->m;
  a.r = c->r;
  a.fl = c->fixed_len;
  a.nwp = c->nwp;
  a.rs = rank_stride(c);
  a.stride = c->stride;
  a.obits = c->obits;
  a.orank = c->orank;
  a.obytes = c->obytes;
  for (uint32_t i = 0; i < 8; ++i) {
    a.oofs[i] = c->oofs[i];
    a.majors[i] = c->majors[i];
    a.olast[i] = c->olast[i];
  }
  a.slices = c->slices;
  a.tail = c->tail;
  a.base = c->base;
  a.dlen = (int)c->dlen;
  a.out = out;
  k_decode_major<<<grid_of(c->n, kThreads), kThreads, 0, s>>>(a);
  count_launch();
  return cudaGetLastError();
}

}  // namespace buffk
