// Batched form: many columns of uneven length and precision per launch.
//
// Work is a device queue of (column or query, row tile) items; persistent
// CTAs take items with one atomic per item, so a launch covers thousands of
// columns with balanced load however their lengths are distributed.
//
//   encode  buff_batch_encode_f64: pass 1 takes per-column min/max on order
//           keys of the raw f64 bits (one persistent launch over all tiles of
//           all columns), a warp per column reads the head rows the
//           reference's `else if` max depends on, the host sizes every column
//           (the same libm log2 as the single-column path) and carves one
//           arena, and pass 2 quantizes and scatters all tiles (one more
//           persistent launch).  Columns whose extremes are not finite, whose
//           shift wraps, or whose max needs a second scan fall back to the
//           single-column encoder.
//   queries buff_plan_*: range/equality filters (with or without the sum),
//           sum, max and decode at a precision, for one query per column or
//           many per column, as one persistent launch that a CUDA graph can
//           replay.  A filter/sum lane owns 32 consecutive rows (one bitmap
//           word) per step, streams 32 bytes of each slice it needs, and
//           accumulates the per-slice byte sums with dp4a; a decode/max lane
//           owns one row of every 32.
//
// The tile size, CTAs per SM and the number of slice-0 loads kept in flight
// are parameters (buff_batch_tune) chosen by buff_batch_autotune.
#include <cuda_runtime.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <new>
#include <vector>

#include "buff_device.cuh"
#include "buff_internal.h"

namespace buffk {
namespace {

using namespace dev;

constexpr int kBT = 256;  // threads per CTA of the persistent kernels
constexpr uint32_t kWarps = kBT / 32;

// ---------------------------------------------------------------- encode

struct EncCol {
  const double *x;
  uint32_t n;
  int32_t pexp;
  uint32_t dlen;
  uint32_t pad;
};

struct EncAcc {
  long long lo;  // min order key over all rows
  long long hi;  // max order key over rows >= 1
};

struct EncHead {
  long long x0, x1;         // first two quantized rows
  unsigned long long brk;   // first i >= 1 with x_i >= x_(i-1); 0: not found in the scanned head
  int ok;                   // extremes finite and their shift does not wrap
  int pad;
};

__global__ void k_benc_init(EncAcc *acc, uint32_t ncols) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < ncols) {
    acc[i].lo = LLONG_MAX;
    acc[i].hi = LLONG_MIN;
  }
}

__global__ void __launch_bounds__(kBT) k_benc_reduce(const EncCol *__restrict__ cols,
                                                     const uint2 *__restrict__ items,
                                                     uint32_t nitems, uint32_t tile,
                                                     unsigned int *counter, EncAcc *acc) {
  __shared__ unsigned int s_item;
  __shared__ long long s_lo[kWarps], s_hi[kWarps];
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (;;) {
    if (threadIdx.x == 0) s_item = atomicAdd(counter, 1u);
    __syncthreads();
    const uint32_t it = s_item;
    if (it >= nitems) return;
    const uint2 item = items[it];
    const EncCol c = cols[item.x];
    const uint32_t r0 = item.y * tile;
    const uint32_t r1 = min(c.n, r0 + tile);
    long long lo = LLONG_MAX, hi = LLONG_MIN;
    const uint32_t nv = (r1 - r0) / 2;
    const ulonglong2 *xv = reinterpret_cast<const ulonglong2 *>(c.x + r0);
    for (uint32_t v0 = threadIdx.x; v0 < nv; v0 += kBT * kU) {
      ulonglong2 raw[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const uint32_t v = v0 + u * kBT;
        if (v < nv) raw[u] = __ldcs(xv + v);
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const uint32_t v = v0 + u * kBT;
        if (v >= nv) break;
        const long long a = order_key(raw[u].x), b = order_key(raw[u].y);
        const uint32_t i0 = r0 + 2 * v;
        lo = min(lo, min(a, b));
        hi = max(hi, b);
        if (i0 >= 1) hi = max(hi, a);
      }
    }
    if (((r1 - r0) & 1u) && threadIdx.x == 0) {
      const uint32_t i = r1 - 1;
      const long long a = order_key((unsigned long long)__double_as_longlong(c.x[i]));
      lo = min(lo, a);
      if (i >= 1) hi = max(hi, a);
    }
    lo = warp_min<long long>(lo);
    hi = warp_max_ll(hi);
    if (lane == 0) {
      s_lo[wid] = lo;
      s_hi[wid] = hi;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (uint32_t w = 1; w < kWarps; ++w) {
        lo = min(lo, s_lo[w]);
        hi = max(hi, s_hi[w]);
      }
      if (lo != LLONG_MAX) atomicMin(&acc[item.x].lo, lo);
      if (hi != LLONG_MIN) atomicMax(&acc[item.x].hi, hi);
    }
    __syncthreads();  // s_item and s_lo/s_hi are reused by the next item
  }
}

// One warp per column: the first two quantized rows, the end of the leading
// strictly decreasing run (scanned over at most `limit` rows) and the
// key-mode validity of the extremes.
__global__ void k_benc_head(const EncCol *__restrict__ cols, const EncAcc *__restrict__ acc,
                            uint32_t ncols, uint32_t limit, EncHead *out) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t col = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (col >= ncols) return;
  const EncCol c = cols[col];
  auto q = [&](uint32_t i) {
    return fetch_bits((unsigned long long)__double_as_longlong(c.x[i]), c.pexp, c.dlen);
  };
  unsigned long long brk = 0;
  const uint32_t end = min(c.n, limit);
  for (uint32_t b0 = 1; b0 < end; b0 += 32) {
    const uint32_t i = b0 + lane;
    const bool hit = i < end && q(i) >= q(i - 1);
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, hit);
    if (m) {
      brk = b0 + (__ffs(m) - 1);
      break;
    }
  }
  if (!brk && end == c.n) brk = c.n;  // the whole column is strictly decreasing
  if (lane == 0) {
    EncHead h;
    h.x0 = c.n > 0 ? q(0) : 0;
    h.x1 = c.n > 1 ? q(1) : 0;
    h.brk = brk;
    const unsigned long long bl = key_bits(acc[col].lo), bh = key_bits(acc[col].hi);
    const int el = (int)((bl >> 52) & 0x7FFu) - 1023, eh = (int)((bh >> 52) & 0x7FFu) - 1023;
    const int lim = 63 - (int)c.dlen;
    h.ok = (el <= lim && eh <= lim) ? 1 : 0;
    h.pad = 0;
    out[col] = h;
  }
}

struct ScatCol {
  const double *x;
  uint8_t *slices;
  uint8_t *tail;
  unsigned long long stride;
  long long base;
  uint32_t n;
  int32_t pexp;
  uint32_t dlen, fl, k, r;
};

// Quantize-and-scatter of one 512-row chunk by one warp (the single-column
// k_encode_scatter with a runtime slice count): codes shifted to the top of
// a 64-bit word, bytes of neighbouring rows gathered with byte permutes into
// shared memory, then one 16-byte store per lane per slice and the packed
// tail of the lane's 16 rows.
template <int K>
__device__ __forceinline__ void scatter_chunk(const ScatCol &c, uint32_t r0, uint32_t lane,
                                              uint8_t *ws) {
  constexpr uint32_t k = K;
  ulonglong2 raw[8];
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const uint32_t i0 = r0 + m * 64 + lane * 2;
    if (i0 + 2 <= c.n) raw[m] = __ldcs(reinterpret_cast<const ulonglong2 *>(c.x + i0));
  }
  const unsigned long long rmask = c.r ? ((1ull << c.r) - 1ull) : 0ull;
  const uint32_t up = 64u - c.fl;
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const uint32_t off = m * 64 + lane * 2;
    const uint32_t i0 = r0 + off;
    unsigned long long cc[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      unsigned long long b = 0;
      if (i0 + 2 <= c.n)
        b = j ? raw[m].y : raw[m].x;
      else if (i0 + j < c.n)
        b = (unsigned long long)__double_as_longlong(c.x[i0 + j]);
      cc[j] = (i0 + j < c.n) ? (unsigned long long)(fetch_bits(b, c.pexp, c.dlen) - c.base) : 0ull;
    }
    if (k) {
      const unsigned long long a0 = (cc[0] << (up & 63)) ^ 0x8080808080808080ull;
      const unsigned long long a1 = (cc[1] << (up & 63)) ^ 0x8080808080808080ull;
      const uint32_t hw0 = (uint32_t)(a0 >> 32), lw0 = (uint32_t)a0;
      const uint32_t hw1 = (uint32_t)(a1 >> 32), lw1 = (uint32_t)a1;
#pragma unroll
      for (uint32_t sl = 0; sl < 8; ++sl) {
        if ((int)sl < K) {
          const bool in_hi = sl < 4;
          const uint32_t b = in_hi ? 3u - sl : 7u - sl;
          const uint32_t sel = b | ((4u + b) << 4);
          const uint32_t v = __byte_perm(in_hi ? hw0 : lw0, in_hi ? hw1 : lw1, sel);
          *reinterpret_cast<uint16_t *>(ws + sl * kRowChunk + off) = (uint16_t)v;
        }
      }
    }
    if (c.r) {
      const uint32_t packed = (uint32_t)(cc[0] & rmask) | ((uint32_t)(cc[1] & rmask) << 8);
      *reinterpret_cast<uint16_t *>(ws + k * kRowChunk + off) = (uint16_t)packed;
    }
  }
  __syncwarp();
#pragma unroll
  for (uint32_t sl = 0; sl < 8; ++sl) {
    if ((int)sl < K) {
      const uint4 v = *reinterpret_cast<const uint4 *>(ws + sl * kRowChunk + lane * 16);
      __stcs(reinterpret_cast<uint4 *>(c.slices + sl * c.stride + r0 + lane * 16), v);
    }
  }
  if (c.r == 1) {
    const ulonglong2 v = *reinterpret_cast<const ulonglong2 *>(ws + k * kRowChunk + lane * 16);
    const uint32_t lo8 = (uint32_t)((v.x * 0x0102040810204080ull) >> 56);
    const uint32_t hi8 = (uint32_t)((v.y * 0x0102040810204080ull) >> 56);
    *reinterpret_cast<uint16_t *>(c.tail + (size_t)2 * ((r0 >> 4) + lane)) =
        (uint16_t)(lo8 | (hi8 << 8));
  } else if (c.r) {
    const uint4 v = *reinterpret_cast<const uint4 *>(ws + k * kRowChunk + lane * 16);
    const uint8_t *b = reinterpret_cast<const uint8_t *>(&v);
    unsigned long long lo = 0, hi = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const uint32_t p = i * c.r;
      const unsigned long long f = b[i];
      if (p >= 64) {
        hi |= f << (p - 64);
      } else {
        lo |= f << p;
        if (p + c.r > 64) hi |= f >> (64 - p);
      }
    }
    uint16_t *dst = reinterpret_cast<uint16_t *>(c.tail + (size_t)2 * c.r * ((r0 >> 4) + lane));
    for (uint32_t i = 0; i < c.r; ++i)
      dst[i] = (uint16_t)(i < 4 ? (lo >> (16 * i)) : (hi >> (16 * (i - 4))));
  }
  __syncwarp();
}

// Persistent scatter for the columns with K slices: every warp takes
// (column, tile) items; a tile is a multiple of 512 rows, and the last tile
// of a column also writes the padding rows up to the slice stride (code 0).
template <int K>
__global__ void __launch_bounds__(kBT) k_benc_scatter(const ScatCol *__restrict__ cols,
                                                      const uint2 *__restrict__ items,
                                                      uint32_t nitems, uint32_t tile,
                                                      unsigned int *counter) {
  __shared__ __align__(16) uint8_t smem[kWarps * 9 * kRowChunk];
  const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint8_t *ws = smem + wid * 9 * kRowChunk;
  for (;;) {
    uint32_t it = 0;
    if (lane == 0) it = atomicAdd(counter, 1u);
    it = __shfl_sync(0xFFFFFFFFu, it, 0);
    if (it >= nitems) return;
    const uint2 item = items[it];
    const ScatCol c = cols[item.x];
    const uint32_t rows = (uint32_t)c.stride;  // n rounded up to 512
    const uint32_t r0 = item.y * tile, r1 = min(rows, r0 + tile);
    for (uint32_t ch = r0; ch < r1; ch += kRowChunk) scatter_chunk<K>(c, ch, lane, ws);
  }
}

cudaError_t launch_benc_scatter(int k, int grid, const ScatCol *cols, const uint2 *items,
                                uint32_t nitems, uint32_t tile, unsigned int *counter,
                                cudaStream_t s) {
  switch (k) {
#define BS(K) \
  case K: k_benc_scatter<K><<<grid, kBT, 0, s>>>(cols, items, nitems, tile, counter); break;
    BS(0) BS(1) BS(2) BS(3) BS(4) BS(5) BS(6) BS(7) BS(8)
#undef BS
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// ---------------------------------------------------------------- queries

struct BQ {
  const uint8_t *slices;
  const uint8_t *tail;
  unsigned long long stride;
  long long base;
  uint32_t n, k, r, ops;
  uint32_t fill;       // filters: 0 compare, 1 every row, 2 no row
  uint32_t full_rows;  // rows a filter may set
  uint32_t k_used;     // slices a filter compares
  uint32_t r_used;     // tail bits a filter compares (0: no tail step)
  uint32_t ttail;
  uint32_t dks, dts;   // decode: slices read, tail bits per row
  int32_t dlen;
  uint8_t tbyte[8];
  unsigned long long keep;
  uint32_t *words;
  double *values;
  unsigned long long *acc;  // [0] count, [1..8] slice sums, [9] tail sum, [10] max code
};

constexpr uint32_t kOpRange = BUFF_Q_RANGE, kOpEqual = BUFF_Q_EQUAL, kOpSum = BUFF_Q_SUM,
                   kOpMax = BUFF_Q_MAX, kOpDecode = BUFF_Q_DECODE;
// Descriptor-only flag: every decoded value base + code fits in 32 bits.
constexpr uint32_t kOpN32 = 0x100;
constexpr int kAcc = kBatchAcc;

// tw[i] for a runtime i without indexing a register array (which would
// place it in local memory).
__device__ __forceinline__ uint32_t pick8(const uint32_t (&tw)[8], uint32_t i) {
  uint32_t v = tw[0];
#pragma unroll
  for (uint32_t j = 1; j < 8; ++j) v = i == j ? tw[j] : v;
  return v;
}

// 32 slice bytes (rows row0..row0+31) with streaming loads.
__device__ __forceinline__ Bytes32 ld32(const uint8_t *p) {
  const uint4 a = __ldcs(reinterpret_cast<const uint4 *>(p));
  const uint4 b = __ldcs(reinterpret_cast<const uint4 *>(p + 16));
  Bytes32 v;
  v.w[0] = a.x;
  v.w[1] = a.y;
  v.w[2] = a.z;
  v.w[3] = a.w;
  v.w[4] = b.x;
  v.w[5] = b.y;
  v.w[6] = b.z;
  v.w[7] = b.w;
  return v;
}

// MSBs of the bytes of four words -> 16 row-ordered bits.
__device__ __forceinline__ uint32_t gather16(const uint32_t *m) {
  return __byte_perm(msb8(m[0], m[1]), msb8(m[2], m[3]), 0x0040);
}

__device__ __forceinline__ uint32_t w4(const uint4 &v, int i) {
  return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}

// Largest byte of a word.
__device__ __forceinline__ uint32_t max4(uint32_t w) {
  const uint32_t a = __vmaxu4(w, w >> 16);
  return max(a & 0xFFu, (a >> 8) & 0xFFu);
}

// Bytes equal to b (b replicated in every byte) -> their MSBs.
__device__ __forceinline__ uint32_t eqb4(uint32_t w, uint32_t bb) {
  const uint32_t x = w ^ bb;  // zero bytes where equal
  return ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x) & 0x80808080u;
}

// byte_fixed_max over rows [r0, r1) (split_double.rs:3919-4105 computes the
// same maximum slice by slice).  One pass over slice 0, 512 rows per warp
// step: the step's largest top byte M is compared with the tile's best code
// so far, and only a step that can reach it refines its candidate rows
// (top byte == M) through the later slices and the tail, each level taking
// the warp-wide largest byte among the remaining candidates.
template <int STAGE>
__device__ __forceinline__ void tile_max(const BQ &q, uint32_t r0, uint32_t r1, uint32_t lane) {
  const uint32_t fl = q.k ? 8 * q.k + q.r : q.r;
  // start from the best code other tiles of the query have published
  unsigned long long best = *reinterpret_cast<volatile unsigned long long *>(q.acc + 10);
  bool have = best != 0;
  for (uint32_t sb = r0; sb < r1; sb += 512 * STAGE) {
    uint4 v[STAGE];
#pragma unroll
    for (int u = 0; u < STAGE; ++u) {
      const uint32_t row0 = sb + u * 512 + lane * 16;
      if (q.k && row0 < r1)
        v[u] = __ldcs(reinterpret_cast<const uint4 *>(q.slices + row0));
      else
        v[u] = make_uint4(H, H, H, H);  // flipped zero bytes
    }
#pragma unroll
    for (int u = 0; u < STAGE; ++u) {
      const uint32_t step = sb + u * 512;
      if (step >= r1) break;  // warp-uniform
      const uint32_t row0 = step + lane * 16;
      const bool act = row0 < r1;
      unsigned long long code;
      uint32_t cand;
      if (q.k) {
        const uint32_t w0 = v[u].x ^ H, w1 = v[u].y ^ H, w2 = v[u].z ^ H, w3 = v[u].w ^ H;
        const uint32_t m = max4(__vmaxu4(__vmaxu4(w0, w1), __vmaxu4(w2, w3)));
        const uint32_t M = __reduce_max_sync(0xFFFFFFFFu, m);
        if (have && M < (uint32_t)(best >> (fl - 8))) continue;  // cannot reach the best
        const uint32_t bb = M * 0x01010101u;
        uint32_t e[4] = {eqb4(w0, bb), eqb4(w1, bb), eqb4(w2, bb), eqb4(w3, bb)};
        cand = act ? gather16(e) : 0u;
        code = M;
        for (uint32_t j = 1; j < q.k; ++j) {
          uint32_t mj = 0;
          uint4 b = make_uint4(0, 0, 0, 0);
          if (cand) {
            b = __ldcs(reinterpret_cast<const uint4 *>(q.slices + j * q.stride + row0));
            const uint32_t bw[4] = {b.x ^ H, b.y ^ H, b.z ^ H, b.w ^ H};
#pragma unroll
            for (int i = 0; i < 16; ++i)
              if (cand >> i & 1u) mj = max(mj, (bw[i >> 2] >> (8 * (i & 3))) & 0xFFu);
          }
          const uint32_t Mj = __reduce_max_sync(0xFFFFFFFFu, mj);
          if (cand) {
            const uint32_t bbj = Mj * 0x01010101u;
            uint32_t ej[4] = {eqb4(b.x ^ H, bbj), eqb4(b.y ^ H, bbj), eqb4(b.z ^ H, bbj),
                              eqb4(b.w ^ H, bbj)};
            cand &= gather16(ej);
          }
          code = (code << 8) | Mj;
        }
      } else {
        cand = act ? ((q.n - row0 >= 16) ? 0xFFFFu : ((1u << (q.n - row0)) - 1u)) : 0u;
        code = 0;
      }
      if (q.r) {
        uint32_t mt = 0;
        if (cand) {
          unsigned long long lo, hi;
          load_tail16(q.tail, row0 >> 4, q.r, lo, hi);
          uint32_t b = cand;
          while (b) {
            const uint32_t i = __ffs(b) - 1;
            b &= b - 1;
            mt = max(mt, field16(lo, hi, i, q.r));
          }
        }
        code = (code << q.r) | __reduce_max_sync(0xFFFFFFFFu, mt);
      }
      if (!have || code > best) {
        // publish it, and take a larger one another tile has published
        unsigned long long g = 0;
        if (lane == 0) g = atomicMax(q.acc + 10, code);
        g = __shfl_sync(0xFFFFFFFFu, g, 0);
        best = g > code ? g : code;
      }
      have = true;
    }
  }
  if (lane == 0 && have) atomicMax(q.acc + 10, best);
}

// Decode over rows [r0, r1), 128-row groups: lane L owns rows 4L..4L+3 of
// each group, so slice bytes come in 4-byte loads covering 128 contiguous
// bytes per warp and values leave as two 16-byte stores per lane; the
// group's dts-bit tail fields (16 dts bytes) are loaded by the first 4 dts
// lanes and handed out with shuffles.  STAGE groups are loaded together.
template <int STAGE>
__device__ __forceinline__ void tile_decode(const BQ &q, uint32_t r0, uint32_t r1,
                                            uint32_t lane) {
  const uint32_t db = q.dts;
  const uint32_t dmask = db ? ((1u << db) - 1u) : 0u;
  for (uint32_t g = r0; g < r1; g += 128 * STAGE) {
    uint32_t sw[STAGE][8];
    uint32_t dw[STAGE];
#pragma unroll
    for (int u = 0; u < STAGE; ++u) {
      const uint32_t base = g + 128 * u;
      dw[u] = 0;
      if (base >= r1) continue;
      const uint32_t row = base + 4 * lane;
#pragma unroll
      for (uint32_t j = 0; j < 8; ++j)
        if (j < q.dks)
          sw[u][j] = __ldcs(reinterpret_cast<const uint32_t *>(q.slices + j * q.stride + row));
      if (db && lane < 4 * db)
        dw[u] = __ldcs(reinterpret_cast<const uint32_t *>(q.tail + (size_t)(base >> 7) * 16 * db) +
                       lane);
    }
#pragma unroll
    for (int u = 0; u < STAGE; ++u) {
      const uint32_t base = g + 128 * u;
      if (base >= r1) break;  // warp-uniform
      const uint32_t row = base + 4 * lane;
      uint32_t f = 0;
      if (db) {
        const uint32_t bit = 4 * lane * db, wi = bit >> 5;
        const uint32_t w0 = __shfl_sync(0xFFFFFFFFu, dw[u], wi);
        const uint32_t w1 = __shfl_sync(0xFFFFFFFFu, dw[u], (wi + 1) & 31);
        f = __funnelshift_r(w0, w1, bit & 31);
      }
      double val[4];
      if (q.ops & kOpN32) {  // 32-bit codes and values (warp-uniform)
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i) {
          uint32_t d = 0;
#pragma unroll
          for (uint32_t j = 0; j < 4; ++j) {
            if (j >= q.dks) break;
            d = (d << 8) | (((sw[u][j] >> (8 * i)) & 0xFFu) ^ 0x80u);
          }
          if (db) d = (d << db) | ((f >> (i * db)) & dmask);
          val[i] = i32_to_f64_scaled((int)((uint32_t)q.base + (d & (uint32_t)q.keep)), q.dlen);
        }
      } else {
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i) {
          unsigned long long d = 0;
#pragma unroll
          for (uint32_t j = 0; j < 8; ++j) {
            if (j >= q.dks) break;
            d = (d << 8) | (((sw[u][j] >> (8 * i)) & 0xFFu) ^ 0x80u);
          }
          if (db) d = (d << db) | ((f >> (i * db)) & dmask);
          val[i] = i64_to_f64_scaled((long long)((unsigned long long)q.base + (d & q.keep)), q.dlen);
        }
      }
      if (row + 4 <= r1) {
        __stcs(reinterpret_cast<double2 *>(q.values + row), make_double2(val[0], val[1]));
        __stcs(reinterpret_cast<double2 *>(q.values + row + 2), make_double2(val[2], val[3]));
      } else {
#pragma unroll
        for (uint32_t i = 0; i < 4; ++i)
          if (row + i < r1) q.values[row + i] = val[i];
      }
    }
  }
}

// Filter only: lane L owns the 32 rows row0 = step + 32L .. +31 (one bitmap
// word) of each 1024-row step; STAGE steps of slice 0 are loaded together,
// later slices and the tail only for words that still hold candidates.
template <int STAGE>
__device__ __forceinline__ void tile_filter32(const BQ &q, uint32_t r0, uint32_t r1,
                                              uint32_t lane) {
  const bool is_range = q.ops & kOpRange;
  const bool cmp = q.fill == 0;
  const uint32_t rmask = q.r ? ((1u << q.r) - 1u) : 0u;
  uint32_t cnt = 0;
  for (uint32_t sb = r0; sb < r1; sb += 1024 * STAGE) {
    Bytes32 v[STAGE];
#pragma unroll
    for (int u = 0; u < STAGE; ++u) {
      const uint32_t row0 = sb + u * 1024 + lane * 32;
      if (cmp && q.k_used && row0 < r1) v[u] = ld32(q.slices + row0);
    }
#pragma unroll
    for (int u = 0; u < STAGE; ++u) {
      const uint32_t row0 = sb + u * 1024 + lane * 32;
      if (row0 >= r1) continue;
      const uint32_t left = q.n - row0;
      const uint32_t valid = left >= 32 ? 0xFFFFFFFFu : ((1u << left) - 1u);
      uint32_t res;
      if (!cmp) {
        res = q.fill == 1 ? valid : 0u;
      } else {
        uint32_t eq = valid, gt = 0;
        if (row0 + 32 > q.full_rows)
          eq &= row0 >= q.full_rows ? 0u : ((1u << (q.full_rows - row0)) - 1u);
        for (uint32_t j = 0; j < q.k_used && eq; ++j) {
          const Bytes32 b = j == 0 ? v[u] : ld32(q.slices + j * q.stride + row0);
          const ByteTarget t = make_target(q.tbyte[j]);
          uint32_t g[8], e[8];
#pragma unroll
          for (int w = 0; w < 8; ++w) cmp4(b.w[w], t, g[w], e[w]);
          gt |= eq & gather32(g);
          eq &= gather32(e);
        }
        if (q.r_used && eq) {
          const uint32_t *tp =
              reinterpret_cast<const uint32_t *>(q.tail + (size_t)(row0 >> 5) * 4 * q.r);
          uint32_t tw[8];
#pragma unroll
          for (uint32_t i = 0; i < 7; ++i) tw[i] = i < q.r ? __ldcs(tp + i) : 0u;
          tw[7] = 0;
          uint32_t gtt = 0, eqt = 0, bb = eq;
          while (bb) {
            const uint32_t i = __ffs(bb) - 1;
            bb &= bb - 1;
            const uint32_t bit = i * q.r, wi = bit >> 5;
            const uint32_t f =
                __funnelshift_r(pick8(tw, wi), pick8(tw, wi + 1), bit & 31) & rmask;
            gtt |= (uint32_t)(f > q.ttail) << i;
            eqt |= (uint32_t)(f == q.ttail) << i;
          }
          gt |= eq & gtt;
          eq &= eqt;
        }
        res = is_range ? gt : eq;
      }
      q.words[row0 >> 5] = res;
      cnt += __popc(res);
    }
  }
  const unsigned long long sc = warp_sum_ull(cnt);
  if (lane == 0 && sc) atomicAdd(q.acc, sc);
}

// ---- filter + sum with the slices staged through shared memory
//
// Lane L owns the 32 rows step + 32L .. +31 of each 1,024-row step -- one
// bitmap word, as in the single-column one-pass kernel -- and copies its own
// 32 bytes of up to 3 slices (a 4th and later slice are loaded directly),
// while the first 8r lanes copy the step's 128r tail bytes, into a per-warp
// ring of kDepth steps with cp.async: kDepth - 1 steps of every slice are in
// flight without holding registers, and a lane reads back only what it
// copied (the tail group excepted, hence the warp barrier around each step).
// Per 32 rows a lane does 8 dp4a per slice, one byte compare of slice 0 with
// the target's top bit specialised, and r weighted popcounts for the tail.
// The 16-rows-per-lane form of this worker (3 steps of 512 rows) ran
// 1.40-1.48 ms per replay of the 4,096-query plan, issue-bound at ~335
// instructions per 512 rows.
constexpr int kDepth = 2;
constexpr uint32_t kStepRows = 1024;
constexpr uint32_t kSlotBytes = 3 * kStepRows + 1024;  // 3 slices + up to 896 tail bytes
constexpr uint32_t kRingBytes = kDepth * kSlotBytes;


// The descriptor fields one filter/sum tile reads, loaded once into
// registers (the descriptor lives in global memory, and reading its fields
// inside the step loop would reload them every step).
struct FsTile {
  const uint8_t *slices, *tail;
  unsigned long long stride;
  uint32_t n, k, r, full_rows, k_used, r_used, ttail, nst;
  uint32_t t0lo0, t0lo1;  // slice-0 compare constants ((t & 0x7f) [+1]) x 0x01010101
  unsigned long long tb;  // target bytes of slices 1..7 (byte j-1 = slice j)
  bool cmp, is_range, th0;
};

__device__ __forceinline__ FsTile fs_tile(const BQ &q, bool do_f) {
  FsTile t;
  t.slices = q.slices;
  t.tail = q.tail;
  t.stride = q.stride;
  t.n = q.n;
  t.k = q.k;
  t.r = q.r;
  t.full_rows = q.full_rows;
  t.k_used = q.k_used;
  t.r_used = q.r_used;
  t.ttail = q.ttail;
  t.nst = q.k < 3 ? q.k : 3u;  // slices staged; later ones load directly
  const uint32_t t0 = q.tbyte[0];
  t.t0lo0 = (t0 & 0x7Fu) * 0x01010101u;
  t.t0lo1 = t.t0lo0 + 0x01010101u;
  t.th0 = t0 & 0x80u;
  t.tb = 0;
  for (int j = 1; j < 8; ++j) t.tb |= (unsigned long long)q.tbyte[j] << (8 * (j - 1));
  t.cmp = do_f && q.fill == 0;
  t.is_range = q.ops & kOpRange;
  return t;
}

__device__ __forceinline__ void fs_issue(const FsTile &q, uint32_t sb, uint32_t r1, uint32_t lane,
                                         uint8_t *slot) {
  if (sb < r1) {
    const uint32_t row0 = sb + lane * 32;
    if (row0 < r1)  // row0 + 32 <= the slice stride (a multiple of 512 >= n)
      for (uint32_t j = 0; j < q.nst; ++j) {
        const uint8_t *src = q.slices + j * q.stride + row0;
        cp16(slot + j * kStepRows + lane * 32, src);
        cp16(slot + j * kStepRows + lane * 32 + 16, src + 16);
      }
    // the step's 128r tail bytes = 8r pieces of 16 (up to 56: a lane copies
    // pieces lane and lane + 32), none past the tail the rows below r1 use
    // (the tail allocation covers that, rounded up to 16)
    const size_t tend = ((size_t)r1 * q.r + 7) / 8;
    for (uint32_t pc = lane; pc < 8 * q.r; pc += 32) {
      const size_t t0 = (size_t)(sb / kStepRows) * 128 * q.r + pc * 16;
      if (t0 < tend) cp16(slot + 3 * kStepRows + pc * 16, q.tail + t0);
    }
  }
  cp_commit();  // every lane commits one group per step, even an empty one
}

// Tail bits of the 32 rows from row0 that lie below n (each row r bits).
__device__ __forceinline__ uint32_t left_bits(uint32_t n, uint32_t row0, uint32_t r) {
  const uint32_t rows = n - row0 >= 32 ? 32u : n - row0;
  return rows * r;
}

// Slice-0 compare of 32 rows (eight words) against a target byte whose top
// bit is TH: the rows above it (gt) and equal to it (eq).
template <bool TH>
__device__ __forceinline__ void cmp32_t(const uint4 &a, const uint4 &b, uint32_t lo0,
                                        uint32_t lo1, uint32_t &gt, uint32_t &eq) {
  uint32_t g[8], e[8];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    g[i] = gt4t<TH>(w4(a, i), lo1);
    e[i] = eq4t<TH>(w4(a, i), lo0, lo1);
    g[4 + i] = gt4t<TH>(w4(b, i), lo1);
    e[4 + i] = eq4t<TH>(w4(b, i), lo0, lo1);
  }
  gt = gather32(g);
  eq = gather32(e);
}

// Sum of the 32 bytes as signed int8: a stored (flipped) byte s holds the
// code byte s ^ 0x80 = int8(s) + 128, so the code-byte sum is this plus 128
// per byte, added once per lane at the end (no per-word flip).
__device__ __forceinline__ int dp4a_sum8(const uint4 &a, const uint4 &b, int acc) {
  acc = __dp4a((int)a.x, 0x01010101, acc);
  acc = __dp4a((int)a.y, 0x01010101, acc);
  acc = __dp4a((int)a.z, 0x01010101, acc);
  acc = __dp4a((int)a.w, 0x01010101, acc);
  acc = __dp4a((int)b.x, 0x01010101, acc);
  acc = __dp4a((int)b.y, 0x01010101, acc);
  acc = __dp4a((int)b.z, 0x01010101, acc);
  acc = __dp4a((int)b.w, 0x01010101, acc);
  return acc;
}

// Bits 0, R, 2R, ... of a word.
template <bool DO_F>
__device__ __forceinline__ void tile_fs_async(const BQ &qd, uint32_t r0, uint32_t r1,
                                              uint32_t lane, uint8_t *ring) {
  const FsTile q = fs_tile(qd, DO_F);
  uint32_t *const words = qd.words;
  unsigned long long *const acc = qd.acc;
  const uint32_t fill = qd.fill;
  const uint32_t c32 = q.r ? 32 % q.r : 0u;  // tail phase step per word
  int sacc[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // signed byte sums (dp4a_sum8)
  uint32_t tacc = 0, cnt = 0, nact = 0;  // nact: steps the lane summed 32 bytes of each slice
  __syncwarp();  // the ring may still be read by the previous item
#pragma unroll
  for (int d = 0; d < kDepth - 1; ++d)
    fs_issue(q, r0 + d * kStepRows, r1, lane, ring + d * kSlotBytes);
  uint32_t t = 0;
  for (uint32_t sb = r0; sb < r1; sb += kStepRows, ++t) {
    fs_issue(q, sb + (kDepth - 1) * kStepRows, r1, lane,
             ring + ((t + kDepth - 1) % kDepth) * kSlotBytes);
    cp_wait<kDepth - 1>();
    __syncwarp();
    const uint8_t *slot = ring + (t % kDepth) * kSlotBytes;
    const uint32_t row0 = sb + lane * 32;
    const bool act = row0 < r1;
    uint32_t valid = 0, eq = 0, gt = 0;
    if (act) {
      ++nact;
      const uint32_t left = q.n - row0;
      valid = left >= 32 ? 0xFFFFFFFFu : ((1u << left) - 1u);
      eq = valid;
      if (row0 + 32 > q.full_rows)
        eq &= row0 >= q.full_rows ? 0u : ((1u << (q.full_rows - row0)) - 1u);
      {  // slice 0: sums and the compare
        const uint4 a = *reinterpret_cast<const uint4 *>(slot + lane * 32);
        const uint4 b = *reinterpret_cast<const uint4 *>(slot + lane * 32 + 16);
        sacc[0] = dp4a_sum8(a, b, sacc[0]);
        if (q.cmp && q.k_used && eq) {
          uint32_t g, e;
          if (q.th0)
            cmp32_t<true>(a, b, q.t0lo0, q.t0lo1, g, e);
          else
            cmp32_t<false>(a, b, q.t0lo0, q.t0lo1, g, e);
          gt = eq & g;
          eq &= e;
        }
      }
#pragma unroll
      for (uint32_t j = 1; j < 8; ++j) {
        if (j >= q.k) break;
        uint4 a, b;
        if (j < 3) {
          a = *reinterpret_cast<const uint4 *>(slot + j * kStepRows + lane * 32);
          b = *reinterpret_cast<const uint4 *>(slot + j * kStepRows + lane * 32 + 16);
        } else {
          const uint8_t *p = q.slices + j * q.stride + row0;
          a = __ldcs(reinterpret_cast<const uint4 *>(p));
          b = __ldcs(reinterpret_cast<const uint4 *>(p + 16));
        }
        sacc[j] = dp4a_sum8(a, b, sacc[j]);
        if (q.cmp && j < q.k_used && eq) {
          const ByteTarget tg = make_target((uint32_t)(q.tb >> (8 * (j - 1))) & 0xFFu);
          uint32_t g[8], e[8];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            cmp4(w4(a, i), tg, g[i], e[i]);
            cmp4(w4(b, i), tg, g[4 + i], e[4 + i]);
          }
          gt |= eq & gather32(g);
          eq &= gather32(e);
        }
      }
      if (q.r) {
        // the lane's 32 fields: r words at byte 4r * lane of the step's tail
        const uint32_t *tp = reinterpret_cast<const uint32_t *>(slot + 3 * kStepRows) + lane * q.r;
        if (valid == 0xFFFFFFFFu) {
          switch (q.r) {  // warp-uniform
            case 1: tacc += tail_sum32<1>(tp); break;
            case 2: tacc += tail_sum32<2>(tp); break;
            case 3: tacc += tail_sum32<3>(tp); break;
            case 4: tacc += tail_sum32<4>(tp); break;
            case 5: tacc += tail_sum32<5>(tp); break;
            case 6: tacc += tail_sum32<6>(tp); break;
            default: tacc += tail_sum32<7>(tp); break;
          }
        } else {  // the column's last rows: only the fields of rows below n
          const uint32_t nbits = left_bits(q.n, row0, q.r);  // stream bits of the lane's rows
          uint32_t ph = 0;  // the lane's fields start at a multiple of r
#pragma unroll
          for (uint32_t i = 0; i < 7; ++i) {
            if (i < q.r) {
              uint32_t word = tp[i];
              if (32 * i >= nbits)
                word = 0;
              else if (32 * i + 32 > nbits)
                word &= (1u << (nbits - 32 * i)) - 1u;
              tacc += wpopc(word, ph, q.r);
              ph += c32;
              if (ph >= q.r) ph -= q.r;
            }
          }
        }
        if (q.cmp && q.r_used && eq) {
          uint32_t tw[8];
#pragma unroll
          for (uint32_t i = 0; i < 8; ++i) tw[i] = i < q.r ? tp[i] : 0u;
          uint32_t gtt = 0, eqt = 0, b = eq;
          while (b) {
            const uint32_t i = __ffs(b) - 1;
            b &= b - 1;
            const uint32_t bit = i * q.r, wi = bit >> 5;
            const uint32_t f =
                __funnelshift_r(pick8(tw, wi), pick8(tw, wi + 1), bit & 31) & ((1u << q.r) - 1u);
            gtt |= (uint32_t)(f > q.ttail) << i;
            eqt |= (uint32_t)(f == q.ttail) << i;
          }
          gt |= eq & gtt;
          eq &= eqt;
        }
      }
    }
    if (DO_F && act) {
      const uint32_t res = fill == 1 ? valid : fill == 2 ? 0u : (q.is_range ? gt : eq);
      words[row0 >> 5] = res;
      cnt += __popc(res);
    }
    __syncwarp();  // the slot is refilled by the next step's copies
  }
  cp_wait<0>();
#pragma unroll
  for (uint32_t j = 0; j < 8; ++j) {
    if (j >= q.k) break;
    const unsigned long long sj =
        warp_sum_ull((unsigned long long)((long long)sacc[j] + 4096ll * nact));
    if (lane == 0 && sj) atomicAdd(acc + 1 + j, sj);
  }
  if (q.r) {
    const unsigned long long st = warp_sum_ull(tacc);
    if (lane == 0 && st) atomicAdd(acc + 9, st);
  }
  if (DO_F) {
    const unsigned long long sc = warp_sum_ull(cnt);
    if (lane == 0 && sc) atomicAdd(acc, sc);
  }
}

// Query classes: each runs in its own persistent launch, compiled for its
// ops only.  A query with a filter and a sum is one FS item; a query with a
// sum (without a filter) and a max or decode is an S item and an MD item.
enum { kClsF = 0, kClsFS = 1, kClsS = 2, kClsMD = 3, kClasses = 4 };
constexpr uint32_t kBqShared = 512;  // class lists up to this size are read from shared memory

// Persistent worker of one class: warp-granular items; the batch's class
// list holds query indices qidx[] and the exclusive prefix of their tile
// counts, so item i belongs to the query found by binary search.
template <int CLS, int STAGE>
__global__ void __launch_bounds__(kBT, (CLS == kClsFS || CLS == kClsS) ? 3 : 0)
    k_bq(const BQ *__restrict__ qs,
                                            const uint32_t *__restrict__ qidx,
                                            const uint32_t *__restrict__ prefix, uint32_t nq,
                                            uint32_t nitems, uint32_t tile,
                                            unsigned int *counter, BatchDone done) {
  extern __shared__ __align__(16) uint8_t dyn_smem[];
  __shared__ bool s_last;
  // a class list of up to kBqShared queries is copied to shared memory once
  // per block, so finding an item's query costs no global round trip
  __shared__ uint32_t s_pf[kBqShared], s_qi[kBqShared];
  const bool lists_shared = nq <= kBqShared;
  if (lists_shared) {
    for (uint32_t i = threadIdx.x; i < nq; i += blockDim.x) {
      s_pf[i] = __ldg(prefix + i);
      s_qi[i] = __ldg(qidx + i);
    }
    __syncthreads();
  }
  const uint32_t lane = threadIdx.x & 31;
  uint8_t *ring = dyn_smem + (threadIdx.x >> 5) * kRingBytes;  // FS / S classes only
  // a warp's first item is its own index; its later items come from the
  // work counter, offset past the items the warps took that way (the counter
  // is one address that every taking warp hits: tens of thousands of small
  // items queued on it for tens of microseconds)
  // the batch's next class launch (programmatic dependent launch) may start
  // once every block of this one runs: the classes are independent
  asm volatile("griddepcontrol.launch_dependents;");
  const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
  uint32_t it = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  // a launch with a few items per warp (a serving batch is split into about
  // eight per launched warp, for latency) strides them statically: warp w
  // takes w, w + nw, ... without the work counter's round trip before each
  // item
  const bool stride = nitems <= 8 * nw;
  for (bool first = true;; first = false) {
    if (!first) {
      if (stride) {
        it += nw;
      } else {
        if (lane == 0) it = nw + atomicAdd(counter, 1u);
        it = __shfl_sync(0xFFFFFFFFu, it, 0);
      }
    }
    if (it >= nitems) break;
    // the query of item `it`: the last i with prefix[i] <= it, found by the
    // whole warp 32-ary (lane l probes lo + l*step), two or three dependent
    // loads for thousands of queries instead of a binary search's dozen
    uint32_t lo = 0, hi = nq;
    while (hi - lo > 1) {
      const uint32_t step = (hi - lo + 31) >> 5;
      const uint32_t pos = lo + lane * step;
      const bool le = pos < hi && (lists_shared ? s_pf[pos] : __ldg(prefix + pos)) <= it;
      const uint32_t b = __ballot_sync(0xFFFFFFFFu, le);  // lane 0 always: prefix[lo] <= it
      const uint32_t j = 31 - __clz(b);
      lo += j * step;
      hi = min(hi, lo + step);
    }
    const BQ &q = qs[lists_shared ? s_qi[lo] : __ldg(qidx + lo)];
    const uint32_t r0 = (it - (lists_shared ? s_pf[lo] : __ldg(prefix + lo))) * tile;
    const uint32_t r1 = min(q.n, r0 + tile);
    if (CLS == kClsF) tile_filter32<STAGE>(q, r0, r1, lane);
    if (CLS == kClsFS) tile_fs_async<true>(q, r0, r1, lane, ring);
    if (CLS == kClsS) tile_fs_async<false>(q, r0, r1, lane, ring);
    if (CLS == kClsMD) {
      if (q.ops & kOpMax) tile_max<STAGE>(q, r0, r1, lane);
      if (q.ops & kOpDecode) tile_decode<STAGE>(q, r0, r1, lane);
    }
  }
  // a class launch started early ends only after the launch before it has
  // ended (a no-op for a launch without a predecessor of its own): so the
  // batch's last launch ends after every class of the batch
  asm volatile("griddepcontrol.wait;" ::: "memory");
  if (!done.flag) return;
  // the batch's completion: the last block to finish (every block's sums
  // added and fenced before its ticket; the earlier class launches of the
  // batch have ended, see above) publishes the accumulators, then the flag,
  // to host memory
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = atomicAdd(done.ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  for (uint32_t i = threadIdx.x; i < done.nacc; i += blockDim.x) done.hacc[i] = __ldcg(done.acc + i);
  __threadfence_system();
  __syncthreads();
  if (threadIdx.x == 0) *reinterpret_cast<volatile uint32_t *>(done.flag) = done.seq;
}

template <int CLS>
const void *bq_fn(int stage) {
  return stage == 4 ? (const void *)k_bq<CLS, 4>
                    : stage == 2 ? (const void *)k_bq<CLS, 2> : (const void *)k_bq<CLS, 1>;
}

const void *class_fn(int cls, int stage) {
  switch (cls) {
    case kClsF: return bq_fn<kClsF>(stage);
    case kClsFS: return bq_fn<kClsFS>(stage);
    case kClsS: return bq_fn<kClsS>(stage);
    default: return bq_fn<kClsMD>(stage);
  }
}

int dev_sms() {
  int d = 0;
  cudaGetDevice(&d);
  return num_sms(d);
}

int plan_query(const buff_query &uq, unsigned long long *acc, BQ *q);

}  // namespace

// Entry points for the serving loop (buff_server.cu).
size_t batch_desc_size() { return sizeof(BQ); }

int batch_plan_query(const buff_query &q, unsigned long long *acc, void *desc) {
  return plan_query(q, acc, static_cast<BQ *>(desc));
}

size_t batch_sched_words(uint32_t nq) { return 4 * (size_t)nq + 2 * kClasses; }

// Class lists of a batch: for class c, qidx (query indices) then the
// exclusive prefix of their tile counts, packed in `buf`.
void batch_schedule(const void *h_desc, uint32_t nq, uint32_t tile, uint32_t *buf,
                    BatchSched *sc) {
  const BQ *qs = static_cast<const BQ *>(h_desc);
  uint32_t nc[kClasses] = {0, 0, 0, 0};
  auto classes = [](const BQ &q, int *out) {
    int m = 0;
    if (q.n == 0) return 0;
    if (q.ops & (kOpRange | kOpEqual))
      out[m++] = (q.ops & kOpSum) ? kClsFS : kClsF;
    else if (q.ops & kOpSum)
      out[m++] = kClsS;
    if (q.ops & (kOpMax | kOpDecode)) out[m++] = kClsMD;
    return m;
  };
  for (uint32_t i = 0; i < nq; ++i) {
    int cl[2];
    const int m = classes(qs[i], cl);
    for (int j = 0; j < m; ++j) nc[cl[j]]++;
  }
  uint32_t off = 0;
  for (int c = 0; c < kClasses; ++c) {
    sc->n[c] = nc[c];
    sc->qidx_off[c] = off;
    sc->prefix_off[c] = off + nc[c];
    sc->items[c] = 0;
    off += 2 * nc[c] + 1;
  }
  uint32_t fill[kClasses] = {0, 0, 0, 0};
  for (uint32_t i = 0; i < nq; ++i) {
    int cl[2];
    const int m = classes(qs[i], cl);
    const uint32_t t = (qs[i].n + tile - 1) / tile;
    for (int j = 0; j < m; ++j) {
      const int c = cl[j];
      buf[sc->qidx_off[c] + fill[c]] = i;
      buf[sc->prefix_off[c] + fill[c]] = sc->items[c];
      fill[c]++;
      sc->items[c] += t;
    }
  }
  for (int c = 0; c < kClasses; ++c) buf[sc->prefix_off[c] + nc[c]] = sc->items[c];
  sc->words = off;
}

size_t class_smem(int cls) {
  return (cls == kClsFS || cls == kClsS) ? (size_t)kWarps * kRingBytes : 0;
}

// Allows the ring's dynamic shared memory once per kernel instance.
void class_prepare(int cls, int stage) {
  static std::atomic<bool> done[4][5];
  if (done[cls][stage].load(std::memory_order_acquire)) return;
  const size_t sm = class_smem(cls);
  if (sm) cudaFuncSetAttribute(class_fn(cls, stage), cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)sm);
  done[cls][stage].store(true, std::memory_order_release);  // setting it twice is harmless
}

// Resident CTAs per SM of a class worker, asked of the runtime once per
// (class, stage): the query costs microseconds of host time, which every
// batch of the serving loop would otherwise pay per class.
int worker_per_sm(int cls, int stage) {
  static std::atomic<int> cache[kClasses][5];
  std::atomic<int> &slot = cache[cls][stage];
  int per_sm = slot.load(std::memory_order_relaxed);
  if (per_sm) return per_sm;
  class_prepare(cls, stage);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, class_fn(cls, stage), kBT,
                                                class_smem(cls));
  if (per_sm < 1) per_sm = 1;
  slot.store(per_sm, std::memory_order_relaxed);
  return per_sm;
}

int class_grid(int cls, const buff_batch_tune &t, uint32_t nitems) {
  const int per_sm = worker_per_sm(cls, (int)t.stage);
  const int bps = (int)t.blocks_per_sm < per_sm ? (int)t.blocks_per_sm : per_sm;
  int grid = bps * dev_sms();
  const uint32_t need = (nitems + kWarps - 1) / kWarps;
  if ((uint32_t)grid > need) grid = need ? (int)need : 1;
  return grid;
}

// One persistent launch per non-empty class, in order on `s`; counters
// holds kClasses zeroed work counters.
cudaError_t batch_launch(const void *d_desc, const uint32_t *d_buf, const BatchSched &sc,
                         const buff_batch_tune &t, unsigned int *counters, cudaStream_t s,
                         const BatchDone *done) {
  const BQ *qs = static_cast<const BQ *>(d_desc);
  const int order[kClasses] = {kClsMD, kClsFS, kClsS, kClsF};
  int last = -1;  // the completion rides on the last class launched
  for (int oi = 0; oi < kClasses; ++oi)
    if (sc.items[order[oi]]) last = oi;
  BatchDone none;
  memset(&none, 0, sizeof(none));
  if (done && last < 0) {  // nothing to launch: one empty worker still completes the batch
    BatchDone d = *done;
    k_bq<kClsF, 1><<<1, kBT, 0, s>>>(qs, d_buf, d_buf, 0, 0, t.tile_rows, counters, d);
    count_launch();
    return cudaGetLastError();
  }
  bool started = false;
  for (int oi = 0; oi < kClasses; ++oi) {
    const int c = order[oi];
    if (!sc.items[c]) continue;
    const BatchDone &bd = (done && oi == last) ? *done : none;
    const uint32_t grid = (uint32_t)class_grid(c, t, sc.items[c]);
    const uint32_t *qi = d_buf + sc.qidx_off[c], *pf = d_buf + sc.prefix_off[c];
    // after the first class of a completed batch, a programmatic dependent
    // launch: it starts while the class before it finishes
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kBT);
    cfg.dynamicSmemBytes = class_smem(c);
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = (done && started) ? 1 : 0;
    started = true;
    cudaError_t e;
#define BQ_LAUNCH(CLS)                                                                          \
  do {                                                                                         \
    if (t.stage == 4)                                                                          \
      e = cudaLaunchKernelEx(&cfg, k_bq<CLS, 4>, qs, qi, pf, sc.n[c], sc.items[c], t.tile_rows, \
                             counters + c, bd);                                               \
    else if (t.stage == 2)                                                                     \
      e = cudaLaunchKernelEx(&cfg, k_bq<CLS, 2>, qs, qi, pf, sc.n[c], sc.items[c], t.tile_rows, \
                             counters + c, bd);                                               \
    else                                                                                       \
      e = cudaLaunchKernelEx(&cfg, k_bq<CLS, 1>, qs, qi, pf, sc.n[c], sc.items[c], t.tile_rows, \
                             counters + c, bd);                                               \
  } while (0)
    switch (c) {
      case kClsF: BQ_LAUNCH(kClsF); break;
      case kClsFS: BQ_LAUNCH(kClsFS); break;
      case kClsS: BQ_LAUNCH(kClsS); break;
      default: BQ_LAUNCH(kClsMD); break;
    }
#undef BQ_LAUNCH
    count_launch();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Result of one query from its accumulators ([0] count, [1..8] slice sums,
// [9] tail sum, [10] max code).
void batch_result(const buff_query &q, const unsigned long long *a, buff_query_result *out) {
  const buff_col *c = q.col;
  buff_query_result &r = *out;
  memset(&r, 0, sizeof(r));
  const uint32_t ops = q.ops;
  r.count = (ops & (kOpRange | kOpEqual)) ? a[0] : 0;
  if (ops & kOpSum) {
    // byte_fixed_sum over the whole code (split_double.rs:2127-2208)
    uint64_t parts[9] = {0};
    uint32_t np = 0;
    for (uint32_t j = 0; j < c->k; ++j) parts[np++] = a[1 + j];
    if (c->r) parts[np++] = a[9];
    r.n_partials = np;
    for (uint32_t j = 0; j < np; ++j) r.partials[j] = parts[j];
    r.sum = buffh::combine_sum(c, c->fixed_len, parts, c->flags & BUFF_FLAG_INTENDED);
  }
  if ((ops & kOpMax) && c->n) {
    r.max_code = a[10];
    r.max_value = (double)(int64_t)((uint64_t)c->base + a[10]) / ldexp(1.0, (int)c->dlen);
  }
}

}  // namespace buffk

// ================================================================ host side

using namespace buffk;

struct buff_plan {
  int device;
  uint32_t nq;
  buff_batch_tune tune;
  std::vector<const buff_col *> cols;
  std::vector<buff_query> queries;
  std::vector<int32_t> status;
  BQ *h_q;                   // pinned
  BQ *d_q;
  uint32_t *h_sched;         // pinned class lists
  uint32_t *d_sched;
  BatchSched sc;
  unsigned long long *d_acc;
  unsigned long long *h_acc;  // pinned
  unsigned int *d_counter;    // one per class
  cudaGraph_t graph;
  cudaGraphExec_t exec;
};

namespace buffk {
namespace {

buff_batch_tune default_tune() {
  buff_batch_tune t;
  t.tile_rows = 32768;
  t.blocks_per_sm = 4;
  t.stage = 2;
  t.reserved = 0;
  return t;
}

bool tune_ok(const buff_batch_tune &t) {
  return t.tile_rows >= 1024 && t.tile_rows % 1024 == 0 && t.tile_rows <= (1u << 24) &&
         t.blocks_per_sm >= 1 && t.blocks_per_sm <= 8 &&
         (t.stage == 1 || t.stage == 2 || t.stage == 4);
}

// Host side of one query: validates it and fills the device descriptor
// with the same plan the single-column entry points use.
int plan_query(const buff_query &uq, unsigned long long *acc, BQ *q) {
  const buff_col *c = uq.col;
  memset(q, 0, sizeof(*q));
  q->acc = acc;
  if (!c || !acc) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;
  const uint32_t ops = uq.ops;
  const uint32_t known = kOpRange | kOpEqual | kOpSum | kOpMax | kOpDecode;
  if (!ops || (ops & ~known) || ((ops & kOpRange) && (ops & kOpEqual))) return BUFF_EINVAL;
  const bool intended = c->flags & BUFF_FLAG_INTENDED;
  q->slices = c->slices;
  q->tail = c->tail;
  q->stride = c->stride;
  q->base = c->base;
  q->n = c->n;
  q->k = c->k;
  q->r = c->r;
  q->ops = ops;
  q->dlen = (int32_t)c->dlen;
  q->words = uq.words;
  q->values = uq.values;
  q->keep = ~0ull;
  if ((ops & (kOpRange | kOpEqual)) && c->n && !uq.words) return BUFF_EINVAL;
  if ((ops & kOpDecode) && c->n && !uq.values) return BUFF_EINVAL;
  if (ops & (kOpRange | kOpEqual)) {
    // buff_simd_range_filter / buff_simd_equal_filter (buff_simd.rs:3361-3733)
    const bool is_range = ops & kOpRange;
    const int64_t fp = buffh::fetch_fixed(uq.pred, c->precision_exp, c->dlen);
    if (fp < c->base) {
      q->fill = is_range ? 1 : 2;  // the early return (:3385-3388, 3573-3576)
    } else {
      const uint64_t t = (uint64_t)(fp - c->base);
      const uint32_t fl = c->fixed_len;
      for (uint32_t j = 0; j < c->k; ++j) q->tbyte[j] = (uint8_t)(t >> (fl - 8 * (j + 1)));
      q->ttail = c->r ? (uint32_t)(t & ((1ull << c->r) - 1)) : 0u;
      q->k_used = c->k;
      q->r_used = c->r;
      if (intended || c->k == 0) {
        q->full_rows = c->n;
        if (fl < 64 && (t >> fl) != 0) q->fill = 2;
      } else {
        q->full_rows = c->n / 32 * 32;
        if (!is_range && c->r == 0) q->fill = 2;  // only the tail step writes `res`
      }
    }
  }
  if (ops & kOpDecode) {
    // buff_simd256_decode / byte_residue_decode_with_precision
    uint32_t total = c->fixed_len;
    if (uq.precision) {
      const int st = buffh::precision_bits(c, uq.precision, &total);
      if (st) return st;
    }
    if (intended) {
      if (total > c->fixed_len) return BUFF_EREFPANIC;
      q->dks = c->k;
      q->dts = c->r;
      const uint32_t drop = c->fixed_len - total;
      q->keep = drop >= 64 ? 0ull : (~0ull << drop);
    } else {
      if (total >= 8 && total / 8 > c->k) return BUFF_EREFPANIC;
      if (total < 8 && c->k && total) return BUFF_ENOTSUP;
      q->dks = total < 8 ? 0 : total / 8;
      q->dts = total < 8 ? total : total % 8;
    }
    const uint32_t bits = 8 * q->dks + q->dts;
    const long long maxc = bits >= 63 ? -1 : (long long)((1ull << bits) - 1ull);
    if (bits <= 32 && c->base >= INT32_MIN && maxc >= 0 && c->base + maxc <= (long long)INT32_MAX)
      q->ops |= kOpN32;
  }
  return BUFF_OK;
}

}  // namespace
}  // namespace buffk

namespace {

#define BCK(expr)                              \
  do {                                         \
    cudaError_t _e = (expr);                   \
    if (_e != cudaSuccess) {                   \
      rc = buffh::cuda_status(_e);             \
      goto done;                               \
    }                                          \
  } while (0)

void release_plan(buff_plan *p) {
  if (!p) return;
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  if (p->h_q) cudaFreeHost(p->h_q);
  if (p->h_acc) cudaFreeHost(p->h_acc);
  if (p->h_sched) cudaFreeHost(p->h_sched);
  if (p->d_q) cudaFree(p->d_q);
  if (p->d_sched) cudaFree(p->d_sched);
  if (p->d_acc) cudaFree(p->d_acc);
  if (p->d_counter) cudaFree(p->d_counter);
  delete p;
}

cudaError_t enqueue(buff_plan *p, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(p->d_q, p->h_q, sizeof(BQ) * p->nq, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(p->d_sched, p->h_sched, sizeof(uint32_t) * p->sc.words,
                        cudaMemcpyHostToDevice, s);
  // the accumulators and the 4 work counters (2 u64 words) zeroed by one kernel
  if (e == cudaSuccess)
    e = zero_u64(p->d_acc, kAcc * p->nq, s,
                 reinterpret_cast<unsigned long long *>(p->d_counter), 2);
  if (e == cudaSuccess) e = batch_launch(p->d_q, p->d_sched, p->sc, p->tune, p->d_counter, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(p->h_acc, p->d_acc, sizeof(unsigned long long) * kAcc * p->nq,
                        cudaMemcpyDeviceToHost, s);
  return e;
}

}  // namespace

extern "C" {

int buff_plan_create(const buff_query *queries, uint32_t nq, const buff_batch_tune *tune,
                     void *stream, buff_plan **out) {
  if (!out || (nq && !queries)) return BUFF_EINVAL;
  *out = nullptr;
  const buff_batch_tune t = tune ? *tune : default_tune();
  if (!tune_ok(t)) return BUFF_EINVAL;
  (void)stream;
  int rc = BUFF_OK;
  buff_plan *p = new (std::nothrow) buff_plan();
  if (!p) return BUFF_ENOMEM;
  cudaGetDevice(&p->device);
  p->nq = nq;
  p->tune = t;
  p->queries.assign(queries, queries + nq);
  p->status.assign(nq, BUFF_OK);
  {
    const size_t qb = sizeof(BQ) * (nq ? nq : 1);
    const size_t ab = sizeof(unsigned long long) * kAcc * (nq ? nq : 1);
    const size_t sb = sizeof(uint32_t) * batch_sched_words(nq);
    BCK(cudaMallocHost(reinterpret_cast<void **>(&p->h_q), qb));
    BCK(cudaMallocHost(reinterpret_cast<void **>(&p->h_acc), ab));
    BCK(cudaMallocHost(reinterpret_cast<void **>(&p->h_sched), sb));
    BCK(cudaMalloc(reinterpret_cast<void **>(&p->d_q), qb));
    BCK(cudaMalloc(reinterpret_cast<void **>(&p->d_acc), ab));
    BCK(cudaMalloc(reinterpret_cast<void **>(&p->d_sched), sb));
    BCK(cudaMalloc(reinterpret_cast<void **>(&p->d_counter), sizeof(unsigned int) * 4));
    for (uint32_t i = 0; i < nq; ++i) {
      const int st = plan_query(queries[i], p->d_acc + (size_t)kAcc * i, &p->h_q[i]);
      if (st) {
        rc = st;
        goto done;
      }
    }
    batch_schedule(p->h_q, nq, t.tile_rows, p->h_sched, &p->sc);
  }
done:
  if (rc != BUFF_OK) {
    release_plan(p);
    return rc;
  }
  *out = p;
  return BUFF_OK;
}

int buff_plan_set_preds(buff_plan *p, const double *preds) {
  if (!p || (p->nq && !preds)) return BUFF_EINVAL;
  for (uint32_t i = 0; i < p->nq; ++i) {
    buff_query q = p->queries[i];
    q.pred = preds[i];
    const int st = plan_query(q, p->d_acc + (size_t)kAcc * i, &p->h_q[i]);
    if (st) return st;
    p->queries[i] = q;
  }
  batch_schedule(p->h_q, p->nq, p->tune.tile_rows, p->h_sched, &p->sc);
  return BUFF_OK;
}

int buff_plan_launch(buff_plan *p, void *stream) {
  if (!p) return BUFF_EINVAL;
  return buffh::cuda_status(enqueue(p, reinterpret_cast<cudaStream_t>(stream)));
}

int buff_plan_capture(buff_plan *p, void *stream) {
  if (!p || !stream) return BUFF_EINVAL;  // capture needs a non-default stream
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  if (p->exec) {
    cudaGraphExecDestroy(p->exec);
    p->exec = nullptr;
  }
  if (p->graph) {
    cudaGraphDestroy(p->graph);
    p->graph = nullptr;
  }
  cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return buffh::cuda_status(e);
  cudaError_t e2 = enqueue(p, s);
  e = cudaStreamEndCapture(s, &p->graph);
  if (e2 != cudaSuccess) return buffh::cuda_status(e2);
  if (e != cudaSuccess) return buffh::cuda_status(e);
  e = cudaGraphInstantiate(&p->exec, p->graph, 0);
  return buffh::cuda_status(e);
}

int buff_plan_replay(buff_plan *p, void *stream) {
  if (!p || !p->exec) return BUFF_EINVAL;
  count_launch();
  return buffh::cuda_status(cudaGraphLaunch(p->exec, reinterpret_cast<cudaStream_t>(stream)));
}

int buff_plan_results(buff_plan *p, buff_query_result *out, void *stream) {
  if (!p || (p->nq && !out)) return BUFF_EINVAL;
  const cudaError_t e = cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return buffh::cuda_status(e);
  for (uint32_t i = 0; i < p->nq; ++i) {
    batch_result(p->queries[i], p->h_acc + (size_t)kAcc * i, &out[i]);
    out[i].status = p->status[i];
  }
  return BUFF_OK;
}

int buff_plan_free(buff_plan *p) {
  if (!p) return BUFF_EINVAL;
  cudaDeviceSynchronize();
  release_plan(p);
  return BUFF_OK;
}

int buff_batch_autotune(const buff_query *queries, uint32_t nq, void *stream,
                        buff_batch_tune *best, float *best_ms) {
  if (!best || (nq && !queries)) return BUFF_EINVAL;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const uint32_t tiles[] = {8192, 16384, 32768, 65536};
  const uint32_t bps[] = {3, 4, 6, 8};
  const uint32_t stages[] = {1, 2, 4};
  float bms = 1e30f;
  buff_batch_tune bt = default_tune();
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return BUFF_ECUDA;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return BUFF_ECUDA;
  }
  int rc = BUFF_OK;
  for (uint32_t ti : tiles)
    for (uint32_t b : bps)
      for (uint32_t st : stages) {
        buff_batch_tune t;
        t.tile_rows = ti;
        t.blocks_per_sm = b;
        t.stage = st;
        t.reserved = 0;
        buff_plan *p = nullptr;
        rc = buff_plan_create(queries, nq, &t, stream, &p);
        if (rc) goto out;
        float ms = 1e30f;
        for (int rep = 0; rep < 4 && rc == BUFF_OK; ++rep) {
          cudaEventRecord(e0, s);
          rc = buff_plan_launch(p, stream);
          cudaEventRecord(e1, s);
          if (cudaEventSynchronize(e1) != cudaSuccess) rc = BUFF_ECUDA;
          float m = 0;
          cudaEventElapsedTime(&m, e0, e1);
          if (rep > 0 && m < ms) ms = m;  // the first launch warms caches and the allocator
        }
        buff_plan_free(p);
        if (rc) goto out;
        if (ms < bms) {
          bms = ms;
          bt = t;
        }
      }
out:
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  *best = bt;
  if (best_ms) *best_ms = bms;
  return BUFF_OK;
}

// ---------------------------------------------------------------- batched encode

int buff_batch_encode_f64(const double *const *values, const uint64_t *lens,
                          const uint64_t *scales, uint32_t ncols, uint32_t flags,
                          const buff_batch_tune *tune, void *stream, buff_col **out) {
  if (!out || (ncols && (!values || !lens || !scales))) return BUFF_EINVAL;
  if (flags & ~(BUFF_FLAG_INTENDED | BUFF_FLAG_BUFF_LAYOUT)) return BUFF_EINVAL;
  const buff_batch_tune t = tune ? *tune : default_tune();
  if (!tune_ok(t)) return BUFF_EINVAL;
  for (uint32_t i = 0; i < ncols; ++i) out[i] = nullptr;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const bool intended = flags & BUFF_FLAG_INTENDED;
  int rc = BUFF_OK;
  std::vector<EncCol> ec(ncols);
  std::vector<EncHead> heads(ncols);
  std::vector<EncAcc> accs(ncols);
  std::vector<const double *> staged(ncols, nullptr);
  std::vector<uint8_t> fast(ncols, 0);
  std::vector<uint2> items;
  std::vector<ScatCol> sc;
  std::vector<uint32_t> scol;  // column of each ScatCol
  EncCol *d_ec = nullptr;
  EncAcc *d_acc = nullptr;
  EncHead *d_head = nullptr;
  uint2 *d_items = nullptr;
  ScatCol *d_sc = nullptr;
  unsigned int *d_counter = nullptr;
  buff_arena *arena = nullptr;
  uint8_t *abase = nullptr;
  const uint32_t enc_tile = t.tile_rows * 4;
  const int grid = (int)t.blocks_per_sm * dev_sms();
  // pass 1 inputs: every column with >= 2 rows, a PRECISION_MAP entry, key-mode
  // precision and a 16-byte aligned device pointer takes the batched path
  for (uint32_t i = 0; i < ncols; ++i) {
    if (lens[i] > BUFF_MAX_ROWS) {
      rc = BUFF_EINVAL;
      goto done;
    }
    const int dl = buffh::dlen_of_scale(scales[i]);
    if (dl < 0) {
      rc = BUFF_EREFPANIC;
      goto done;
    }
    buff_col probe;
    memset(&probe, 0, sizeof(probe));
    buff_col *pc = buffh::new_col(scales[i], flags);
    if (!pc) {
      rc = BUFF_ENOMEM;
      goto done;
    }
    probe = *pc;
    delete pc;
    ec[i].x = values[i];
    ec[i].n = (uint32_t)lens[i];
    ec[i].pexp = probe.precision_exp;
    ec[i].dlen = (uint32_t)dl;
    ec[i].pad = 0;
    const bool keys = probe.precision_exp >= -dl;
    const bool aligned =
        buffh::is_device_ptr(values[i]) && (reinterpret_cast<uintptr_t>(values[i]) & 15) == 0;
    fast[i] = (lens[i] >= 2 && keys && aligned) ? 1 : 0;
    if (fast[i])
      for (uint32_t tt = 0; (uint64_t)tt * enc_tile < lens[i]; ++tt)
        items.push_back(make_uint2(i, tt));
  }
  if (!items.empty()) {
    BCK(cudaMallocAsync(reinterpret_cast<void **>(&d_ec), sizeof(EncCol) * ncols, s));
    BCK(cudaMallocAsync(reinterpret_cast<void **>(&d_acc), sizeof(EncAcc) * ncols, s));
    BCK(cudaMallocAsync(reinterpret_cast<void **>(&d_head), sizeof(EncHead) * ncols, s));
    BCK(cudaMallocAsync(reinterpret_cast<void **>(&d_items), sizeof(uint2) * items.size(), s));
    BCK(cudaMallocAsync(reinterpret_cast<void **>(&d_counter), sizeof(unsigned int), s));
    BCK(cudaMemcpyAsync(d_ec, ec.data(), sizeof(EncCol) * ncols, cudaMemcpyHostToDevice, s));
    BCK(cudaMemcpyAsync(d_items, items.data(), sizeof(uint2) * items.size(),
                        cudaMemcpyHostToDevice, s));
    BCK(cudaMemsetAsync(d_counter, 0, sizeof(unsigned int), s));
    k_benc_init<<<(ncols + 255) / 256, 256, 0, s>>>(d_acc, ncols);
    k_benc_reduce<<<grid, kBT, 0, s>>>(d_ec, d_items, (uint32_t)items.size(), enc_tile, d_counter,
                                       d_acc);
    k_benc_head<<<(ncols + kWarps - 1) / kWarps, kBT, 0, s>>>(d_ec, d_acc, ncols, 65536, d_head);
    count_launch(3);
    BCK(cudaGetLastError());
    BCK(cudaMemcpyAsync(heads.data(), d_head, sizeof(EncHead) * ncols, cudaMemcpyDeviceToHost, s));
    BCK(cudaMemcpyAsync(accs.data(), d_acc, sizeof(EncAcc) * ncols, cudaMemcpyDeviceToHost, s));
    BCK(cudaStreamSynchronize(s));
  }
  {
    // sizes: exact min and the reference's max (Q1: rows after the leading
    // strictly decreasing run), then fixed_len = ceil(log2(delta)) on the host
    size_t total = 0;
    std::vector<size_t> offs(ncols, 0);
    std::vector<buff_col *> cols(ncols, nullptr);
    auto key_bits_h = [](long long k) {
      const uint64_t u = (uint64_t)k;
      return u ^ ((uint64_t)(k >> 63) >> 1);
    };
    for (uint32_t i = 0; i < ncols; ++i) {
      if (!fast[i]) continue;
      const EncHead &h = heads[i];
      if (!h.ok) {
        fast[i] = 0;
        continue;
      }
      double lo_v, hi_v;
      const uint64_t bl = key_bits_h(accs[i].lo), bh = key_bits_h(accs[i].hi);
      memcpy(&lo_v, &bl, 8);
      memcpy(&hi_v, &bh, 8);
      const int64_t mn = buffh::fetch_fixed(lo_v, ec[i].pexp, ec[i].dlen);
      const int64_t mx1 = buffh::fetch_fixed(hi_v, ec[i].pexp, ec[i].dlen);
      int64_t mx;
      if (intended) {
        mx = h.x0 > mx1 ? h.x0 : mx1;
      } else if (h.brk == 1 || mx1 > h.x1) {
        mx = mx1;
      } else if (h.brk >= ec[i].n) {
        mx = INT64_MIN;
      } else {
        fast[i] = 0;  // needs the max over rows >= brk: single-column path
        continue;
      }
      const int64_t delta = (int64_t)((uint64_t)mx - (uint64_t)mn);
      uint32_t fl;
      if (intended) {
        fl = delta == 0 ? 0u : (uint32_t)(64 - __builtin_clzll((uint64_t)delta));
      } else if (delta == 0) {
        fl = 0;
      } else {
        const double cl = ceil(log2((double)delta));
        fl = (isnan(cl) || cl <= 0.0) ? 0u : (uint32_t)cl;
      }
      if (!intended && fl == 0) {
        rc = BUFF_EREFPANIC;  // constant column: write_bits(_, 0) (bit_packing.rs:117)
        goto done;
      }
      buff_col *c = buffh::new_col(scales[i], flags);
      if (!c) {
        rc = BUFF_ENOMEM;
        goto done;
      }
      cols[i] = c;
      c->n = ec[i].n;
      c->dlen = ec[i].dlen;
      c->base = mn;
      buffh::set_layout(c, fl);
      c->ilen = (uint32_t)((uint64_t)fl - (uint64_t)c->dlen);
      c->stride = round_up(c->n, kRowChunk);
      c->tail_bytes = ((uint64_t)c->n * c->r + 7) / 8;
      c->tail_alloc = c->stride / 8 * c->r + 64;
      offs[i] = total;
      total += round_up((size_t)c->k * c->stride, 256) + round_up(c->tail_alloc, 256);
    }
    if (total) {
      BCK(cudaMallocAsync(reinterpret_cast<void **>(&abase), total, s));
      arena = new (std::nothrow) buff_arena;
      if (!arena) {
        rc = BUFF_ENOMEM;
        goto done;
      }
      arena->base = abase;
      arena->refs.store(0);
    }
    items.clear();
    const uint32_t sc_tile = t.tile_rows;
    for (uint32_t i = 0; i < ncols; ++i) {
      if (!fast[i]) continue;
      buff_col *c = cols[i];
      c->slices = c->k ? abase + offs[i] : nullptr;
      c->tail = abase + offs[i] + round_up((size_t)c->k * c->stride, 256);
      c->arena = arena;
      arena->refs.fetch_add(1);
      out[i] = c;
      cols[i] = nullptr;
      ScatCol d;
      d.x = ec[i].x;
      d.slices = c->slices;
      d.tail = c->tail;
      d.stride = c->stride;
      d.base = c->base;
      d.n = c->n;
      d.pexp = ec[i].pexp;
      d.dlen = c->dlen;
      d.fl = c->fixed_len;
      d.k = c->k;
      d.r = c->r;
      sc.push_back(d);
      scol.push_back(i);
      // tail padding past the last full 512-row chunk is never written by the scatter
      BCK(cudaMemsetAsync(c->tail + c->stride / 8 * c->r, 0, 64, s));
    }
    // items grouped by slice count: one launch per count, compiled for it
    std::vector<uint32_t> kstart(10, 0);
    {
      std::vector<std::vector<uint2>> byk(9);
      for (uint32_t ci = 0; ci < sc.size(); ++ci)
        for (uint32_t tt = 0; (uint64_t)tt * sc_tile < sc[ci].stride; ++tt)
          byk[sc[ci].k].push_back(make_uint2(ci, tt));
      for (int k = 0; k <= 8; ++k) {
        kstart[k] = (uint32_t)items.size();
        items.insert(items.end(), byk[k].begin(), byk[k].end());
      }
      kstart[9] = (uint32_t)items.size();
    }
    for (uint32_t i = 0; i < ncols; ++i)
      if (cols[i]) buffh::free_col(cols[i]);
    if (!sc.empty()) {
      unsigned int *d_cnt9 = nullptr;
      BCK(cudaMallocAsync(reinterpret_cast<void **>(&d_sc), sizeof(ScatCol) * sc.size(), s));
      if (d_items) BCK(cudaFreeAsync(d_items, s));
      d_items = nullptr;
      BCK(cudaMallocAsync(reinterpret_cast<void **>(&d_items), sizeof(uint2) * items.size(), s));
      BCK(cudaMallocAsync(reinterpret_cast<void **>(&d_cnt9), sizeof(unsigned int) * 9, s));
      BCK(cudaMemcpyAsync(d_sc, sc.data(), sizeof(ScatCol) * sc.size(), cudaMemcpyHostToDevice, s));
      BCK(cudaMemcpyAsync(d_items, items.data(), sizeof(uint2) * items.size(),
                          cudaMemcpyHostToDevice, s));
      BCK(cudaMemsetAsync(d_cnt9, 0, sizeof(unsigned int) * 9, s));
      for (int k = 0; k <= 8; ++k) {
        const uint32_t ni = kstart[k + 1] - kstart[k];
        if (!ni) continue;
        int g = grid;
        if ((uint32_t)g > (ni + kWarps - 1) / kWarps) g = (int)((ni + kWarps - 1) / kWarps);
        const cudaError_t e =
            launch_benc_scatter(k, g, d_sc, d_items + kstart[k], ni, sc_tile, d_cnt9 + k, s);
        count_launch();
        if (e != cudaSuccess) {
          cudaFreeAsync(d_cnt9, s);
          rc = buffh::cuda_status(e);
          goto done;
        }
      }
      cudaFreeAsync(d_cnt9, s);
      BCK(cudaStreamSynchronize(s));  // the descriptors above live on this stack frame
    }
  }
  // everything else through the single-column encoder
  for (uint32_t i = 0; i < ncols; ++i) {
    if (out[i]) continue;
    rc = buff_encode_f64(values[i], lens[i], scales[i], flags, stream, &out[i]);
    if (rc) goto done;
  }
done:
  if (d_ec) cudaFreeAsync(d_ec, s);
  if (d_acc) cudaFreeAsync(d_acc, s);
  if (d_head) cudaFreeAsync(d_head, s);
  if (d_items) cudaFreeAsync(d_items, s);
  if (d_sc) cudaFreeAsync(d_sc, s);
  if (d_counter) cudaFreeAsync(d_counter, s);
  if (arena && arena->refs.load() == 0) {
    cudaFreeAsync(abase, s);
    delete arena;
  }
  if (rc != BUFF_OK) {
    for (uint32_t i = 0; i < ncols; ++i) {
      if (out[i]) buff_col_free(out[i]);
      out[i] = nullptr;
    }
  }
  (void)staged;
  (void)scol;
  return rc;
}

}  // extern "C"
