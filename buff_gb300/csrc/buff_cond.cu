// Row-conditioned decode: values of listed rows or of the rows set in a
// bitmap (buff_decode_condition, compress/buff_simd.rs:1528-1712, and
// buff_major_decode_condition, :1714-1914).
//
// The reference walks each slice once per listed row with the BitPack
// reader; here every selected row is rebuilt independently from its k slice
// bytes and its packed tail field.  For the bitmap form a lane owns 4
// consecutive rows, so a warp covers four 32-row bitmap words and its slice
// reads coalesce; the output slot of a row is the prefix count of set bits
// before its word plus the set bits below it in the word.
#include <cuda_runtime.h>
#include <limits.h>
#include <stdint.h>

#include "buff_device.cuh"
#include "buff_internal.h"

namespace buffk {
namespace {

using namespace dev;

struct RowArgs {
  const uint8_t *slices, *tail;
  size_t stride;
  uint32_t n, k, r;
  int tail_shift;
  long long base;
  int dlen;
  double *out;
};

// The code the reference rebuilds for one row.  tail_shift reproduces
// `fixed | (cur << remain)` (:1693, :1701): the tail field lands r bits too
// high, over the low bits of the last byte.
__device__ __forceinline__ unsigned long long row_code(const RowArgs &a, uint32_t row) {
  unsigned long long v = 0;
  for (uint32_t j = 0; j < a.k; ++j)
    v = (v << 8) | (uint32_t)(__ldg(a.slices + (size_t)j * a.stride + row) ^ 0x80u);
  if (a.r) {
    const unsigned long long bit = (unsigned long long)row * a.r;
    const uint32_t b0 = __ldg(a.tail + (bit >> 3));
    const uint32_t b1 = ((bit & 7) + a.r > 8) ? __ldg(a.tail + (bit >> 3) + 1) : 0u;
    const unsigned long long t = ((b0 | (b1 << 8)) >> (bit & 7)) & ((1u << a.r) - 1u);
    if (a.k == 0)
      v = t;
    else
      v = (v << a.r) | (a.tail_shift ? (t << a.r) : t);
  }
  return v;
}

__device__ __forceinline__ double row_value(const RowArgs &a, uint32_t row) {
  return i64_to_f64_scaled((long long)((unsigned long long)a.base + row_code(a, row)), a.dlen);
}

__global__ void __launch_bounds__(kThreads) k_decode_list(RowArgs a, const uint32_t *__restrict__ rows,
                                                          uint64_t nrows) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nrows;
       i += (uint64_t)gridDim.x * blockDim.x)
    a.out[i] = row_value(a, rows[i]);
}

// The bitmap form with 4 rows per lane: a warp covers 128 rows (4 bitmap
// words) per step and takes kDecSteps steps per iteration, their bitmap
// words loaded together so that sparse selections skip empty steps
// kDecSteps at a time; a step's first output slot is its entry of `rank`
// (selected rows before the step), a lane's place within it a warp scan.  For a step with selected rows each lane reads
// its 4 rows of every slice with one 4-byte load (128 bytes per warp
// request) and their 4 tail fields from at most 5 tail bytes, and writes the
// selected values to their slots.  N32: every base + code fits in 32 bits
// (the exact 32-bit conversion).
constexpr uint32_t kDecSteps = 4;

template <bool N32, int KS>
__global__ void __launch_bounds__(kThreads) k_decode_words4(RowArgs a, const uint32_t *__restrict__ words,
                                                            const uint32_t *__restrict__ rank) {
  // KS > 0: the slice count is a constant, so every step's slice words are
  // loaded together before any is used; KS == 0: a.k slices, loaded in turn
  const uint32_t ks = KS > 0 ? (uint32_t)KS : a.k;
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t nsteps = (uint32_t)(((uint64_t)a.n + 127) / 128);
  const uint32_t rmask = a.r ? ((1u << a.r) - 1u) : 0u;
  for (uint32_t st0 = warp * kDecSteps; st0 < nsteps; st0 += nwarps * kDecSteps) {
    uint32_t word[kDecSteps], nib[kDecSteps], any = 0;
#pragma unroll
    for (uint32_t u = 0; u < kDecSteps; ++u) {
      const uint32_t row0 = (st0 + u) * 128 + lane * 4;
      word[u] = (st0 + u < nsteps && row0 < a.n) ? __ldg(words + (row0 >> 5)) : 0u;
      nib[u] = (word[u] >> (row0 & 31)) & 0xFu;
      if (row0 + 4 > a.n) nib[u] &= row0 < a.n ? (1u << (a.n - row0)) - 1u : 0u;  // rows past n
      any |= nib[u];
    }
    if (!__any_sync(0xFFFFFFFFu, any != 0)) continue;
    // each lane's place among the selected rows of its step (lanes in row order)
    uint32_t excl[kDecSteps];
#pragma unroll
    for (uint32_t u = 0; u < kDecSteps; ++u) {
      const uint32_t cl = __popc(nib[u]);
      uint32_t incl = cl;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (uint32_t)o) incl += y;
      }
      excl[u] = incl - cl;
    }
    constexpr int KL = KS > 0 ? KS : 1;
    uint32_t xs[kDecSteps][KL];
    // the 5 tail bytes holding each step's 4 fields (the tail buffer is padded
    // past its last row), loaded with the slices
    unsigned long long tf[kDecSteps];
#pragma unroll
    for (uint32_t u = 0; u < kDecSteps; ++u) {
      tf[u] = 0;
      if (a.r && nib[u]) {
        const unsigned long long bit = (unsigned long long)((st0 + u) * 128 + lane * 4) * a.r;
        const uint8_t *tb = a.tail + (bit >> 3);
#pragma unroll
        for (int b = 0; b < 5; ++b) tf[u] |= (unsigned long long)__ldg(tb + b) << (8 * b);
        tf[u] >>= (bit & 7);
      }
    }
    if (KS > 0) {
#pragma unroll
      for (uint32_t u = 0; u < kDecSteps; ++u)
#pragma unroll
        for (int j = 0; j < KL; ++j)
          xs[u][j] = nib[u] ? __ldg(reinterpret_cast<const uint32_t *>(
                                  a.slices + (size_t)j * a.stride + (st0 + u) * 128 + lane * 4))
                            : 0u;
    }
#pragma unroll
    for (uint32_t u = 0; u < kDecSteps; ++u) {
      if (!nib[u]) continue;
      const uint32_t row0 = (st0 + u) * 128 + lane * 4;
      unsigned long long c[4] = {0, 0, 0, 0};
      for (uint32_t j = 0; j < ks; ++j) {
        const uint32_t x =
            (KS > 0 ? xs[u][j < (uint32_t)KL ? j : 0]
                    : __ldg(reinterpret_cast<const uint32_t *>(a.slices + (size_t)j * a.stride +
                                                               row0))) ^
            0x80808080u;
#pragma unroll
        for (int i = 0; i < 4; ++i) c[i] = (c[i] << 8) | ((x >> (8 * i)) & 0xFFu);
      }
      if (a.r) {
        // fields of rows row0..row0+3: bits row0*r .. +4r (4r <= 28) of the tail
        const unsigned long long f = tf[u];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const unsigned long long t = (f >> (i * a.r)) & rmask;
          if (a.k == 0)
            c[i] = t;
          else
            c[i] = (c[i] << a.r) | (a.tail_shift ? (t << a.r) : t);
        }
      }
      uint32_t at = __ldg(rank + st0 + u) + excl[u];
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (nib[u] >> i & 1u)
          a.out[at++] = N32 ? i32_to_f64_scaled((int)((uint32_t)a.base + (uint32_t)c[i]), a.dlen)
                            : i64_to_f64_scaled((long long)((unsigned long long)a.base + c[i]),
                                                a.dlen);
    }
  }
}

// Selected rows of each 128-row step (rows below n only), for step_ranks.
__global__ void k_step_popc(const uint32_t *__restrict__ words, uint32_t n, uint32_t nsteps,
                            uint32_t *cnt) {
  const uint32_t nw = (uint32_t)(((uint64_t)n + 31) / 32);
  for (uint32_t st = blockIdx.x * blockDim.x + threadIdx.x; st < nsteps;
       st += gridDim.x * blockDim.x) {
    uint32_t c = 0;
#pragma unroll
    for (uint32_t i = 0; i < 4; ++i) {
      const uint32_t w = st * 4 + i;
      if (w >= nw) break;
      uint32_t b = __ldg(words + w);
      if (w == nw - 1 && (n & 31)) b &= (1u << (n & 31)) - 1u;
      c += __popc(b);
    }
    cnt[st] = c;
  }
}

__global__ void k_check_rows(const uint32_t *__restrict__ rows, uint64_t nrows, uint32_t n,
                             uint32_t *bad) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nrows;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t r = rows[i];
    if (r >= n || (i > 0 && r <= rows[i - 1])) atomicOr(bad, 1u);
  }
}

// ---------------------------------------------------------------- windowed max

struct WinArgs {
  const uint8_t *slices, *tail;
  size_t stride;
  uint32_t k, r, lo, hi, s, w;
  unsigned long long *codes;  // one per window, zeroed
};

// The full codes of rows row0..row0+3 (row0 a multiple of 4): 4-byte slice
// loads and one 4r-bit field group of the tail.
__device__ __forceinline__ void codes4(const WinArgs &a, uint32_t row0, unsigned long long *c) {
#pragma unroll
  for (int i = 0; i < 4; ++i) c[i] = 0;
  for (uint32_t j = 0; j < a.k; ++j) {
    const uint32_t w = __ldg(reinterpret_cast<const uint32_t *>(a.slices + j * a.stride + row0));
#pragma unroll
    for (int i = 0; i < 4; ++i) c[i] = (c[i] << 8) | (((w >> (8 * i)) & 0xFFu) ^ 0x80u);
  }
  if (a.r) {
    const unsigned long long bit = (unsigned long long)row0 * a.r;
    const uint32_t *tp = reinterpret_cast<const uint32_t *>(a.tail) + (bit >> 5);
    const uint32_t f = __funnelshift_r(__ldg(tp), __ldg(tp + 1), (uint32_t)(bit & 31));
    const uint32_t m = (1u << a.r) - 1u;
#pragma unroll
    for (int i = 0; i < 4; ++i) c[i] = (c[i] << a.r) | ((f >> (i * a.r)) & m);
  }
}

// Per-window maxima of the codes of rows [lo, hi), windows of w rows from s.
// A warp covers 128 rows per step (lane: 4 rows).  With w >= 128 a step
// touches at most two windows, reduced across the warp; narrower windows
// flush each lane's running maximum at every window change.
template <bool WIDE>
__global__ void __launch_bounds__(kThreads) k_max_range(WinArgs a) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t first = a.lo & ~127u;
  const uint32_t nsteps = (a.hi - first + 127) / 128;
  for (uint32_t st = warp; st < nsteps; st += nwarps) {
    const uint32_t c0 = first + st * 128;
    const uint32_t row0 = c0 + lane * 4;
    unsigned long long c[4] = {0, 0, 0, 0};
    const bool any = row0 < a.hi && row0 + 4 > a.lo;
    if (any) codes4(a, row0, c);
    if (WIDE) {
      const uint32_t wa = ((c0 > a.lo ? c0 : a.lo) - a.s) / a.w;
      const uint32_t split = a.s + (wa + 1) * a.w;  // first row of window wa + 1
      unsigned long long ma = 0, mb = 0;
      bool ha = false, hb = false;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t row = row0 + i;
        if (!any || row < a.lo || row >= a.hi) continue;
        if (row < split) {
          ma = c[i] > ma ? c[i] : ma;
          ha = true;
        } else {
          mb = c[i] > mb ? c[i] : mb;
          hb = true;
        }
      }
      ma = warp_max_ull(ma);
      const bool anya = __any_sync(0xFFFFFFFFu, ha);
      if (lane == 0 && anya) atomicMax(a.codes + wa, ma);
      if (__any_sync(0xFFFFFFFFu, hb)) {
        mb = warp_max_ull(mb);
        if (lane == 0) atomicMax(a.codes + wa + 1, mb);
      }
    } else if (any) {
      uint32_t cur = 0xFFFFFFFFu;
      unsigned long long m = 0;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t row = row0 + i;
        if (row < a.lo || row >= a.hi) continue;
        const uint32_t win = (row - a.s) / a.w;
        if (win != cur) {
          if (cur != 0xFFFFFFFFu) atomicMax(a.codes + cur, m);
          cur = win;
          m = 0;
        }
        m = c[i] > m ? c[i] : m;
      }
      if (cur != 0xFFFFFFFFu) atomicMax(a.codes + cur, m);
    }
  }
}

// The same maxima for windows of at least 1,024 rows on columns with byte
// slices, as the progressive max of byte_fixed_max per window, in two
// passes over 1,024-row chunks (a warp per chunk, a lane per 32-row block;
// a chunk touches at most two windows).  Pass 1 reads slice 0 only: the
// largest leading byte of each (chunk, window) part goes to tops[] and is
// folded into the window's wtop[].  Pass 2 revisits only the parts whose
// leading byte equals their window's, refines the rows holding it through
// the later slices and the tail (max_in_block) and folds the code into the
// window with one atomic.  Rows outside a window read as the zero code.

// This lane's rows of [ra, re) among its 32 rows from row0, and the
// unflipped slice-0 bytes of those rows (others zero).
__device__ __forceinline__ uint32_t window_bytes(const Bytes32 &d, uint32_t row0, uint32_t ra,
                                                 uint32_t re, uint32_t *u) {
  uint32_t live = 0;
  if (row0 < re && row0 + 32 > ra) {
    const uint32_t from = ra > row0 ? ra - row0 : 0u;
    const uint32_t to = re - row0 < 32 ? re - row0 : 32u;
    live = (to >= 32 ? 0xFFFFFFFFu : ((1u << to) - 1u)) & ~((1u << from) - 1u);
  }
#pragma unroll
  for (int q = 0; q < 8; ++q) u[q] = (d.w[q] ^ H) & expand4((live >> (4 * q)) & 0xFu);
  return live;
}

__device__ __forceinline__ Bytes32 chunk_block(const WinArgs &a, uint32_t row0) {
  Bytes32 d;
  if (row0 < a.hi && row0 + 32 > a.lo) {
    d = ld_cand32(a.slices + row0);
  } else {
#pragma unroll
    for (int q = 0; q < 8; ++q) d.w[q] = H;
  }
  return d;
}

// The window rows [ra, re) of window x.
__device__ __forceinline__ void window_rows(const WinArgs &a, uint32_t x, uint32_t &ra,
                                            uint32_t &re) {
  const uint32_t ws = a.s + x * a.w;
  const uint64_t we = (uint64_t)ws + a.w;
  ra = ws > a.lo ? ws : a.lo;
  re = we < a.hi ? (uint32_t)we : a.hi;
}

__device__ __forceinline__ void chunk_windows(const WinArgs &a, uint32_t cr0, uint32_t &wa,
                                              uint32_t &wb) {
  const uint32_t first = cr0 > a.lo ? cr0 : a.lo;
  const uint32_t last = cr0 + 1023 < a.hi - 1 ? cr0 + 1023 : a.hi - 1;
  wa = (first - a.s) / a.w;
  wb = (last - a.s) / a.w;
}

__global__ void __launch_bounds__(kThreads) k_max_range_tops(WinArgs a, uint8_t *tops,
                                                             unsigned int *wtop) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t c0 = a.lo / 1024, c1 = (a.hi - 1) / 1024;
  for (uint32_t ch = c0 + warp; ch <= c1; ch += nwarps) {
    const uint32_t cr0 = ch * 1024, row0 = cr0 + lane * 32;
    const Bytes32 d = chunk_block(a, row0);
    uint32_t wa, wb;
    chunk_windows(a, cr0, wa, wb);
    for (uint32_t x = wa; x <= wb; ++x) {
      uint32_t ra, re, u[8], mx = 0;
      window_rows(a, x, ra, re);
      window_bytes(d, row0, ra, re, u);
#pragma unroll
      for (int q = 0; q < 8; ++q) mx = __vmaxu4(mx, u[q]);
      mx = __vmaxu4(mx, mx >> 16);
      mx = __vmaxu4(mx, mx >> 8);
      const uint32_t top = __reduce_max_sync(0xFFFFFFFFu, mx & 0xFFu);
      if (lane == 0) {
        tops[2 * (size_t)(ch - c0) + (x - wa)] = (uint8_t)top;
        atomicMax(wtop + x, top);
      }
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_max_range_refine(WinArgs a,
                                                               const uint8_t *__restrict__ tops,
                                                               const unsigned int *__restrict__ wtop) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
  const uint32_t c0 = a.lo / 1024, c1 = (a.hi - 1) / 1024;
  for (uint32_t ch = c0 + warp; ch <= c1; ch += nwarps) {
    const uint32_t cr0 = ch * 1024, row0 = cr0 + lane * 32;
    uint32_t wa, wb;
    chunk_windows(a, cr0, wa, wb);
    bool any = false;
    for (uint32_t x = wa; x <= wb; ++x)
      any |= tops[2 * (size_t)(ch - c0) + (x - wa)] == (uint8_t)wtop[x];
    if (!any) continue;  // no row of this chunk can hold a window's maximum
    const Bytes32 d = chunk_block(a, row0);
    for (uint32_t x = wa; x <= wb; ++x) {
      const uint32_t top = wtop[x];
      if (tops[2 * (size_t)(ch - c0) + (x - wa)] != (uint8_t)top) continue;
      uint32_t ra, re, u[8], e[8];
      window_rows(a, x, ra, re);
      const uint32_t live = window_bytes(d, row0, ra, re, u);
#pragma unroll
      for (int q = 0; q < 8; ++q) e[q] = eqbytes(u[q], top * 0x01010101u);
      const uint32_t cand = gather32(e) & live;
      const unsigned long long code =
          cand ? max_in_block(a.slices, a.stride, a.k, a.tail, a.r, row0, cand, top) : 0ull;
      const unsigned long long m = warp_max_ull(code);
      if (lane == 0) atomicMax(a.codes + x, m);
    }
  }
}

// Window maxima as values.  `shift` drops the right padding of a buff-slice
// code; `empty` marks windows that read no row (f64::min_value()).
__global__ void k_codes_to_values(const unsigned long long *codes, uint32_t n, long long base,
                                  int dlen, uint32_t shift, uint32_t empty_from, double *out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = i >= empty_from
               ? -1.7976931348623157e308
               : i64_to_f64_scaled((long long)((unsigned long long)base + (codes[i] >> shift)), dlen);
}

int grid_for_items(uint64_t items) {
  uint64_t g = (items + kThreads - 1) / kThreads;
  int dev = 0;
  cudaGetDevice(&dev);
  const uint64_t cap = (uint64_t)16 * num_sms(dev);
  if (g > cap) g = cap;
  return g < 1 ? 1 : (int)g;
}

}  // namespace

cudaError_t decode_rows(const buff_col *c, const uint32_t *rows, uint64_t nrows,
                        const uint32_t *words, const uint32_t *rank, int tail_shift, double *out,
                        cudaStream_t s) {
  RowArgs a;
  a.slices = c->slices;
  a.tail = c->tail;
  a.stride = c->stride;
  a.n = c->n;
  a.k = c->k - c->m;  // a buff-major column decodes here only without sparse columns
  a.r = c->r;
  a.tail_shift = tail_shift;
  a.base = c->base;
  a.dlen = (int)c->dlen;
  a.out = out;
  if (rows) {
    if (!nrows) return cudaSuccess;
    k_decode_list<<<grid_for_items(nrows), kThreads, 0, s>>>(a, rows, nrows);
  } else {
    if (!c->n) return cudaSuccess;
    // every value base + code in 32 bits: the exact 32-bit conversion
    const uint32_t bits = 8 * a.k + a.r + (tail_shift && a.k && a.r ? a.r : 0u);
    const long long maxc = bits >= 63 ? -1 : (long long)((1ull << bits) - 1ull);
    const bool n32 = bits <= 32 && c->base >= INT32_MIN && maxc >= 0 &&
                     c->base + maxc <= (long long)INT32_MAX;
    const int g = grid_for_items(((uint64_t)c->n + 3) / 4);
#define DW4(KSV)                                                           \
  (n32 ? k_decode_words4<true, KSV><<<g, kThreads, 0, s>>>(a, words, rank) \
       : k_decode_words4<false, KSV><<<g, kThreads, 0, s>>>(a, words, rank))
    switch (a.k) {
      case 1: DW4(1); break;
      case 2: DW4(2); break;
      case 3: DW4(3); break;
      case 4: DW4(4); break;
      default: DW4(0); break;
    }
#undef DW4
  }
  count_launch();
  return cudaGetLastError();
}

cudaError_t step_ranks(const uint32_t *words, uint32_t n, uint32_t *rank, cudaStream_t s) {
  const uint32_t nsteps = (uint32_t)(((uint64_t)n + 127) / 128);
  if (!nsteps) return cudaMemsetAsync(rank, 0, sizeof(uint32_t), s);
  uint32_t *tmp = nullptr;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&tmp),
                                  sizeof(uint32_t) * exclusive_scan_tmp(nsteps), s);
  if (e != cudaSuccess) return e;
  k_step_popc<<<grid_for_items(nsteps), kThreads, 0, s>>>(words, n, nsteps, rank);
  count_launch();
  e = exclusive_scan(rank, nsteps, tmp, s);  // rank[nsteps] = the total
  cudaFreeAsync(tmp, s);
  return e;
}

cudaError_t max_range(const buff_col *c, uint32_t lo, uint32_t hi, uint32_t s, uint32_t w,
                      uint32_t nwin, unsigned long long *codes, double *out, cudaStream_t st,
                      uint32_t shift, uint32_t empty_from) {
  WinArgs a;
  a.slices = c->slices;
  a.tail = c->tail;
  a.stride = c->stride;
  a.k = c->k;
  a.r = c->r;
  a.lo = lo;
  a.hi = hi;
  a.s = s;
  a.w = w;
  a.codes = codes;
  cudaError_t e = cudaMemsetAsync(codes, 0, sizeof(unsigned long long) * nwin, st);
  if (e != cudaSuccess || !nwin) return e;
  if (hi > lo) {
    const uint64_t steps = (hi - (lo & ~127u) + 127) / 128;
    const int grid = grid_for_items(steps * 32);
    if (w >= 1024 && c->k >= 1) {
      const uint64_t chunks = (hi - 1) / 1024 - lo / 1024 + 1;
      uint8_t *tops = nullptr;
      unsigned int *wtop = nullptr;
      e = cudaMallocAsync(reinterpret_cast<void **>(&tops), 2 * chunks, st);
      if (e == cudaSuccess)
        e = cudaMallocAsync(reinterpret_cast<void **>(&wtop), sizeof(unsigned int) * nwin, st);
      if (e == cudaSuccess) e = cudaMemsetAsync(wtop, 0, sizeof(unsigned int) * nwin, st);
      if (e == cudaSuccess) {
        const int g = grid_for_items(chunks * 32);
        k_max_range_tops<<<g, kThreads, 0, st>>>(a, tops, wtop);
        k_max_range_refine<<<g, kThreads, 0, st>>>(a, tops, wtop);
        count_launch();  // with the one below: two launches
      }
      if (tops) cudaFreeAsync(tops, st);
      if (wtop) cudaFreeAsync(wtop, st);
      if (e != cudaSuccess) return e;
    } else if (w >= 128)
      k_max_range<true><<<grid, kThreads, 0, st>>>(a);
    else
      k_max_range<false><<<grid, kThreads, 0, st>>>(a);
    count_launch();
  }
  k_codes_to_values<<<(nwin + 255) / 256, 256, 0, st>>>(codes, nwin, c->base, (int)c->dlen, shift,
                                                         empty_from, out);
  count_launch();
  return cudaGetLastError();
}

cudaError_t check_rows(const uint32_t *rows, uint64_t nrows, uint32_t n, uint32_t *bad,
                       cudaStream_t s) {
  if (!nrows) return cudaSuccess;
  k_check_rows<<<grid_for_items(nrows), kThreads, 0, s>>>(rows, nrows, n, bad);
  count_launch();
  return cudaGetLastError();
}

}  // namespace buffk
