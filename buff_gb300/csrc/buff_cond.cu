// Row-conditioned decode: values of listed rows or of the rows set in a
// bitmap (buff_decode_condition, compress/buff_simd.rs:1528-1712, and
// buff_major_decode_condition, :1714-1914).
//
// The reference walks each slice once per listed row with the BitPack
// reader; here every selected row is rebuilt independently from its k slice
// bytes and its packed tail field.  For the bitmap form one thread owns one
// row, so a warp covers one 32-row bitmap word and its slice reads coalesce;
// the output slot of a row is the prefix count of set bits before its word
// plus the set bits below it in the word.
#include <cuda_runtime.h>
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

__global__ void __launch_bounds__(kThreads) k_decode_words(RowArgs a, const uint32_t *__restrict__ words,
                                                           const uint32_t *__restrict__ rank) {
  const uint32_t lane = threadIdx.x & 31;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < a.n;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t w = i >> 5;
    const uint32_t b = __ldg(words + w);
    if (!(b >> lane & 1u)) continue;
    const uint32_t at = __ldg(rank + w) + __popc(b & ((1u << lane) - 1u));
    a.out[at] = row_value(a, (uint32_t)i);
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
    k_decode_words<<<grid_for_items(c->n), kThreads, 0, s>>>(a, words, rank);
  }
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
