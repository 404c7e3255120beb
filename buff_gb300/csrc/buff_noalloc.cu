// Range filter that allocates nothing (buff_range_filter_noalloc).
//
// Some callers cannot allocate device memory per query: a query server that
// has reserved the whole HBM budget for resident columns, or a host process
// whose device memory belongs to another allocator, must not call
// cudaMalloc / cudaMallocAsync from a query path.  The regular
// buff_range_filter stages its bitmap and count in per-call scratch when the
// outputs are host memory; this variant uses a fixed scratch array that lives
// in the library's device image instead.
//
// The scratch array below is part of this library's device code.  CUDA loads
// device code lazily, so a device reserves the array (about 8 MiB) the first
// time this entry point runs on it, and holds it until the process exits.  All
// calls share it: two calls whose work overlaps on the GPU (for example on two
// streams) race on it, so callers must order them.
#include <cuda_runtime.h>
#include <stdint.h>
#include <mutex>

#include "buff_internal.h"

namespace {

constexpr uint32_t kNoallocWords = BUFF_NOALLOC_MAX_ROWS / 32;
// Bitmap words for up to BUFF_NOALLOC_MAX_ROWS rows, then the 64-bit count.
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoallocWords + 64];

// Device address of g_noalloc_scratch, looked up once per device.  In host
// code the symbol itself is only a host-side stand-in, never a device address.
std::mutex g_mu;
uint32_t *g_addr[64] = {nullptr};

int scratch_address(int device, uint32_t **out) {
  if (device < 0 || device >= 64) return BUFF_EINVAL;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[device]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      // the lookup loads this file's device code, which reserves the array
      return e == cudaErrorMemoryAllocation ? BUFF_ENOMEM : BUFF_ECUDA;
    }
    g_addr[device] = static_cast<uint32_t *>(p);
  }
  *out = g_addr[device];
  return BUFF_OK;
}

}  // namespace

extern "C" int buff_range_filter_noalloc(const buff_col *c, double pred, uint32_t *words,
                                         uint64_t *count, void *stream) {
  if (!c || (!words && c->n > 0)) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;  // buff-major columns are not supported here
  if (c->n > BUFF_NOALLOC_MAX_ROWS) return BUFF_ESCRATCH;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return BUFF_ECUDA;
  uint32_t *scratch = nullptr;
  int rc = scratch_address(dev, &scratch);
  if (rc != BUFF_OK) return rc;
  const uint32_t n = c->n, nw = (n + 31) / 32;
  unsigned long long *dcount = reinterpret_cast<unsigned long long *>(scratch + kNoallocWords);
  // The plan of buff_simd_range_filter (compress/buff_simd.rs:3361-3547), the
  // one buff_range_filter runs: early return, full compare for fixed_len < 8
  // (or the intended semantics), truncated per-slice target bytes otherwise.
  int action = 2;  // 0: no rows, 1: all rows, 2: kernel
  buffk::FilterArgs a;
  rc = buffh::plan_filter(c, pred, 0 /* range */, &a, &action);
  if (rc != BUFF_OK) return rc;
  a.slices = c->slices;
  a.stride = c->stride;
  a.tail = c->tail;
  if (n == 0) {
    if (!count) return BUFF_OK;
    if (!buffh::is_device_ptr(count)) {
      *count = 0;
      return BUFF_OK;
    }
    cudaError_t e = cudaMemsetAsync(count, 0, sizeof(uint64_t), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    return e == cudaSuccess ? BUFF_OK : buffh::cuda_status(e);
  }
  cudaError_t e = cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess) {
    if (action == 2) {
      a.words = scratch;
      a.count = dcount;
      e = buffk::launch_filter(a, s);
    } else {
      e = buffk::launch_fill_words(scratch, n, action ? 0xFFFFFFFFu : 0u, dcount, s);
    }
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(words, scratch, (size_t)nw * 4, cudaMemcpyDefault, s);
  if (e == cudaSuccess && count)
    e = cudaMemcpyAsync(count, dcount, sizeof(uint64_t), cudaMemcpyDefault, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return buffh::cuda_status(e);
  }
  return BUFF_OK;
}
