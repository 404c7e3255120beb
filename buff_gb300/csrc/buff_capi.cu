// C ABI of the GB300 BUFF column codec (include/buff_gpu.h).
//
// Host side of every entry point: argument checks, the scalar steps the
// reference runs once per column or query (precision, bit width, predicate
// target, the f64 combine of the sum), staging of host buffers, and the
// launch of the kernels in buff_kernels.cu.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <new>
#include <vector>

#include "buff_device.cuh"
#include "buff_internal.h"
#include "buff_roaring.h"
#include "buff_snappy.h"

using buffk::EncStats;
using buffk::FilterArgs;

namespace {

thread_local int g_last_cuda = 0;

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return BUFF_OK;
  g_last_cuda = (int)e;
  if (e == cudaErrorMemoryAllocation) return BUFF_ENOMEM;
  return BUFF_ECUDA;
}

#define CK(expr)                              \
  do {                                        \
    cudaError_t _e = (expr);                  \
    if (_e != cudaSuccess) {                  \
      rc = cuda_status(_e);                   \
      goto done;                              \
    }                                         \
  } while (0)

inline cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// True when `p` can be dereferenced by the device (device or managed memory).
bool is_device_ptr(const void *p) {
  if (!p) return false;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, p);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// ---- scalar steps of the reference (host, once per column / query) ----

// `(scale as f32).log10() as i32` (compress/buff_simd.rs:3127); scale 0 -> 0.
int prec_of_scale(uint64_t scale) {
  if (scale == 0) return 0;
  float l = log10f((float)scale);
  if (isnan(l)) return 0;
  if (l >= 2147483647.0f) return 2147483647;
  if (l <= -2147483648.0f) return -2147483647 - 1;
  return (int)l;
}

// PRECISION_MAP (compress/mod.rs:29-46): decimals -> fractional bits.
int dlen_of_prec(int prec) {
  static const int kMap[16] = {-1, 5, 8, 11, 15, 18, 21, 25, 28, 31, 35, 38, 50, 10, 10, 10};
  return (prec >= 1 && prec <= 15) ? kMap[prec] : -1;
}

// Exponent of get_precision_bound(prec) (methods/prec_double.rs:273-281,
// PrecisionBound::new :28-33): the decimal string "0.<prec zeros>49".
int precision_exp_of(int prec) {
  char buf[64];
  int p = 0;
  buf[p++] = '0';
  buf[p++] = '.';
  for (int i = 0; i < prec && p < 60; ++i) buf[p++] = '0';
  buf[p++] = '4';
  buf[p++] = '9';
  buf[p] = 0;
  double d = strtod(buf, nullptr);
  uint64_t u;
  memcpy(&u, &d, 8);
  return (int)((u >> 52) & 0x7FF) - 1023;
}

// PrecisionBound::fetch_fixed_aligned (methods/prec_double.rs:190-205).
int64_t fetch_fixed_host(double v, int pexp, uint32_t dlen) {
  uint64_t b;
  memcpy(&b, &v, 8);
  int exp = (int)((b >> 52) & 0x7FF) - 1023;
  if (exp < pexp) return 0;
  int sh = 63 - exp - (int)dlen;
  uint64_t f = ((b << 11) | 0x8000000000000000ull) >> (sh & 63);
  if (b >> 63) f = ~(f - 1);
  return (int64_t)f;
}

void set_layout(buff_col *c, uint32_t fl) {
  c->fixed_len = fl;
  if (fl < 8) {
    c->k = 0;
    c->r = fl;
  } else {
    c->k = fl / 8;
    c->r = fl % 8;
  }
}

uint64_t serialized_size(const buff_col *c) {
  return 20ull + (uint64_t)c->k * c->n + ((uint64_t)c->n * c->r + 7) / 8;
}

// Column storage comes from the device's stream-ordered pool, whose release
// threshold is raised once per device so that freed columns stay cached for
// the next encode/deserialize instead of going back to the driver.
void init_pool(int device) {
  static std::atomic<bool> done[64];
  if (device < 0 || device >= 64 || done[device].load(std::memory_order_acquire)) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  cudaGetLastError();
  done[device].store(true, std::memory_order_release);  // setting it twice is harmless
}

int alloc_col(buff_col *c, cudaStream_t s) {
  init_pool(c->device);
  const size_t rows = buffk::round_up(c->n ? c->n : 1, buffk::kRowChunk);
  c->stride = rows;
  c->tail_bytes = ((uint64_t)c->n * c->r + 7) / 8;
  c->tail_alloc = rows / 8 * c->r + 64;
  cudaError_t e = cudaSuccess;
  if (c->k) e = cudaMallocAsync(reinterpret_cast<void **>(&c->slices), (size_t)c->k * c->stride, s);
  if (e != cudaSuccess) return cuda_status(e);
  e = cudaMallocAsync(reinterpret_cast<void **>(&c->tail), c->tail_alloc, s);
  if (e != cudaSuccess) return cuda_status(e);
  return BUFF_OK;
}

// Frees on `s` (stream-ordered after the work already queued there); with
// s == nullptr the whole device is drained first, so any stream may still
// have been reading the column.
void free_col(buff_col *c, cudaStream_t s = nullptr, bool ordered = false) {
  if (!c) return;
  if (c->arena) {  // slices and tail belong to the arena of a batched encode
    if (c->arena->refs.fetch_sub(1) == 1) {
      if (!ordered) cudaDeviceSynchronize();
      cudaFreeAsync(c->arena->base, s);
      if (!ordered) cudaStreamSynchronize(s);
      delete c->arena;
    }
    c->slices = nullptr;
    c->tail = nullptr;
  }
  void *bufs[5] = {c->slices, c->tail, c->obits, c->orank, c->obytes};
  bool any = false;
  for (void *b : bufs) any |= b != nullptr;
  if (any) {
    if (!ordered) cudaDeviceSynchronize();
    for (void *b : bufs)
      if (b) cudaFreeAsync(b, s);
    if (!ordered) cudaStreamSynchronize(s);
  }
  delete c;
}

buff_col *new_col(uint64_t scale, uint32_t flags) {
  buff_col *c = new (std::nothrow) buff_col;
  if (!c) return nullptr;
  memset(c, 0, sizeof(*c));
  c->scale = scale;
  c->flags = flags;
  c->prec = prec_of_scale(scale);
  c->precision_exp = precision_exp_of(c->prec);
  cudaGetDevice(&c->device);
  return c;
}

// Bits rebuilt by a precision-limited read (compress/split_double.rs:1642-1664).
int precision_bits(const buff_col *c, uint32_t precision, uint32_t *total) {
  const uint32_t ilen = c->ilen, dlen = c->dlen;
  if (precision == 0) {
    uint32_t rm = ilen;
    if (ilen % 8 > 0) rm = (ilen / 8 + 1) * 8;
    *total = rm;
    return BUFF_OK;
  }
  const int bn = dlen_of_prec(precision > 15 ? -1 : (int)precision);
  if (bn < 0) return BUFF_EREFPANIC;          // PRECISION_MAP.get(..).unwrap()
  const uint32_t bits_needed = (uint32_t)bn;
  if (!(dlen >= bits_needed)) return BUFF_EREFPANIC;  // assert!(dlen >= bits_needed)
  uint32_t rm = ilen + bits_needed;
  const uint32_t fixed_byte = (dlen + ilen) / 8;
  uint32_t byte_needed = (ilen + bits_needed) / 8;
  const uint32_t extra = (ilen + bits_needed) % 8;
  if (byte_needed < fixed_byte && extra > 0) {
    byte_needed += 1;
    rm = byte_needed * 8;
  }
  *total = rm;
  return BUFF_OK;
}

// The reference's f64 accumulation of byte_fixed_sum (split_double.rs:2141-2205)
// over `total` leading bits, from the exact per-slice sums.
double combine_sum(const buff_col *c, uint32_t total, const uint64_t *parts, bool intended) {
  const int32_t ilen_i = (int32_t)c->ilen;
  double sum_base = (double)c->n * (double)c->base;
  sum_base = sum_base / ldexp(1.0, (int)c->dlen);
  double sum = 0.0;
  int32_t processed = 0;
  uint32_t remain = total, slot = 0;
  while (remain >= 8) {
    remain -= 8;
    processed += 8;
    sum = sum + (double)parts[slot++] / ldexp(1.0, processed - ilen_i);
    if (remain == 0 && !intended) return sum;  // no base term when nothing follows
  }
  if (remain > 0) {
    processed += (int32_t)remain;
    sum = sum + (double)parts[slot] / ldexp(1.0, processed - ilen_i);
  }
  sum += sum_base;
  return sum;
}

// Device scratch for one call (stream-ordered pool allocation).
template <typename T>
cudaError_t scratch(T **p, size_t count, cudaStream_t s) {
  return cudaMallocAsync(reinterpret_cast<void **>(p), count * sizeof(T) + 16, s);
}

// ---------------------------------------------------------------- encode

cudaError_t reduce(const double *x, uint32_t n, uint32_t from, const buff_col *c, int keys,
                   int find_brk, EncStats *d, cudaStream_t s) {
  return buffk::launch_encode_reduce_f64(x, n, from, c->precision_exp, c->dlen, keys, find_brk, d,
                                         s);
}
cudaError_t reduce(const float *x, uint32_t n, uint32_t from, const buff_col *c, int keys,
                   int find_brk, EncStats *d, cudaStream_t s) {
  return buffk::launch_encode_reduce_f32(x, n, from, c->precision_exp, c->dlen, keys, find_brk, d,
                                         s);
}

// Slice layout (buff_slice_encode, compress/buff_slice.rs:298-437): every
// slice byte aligned, the last holding the low code bits left-aligned.
void set_slice_layout(buff_col *c, uint32_t fl) {
  c->layout = 2;
  c->k = fl < 8 ? 1u : (fl + 7) / 8;
  c->r = 0;
  c->fixed_len = 8 * c->k;
  c->pad = c->fixed_len - fl;
}

// Device bytes alloc_col takes for a column (slices and padded tail).
uint64_t col_alloc_bytes(const buff_col *c) {
  const uint64_t rows = buffk::round_up(c->n ? c->n : 1, buffk::kRowChunk);
  return (uint64_t)c->k * rows + rows / 8 * c->r + 64;
}

// `admit` (may be null) is asked for the column's device bytes once its
// width is known, before the column is allocated; a nonzero answer ends the
// encode with that status.
template <typename T>
int encode_impl(const T *values, uint64_t n64, uint64_t scale, uint32_t flags, cudaStream_t s,
                buff_col **out, bool slice = false, const buffh::EncodeAdmit *admit = nullptr) {
  if (!out) return BUFF_EINVAL;
  *out = nullptr;
  if (slice && (flags & BUFF_FLAG_INTENDED)) return BUFF_ENOTSUP;
  if (n64 > BUFF_MAX_ROWS) return BUFF_EINVAL;  // the header stores n as u32 (BUFF_MAX_ROWS)
  if (n64 > 0 && !values) return BUFF_EINVAL;
  const uint32_t n = (uint32_t)n64;
  const bool intended = flags & BUFF_FLAG_INTENDED;
  const int prec = prec_of_scale(scale);
  const int dl = dlen_of_prec(prec);
  if (dl < 0) return BUFF_EREFPANIC;  // PRECISION_MAP has no entry (scale < 10 or > 10^15)
  int rc = BUFF_OK;
  buff_col *c = new_col(scale, flags);
  if (!c) return BUFF_ENOMEM;
  c->n = n;
  c->dlen = (uint32_t)dl;
  T *staged = nullptr;
  EncStats *dst = nullptr;
  const T *dx = values;
  EncStats st;
  memset(&st, 0, sizeof(st));
  int64_t mn = INT64_MAX, mx = INT64_MIN;
  if (n > 0) {
    if (!is_device_ptr(values) || (reinterpret_cast<uintptr_t>(values) & 15)) {
      CK(scratch(&staged, n, s));
      CK(cudaMemcpyAsync(staged, values, (size_t)n * sizeof(T), cudaMemcpyDefault, s));
      dx = staged;
    }
    CK(scratch(&dst, 1, s));
    // Min/max on order keys of the raw values; quantize every row instead when
    // an extreme is non-finite or too large for the shift, or when small
    // magnitudes wrap the shift (precision bound below 2^-dlen: 13-15 decimals).
    int keys = c->precision_exp >= -(int)c->dlen ? 1 : 0;
    CK(reduce(dx, n, 1, c, keys, 1, dst, s));
    CK(cudaMemcpyAsync(&st, dst, sizeof(st), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (!st.ok) {
      keys = 0;
      CK(reduce(dx, n, 1, c, keys, 1, dst, s));
      CK(cudaMemcpyAsync(&st, dst, sizeof(st), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    }
    mn = st.mn;
    if (intended) {
      mx = st.mx0;
    } else if (n >= 2) {
      // Reference max (`else if`, compress/buff_simd.rs:3141-3146) = max of the
      // rows after the leading strictly decreasing run x_0 > x_1 > ... .
      const uint64_t brk = st.brk;
      if (brk == 1 || st.mx1 > st.x1) {
        mx = st.mx1;
      } else if (brk >= n) {
        mx = INT64_MIN;
      } else {
        EncStats s2;
        CK(reduce(dx, n, (uint32_t)brk, c, keys, 0, dst, s));
        CK(cudaMemcpyAsync(&s2, dst, sizeof(s2), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        mx = s2.mx1;
      }
    }
  }
  {
    const int64_t delta = (int64_t)((uint64_t)mx - (uint64_t)mn);
    uint32_t fl;
    if (intended) {
      fl = (n == 0 || delta == 0) ? 0u : (uint32_t)(64 - __builtin_clzll((uint64_t)delta));
    } else if (delta == 0) {
      fl = 0;
    } else {
      // `(delta as f64).log2().ceil() as usize` (buff_simd.rs:3156-3161)
      const double cl = ceil(log2((double)delta));
      fl = (isnan(cl) || cl <= 0.0) ? 0u : (uint32_t)cl;
    }
    if (!intended && !slice && fl == 0 && n > 0) {
      // write_bits(_, 0) indexes one past the buffer (bit_packing.rs:117)
      rc = BUFF_EREFPANIC;
      goto done;
    }
    c->base = mn;
    if (slice)
      set_slice_layout(c, fl);
    else
      set_layout(c, fl);
    c->ilen = (uint32_t)((uint64_t)fl - (uint64_t)c->dlen);
    if (admit && (rc = admit->fn(admit->ctx, col_alloc_bytes(c)))) goto done;
    if ((rc = alloc_col(c, s))) goto done;
    if (n > 0) {
      if (sizeof(T) == 8)
        CK(buffk::launch_encode_scatter_f64(reinterpret_cast<const double *>(dx), c, s));
      else
        CK(buffk::launch_encode_scatter_f32(reinterpret_cast<const float *>(dx), c, s));
    }
  }
done:
  if (staged) cudaFreeAsync(staged, s);
  if (dst) cudaFreeAsync(dst, s);
  if (rc != BUFF_OK) {
    cudaStreamSynchronize(s);
    free_col(c);
    return rc;
  }
  *out = c;
  return BUFF_OK;
}

// ---------------------------------------------------------------- filters

enum FilterKind {
  kRange = 0,
  kEqual = 1,
  kRangeSlice = 2,
  kEqualSlice = 3,
  kRangeScalar = 4,  // buff_range_filter (buff_simd.rs:4507-4679): every row
  kEqualScalar = 5   // buff_equal_filter (buff_simd.rs:4925-5094): every row
};

// The filter plan of buff_simd_range_filter / _equal_filter and their
// `_with_slice` forms for a buff-simd column: *action = 0 (no row set),
// 1 (every row set) or 2 (the filter kernel with *a, whose device pointers
// the caller fills in).  Returns BUFF_EREFPANIC where the reference panics.
int plan_filter(const buff_col *c, double pred, int kind, FilterArgs *a, int *action) {
  const bool intended = c->flags & BUFF_FLAG_INTENDED;
  const bool is_range = (kind == kRange || kind == kRangeSlice || kind == kRangeScalar);
  const bool with_slice = (kind == kRangeSlice || kind == kEqualSlice);
  // the scalar buff-layout filters read slice 0 byte by byte for every row,
  // so rows after the last full 32-row block are compared too
  const bool scalar = (kind == kRangeScalar || kind == kEqualScalar);
  const uint32_t n = c->n;
  *action = 2;
  memset(a, 0, sizeof(*a));
  const int64_t fixed_part = fetch_fixed_host(pred, c->precision_exp, c->dlen);
  if (fixed_part < c->base) {
    // early return (buff_simd.rs:3385-3388, 3573-3576, 3769-3772, 3919-3922):
    // the printed count is n for range and both fused forms, 0 for equality.
    *action = (kind == kEqual || kind == kEqualScalar) ? 0 : 1;
    return BUFF_OK;
  }
  const uint64_t t = (uint64_t)(fixed_part - c->base);
  const uint32_t fl = c->fixed_len;
  if (with_slice && !intended && (c->k == 0 || n < 32)) return BUFF_EREFPANIC;
  a->n = n;
  a->is_range = is_range ? 1u : 0u;
  if (intended || c->k == 0) {
    // full compare of every row against the untruncated target
    // (fixed_len < 8: buff_simd.rs:3395-3402, 3583-3590)
    const bool above = fl < 64 && (t >> fl) != 0;
    if (above) {
      *action = 0;
    } else {
      a->full_rows = n;
      a->k_used = c->k;
      a->r = c->r;
      for (uint32_t j = 0; j < c->k; ++j) a->tbyte[j] = (uint8_t)(t >> (fl - 8 * (j + 1)));
      a->ttail = c->r ? (uint32_t)(t & ((1ull << c->r) - 1)) : 0u;
    }
  } else {
    // byte slices with truncated per-slice targets (buff_simd.rs:3407, 3425, 3448)
    a->full_rows = scalar ? n : n / 32 * 32;
    a->k_used = with_slice ? (c->k < 4 ? c->k : 4u) : c->k;
    a->r = c->r;
    for (uint32_t j = 0; j < a->k_used; ++j) a->tbyte[j] = (uint8_t)(t >> (fl - 8 * (j + 1)));
    a->ttail = c->r ? (uint32_t)(t & ((1ull << c->r) - 1)) : 0u;
    if (!is_range) {
      a->tail_only_eq = 1;  // only the tail step writes `res` (buff_simd.rs:3684-3729)
      if (c->r == 0) *action = 0;
    }
  }
  return BUFF_OK;
}

int filter_impl(const buff_col *c, double pred, uint32_t *words, uint64_t *count, cudaStream_t s,
                FilterKind kind) {
  if (!c || (!words && c->n > 0)) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;  // buff-major columns: the *_majority calls
  const uint32_t n = c->n, nw = (n + 31) / 32;
  int rc = BUFF_OK;
  uint32_t *dwords = words;
  unsigned long long *dcount = nullptr;
  const bool words_host = n > 0 && !is_device_ptr(words);
  const bool count_host = count && !is_device_ptr(count);
  bool need_sync = words_host || count_host;
  // 0: fill zeros, 1: fill ones, 2: kernel
  int action = 2;
  FilterArgs a;
  if ((rc = plan_filter(c, pred, kind, &a, &action))) return rc;
  a.slices = c->slices;
  a.stride = c->stride;
  a.tail = c->tail;
  if (n == 0) {
    if (count) {
      if (count_host)
        *count = 0;
      else
        return cuda_status(cudaMemsetAsync(count, 0, sizeof(uint64_t), S(s)));
    }
    return BUFF_OK;
  }
  if (words_host) CK(scratch(&dwords, nw, s));
  if (count) {
    if (count_host)
      CK(scratch(&dcount, 1, s));
    else
      dcount = reinterpret_cast<unsigned long long *>(count);
    CK(buffk::zero_u64(dcount, 1, s));
  }
  if (action == 2) {
    a.words = dwords;
    a.count = dcount;
    CK(buffk::launch_filter(a, s));
  } else {
    CK(buffk::launch_fill_words(dwords, n, action ? 0xFFFFFFFFu : 0u, dcount, s));
  }
  if (words_host) CK(cudaMemcpyAsync(words, dwords, (size_t)nw * 4, cudaMemcpyDeviceToHost, s));
  if (count_host) CK(cudaMemcpyAsync(count, dcount, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  if (need_sync) CK(cudaStreamSynchronize(s));
done:
  if (words_host && dwords && dwords != words) cudaFreeAsync(dwords, s);
  if (count_host && dcount) cudaFreeAsync(dcount, s);
  return rc;
}

// ---------------------------------------------------------------- sum

int sum_partials(const buff_col *c, uint32_t total, unsigned long long *d, cudaStream_t s) {
  // slices read: total/8 (<= k); packed bits per row after them: total % 8
  // (for fixed_len < 8 and total < 8 the packed region itself).
  uint32_t ks, ts;
  if (total < 8) {
    ks = 0;
    ts = total;
  } else {
    ks = total / 8;
    ts = total % 8;
  }
  if (ks > c->k) return BUFF_EREFPANIC;  // reads past the slices (slice index panic)
  if (c->k && ks < c->k && ts) return BUFF_ENOTSUP;
  if (c->k && total < 8 && total > 0) return BUFF_ENOTSUP;
  cudaError_t e = buffk::zero_u64(d, 9, s);
  if (e != cudaSuccess) return cuda_status(e);
  return cuda_status(buffk::launch_sum(c, ks, ts, d, s));
}

// ---------------------------------------------------------------- buff-major

// Boyer-Moore majority vote of one byte over the sample (buff_simd.rs:382-446).
static void bm_vote(const uint64_t *codes, uint32_t cnt, uint32_t sh, uint8_t *major, int32_t *freq) {
  int32_t f = 0;
  uint8_t m = 0;
  for (uint32_t i = 0; i < cnt; ++i) {
    const uint8_t b = (uint8_t)(codes[i] >> sh);
    if (f == 0) {
      m = b;
      f = 1;
    } else if (m == b) {
      ++f;
    } else {
      --f;
    }
  }
  *major = m;
  *freq = f;
}

// forced_major >= 0: byte_residue_encode_outlieru8 (compress/split_double.rs:
// 957-1240), whose vote result is overwritten with MAJOR = 69 and whose count
// is never negative, so the leading byte is always the one sparse column; its
// bitmaps are croaring images.
template <typename T>
int encode_major_impl(const T *values, uint64_t n64, uint64_t scale, uint32_t flags, cudaStream_t s,
                      buff_col **out, int forced_major = -1) {
  if (!out) return BUFF_EINVAL;
  *out = nullptr;
  if (flags & BUFF_FLAG_INTENDED) return BUFF_ENOTSUP;
  if (n64 > BUFF_MAX_ROWS) return BUFF_EINVAL;
  if (n64 > 0 && !values) return BUFF_EINVAL;
  const uint32_t n = (uint32_t)n64;
  const int prec = prec_of_scale(scale);
  const int dl = dlen_of_prec(prec);
  if (dl < 0) return BUFF_EREFPANIC;
  if (n < 2000) return BUFF_EREFPANIC;  // fixed_vec[0..SAMPLE] (buff_simd.rs:382)
  int rc = BUFF_OK;
  buff_col *c = new_col(scale, flags);
  if (!c) return BUFF_ENOMEM;
  c->layout = 1;
  c->n = n;
  c->dlen = (uint32_t)dl;
  T *staged = nullptr;
  EncStats *dst = nullptr;
  uint8_t *lead = nullptr;
  const T *dx = values;
  EncStats st;
  memset(&st, 0, sizeof(st));
  T head[2000];
  uint64_t codes[2000];
  uint32_t fl = 0, m = 0;
  if (!is_device_ptr(values) || (reinterpret_cast<uintptr_t>(values) & 15)) {
    CK(scratch(&staged, n, s));
    CK(cudaMemcpyAsync(staged, values, (size_t)n * sizeof(T), cudaMemcpyDefault, s));
    dx = staged;
  }
  CK(scratch(&dst, 1, s));
  {
    int keys = c->precision_exp >= -(int)c->dlen ? 1 : 0;
    CK(reduce(dx, n, 1, c, keys, 0, dst, s));
    CK(cudaMemcpyAsync(&st, dst, sizeof(st), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(head, dx, sizeof(head), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (!st.ok) {
      CK(reduce(dx, n, 1, c, 0, 0, dst, s));
      CK(cudaMemcpyAsync(&st, dst, sizeof(st), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    }
  }
  {
    // exact min/max here (two ifs, buff_simd.rs:340-347)
    const int64_t mn = st.mn, mx = st.mx0;
    const int64_t delta = (int64_t)((uint64_t)mx - (uint64_t)mn);
    if (delta != 0) {
      const double cl = ceil(log2((double)delta));
      fl = (isnan(cl) || cl <= 0.0) ? 0u : (uint32_t)cl;
    }
    for (uint32_t i = 0; i < 2000; ++i)
      codes[i] = (uint64_t)(fetch_fixed_host((double)head[i], c->precision_exp, c->dlen) - mn);
    uint32_t rsf = fl >= 8 ? fl - 8 : 0;
    const int32_t limit = (int32_t)(2000.0f * 0.6f);
    uint8_t major;
    int32_t freq;
    bm_vote(codes, 2000, rsf, &major, &freq);
    if (forced_major >= 0) {
      c->majors[m++] = (uint8_t)forced_major;
      c->bm_roaring = 1;
    } else if (freq > limit) {
      c->majors[m++] = major;
      while (rsf > 7 && m < 8) {
        rsf -= 8;
        bm_vote(codes, 2000, rsf, &major, &freq);
        if (freq > limit)
          c->majors[m++] = major;
        else
          break;
      }
    }
    if (fl < 8) {
      // with a sparse column `remain -= 8` underflows; without one the packed
      // codes overwrite the column-count byte, so neither image is decodable
      rc = m ? BUFF_EREFPANIC : BUFF_ENOTSUP;
      goto done;
    }
    c->base = mn;
    set_layout(c, fl);
    c->m = m;
    c->ilen = (uint32_t)((uint64_t)fl - (uint64_t)c->dlen);
    const uint32_t k = c->k;
    c->k = k - m;  // allocate the dense slices only
    rc = alloc_col(c, s);
    c->k = k;
    if (rc) goto done;
    c->nwp = c->stride / 32;
    if (m) CK(scratch(&lead, (size_t)m * c->stride, s));
    if (sizeof(T) == 8)
      CK(buffk::launch_encode_scatter_f64(reinterpret_cast<const double *>(dx), c, s, lead, m));
    else
      CK(buffk::launch_encode_scatter_f32(reinterpret_cast<const float *>(dx), c, s, lead, m));
    if (m) CK(buffk::major_build_sparse(c, lead, s));
  }
done:
  if (staged) cudaFreeAsync(staged, s);
  if (dst) cudaFreeAsync(dst, s);
  if (lead) cudaFreeAsync(lead, s);
  if (rc != BUFF_OK) {
    cudaStreamSynchronize(s);
    free_col(c);
    return rc;
  }
  *out = c;
  return BUFF_OK;
}

// The byte image of a buff-major column (buff_simd.rs:449-528): header,
// column count, per sparse column (major, bitmap size, bitmap, outlier
// count, outlier bytes), a pad byte, the unflipped dense slices, the tail.
// The buff-major image (buff_simd.rs:317-630).  prefix_only: only the header
// and the sparse columns (up to the dense slices), which buff_serialize
// follows with the dense slices and tail written in place.
int major_image(const buff_col *c, std::vector<uint8_t> &img, cudaStream_t s,
                bool prefix_only = false) {
  int rc = BUFF_OK;
  const uint32_t n = c->n, kd = c->k - c->m;
  const size_t nw = ((size_t)n + 31) / 32;
  std::vector<uint32_t> bits((size_t)c->m * nw);
  std::vector<uint8_t> ob(c->oofs[c->m]);
  std::vector<uint8_t> dense(prefix_only ? 0 : (size_t)kd * n), tail(prefix_only ? 0 : c->tail_bytes);
  for (uint32_t col = 0; col < c->m; ++col)
    CK(cudaMemcpyAsync(bits.data() + col * nw, c->obits + col * c->nwp, nw * 4,
                       cudaMemcpyDeviceToHost, s));
  if (!ob.empty()) CK(cudaMemcpyAsync(ob.data(), c->obytes, ob.size(), cudaMemcpyDeviceToHost, s));
  if (!prefix_only && kd && n)
    CK(cudaMemcpy2DAsync(dense.data(), n, c->slices, c->stride, n, kd, cudaMemcpyDeviceToHost, s));
  if (!tail.empty())
    CK(cudaMemcpyAsync(tail.data(), c->tail, tail.size(), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  {
    img.clear();
    auto put32 = [&](uint32_t v) {
      for (int b = 0; b < 4; ++b) img.push_back((uint8_t)(v >> (8 * b)));
    };
    const uint64_t ub = (uint64_t)c->base;
    put32((uint32_t)ub);
    put32((uint32_t)(ub >> 32));
    put32(n);
    put32(c->ilen);
    put32(c->dlen);
    img.push_back((uint8_t)c->m);
    std::vector<uint8_t> bin(8 + 4 * nw);
    for (uint32_t col = 0; col < c->m; ++col) {
      // BitVec::to_binary: u64 nbits, then the words (bit-vec lib.rs:399-406)
      for (int b = 0; b < 8; ++b) bin[b] = (uint8_t)((uint64_t)n >> (8 * b));
      for (size_t w = 0; w < nw; ++w)
        for (int b = 0; b < 4; ++b) bin[8 + 4 * w + b] = (uint8_t)(bits[col * nw + w] >> (8 * b));
      std::vector<uint8_t> bm = c->bm_roaring ? buffroaring::serialize(bits.data() + col * nw, n)
                                : (c->flags & BUFF_FLAG_RAW_BITMAPS)
                                    ? bin
                                    : buffsnappy::compress(bin.data(), bin.size());
      img.push_back(c->majors[col]);
      put32((uint32_t)bm.size());
      img.insert(img.end(), bm.begin(), bm.end());
      put32(c->nout[col]);
      img.insert(img.end(), ob.begin() + c->oofs[col], ob.begin() + c->oofs[col] + c->nout[col]);
    }
    if (c->m) img.push_back(0);  // finish_write_byte before the dense region
    if (prefix_only) return BUFF_OK;
    for (uint8_t &b : dense) b ^= 0x80;  // the dense slices are stored unflipped
    img.insert(img.end(), dense.begin(), dense.end());
    img.insert(img.end(), tail.begin(), tail.end());
  }
done:
  return rc;
}

int filter_major_impl(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                      cudaStream_t s, bool is_range) {
  if (!c || (!words && c->n > 0)) return BUFF_EINVAL;
  if (c->layout != 1) return BUFF_ENOTSUP;
  const uint32_t n = c->n, nw = (n + 31) / 32;
  int rc = BUFF_OK;
  uint32_t *dwords = words;
  unsigned long long *dcount = nullptr;
  const bool words_host = n > 0 && !is_device_ptr(words);
  const bool count_host = count && !is_device_ptr(count);
  const int64_t fp = fetch_fixed_host(pred, c->precision_exp, c->dlen);
  const bool early = fp < c->base;  // (buff_simd.rs:886-889, 1939-1942)
  uint8_t tb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  uint32_t ttail = 0;
  if (!early) {
    const uint64_t t = (uint64_t)(fp - c->base);
    for (uint32_t j = 0; j < c->k; ++j) tb[j] = (uint8_t)(t >> (c->fixed_len - 8 * (j + 1)));
    ttail = c->r ? (uint32_t)(t & ((1ull << c->r) - 1)) : 0u;
  }
  if (words_host) CK(scratch(&dwords, nw, s));
  if (count) {
    if (count_host)
      CK(scratch(&dcount, 1, s));
    else
      dcount = reinterpret_cast<unsigned long long *>(count);
    CK(buffk::zero_u64(dcount, 1, s));
  }
  if (early)
    CK(buffk::launch_fill_words(dwords, n, is_range ? 0xFFFFFFFFu : 0u, dcount, s));
  else
    CK(buffk::major_filter(c, is_range ? 1 : 0, tb, ttail, dwords, dcount, s));
  if (words_host) CK(cudaMemcpyAsync(words, dwords, (size_t)nw * 4, cudaMemcpyDeviceToHost, s));
  if (count_host) CK(cudaMemcpyAsync(count, dcount, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  if (words_host || count_host) CK(cudaStreamSynchronize(s));
done:
  if (words_host && dwords && dwords != words) cudaFreeAsync(dwords, s);
  if (count_host && dcount) cudaFreeAsync(dcount, s);
  return rc;
}


// ---------------------------------------------------------------- row-conditioned reads

// Device copy of a row list (host lists are checked here, device lists by a
// kernel); BUFF_EINVAL unless strictly ascending and below n, as the
// reference's `entry - pre` walk requires.
int stage_rows(const buff_col *c, const uint32_t *rows, uint64_t nrows, const uint32_t **drows,
               uint32_t **owned, cudaStream_t s) {
  int rc = BUFF_OK;
  *owned = nullptr;
  *drows = rows;
  if (is_device_ptr(rows)) {
    uint32_t *bad = nullptr, hbad = 0;
    CK(scratch(&bad, 1, s));
    CK(cudaMemsetAsync(bad, 0, 4, s));
    CK(buffk::check_rows(rows, nrows, c->n, bad, s));
    CK(cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    cudaFreeAsync(bad, s);
    if (hbad) return BUFF_EINVAL;
    return BUFF_OK;
  }
  for (uint64_t i = 0; i < nrows; ++i)
    if (rows[i] >= c->n || (i && rows[i] <= rows[i - 1])) return BUFF_EINVAL;
  CK(scratch(owned, nrows, s));
  CK(cudaMemcpyAsync(*owned, rows, nrows * 4, cudaMemcpyHostToDevice, s));
  *drows = *owned;
done:
  return rc;
}

int decode_list_impl(const buff_col *c, const uint32_t *rows, uint64_t nrows, double *out,
                     int tail_shift, cudaStream_t s) {
  int rc = BUFF_OK;
  const uint32_t *drows = nullptr;
  uint32_t *owned = nullptr;
  const bool stage = !is_device_ptr(out);
  double *d = stage ? nullptr : out;
  if ((rc = stage_rows(c, rows, nrows, &drows, &owned, s))) goto done;
  if (stage) CK(scratch(&d, nrows, s));
  CK(buffk::decode_rows(c, drows, nrows, nullptr, nullptr, tail_shift, d, s));
  if (stage) {
    CK(cudaMemcpyAsync(out, d, nrows * 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
done:
  if (owned) cudaFreeAsync(owned, s);
  if (stage && d) cudaFreeAsync(d, s);
  return rc;
}

// Rows set in device words `dwords` (bits at or past n ignored): their
// ranks, the count, and the decoded values into `out` (host or device).
int decode_words_impl(const buff_col *c, const uint32_t *dwords, double *out, uint64_t *count,
                      int tail_shift, cudaStream_t s) {
  int rc = BUFF_OK;
  const uint32_t n = c->n;
  uint32_t *rank = nullptr;
  uint32_t tailw[2] = {0, 0};
  uint64_t cnt = 0;
  const bool stage = out && !is_device_ptr(out);
  double *d = stage ? nullptr : out;
  if (n == 0) {
    if (count) *count = 0;
    return BUFF_OK;
  }
  {
    const size_t nsteps = ((size_t)n + 127) / 128;
    CK(scratch(&rank, nsteps + 1, s));
    CK(buffk::step_ranks(dwords, n, rank, s));
    CK(cudaMemcpyAsync(&tailw[0], rank + nsteps, 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    cnt = tailw[0];
  }
  if (count) *count = cnt;
  if (out && cnt) {
    if (stage) CK(scratch(&d, cnt, s));
    CK(buffk::decode_rows(c, nullptr, 0, dwords, rank, tail_shift, d, s));
    if (stage) {
      CK(cudaMemcpyAsync(out, d, cnt * 8, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    }
  }
done:
  if (rank) cudaFreeAsync(rank, s);
  if (stage && d) cudaFreeAsync(d, s);
  return rc;
}

// buff_range_filter_condition (buff_simd.rs:4683-4921): candidate rows only,
// no early "all rows" (the reference returns its empty res), truncated
// target bytes, no 32-row restriction.
int filter_cond_impl(const buff_col *c, double pred, const uint32_t *cand, uint32_t *words,
                     uint64_t *count, cudaStream_t s) {
  const uint32_t n = c->n, nw = (n + 31) / 32;
  int rc = BUFF_OK;
  uint32_t *dwords = words, *dcand = const_cast<uint32_t *>(cand);
  unsigned long long *dcount = nullptr;
  const bool words_host = n > 0 && !is_device_ptr(words);
  const bool count_host = count && !is_device_ptr(count);
  const bool cand_host = n > 0 && !is_device_ptr(cand);
  const int64_t fp = fetch_fixed_host(pred, c->precision_exp, c->dlen);
  bool none = fp < c->base;
  uint8_t tb[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  uint32_t ttail = 0;
  if (!none) {
    const uint64_t t = (uint64_t)(fp - c->base);
    if (c->k == 0) {  // fixed_len < 8: `dec > fixed_target as u8` (:4713-4748)
      const uint32_t tt = (uint32_t)(t & 0xFF);
      if (c->r < 8 && tt >= (1u << c->r)) none = true;
      ttail = tt;
    } else {
      for (uint32_t j = 0; j < c->k; ++j) tb[j] = (uint8_t)(t >> (c->fixed_len - 8 * (j + 1)));
      ttail = c->r ? (uint32_t)(t & ((1ull << c->r) - 1)) : 0u;
    }
  }
  if (n == 0) {
    if (count) {
      if (count_host)
        *count = 0;
      else
        return cuda_status(cudaMemsetAsync(count, 0, sizeof(uint64_t), s));
    }
    return BUFF_OK;
  }
  if (words_host) CK(scratch(&dwords, nw, s));
  if (count) {
    if (count_host)
      CK(scratch(&dcount, 1, s));
    else
      dcount = reinterpret_cast<unsigned long long *>(count);
    CK(buffk::zero_u64(dcount, 1, s));
  }
  if (none) {
    CK(buffk::launch_fill_words(dwords, n, 0u, dcount, s));
  } else {
    if (cand_host) {
      CK(scratch(&dcand, nw, s));
      CK(cudaMemcpyAsync(dcand, cand, (size_t)nw * 4, cudaMemcpyHostToDevice, s));
    }
    CK(buffk::major_filter(c, 1, tb, ttail, dwords, dcount, s, dcand));
  }
  if (words_host) CK(cudaMemcpyAsync(words, dwords, (size_t)nw * 4, cudaMemcpyDeviceToHost, s));
  if (count_host) CK(cudaMemcpyAsync(count, dcount, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  if (words_host || count_host || cand_host) CK(cudaStreamSynchronize(s));
done:
  if (words_host && dwords && dwords != words) cudaFreeAsync(dwords, s);
  if (count_host && dcount) cudaFreeAsync(dcount, s);
  if (cand_host && dcand && dcand != cand) cudaFreeAsync(dcand, s);
  return rc;
}

// (defined with the RAPG entry points below)
int rapg_image(const buff_col *c, std::vector<uint8_t> &img, cudaStream_t s,
               bool prefix_only = false, bool *complete = nullptr);
}  // namespace

// ================================================================ C ABI

extern "C" {

int buff_encode_f64(const double *values, uint64_t n, uint64_t scale, uint32_t flags, void *stream,
                    buff_col **out) {
  return encode_impl<double>(values, n, scale, flags, S(stream), out);
}

int buff_encode_f32(const float *values, uint64_t n, uint64_t scale, uint32_t flags, void *stream,
                    buff_col **out) {
  return encode_impl<float>(values, n, scale, flags, S(stream), out);
}

int buff_col_free(buff_col *col) {
  if (!col) return BUFF_EINVAL;
  free_col(col);
  return BUFF_OK;
}

int buff_col_free_async(buff_col *col, void *stream) {
  if (!col) return BUFF_EINVAL;
  free_col(col, S(stream), true);
  return BUFF_OK;
}

int buff_col_get_info(const buff_col *c, buff_col_info *info) {
  if (!c || !info) return BUFF_EINVAL;
  memset(info, 0, sizeof(*info));
  info->base = c->base;
  info->n = c->n;
  info->ilen = c->ilen;
  info->dlen = c->dlen;
  info->fixed_len = c->fixed_len;
  info->k = c->k;
  info->r = c->r;
  info->scale = c->scale;
  info->prec = c->prec;
  info->precision_exp = c->precision_exp;
  info->flags = c->flags;
  info->outlier_cols = c->m;
  info->serialized_bytes = serialized_size(c);
  info->device_bytes = (uint64_t)c->k * c->stride + c->tail_alloc;
  if (c->layout == 1 || c->layout == 3) {
    info->device_bytes = (uint64_t)(c->k - c->m) * c->stride + c->tail_alloc +
                         (uint64_t)c->m * c->nwp * 8 + c->oofs[c->m];
    info->serialized_bytes = 0;  // known after compressing the bitmaps (buff_serialize)
  }
  return BUFF_OK;
}

int buff_serialize(const buff_col *c, uint8_t *out, uint64_t cap, uint64_t *len, void *stream) {
  if (!c || !len) return BUFF_EINVAL;
  if (c->layout == 1 || c->layout == 3) {
    std::vector<uint8_t> img;
    // the header and sparse columns first; the dense slices and tail follow
    // it from one kernel (in place into pinned memory, else staged and copied)
    bool complete = false;
    int st = c->layout == 1 ? major_image(c, img, S(stream), true)
                            : rapg_image(c, img, S(stream), true, &complete);
    if (st) return st;
    const uint64_t body = complete ? 0 : (uint64_t)(c->k - c->m) * c->n + c->tail_bytes;
    *len = img.size() + body;
    if (!out || cap < *len) return BUFF_EINVAL;
    if (!complete && !is_device_ptr(out)) {
      cudaError_t e = cudaSuccess;
      memcpy(out, img.data(), img.size());
      if (buffk::body_to_host(c, out + img.size(), body, c->k - c->m, 0x80808080u, S(stream),
                              &e)) {
        if (e == cudaSuccess) e = cudaStreamSynchronize(S(stream));
        return cuda_status(e);
      }
    }
    if (!complete) {  // the whole image on the host, then copied
      st = c->layout == 1 ? major_image(c, img, S(stream)) : rapg_image(c, img, S(stream));
      if (st) return st;
    }
    if (is_device_ptr(out)) {
      const cudaError_t e = cudaMemcpy(out, img.data(), img.size(), cudaMemcpyHostToDevice);
      return cuda_status(e);
    }
    memcpy(out, img.data(), img.size());
    return BUFF_OK;
  }
  const uint64_t need = serialized_size(c);
  *len = need;
  if (!out || cap < need) return BUFF_EINVAL;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  const bool dev = is_device_ptr(out);
  uint8_t hdr[20];
  const uint64_t ub = (uint64_t)c->base;
  const uint32_t words5[5] = {(uint32_t)ub, (uint32_t)(ub >> 32), c->n, c->ilen, c->dlen};
  for (int i = 0; i < 5; ++i)
    for (int b = 0; b < 4; ++b) hdr[4 * i + b] = (uint8_t)(words5[i] >> (8 * b));
  if (dev) {
    CK(cudaMemcpyAsync(out, hdr, 20, cudaMemcpyHostToDevice, s));
  } else {
    memcpy(out, hdr, 20);
    // every slice and tail byte (unflipped for the buff layout) from one
    // kernel: written in place into pinned memory, else staged on the device
    // and copied once
    cudaError_t e = cudaSuccess;
    const uint32_t flipx = (c->flags & BUFF_FLAG_BUFF_LAYOUT) ? 0x80808080u : 0u;
    if (buffk::body_to_host(c, out + 20, need - 20, c->k, flipx, s, &e)) {
      CK(e);
      CK(cudaStreamSynchronize(s));
      goto done;
    }
  }
  if (c->k && c->n)
    CK(cudaMemcpy2DAsync(out + 20, c->n, c->slices, c->stride, c->n, c->k, cudaMemcpyDefault, s));
  // the buff layout (byte_fixed_encode) stores the slice bytes unflipped
  if (dev && (c->flags & BUFF_FLAG_BUFF_LAYOUT))
    CK(buffk::flip_bytes(out + 20, (size_t)c->k * c->n, s));
  if (c->tail_bytes)
    CK(cudaMemcpyAsync(out + 20 + (uint64_t)c->k * c->n, c->tail, c->tail_bytes, cudaMemcpyDefault,
                       s));
  CK(cudaStreamSynchronize(s));  // hdr lives on this stack frame
  if (!dev && (c->flags & BUFF_FLAG_BUFF_LAYOUT))
    for (uint64_t i = 0; i < (uint64_t)c->k * c->n; ++i) out[20 + i] ^= 0x80u;
done:
  return rc;
}

int buff_deserialize(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                     void *stream, buff_col **out) {
  if (!out || !bytes) return BUFF_EINVAL;
  *out = nullptr;
  if (len < 20) return BUFF_ECORRUPT;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  const bool dev = is_device_ptr(bytes);
  uint8_t hdr[20];
  buff_col *c = nullptr;
  uint32_t w[5];
  if (dev) {
    CK(cudaMemcpyAsync(hdr, bytes, 20, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  } else {
    memcpy(hdr, bytes, 20);
  }
  for (int i = 0; i < 5; ++i)
    w[i] = (uint32_t)hdr[4 * i] | ((uint32_t)hdr[4 * i + 1] << 8) |
           ((uint32_t)hdr[4 * i + 2] << 16) | ((uint32_t)hdr[4 * i + 3] << 24);
  c = new_col(scale, flags);
  if (!c) return BUFF_ENOMEM;
  c->base = (int64_t)((uint64_t)w[0] | ((uint64_t)w[1] << 32));
  c->n = w[2];
  c->ilen = w[3];
  c->dlen = w[4];
  if (c->n > BUFF_MAX_ROWS) {
    rc = BUFF_ENOTSUP;
    goto done;
  }
  {
    const uint32_t fl = c->ilen + c->dlen;  // the decoders' `dlen + ilen` (u32)
    if (fl > 64 || c->dlen > 1000) {
      rc = BUFF_ECORRUPT;
      goto done;
    }
    set_layout(c, fl);
    if (serialized_size(c) > len) {
      rc = BUFF_ECORRUPT;
      goto done;
    }
    if ((rc = alloc_col(c, s))) goto done;
    cudaError_t ue = cudaSuccess;
    if (!dev && buffk::upload_slices(bytes, c,
                                     (flags & BUFF_FLAG_BUFF_LAYOUT) ? 0x80808080u : 0u, s,
                                     &ue)) {
      // slices read in place by the device, flipped and padded on the way
      CK(ue);
    } else {
      if (c->k && c->n)
        CK(cudaMemcpy2DAsync(c->slices, c->stride, bytes + 20, c->n, c->n, c->k,
                             cudaMemcpyDefault, s));
      if (c->k && c->n && (flags & BUFF_FLAG_BUFF_LAYOUT))
        CK(buffk::flip_bytes(c->slices, (size_t)c->k * c->stride, s));
      // padding rows of every slice hold the flipped zero byte (what encode writes)
      if (c->k && c->stride > c->n)
        CK(cudaMemset2DAsync(c->slices + c->n, c->stride, 0x80, c->stride - c->n, c->k, s));
    }
    CK(cudaMemsetAsync(c->tail, 0, c->tail_alloc, s));
    if (c->tail_bytes)
      CK(cudaMemcpyAsync(c->tail, bytes + 20 + (uint64_t)c->k * c->n, c->tail_bytes,
                         cudaMemcpyDefault, s));
    if (!dev) CK(cudaStreamSynchronize(s));
  }
done:
  if (rc != BUFF_OK) {
    free_col(c);
    return rc;
  }
  *out = c;
  return BUFF_OK;
}

int buff_decode(const buff_col *c, double *out, void *stream) {
  if (!c || (!out && c->n)) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;  // buff-major columns: the *_majority calls
  if (c->n == 0) return BUFF_OK;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  const bool stage = !is_device_ptr(out) || (reinterpret_cast<uintptr_t>(out) & 15);
  double *d = stage ? nullptr : out;
  if (stage) CK(scratch(&d, c->n, s));
  CK(buffk::launch_decode(c, c->fixed_len, 0, d, s));
  if (stage) {
    CK(cudaMemcpyAsync(out, d, (size_t)c->n * 8, cudaMemcpyDefault, s));
    CK(cudaStreamSynchronize(s));
  }
done:
  if (stage && d) cudaFreeAsync(d, s);
  return rc;
}

int buff_decode_at_precision(const buff_col *c, uint32_t precision, double *out, void *stream) {
  if (!c || (!out && c->n)) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;  // buff-major columns: the *_majority calls
  uint32_t total = 0;
  int rc = precision_bits(c, precision, &total);
  if (rc) return rc;
  const bool intended = c->flags & BUFF_FLAG_INTENDED;
  if (intended) {
    if (total > c->fixed_len) return BUFF_EREFPANIC;
  } else {
    if (total >= 8 && total / 8 > c->k) return BUFF_EREFPANIC;  // reads past the slices
    if (total < 8 && c->k && total) return BUFF_ENOTSUP;
  }
  if (c->n == 0) return BUFF_OK;
  cudaStream_t s = S(stream);
  const bool stage = !is_device_ptr(out) || (reinterpret_cast<uintptr_t>(out) & 15);
  double *d = stage ? nullptr : out;
  if (stage) CK(scratch(&d, c->n, s));
  CK(buffk::launch_decode(c, total, intended ? 1 : 0, d, s));
  if (stage) {
    CK(cudaMemcpyAsync(out, d, (size_t)c->n * 8, cudaMemcpyDefault, s));
    CK(cudaStreamSynchronize(s));
  }
done:
  if (stage && d) cudaFreeAsync(d, s);
  return rc;
}

int buff_range_filter(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                      void *stream) {
  return filter_impl(c, pred, words, count, S(stream), kRange);
}
int buff_equal_filter(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                      void *stream) {
  return filter_impl(c, pred, words, count, S(stream), kEqual);
}
int buff_scalar_range_filter(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                             void *stream) {
  return filter_impl(c, pred, words, count, S(stream), kRangeScalar);
}
int buff_scalar_equal_filter(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                             void *stream) {
  return filter_impl(c, pred, words, count, S(stream), kEqualScalar);
}
int buff_range_filter_with_slice(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                                 void *stream) {
  return filter_impl(c, pred, words, count, S(stream), kRangeSlice);
}
int buff_equal_filter_with_slice(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                                 void *stream) {
  return filter_impl(c, pred, words, count, S(stream), kEqualSlice);
}

int buff_sum_partials_async(const buff_col *c, uint64_t *dev_partials, void *stream) {
  if (!c || !dev_partials) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;  // buff-major columns: the *_majority calls
  return sum_partials(c, c->fixed_len, reinterpret_cast<unsigned long long *>(dev_partials),
                      S(stream));
}

int buff_range_filter_sum(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                          uint64_t *partials, void *stream) {
  if (!c || !partials || (!words && c->n > 0)) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  const uint32_t n = c->n, nw = (n + 31) / 32;
  const bool intended = c->flags & BUFF_FLAG_INTENDED;
  const int64_t fp = fetch_fixed_host(pred, c->precision_exp, c->dlen);
  uint32_t *dwords = words;
  unsigned long long *dcount = nullptr, *dparts = nullptr;
  const bool words_host = n > 0 && !is_device_ptr(words);
  const bool count_host = count && !is_device_ptr(count);
  const bool parts_host = !is_device_ptr(partials);
  if (intended || c->k == 0 || fp < c->base || n == 0) {
    // plans without a single pass: the two calls
    if ((rc = filter_impl(c, pred, words, count, s, kRange))) return rc;
    if (parts_host) {
      buff_sum_result r;
      if ((rc = buff_sum(c, &r, stream))) return rc;
      for (uint32_t j = 0; j < 9; ++j) partials[j] = j < r.n_partials ? r.partials[j] : 0;
      return BUFF_OK;
    }
    return sum_partials(c, c->fixed_len, reinterpret_cast<unsigned long long *>(partials), s);
  }
  {
    buffk::FilterArgs a;
    memset(&a, 0, sizeof(a));
    const uint64_t t = (uint64_t)(fp - c->base);
    const uint32_t fl = c->fixed_len;
    a.slices = c->slices;
    a.stride = c->stride;
    a.tail = c->tail;
    a.n = n;
    a.is_range = 1;
    a.full_rows = n / 32 * 32;
    a.k_used = c->k;
    a.r = c->r;
    for (uint32_t j = 0; j < c->k; ++j) a.tbyte[j] = (uint8_t)(t >> (fl - 8 * (j + 1)));
    a.ttail = c->r ? (uint32_t)(t & ((1ull << c->r) - 1)) : 0u;
    if (words_host) CK(scratch(&dwords, nw, s));
    if (count) {
      if (count_host)
        CK(scratch(&dcount, 1, s));
      else
        dcount = reinterpret_cast<unsigned long long *>(count);
    }
    if (parts_host)
      CK(scratch(&dparts, 9, s));
    else
      dparts = reinterpret_cast<unsigned long long *>(partials);
    CK(buffk::zero_u64(dparts, 9, s, dcount, 1));
    a.words = dwords;
    a.count = dcount;
    CK(buffk::launch_filter_sum(a, c, dparts, s));
    if (words_host) CK(cudaMemcpyAsync(words, dwords, (size_t)nw * 4, cudaMemcpyDeviceToHost, s));
    if (count_host) CK(cudaMemcpyAsync(count, dcount, 8, cudaMemcpyDeviceToHost, s));
    if (parts_host) CK(cudaMemcpyAsync(partials, dparts, 72, cudaMemcpyDeviceToHost, s));
    if (words_host || count_host || parts_host) CK(cudaStreamSynchronize(s));
  }
done:
  if (words_host && dwords && dwords != words) cudaFreeAsync(dwords, s);
  if (count_host && dcount) cudaFreeAsync(dcount, s);
  if (parts_host && dparts) cudaFreeAsync(dparts, s);
  return rc;
}

int buff_sum_finish(const buff_col *c, const uint64_t *parts, buff_sum_result *out) {
  if (!c || !parts || !out) return BUFF_EINVAL;
  memset(out, 0, sizeof(*out));
  const bool intended = c->flags & BUFF_FLAG_INTENDED;
  out->sum = combine_sum(c, c->fixed_len, parts, intended);
  __int128 acc = (__int128)c->n * (__int128)c->base;
  for (uint32_t j = 0; j < c->k; ++j) acc += (__int128)parts[j] << (c->fixed_len - 8 * (j + 1));
  if (c->r) acc += (__int128)parts[c->k];
  out->exact_num_lo = (int64_t)(uint64_t)acc;
  out->exact_num_hi = (int64_t)(acc >> 64);
  // exact / 2^dlen, rounded once (int128 -> double is round-to-nearest-even)
  out->exact = ldexp((double)acc, -(int)c->dlen);
  out->n_partials = c->k + (c->r ? 1u : 0u);
  for (uint32_t j = 0; j < out->n_partials && j < 9; ++j) out->partials[j] = parts[j];
  return BUFF_OK;
}

int buff_sum(const buff_col *c, buff_sum_result *out, void *stream) {
  if (!c || !out) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;  // buff-major columns: the *_majority calls
  cudaStream_t s = S(stream);
  uint64_t parts[9] = {0};
  unsigned long long *d = nullptr;
  int rc = BUFF_OK;
  if (c->n) {
    CK(scratch(&d, 9, s));
    if ((rc = sum_partials(c, c->fixed_len, d, s))) goto done;
    CK(cudaMemcpyAsync(parts, d, sizeof(parts), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  rc = buff_sum_finish(c, parts, out);
done:
  if (d) cudaFreeAsync(d, s);
  return rc;
}

int buff_sum_at_precision(const buff_col *c, uint32_t precision, double *out, void *stream) {
  if (!c || !out) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;  // buff-major columns: the *_majority calls
  uint32_t total = 0;
  int rc = precision_bits(c, precision, &total);
  if (rc) return rc;
  cudaStream_t s = S(stream);
  uint64_t parts[9] = {0};
  unsigned long long *d = nullptr;
  if (c->n) {
    CK(scratch(&d, 9, s));
    if ((rc = sum_partials(c, total, d, s))) goto done;
    CK(cudaMemcpyAsync(parts, d, sizeof(parts), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  } else if (total >= 8 && total / 8 > c->k) {
    rc = BUFF_EREFPANIC;
    goto done;
  }
  *out = combine_sum(c, total, parts, c->flags & BUFF_FLAG_INTENDED);
done:
  if (d) cudaFreeAsync(d, s);
  return rc;
}

int buff_max_async(const buff_col *c, uint64_t *dev_max_code, void *stream) {
  if (!c || !dev_max_code) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;  // buff-major columns: the *_majority calls
  cudaStream_t s = S(stream);
  cudaError_t e = buffk::zero_u64(reinterpret_cast<unsigned long long *>(dev_max_code), 1, s);
  if (e != cudaSuccess) return cuda_status(e);
  return cuda_status(
      buffk::launch_max(c, reinterpret_cast<unsigned long long *>(dev_max_code), s));
}

int buff_max(const buff_col *c, double *max_value, uint64_t *max_code, uint32_t *argmax_words,
             uint64_t *argmax_count, void *stream) {
  if (!c) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;  // buff-major columns: the *_majority calls
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  const uint32_t nw = (c->n + 31) / 32;
  unsigned long long *d = nullptr;
  uint32_t *dwords = nullptr;
  uint64_t m = 0, cnt = 0;
  const bool intended = c->flags & BUFF_FLAG_INTENDED;
  const bool words_dev = argmax_words && is_device_ptr(argmax_words);
  CK(scratch(&d, 2, s));
  CK(buffk::zero_u64(d, 2, s));
  if (c->n) CK(buffk::launch_max(c, d, s));
  if (argmax_words || argmax_count) {
    // byte_fixed_max fills `res` only in the tail step (or for fixed_len < 8).
    const bool empty = !intended && c->k > 0 && c->r == 0;
    if (c->n) {
      if (argmax_words) {
        if (words_dev)
          dwords = argmax_words;
        else
          CK(scratch(&dwords, nw, s));
      }
      if (empty) {
        if (dwords) CK(buffk::launch_fill_words(dwords, c->n, 0u, nullptr, s));
      } else {
        uint32_t *tmp = dwords;
        if (!tmp) CK(scratch(&tmp, nw, s));
        CK(buffk::launch_argmax(c, d, tmp, d + 1, s));
        if (!dwords) cudaFreeAsync(tmp, s);
      }
      if (argmax_words && !words_dev)
        CK(cudaMemcpyAsync(argmax_words, dwords, (size_t)nw * 4, cudaMemcpyDeviceToHost, s));
    }
  }
  CK(cudaMemcpyAsync(&m, d, sizeof(m), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&cnt, d + 1, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (max_code) *max_code = m;
  if (max_value)
    *max_value = (double)(int64_t)((uint64_t)c->base + m) / ldexp(1.0, (int)c->dlen);
  if (argmax_count) *argmax_count = cnt;
done:
  if (d) cudaFreeAsync(d, s);
  if (dwords && !words_dev) cudaFreeAsync(dwords, s);
  return rc;
}

// ---------------------------------------------------------------- buff-major ABI

int buff_encode_majority_f64(const double *values, uint64_t n, uint64_t scale, uint32_t flags,
                             void *stream, buff_col **out) {
  return encode_major_impl<double>(values, n, scale, flags, S(stream), out);
}

int buff_encode_majority_f32(const float *values, uint64_t n, uint64_t scale, uint32_t flags,
                             void *stream, buff_col **out) {
  return encode_major_impl<float>(values, n, scale, flags, S(stream), out);
}

}  // extern "C"

namespace {

// A buff-major image (snappy or raw BitVec bitmaps), or with `roaring` the
// RAPG-major image of byte_residue_encode_outlieru8 (croaring bitmaps, one
// sparse column: its queries equal the buff-major ones only there).
int deserialize_major_impl(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                           void *stream, buff_col **out, bool roaring) {
  if (!out || !bytes) return BUFF_EINVAL;
  *out = nullptr;
  if (flags & BUFF_FLAG_INTENDED) return BUFF_ENOTSUP;
  if (len < 21) return BUFF_ECORRUPT;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  std::vector<uint8_t> host;
  const uint8_t *b = bytes;
  buff_col *c = nullptr;
  std::vector<std::vector<uint32_t>> bms;
  std::vector<const uint8_t *> outl;
  size_t pos = 21, dense_at = 21;
  uint32_t w5[5], m;
  if (is_device_ptr(bytes)) {
    host.resize(len);
    CK(cudaMemcpyAsync(host.data(), bytes, len, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    b = host.data();
  }
  for (int i = 0; i < 5; ++i)
    w5[i] = (uint32_t)b[4 * i] | ((uint32_t)b[4 * i + 1] << 8) | ((uint32_t)b[4 * i + 2] << 16) |
            ((uint32_t)b[4 * i + 3] << 24);
  m = b[20];
  if (roaring && m != 1) return BUFF_ENOTSUP;
  c = new_col(scale, flags);
  if (!c) return BUFF_ENOMEM;
  c->layout = 1;
  c->bm_roaring = roaring ? 1u : 0u;
  c->base = (int64_t)((uint64_t)w5[0] | ((uint64_t)w5[1] << 32));
  c->n = w5[2];
  c->ilen = w5[3];
  c->dlen = w5[4];
  if (c->n > BUFF_MAX_ROWS) {
    rc = BUFF_ENOTSUP;
    goto done;
  }
  {
    const uint32_t fl = c->ilen + c->dlen;
    if (fl > 64 || c->dlen > 1000 || fl < 8 || m > fl / 8) {
      rc = fl < 8 ? BUFF_ENOTSUP : BUFF_ECORRUPT;
      goto done;
    }
    set_layout(c, fl);
    c->m = m;
    const size_t nw = ((size_t)c->n + 31) / 32;
    auto rd32 = [&](size_t at) -> uint32_t {
      return (uint32_t)b[at] | ((uint32_t)b[at + 1] << 8) | ((uint32_t)b[at + 2] << 16) |
             ((uint32_t)b[at + 3] << 24);
    };
    uint64_t off = 0;
    for (uint32_t col = 0; col < m; ++col) {
      if (pos + 5 > len) {
        rc = BUFF_ECORRUPT;
        goto done;
      }
      c->majors[col] = b[pos];
      const uint32_t bml = rd32(pos + 1);
      if (pos + 5 + (uint64_t)bml + 4 > len) {
        rc = BUFF_ECORRUPT;
        goto done;
      }
      std::vector<uint8_t> bin;
      std::vector<uint32_t> words(nw, 0);
      const size_t np = pos + 5 + bml;
      const uint32_t nout = rd32(np);
      if (roaring) {
        // Bitmap::deserialize: rows below n, one per outlier byte
        std::vector<uint32_t> rows;
        if (!buffroaring::parse(b + pos + 5, bml, rows) || rows.size() != nout ||
            (nout && rows.back() >= c->n)) {
          rc = BUFF_ECORRUPT;
          goto done;
        }
        for (uint32_t r : rows) words[r >> 5] |= 1u << (r & 31);
      } else {
        if (flags & BUFF_FLAG_RAW_BITMAPS) {
          bin.assign(b + pos + 5, b + pos + 5 + bml);
        } else if (!buffsnappy::decompress(b + pos + 5, bml, bin)) {
          rc = BUFF_ECORRUPT;
          goto done;
        }
        // BitVec::from_binary (bit-vec lib.rs:409-428)
        for (size_t at = 8, w = 0; at + 4 <= bin.size() && w < nw; at += 4, ++w)
          words[w] = (uint32_t)bin[at] | ((uint32_t)bin[at + 1] << 8) |
                     ((uint32_t)bin[at + 2] << 16) | ((uint32_t)bin[at + 3] << 24);
        if (nw && (c->n & 31)) words[nw - 1] &= (1u << (c->n & 31)) - 1u;
      }
      bms.push_back(std::move(words));
      if (np + 4 + (uint64_t)nout > len) {
        rc = BUFF_ECORRUPT;
        goto done;
      }
      c->nout[col] = nout;
      c->oofs[col] = off;
      off += nout;
      outl.push_back(b + np + 4);
      pos = np + 4 + nout;  // the pad written after the outliers holds the next major
    }
    c->oofs[m] = off;
    dense_at = m ? pos + 1 : 21;
    const uint32_t kd = c->k - m;
    const uint64_t need = dense_at + (uint64_t)kd * c->n + ((uint64_t)c->n * c->r + 7) / 8;
    if (need > len) {
      rc = BUFF_ECORRUPT;
      goto done;
    }
    const uint32_t k = c->k;
    c->k = kd;
    rc = alloc_col(c, s);
    c->k = k;
    if (rc) goto done;
    c->nwp = c->stride / 32;
    if (kd && c->n) {
      CK(cudaMemcpy2DAsync(c->slices, c->stride, b + dense_at, c->n, c->n, kd,
                           cudaMemcpyHostToDevice, s));
      CK(buffk::flip_bytes(c->slices, (size_t)kd * c->stride, s));
      if (c->stride > c->n)
        CK(cudaMemset2DAsync(c->slices + c->n, c->stride, 0x80, c->stride - c->n, kd, s));
    }
    CK(cudaMemsetAsync(c->tail, 0, c->tail_alloc, s));
    if (c->tail_bytes)
      CK(cudaMemcpyAsync(c->tail, b + dense_at + (uint64_t)kd * c->n, c->tail_bytes,
                         cudaMemcpyHostToDevice, s));
    if (m) {
      CK(scratch(&c->obits, (size_t)m * c->nwp, s));
      CK(scratch(&c->orank, (size_t)m * (c->nwp + 16), s));
      CK(scratch(&c->obytes, off + 16, s));
      CK(cudaMemsetAsync(c->obits, 0, sizeof(uint32_t) * m * c->nwp, s));
      for (uint32_t col = 0; col < m; ++col) {
        CK(cudaMemcpyAsync(c->obits + col * c->nwp, bms[col].data(), nw * 4,
                           cudaMemcpyHostToDevice, s));
        if (c->nout[col])
          CK(cudaMemcpyAsync(c->obytes + c->oofs[col], outl[col], c->nout[col],
                             cudaMemcpyHostToDevice, s));
      }
      CK(buffk::major_index(c, s));
    }
    CK(cudaStreamSynchronize(s));
  }
done:
  if (rc != BUFF_OK) {
    free_col(c);
    return rc;
  }
  *out = c;
  return BUFF_OK;
}

}  // namespace

extern "C" {

int buff_deserialize_majority(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                              void *stream, buff_col **out) {
  return deserialize_major_impl(bytes, len, scale, flags, stream, out, false);
}

// ---- RAPG-major (byte_residue_encode_outlieru8 and its queries) ----

int buff_rapg_encode_outlieru8_f64(const double *values, uint64_t n, uint64_t scale, uint32_t flags,
                                   void *stream, buff_col **out) {
  if (flags & BUFF_FLAG_RAW_BITMAPS) return BUFF_ENOTSUP;
  return encode_major_impl<double>(values, n, scale, flags, S(stream), out, 69);
}

int buff_rapg_encode_outlieru8_f32(const float *values, uint64_t n, uint64_t scale, uint32_t flags,
                                   void *stream, buff_col **out) {
  if (flags & BUFF_FLAG_RAW_BITMAPS) return BUFF_ENOTSUP;
  return encode_major_impl<float>(values, n, scale, flags, S(stream), out, 69);
}

int buff_rapg_major_deserialize(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                                void *stream, buff_col **out) {
  if (flags & BUFF_FLAG_RAW_BITMAPS) return BUFF_ENOTSUP;
  return deserialize_major_impl(bytes, len, scale, flags, stream, out, true);
}

int buff_rapg_decode_majority(const buff_col *c, double *out, void *stream) {
  if (c && !c->bm_roaring) return BUFF_ENOTSUP;
  return buff_decode_majority(c, out, stream);
}

int buff_rapg_range_filter_majority(const buff_col *c, double pred, uint32_t *words,
                                    uint64_t *count, void *stream) {
  if (c && !c->bm_roaring) return BUFF_ENOTSUP;
  return buff_range_filter_majority(c, pred, words, count, stream);
}

int buff_rapg_equal_filter_majority(const buff_col *c, double pred, uint32_t *words,
                                    uint64_t *count, void *stream) {
  if (c && !c->bm_roaring) return BUFF_ENOTSUP;
  return buff_equal_filter_majority(c, pred, words, count, stream);
}

int buff_rapg_sum_majority(const buff_col *c, buff_sum_result *out, void *stream) {
  if (c && !c->bm_roaring) return BUFF_ENOTSUP;
  return buff_sum_majority(c, out, stream);
}

int buff_rapg_max_majority(const buff_col *c, double *value, uint64_t *code, uint32_t *argmax,
                           uint64_t *argmax_count, void *stream) {
  if (c && !c->bm_roaring) return BUFF_ENOTSUP;
  return buff_max_majority(c, value, code, argmax, argmax_count, stream);
}

int buff_range_filter_majority(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                               void *stream) {
  return filter_major_impl(c, pred, words, count, S(stream), true);
}

int buff_equal_filter_majority(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                               void *stream) {
  return filter_major_impl(c, pred, words, count, S(stream), false);
}

int buff_decode_majority(const buff_col *c, double *out, void *stream) {
  if (!c || (!out && c->n)) return BUFF_EINVAL;
  if (c->layout != 1) return BUFF_ENOTSUP;
  for (uint32_t col = 0; col < c->m; ++col)
    if (c->nout[col] == 0) return BUFF_EREFPANIC;  // outlier_iter.next().unwrap() (:680)
  if (c->n == 0) return BUFF_OK;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  const bool stage = !is_device_ptr(out) || (reinterpret_cast<uintptr_t>(out) & 15);
  double *d = stage ? nullptr : out;
  if (stage) CK(scratch(&d, c->n, s));
  if (c->m)
    CK(buffk::major_decode(c, d, s));
  else
    CK(buffk::launch_decode(c, c->fixed_len, 0, d, s));
  if (stage) {
    CK(cudaMemcpyAsync(out, d, (size_t)c->n * 8, cudaMemcpyDefault, s));
    CK(cudaStreamSynchronize(s));
  }
done:
  if (stage && d) cudaFreeAsync(d, s);
  return rc;
}

namespace {
buffk::dev::MajorSumArgs major_sum_args(const buff_col *c) {
  buffk::dev::MajorSumArgs a;
  memset(&a, 0, sizeof(a));
  a.n = c->n;
  a.base = c->base;
  a.m = c->m;
  a.k = c->k;
  a.r = c->r;
  a.fixed_len = c->fixed_len;
  a.ilen = (int32_t)c->ilen;
  a.dlen = (int32_t)c->dlen;
  for (uint32_t i = 0; i < 8; ++i) {
    a.majors[i] = c->majors[i];
    a.nout[i] = c->nout[i];
  }
  return a;
}

// The raw byte sums of a buff-major column into d (24 u64, device): sparse
// columns' outlier bytes at d[0..m), dense slices and tail from d[8].
int major_raw_sums(const buff_col *c, unsigned long long *d, cudaStream_t s) {
  return cuda_status(buffk::major_sums(c, major_sum_args(c), d, nullptr, nullptr, s));
}
}  // namespace

int buff_sum_majority(const buff_col *c, buff_sum_result *out, void *stream) {
  if (!c || !out) return BUFF_EINVAL;
  if (c->layout != 1) return BUFF_ENOTSUP;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  unsigned long long *d = nullptr;
  unsigned long long h[24] = {0};
  CK(scratch(&d, 24, s));
  if ((rc = major_raw_sums(c, d, s))) goto done;
  CK(cudaMemcpyAsync(h, d, sizeof(uint64_t) * 24, cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  {
    // buff_sum_majority (buff_simd.rs:2294-2442)
    const buffk::dev::MajorSumArgs a = major_sum_args(c);
    unsigned long long parts[9] = {0};
    memset(out, 0, sizeof(*out));
    const uint32_t np = buffk::dev::major_sum_parts(a, h, parts);
    out->sum = buffk::dev::major_sum_f64(a, parts);
    __int128 acc = (__int128)c->n * (__int128)c->base;
    for (uint32_t j = 0; j < c->k; ++j) acc += (__int128)parts[j] << (c->fixed_len - 8 * (j + 1));
    if (c->r) acc += (__int128)parts[c->k];
    out->exact_num_lo = (int64_t)(uint64_t)acc;
    out->exact_num_hi = (int64_t)(acc >> 64);
    out->exact = ldexp((double)acc, -(int)c->dlen);
    out->n_partials = np;
    for (uint32_t j = 0; j < np; ++j) out->partials[j] = parts[j];
  }
done:
  if (d) cudaFreeAsync(d, s);
  return rc;
}

int buff_sum_majority_async(const buff_col *c, double *dev_sum, uint64_t *dev_partials,
                            void *stream) {
  if (!c || !dev_sum) return BUFF_EINVAL;
  if (c->layout != 1) return BUFF_ENOTSUP;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  unsigned long long *d = nullptr;
  CK(scratch(&d, 24, s));
  CK(buffk::major_sums(c, major_sum_args(c), d, dev_sum,
                       reinterpret_cast<unsigned long long *>(dev_partials), s));
done:
  if (d) cudaFreeAsync(d, s);
  return rc;
}

int buff_max_majority(const buff_col *c, double *max_value, uint64_t *max_code,
                      uint32_t *argmax_words, uint64_t *argmax_count, void *stream) {
  if (!c) return BUFF_EINVAL;
  if (c->layout != 1) return BUFF_ENOTSUP;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  uint32_t *cand = nullptr;
  unsigned char *st = nullptr;
  uint64_t res[2] = {0, 0};  // max code, arg-max count
  const size_t nw = ((size_t)c->n + 31) / 32;
  const size_t sb = buffk::major_max_state_bytes(), mo = buffk::major_max_state_mx_offset();
  if (c->n && !argmax_words && !argmax_count && buffk::major1_max_applies(c)) {
    // the value alone: one pass (the arg-max rows need the candidate steps)
    CK(scratch(&st, sb, s));
    unsigned long long *mx = reinterpret_cast<unsigned long long *>(st + mo);
    CK(buffk::major1_max(c, mx, s));
    CK(cudaMemcpyAsync(res, mx, 8, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (max_code) *max_code = res[0];
    if (max_value)
      *max_value = (double)(int64_t)((uint64_t)c->base + res[0]) / ldexp(1.0, (int)c->dlen);
    goto done;
  }
  CK(scratch(&cand, c->nwp, s));
  CK(scratch(&st, sb, s));
  if (c->n) {
    CK(buffk::launch_fill_words(cand, c->n, 0xFFFFFFFFu, nullptr, s));
    CK(buffk::major_max(c, cand, st, s));
    if (argmax_words) CK(cudaMemcpyAsync(argmax_words, cand, nw * 4, cudaMemcpyDefault, s));
    CK(cudaMemcpyAsync(res, st + mo, 16, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaStreamSynchronize(s));
  if (max_code) *max_code = res[0];
  if (max_value)
    *max_value = (double)(int64_t)((uint64_t)c->base + res[0]) / ldexp(1.0, (int)c->dlen);
  if (argmax_count) *argmax_count = res[1];
done:
  if (cand) cudaFreeAsync(cand, s);
  if (st) cudaFreeAsync(st, s);
  return rc;
}

int buff_max_majority_async(const buff_col *c, uint64_t *dev_max_code, void *stream) {
  if (!c || !dev_max_code) return BUFF_EINVAL;
  if (c->layout != 1) return BUFF_ENOTSUP;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  uint32_t *cand = nullptr;
  unsigned char *st = nullptr;
  const size_t sb = buffk::major_max_state_bytes(), mo = buffk::major_max_state_mx_offset();
  if (!c->n) return cuda_status(cudaMemsetAsync(dev_max_code, 0, 8, s));
  if (buffk::major1_max_applies(c))
    return cuda_status(
        buffk::major1_max(c, reinterpret_cast<unsigned long long *>(dev_max_code), s));
  CK(scratch(&cand, c->nwp, s));
  CK(scratch(&st, sb, s));
  CK(buffk::launch_fill_words(cand, c->n, 0xFFFFFFFFu, nullptr, s));
  CK(buffk::major_max(c, cand, st, s));
  CK(cudaMemcpyAsync(dev_max_code, st + mo, 8, cudaMemcpyDeviceToDevice, s));
done:
  if (cand) cudaFreeAsync(cand, s);
  if (st) cudaFreeAsync(st, s);
  return rc;
}

// ---------------------------------------------------------------- row-conditioned ABI

int buff_decode_condition(const buff_col *c, const uint32_t *rows, uint64_t nrows, double *out,
                          void *stream) {
  if (!c || (nrows && (!rows || !out))) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;
  const bool intended = c->flags & BUFF_FLAG_INTENDED;
  if (nrows == 0) return intended ? BUFF_OK : BUFF_EREFPANIC;  // iter.next().unwrap() (:1559)
  return decode_list_impl(c, rows, nrows, out, intended ? 0 : 1, S(stream));
}

int buff_major_decode_condition(const buff_col *c, const uint32_t *rows, uint64_t nrows,
                                double *out, uint64_t *nout, void *stream) {
  if (!c || !nout || (nrows && (!rows || !out))) return BUFF_EINVAL;
  if (c->layout != 1) return BUFF_ENOTSUP;
  *nout = 0;
  if (c->m > 0 || nrows == 0) return BUFF_OK;  // "not implemented yet": empty (:1741-1743)
  const int rc = decode_list_impl(c, rows, nrows, out, 0, S(stream));
  if (rc == BUFF_OK) *nout = nrows;
  return rc;
}

int buff_decode_selected(const buff_col *c, const uint32_t *words, double *out, uint64_t *count,
                         void *stream) {
  if (!c || !count || (c->n && !words)) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  const size_t nw = ((size_t)c->n + 31) / 32;
  uint32_t *dw = const_cast<uint32_t *>(words);
  const bool host = c->n && !is_device_ptr(words);
  if (host) {
    CK(scratch(&dw, nw, s));
    CK(cudaMemcpyAsync(dw, words, nw * 4, cudaMemcpyHostToDevice, s));
  }
  rc = decode_words_impl(c, dw, out, count, (c->flags & BUFF_FLAG_INTENDED) ? 0 : 1, s);
done:
  if (host && dw && dw != words) cudaFreeAsync(dw, s);
  return rc;
}

int buff_range_filter_condition(const buff_col *c, double pred, const uint32_t *cand_words,
                                uint32_t *words, uint64_t *count, void *stream) {
  if (!c || (c->n && (!cand_words || !words))) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;
  return filter_cond_impl(c, pred, cand_words, words, count, S(stream));
}

int buff_range_filter_majority_condition(const buff_col *c, double pred,
                                         const uint32_t *cand_words, uint32_t *words,
                                         uint64_t *count, void *stream) {
  if (!c || (c->n && (!cand_words || !words))) return BUFF_EINVAL;
  if (c->layout != 1) return BUFF_ENOTSUP;
  if (c->m > 0) {  // "not implemented yet": the empty res (:1313-1315)
    cudaStream_t s = S(stream);
    int rc = BUFF_OK;
    const size_t nw = ((size_t)c->n + 31) / 32;
    if (nw) CK(cudaMemsetAsync(words, 0, nw * 4, s));
    if (count) CK(cudaMemsetAsync(count, 0, sizeof(uint64_t), s));
    CK(cudaStreamSynchronize(s));
  done:
    return rc;
  }
  return filter_cond_impl(c, pred, cand_words, words, count, S(stream));
}

int buff_range_filter_decode(const buff_col *c, double pred, uint32_t *words, double *out,
                             uint64_t *count, void *stream) {
  if (!c || !count || (c->n && !out)) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  const size_t nw = ((size_t)c->n + 31) / 32;
  const bool own = !words || !is_device_ptr(words);
  uint32_t *dw = own ? nullptr : words;
  if (c->n == 0) {
    *count = 0;
    return BUFF_OK;
  }
  if (own) CK(scratch(&dw, nw, s));
  if ((rc = filter_impl(c, pred, dw, nullptr, s, kRange))) goto done;
  rc = decode_words_impl(c, dw, out, count, (c->flags & BUFF_FLAG_INTENDED) ? 0 : 1, s);
  if (rc == BUFF_OK && words && own) {
    CK(cudaMemcpyAsync(words, dw, nw * 4, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
done:
  if (own && dw) cudaFreeAsync(dw, s);
  return rc;
}

// ---------------------------------------------------------------- windowed max

int buff_max_majority_range(const buff_col *c, uint32_t start, uint32_t end, uint32_t window,
                            double *out, uint64_t *nout, void *stream) {
  if (!c || !nout) return BUFF_EINVAL;
  if (c->layout != 1) return BUFF_ENOTSUP;
  *nout = 0;
  // with sparse columns the reference logs "not implemented" and returns no
  // windows (buff_simd.rs:2898-2902); without, it is buff_max_range on the
  // slices and tail that follow the count byte
  if (c->m) return BUFF_OK;
  buff_col view = *c;
  view.layout = 0;
  return buff_max_range(&view, start, end, window, out, nout, stream);
}

int buff_max_range(const buff_col *c, uint32_t start, uint32_t end, uint32_t window, double *out,
                   uint64_t *nout, void *stream) {
  if (!c || !nout) return BUFF_EINVAL;
  if (c->layout != 0) return BUFF_ENOTSUP;
  *nout = 0;
  const bool intended = c->flags & BUFF_FLAG_INTENDED;
  // the reference divides by the window, reads rows [start, end) and, for
  // codes wider than a byte, asserts that the windows cover the range exactly
  if (window == 0 || end < start || end > c->n) return intended ? BUFF_EINVAL : BUFF_EREFPANIC;
  const uint32_t full = (end - start) / window;
  const bool ragged = (end - start) % window != 0;
  if (!intended && c->fixed_len > 8 && (ragged || full == 0)) return BUFF_EREFPANIC;
  const uint32_t nwin = full + (intended && ragged ? 1u : 0u);
  if (nwin && !out) return BUFF_EINVAL;
  const uint32_t hi = intended ? end : start + full * window;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  unsigned long long *codes = nullptr;
  double *d = nullptr;
  const bool stage = nwin && !is_device_ptr(out);
  if (!nwin) return BUFF_OK;
  CK(scratch(&codes, nwin, s));
  if (stage)
    CK(scratch(&d, nwin, s));
  else
    d = out;
  CK(buffk::max_range(c, start, hi, start, window, nwin, codes, d, s));
  if (stage) {
    CK(cudaMemcpyAsync(out, d, sizeof(double) * nwin, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  *nout = nwin;
done:
  if (codes) cudaFreeAsync(codes, s);
  if (stage && d) cudaFreeAsync(d, s);
  return rc;
}

}  // extern "C"

namespace {

// ---------------------------------------------------------------- RAPG byte_residue

// byte_residue_encode (compress/split_double.rs:624-955): exact min and max
// (two ifs), width ceil(log2(max - min)).  When ilen > 15 -- a u32 compare,
// so also when ilen wrapped because the codes are narrower than dlen -- the
// image carries an outlier-column count byte, and the leading code bytes
// that are nonzero in fewer than 200 of the first 2000 codes (counted
// cumulatively from the top byte down, :693-716) become sparse columns: the
// rows whose byte is nonzero and those bytes.  The remaining bytes are dense
// slices, then the packed tail.
template <typename T>
int encode_rapg_impl(const T *values, uint64_t n64, uint64_t scale, uint32_t flags, cudaStream_t s,
                     buff_col **out) {
  if (!out) return BUFF_EINVAL;
  *out = nullptr;
  if (flags & BUFF_FLAG_INTENDED) return BUFF_ENOTSUP;
  if (n64 > BUFF_MAX_ROWS) return BUFF_EINVAL;
  if (n64 > 0 && !values) return BUFF_EINVAL;
  const uint32_t n = (uint32_t)n64;
  const int dl = dlen_of_prec(prec_of_scale(scale));
  if (dl < 0) return BUFF_EREFPANIC;  // PRECISION_MAP.get(&prec).unwrap()
  int rc = BUFF_OK;
  buff_col *c = new_col(scale, flags);
  if (!c) return BUFF_ENOMEM;
  c->layout = 3;
  c->n = n;
  c->dlen = (uint32_t)dl;
  T *staged = nullptr;
  EncStats *dst = nullptr;
  uint8_t *lead = nullptr;
  const T *dx = values;
  EncStats st;
  memset(&st, 0, sizeof(st));
  st.mn = INT64_MAX;
  st.mx0 = INT64_MIN;
  std::vector<T> head(n < 2000 ? n : 2000);
  uint32_t fl = 0, m = 0;
  if (n) {
    if (!is_device_ptr(values) || (reinterpret_cast<uintptr_t>(values) & 15)) {
      CK(scratch(&staged, n, s));
      CK(cudaMemcpyAsync(staged, values, (size_t)n * sizeof(T), cudaMemcpyDefault, s));
      dx = staged;
    }
    CK(scratch(&dst, 1, s));
    const int keys = c->precision_exp >= -(int)c->dlen ? 1 : 0;
    CK(reduce(dx, n, 1, c, keys, 0, dst, s));
    CK(cudaMemcpyAsync(&st, dst, sizeof(st), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(head.data(), dx, head.size() * sizeof(T), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if (!st.ok) {
      CK(reduce(dx, n, 1, c, 0, 0, dst, s));
      CK(cudaMemcpyAsync(&st, dst, sizeof(st), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
    }
  }
  {
    const int64_t mn = st.mn, mx = st.mx0;
    const int64_t delta = (int64_t)((uint64_t)mx - (uint64_t)mn);
    if (delta != 0) {
      const double cl = ceil(log2((double)delta));
      fl = (isnan(cl) || cl <= 0.0) ? 0u : (uint32_t)cl;
    }
    const uint64_t ilen64 = (uint64_t)fl - (uint64_t)c->dlen;  // usize, wraps
    c->rg_count_byte = ilen64 > 15;
    if (c->rg_count_byte) {
      if (n < 2000) {  // fixed_vec[0..SAMPLE]
        rc = BUFF_EREFPANIC;
        goto done;
      }
      // leading zeros of each sample code within fixed_len bits; a code at
      // 2^fixed_len (the width's lost top bit) wraps and is not counted
      uint32_t counter[32] = {0};
      const uint64_t head_len = 64u - fl;
      for (uint32_t i = 0; i < 2000; ++i) {
        const uint64_t u =
            (uint64_t)fetch_fixed_host((double)head[i], c->precision_exp, c->dlen) - (uint64_t)mn;
        const uint64_t lz = (uint64_t)(u ? __builtin_clzll(u) : 64) - head_len;
        if (lz < 32) ++counter[lz];
      }
      const uint32_t ol = (uint32_t)(2000.0f * 0.1f);
      const uint64_t adjusted = ilen64 / 8 * 8;
      uint32_t sum = 0;
      for (uint64_t i = 0; i < adjusted; ++i) {
        if (i >= 32) {  // bits_counter[i]: index out of bounds
          rc = BUFF_EREFPANIC;
          goto done;
        }
        sum += counter[i];
        if (i % 8 == 7) {
          if (sum < ol)
            ++m;
          else
            break;
        }
      }
    }
    c->base = mn;
    set_layout(c, fl);
    c->m = m;
    c->ilen = (uint32_t)ilen64;
    const uint32_t k = c->k;
    c->k = k - m;  // allocate the dense slices only
    rc = alloc_col(c, s);
    c->k = k;
    if (rc) goto done;
    c->nwp = c->stride / 32;
    if (n && fl) {
      if (m) CK(scratch(&lead, (size_t)m * c->stride, s));
      if (sizeof(T) == 8)
        CK(buffk::launch_encode_scatter_f64(reinterpret_cast<const double *>(dx), c, s, lead, m));
      else
        CK(buffk::launch_encode_scatter_f32(reinterpret_cast<const float *>(dx), c, s, lead, m));
      if (m) CK(buffk::major_build_sparse(c, lead, s));
    }
    if (c->rg_count_byte && fl > 0 && fl < 8) {
      // packed codes narrower than a byte overwrite the count byte; the
      // readers take that byte as the column count and read on from the next
      uint8_t first = 0;
      CK(cudaMemcpyAsync(&first, c->tail, 1, cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      c->rg_skip = 1;
      c->rg_bad = first != 0;
    }
    CK(cudaStreamSynchronize(s));
  }
done:
  if (staged) cudaFreeAsync(staged, s);
  if (dst) cudaFreeAsync(dst, s);
  if (lead) cudaFreeAsync(lead, s);
  if (rc != BUFF_OK) {
    cudaStreamSynchronize(s);
    free_col(c);
    return rc;
  }
  *out = c;
  return BUFF_OK;
}

// The byte image byte_residue_encode writes: header; [count byte]; per
// sparse column u32 bitmap size, roaring bitmap, u32 outlier count, outlier
// bytes (each column's pad byte is overwritten by the next write, so one pad
// byte follows the last column); unflipped dense slices; packed tail.  Codes
// narrower than a byte are packed from byte 20, over the count byte.
// The RAPG image (split_double.rs:624-955).  prefix_only: as major_image,
// except that codes narrower than a byte (the image is the header and the
// packed codes) are built whole, *complete set.
int rapg_image(const buff_col *c, std::vector<uint8_t> &img, cudaStream_t s, bool prefix_only,
               bool *complete) {
  int rc = BUFF_OK;
  const uint32_t n = c->n, kd = c->k - c->m;
  const size_t nw = ((size_t)n + 31) / 32;
  if (c->fixed_len < 8) prefix_only = false;
  if (complete) *complete = !prefix_only;
  std::vector<uint32_t> bits((size_t)c->m * nw);
  std::vector<uint8_t> ob(c->oofs[c->m]);
  std::vector<uint8_t> dense(prefix_only ? 0 : (size_t)kd * n), tail(prefix_only ? 0 : c->tail_bytes);
  for (uint32_t col = 0; col < c->m; ++col)
    CK(cudaMemcpyAsync(bits.data() + col * nw, c->obits + col * c->nwp, nw * 4,
                       cudaMemcpyDeviceToHost, s));
  if (!ob.empty()) CK(cudaMemcpyAsync(ob.data(), c->obytes, ob.size(), cudaMemcpyDeviceToHost, s));
  if (!prefix_only && kd && n)
    CK(cudaMemcpy2DAsync(dense.data(), n, c->slices, c->stride, n, kd, cudaMemcpyDeviceToHost, s));
  if (!tail.empty())
    CK(cudaMemcpyAsync(tail.data(), c->tail, tail.size(), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  {
    img.clear();
    auto put32 = [&](uint32_t v) {
      for (int b = 0; b < 4; ++b) img.push_back((uint8_t)(v >> (8 * b)));
    };
    const uint64_t ub = (uint64_t)c->base;
    put32((uint32_t)ub);
    put32((uint32_t)(ub >> 32));
    put32(n);
    put32(c->ilen);
    put32(c->dlen);
    if (c->fixed_len < 8) {
      if (c->rg_count_byte && tail.empty()) img.push_back(0);
      img.insert(img.end(), tail.begin(), tail.end());
      return BUFF_OK;
    }
    if (c->rg_count_byte) img.push_back((uint8_t)c->m);
    for (uint32_t col = 0; col < c->m; ++col) {
      const std::vector<uint8_t> bm = buffroaring::serialize(bits.data() + col * nw, n);
      put32((uint32_t)bm.size());
      img.insert(img.end(), bm.begin(), bm.end());
      put32(c->nout[col]);
      img.insert(img.end(), ob.begin() + c->oofs[col], ob.begin() + c->oofs[col] + c->nout[col]);
    }
    if (c->m) img.push_back(0);
    if (prefix_only) return BUFF_OK;
    for (uint8_t &b : dense) b ^= 0x80;  // the dense slices are stored unflipped
    img.insert(img.end(), dense.begin(), dense.end());
    img.insert(img.end(), tail.begin(), tail.end());
  }
done:
  return rc;
}

// The reads byte_residue_decode / byte_residue_sum make for R code bits
// (compress/split_double.rs:1353-1610, 2211-2407; R < fixed_len for the
// _with_precision forms, :1642-1664): one byte per sparse column, then
// slices while at least 8 bits remain -- past the dense ones the reader
// takes the bytes after them -- then ts-bit fields.  Reads past the image
// panic there.
struct RapgPlan {
  uint32_t ks, ts;
  uint64_t tbit0;  // bit of `tail` where the ts-bit fields start
  bool emit;       // the decode returns values (not when R ends with the sparse columns)
  bool no_base;    // the sum returns at its last slice, before the base term
};

int rapg_plan(const buff_col *c, uint32_t R, RapgPlan *p) {
  if (c->rg_bad) return BUFF_EREFPANIC;
  const uint32_t m = c->m, kd = c->k - m;
  uint32_t remain = R;
  if (m) {
    if (R < 8 * m) return BUFF_EREFPANIC;  // `remain -= 8` wraps: slices read past the image
    remain = R - 8 * m;
  }
  p->ks = remain / 8;
  p->ts = remain % 8;
  p->emit = !(m && remain == 0);
  p->no_base = p->ks > 0 && p->ts == 0;
  uint64_t at = c->rg_skip;  // bytes of the tail region consumed so far
  if (p->ks > kd) at += (uint64_t)(p->ks - kd) * c->n;
  if (at > c->tail_bytes) return BUFF_EREFPANIC;  // read_n_byte past the image
  p->tbit0 = 8 * at;
  if (p->ts) {
    if (p->ks < kd) return BUFF_ENOTSUP;  // bit fields from inside a slice
    if (p->tbit0 + (uint64_t)c->n * p->ts > 8ull * c->tail_bytes) return BUFF_EREFPANIC;
  }
  return BUFF_OK;
}

int rapg_bits(const buff_col *c, int precision, uint32_t *R) {
  if (precision < 0) {
    *R = c->ilen + c->dlen;
    return BUFF_OK;
  }
  return precision_bits(c, (uint32_t)precision, R);
}

int rapg_decode_impl(const buff_col *c, int precision, double *out, uint64_t *nout,
                     cudaStream_t s) {
  if (!c || !nout || (!out && c->n)) return BUFF_EINVAL;
  if (c->layout != 3) return BUFF_ENOTSUP;
  *nout = 0;
  uint32_t R;
  int rc = rapg_bits(c, precision, &R);
  if (rc) return rc;
  RapgPlan p;
  if ((rc = rapg_plan(c, R, &p))) return rc;
  for (uint32_t col = 0; col < c->m; ++col)
    if (c->nout[col] == 0) return BUFF_EREFPANIC;  // outlier_iter.next().unwrap() (:1393)
  if (!p.emit || c->n == 0) return BUFF_OK;
  const bool stage = !is_device_ptr(out) || (reinterpret_cast<uintptr_t>(out) & 15);
  double *d = stage ? nullptr : out;
  if (stage) CK(scratch(&d, c->n, s));
  CK(buffk::rapg_decode(c, R, p.ks, p.ts, p.tbit0, d, s));
  if (stage) {
    CK(cudaMemcpyAsync(out, d, (size_t)c->n * 8, cudaMemcpyDefault, s));
    CK(cudaStreamSynchronize(s));
  }
  *nout = c->n;
done:
  if (stage && d) cudaFreeAsync(d, s);
  return rc;
}

int rapg_sum_impl(const buff_col *c, int precision, double *sum, cudaStream_t s) {
  if (!c || !sum) return BUFF_EINVAL;
  if (c->layout != 3) return BUFF_ENOTSUP;
  uint32_t R;
  int rc = rapg_bits(c, precision, &R);
  if (rc) return rc;
  RapgPlan p;
  if ((rc = rapg_plan(c, R, &p))) return rc;
  const uint32_t m = c->m, kd = c->k - m, n = c->n;
  const uint32_t ks_dense = p.ks < kd ? p.ks : kd;
  unsigned long long *d = nullptr;
  uint64_t h[40] = {0};
  // a plan that reads every dense slice and the whole tail fields is the
  // buff-major sum's one launch (outlier bytes, slices and tail together:
  // raw[col], raw[8 + j], raw[8 + kd]); other plans sum their parts one by one
  const bool one = p.ks == kd && p.tbit0 == 0 && p.ts == c->r && n;
  CK(scratch(&d, 40, s));
  if (one) {
    CK(buffk::major_sums(c, major_sum_args(c), d, nullptr, nullptr, s));
  } else {
    CK(buffk::zero_u64(d, 40, s));
    for (uint32_t col = 0; col < m; ++col)
      if (c->nout[col])
        CK(buffk::major_bytesum(c->obytes + c->oofs[col], c->nout[col], d + col, s));
    if (n && ks_dense) CK(buffk::launch_sum(c, ks_dense, 0, d + 8, s));
    for (uint32_t j = kd; j < p.ks && n; ++j)
      CK(buffk::major_bytesum(c->tail + c->rg_skip + (size_t)(j - kd) * n, n, d + 8 + j, s));
    if (p.ts) CK(buffk::field_sum(c->tail, p.tbit0, p.ts, n, d + 32, s));
  }
  CK(cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (one) {
    h[32] = p.ts ? h[8 + kd] : 0;
    h[8 + kd] = 0;
  }
  {
    // the f64 steps of byte_residue_sum (:2229-2404): each partial over
    // 2^(processed - ilen), the base term n * base / 2^dlen last
    auto powi2 = [](int32_t e) -> double {
      if (e >= 1024) return INFINITY;
      if (e <= -1024) return 0.0;
      return ldexp(1.0, e);
    };
    const int32_t ilen_i = (int32_t)c->ilen;
    const double sum_base = ((double)n * (double)c->base) / ldexp(1.0, (int)c->dlen);
    double acc = 0.0;
    int32_t processed = 0;
    for (uint32_t col = 0; col < m; ++col) {
      processed += 8;
      acc = acc + (double)h[col] / powi2(processed - ilen_i);
    }
    for (uint32_t j = 0; j < p.ks; ++j) {
      processed += 8;
      acc = acc + (double)h[8 + j] / powi2(processed - ilen_i);
    }
    if (!p.no_base) {
      if (p.ts) {
        processed += (int32_t)p.ts;
        acc = acc + (double)h[32] / powi2(processed - ilen_i);
      }
      acc += sum_base;
    }
    *sum = acc;
  }
done:
  if (d) cudaFreeAsync(d, s);
  return rc;
}

}  // namespace

extern "C" {

int buff_rapg_encode_f64(const double *values, uint64_t n, uint64_t scale, uint32_t flags,
                         void *stream, buff_col **out) {
  return encode_rapg_impl<double>(values, n, scale, flags, S(stream), out);
}

int buff_rapg_encode_f32(const float *values, uint64_t n, uint64_t scale, uint32_t flags,
                         void *stream, buff_col **out) {
  return encode_rapg_impl<float>(values, n, scale, flags, S(stream), out);
}

// Reads an image the way the reference's decoders walk it (BitPack reads of
// the header, the count byte, each column's directory) and rejects images
// whose length differs from what byte_residue_encode writes for that
// directory, or whose bitmaps do not list exactly their outlier rows.
int buff_rapg_deserialize(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                          void *stream, buff_col **out) {
  if (!out || !bytes) return BUFF_EINVAL;
  *out = nullptr;
  if (flags & BUFF_FLAG_INTENDED) return BUFF_ENOTSUP;
  if (len < 20) return BUFF_ECORRUPT;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  std::vector<uint8_t> host;
  const uint8_t *b = bytes;
  buff_col *c = nullptr;
  std::vector<std::vector<uint32_t>> rows;
  std::vector<const uint8_t *> outl;
  if (is_device_ptr(bytes)) {
    host.resize(len);
    CK(cudaMemcpyAsync(host.data(), bytes, len, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    b = host.data();
  }
  {
    auto rd32 = [&](uint64_t at) -> uint32_t {
      return (uint32_t)b[at] | ((uint32_t)b[at + 1] << 8) | ((uint32_t)b[at + 2] << 16) |
             ((uint32_t)b[at + 3] << 24);
    };
    c = new_col(scale, flags);
    if (!c) return BUFF_ENOMEM;
    c->layout = 3;
    c->base = (int64_t)((uint64_t)rd32(0) | ((uint64_t)rd32(4) << 32));
    c->n = rd32(8);
    c->ilen = rd32(12);
    c->dlen = rd32(16);
    const uint32_t fl = c->ilen + c->dlen, n = c->n;
    if (n > BUFF_MAX_ROWS) {
      rc = BUFF_ENOTSUP;
      goto done;
    }
    if (fl > 64) {
      rc = BUFF_ECORRUPT;
      goto done;
    }
    set_layout(c, fl);
    c->rg_count_byte = c->ilen > 15;
    uint32_t m = 0;
    uint64_t pos = 20, dense_at = 20;
    if (c->rg_count_byte && fl >= 8) {
      if (len < 21) {
        rc = BUFF_ECORRUPT;
        goto done;
      }
      m = b[20];
      pos = 21;
      if (m > c->k) {
        rc = BUFF_ECORRUPT;
        goto done;
      }
      uint64_t off = 0;
      for (uint32_t col = 0; col < m; ++col) {
        if (pos + 4 > len) {
          rc = BUFF_ECORRUPT;
          goto done;
        }
        const uint32_t bml = rd32(pos);
        if (pos + 8 + (uint64_t)bml > len) {
          rc = BUFF_ECORRUPT;
          goto done;
        }
        std::vector<uint32_t> r;
        const uint32_t no = rd32(pos + 4 + bml);
        if (!buffroaring::parse(b + pos + 4, bml, r) || r.size() != no ||
            (no && r.back() >= n) || pos + 8 + (uint64_t)bml + no > len) {
          rc = BUFF_ECORRUPT;
          goto done;
        }
        rows.push_back(std::move(r));
        outl.push_back(b + pos + 8 + bml);
        c->nout[col] = no;
        c->oofs[col] = off;
        off += no;
        pos += 8 + (uint64_t)bml + no;
      }
      c->oofs[m] = off;
      dense_at = m ? pos + 1 : 21;
    }
    c->m = m;
    // codes narrower than a byte are packed from byte 20, over the count byte
    const uint64_t tail_len = ((uint64_t)n * c->r + 7) / 8;
    const uint64_t need =
        fl < 8 ? 20 + (tail_len > c->rg_count_byte ? tail_len : (uint64_t)c->rg_count_byte)
               : dense_at + (uint64_t)(c->k - m) * n + tail_len;
    if (need != len) {
      rc = BUFF_ECORRUPT;
      goto done;
    }
    if (fl < 8 && c->rg_count_byte && fl > 0) {
      // the readers take byte 20 (the first packed byte) as the column count
      // and read on from byte 21
      c->rg_skip = 1;
      c->rg_bad = b[20] != 0;
    }
    const uint32_t k = c->k, kd = k - m;
    c->k = kd;
    rc = alloc_col(c, s);
    c->k = k;
    if (rc) goto done;
    c->nwp = c->stride / 32;
    if (kd && n) {
      CK(cudaMemcpy2DAsync(c->slices, c->stride, b + dense_at, n, n, kd, cudaMemcpyHostToDevice, s));
      CK(buffk::flip_bytes(c->slices, (size_t)kd * c->stride, s));
      if (c->stride > n)
        CK(cudaMemset2DAsync(c->slices + n, c->stride, 0x80, c->stride - n, kd, s));
    }
    CK(cudaMemsetAsync(c->tail, 0, c->tail_alloc, s));
    if (c->tail_bytes)
      CK(cudaMemcpyAsync(c->tail, b + (fl < 8 ? 20 : dense_at + (uint64_t)kd * n), c->tail_bytes,
                         cudaMemcpyHostToDevice, s));
    if (m) {
      std::vector<uint32_t> words((size_t)m * c->nwp, 0);
      for (uint32_t col = 0; col < m; ++col)
        for (uint32_t r : rows[col]) words[col * c->nwp + (r >> 5)] |= 1u << (r & 31);
      CK(scratch(&c->obits, (size_t)m * c->nwp, s));
      CK(scratch(&c->orank, (size_t)m * (c->nwp + 16), s));
      CK(scratch(&c->obytes, c->oofs[m] + 16, s));
      CK(cudaMemcpyAsync(c->obits, words.data(), words.size() * 4, cudaMemcpyHostToDevice, s));
      for (uint32_t col = 0; col < m; ++col)
        if (c->nout[col])
          CK(cudaMemcpyAsync(c->obytes + c->oofs[col], outl[col], c->nout[col],
                             cudaMemcpyHostToDevice, s));
      CK(buffk::major_index(c, s));
    }
    CK(cudaStreamSynchronize(s));
  }
done:
  if (rc != BUFF_OK) {
    free_col(c);
    return rc;
  }
  *out = c;
  return BUFF_OK;
}

int buff_rapg_decode(const buff_col *c, double *out, uint64_t *nout, void *stream) {
  return rapg_decode_impl(c, -1, out, nout, S(stream));
}

int buff_rapg_decode_at_precision(const buff_col *c, uint32_t precision, double *out,
                                  uint64_t *nout, void *stream) {
  return rapg_decode_impl(c, precision > 0x7FFFFFFFu ? 0x7FFFFFFF : (int)precision, out, nout,
                          S(stream));
}

int buff_rapg_sum(const buff_col *c, double *sum, void *stream) {
  return rapg_sum_impl(c, -1, sum, S(stream));
}

int buff_rapg_sum_at_precision(const buff_col *c, uint32_t precision, double *sum, void *stream) {
  return rapg_sum_impl(c, precision > 0x7FFFFFFFu ? 0x7FFFFFFF : (int)precision, sum, S(stream));
}

// ---------------------------------------------------------------- buff-slice ABI

int buff_slice_encode_f64(const double *values, uint64_t n, uint64_t scale, uint32_t flags,
                          void *stream, buff_col **out) {
  return encode_impl<double>(values, n, scale, flags, S(stream), out, true);
}

int buff_slice_encode_f32(const float *values, uint64_t n, uint64_t scale, uint32_t flags,
                          void *stream, buff_col **out) {
  return encode_impl<float>(values, n, scale, flags, S(stream), out, true);
}

int buff_slice_deserialize(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                           void *stream, buff_col **out) {
  if (!out || !bytes) return BUFF_EINVAL;
  *out = nullptr;
  if (len < 20) return BUFF_ECORRUPT;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  const bool dev = is_device_ptr(bytes);
  uint8_t hdr[20];
  uint32_t w[5];
  buff_col *c = nullptr;
  if (dev) {
    CK(cudaMemcpyAsync(hdr, bytes, 20, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  } else {
    memcpy(hdr, bytes, 20);
  }
  for (int i = 0; i < 5; ++i)
    w[i] = (uint32_t)hdr[4 * i] | ((uint32_t)hdr[4 * i + 1] << 8) |
           ((uint32_t)hdr[4 * i + 2] << 16) | ((uint32_t)hdr[4 * i + 3] << 24);
  c = new_col(scale, flags);
  if (!c) return BUFF_ENOMEM;
  c->base = (int64_t)((uint64_t)w[0] | ((uint64_t)w[1] << 32));
  c->n = w[2];
  c->ilen = w[3];
  c->dlen = w[4];
  if (c->n > BUFF_MAX_ROWS) {
    rc = BUFF_ENOTSUP;
    goto done;
  }
  {
    const uint32_t fl = c->ilen + c->dlen;
    if (fl > 64 || c->dlen > 1000) {
      rc = BUFF_ECORRUPT;
      goto done;
    }
    set_slice_layout(c, fl);
    if (20 + (uint64_t)c->k * c->n > len) {
      rc = BUFF_ECORRUPT;
      goto done;
    }
    if ((rc = alloc_col(c, s))) goto done;
    cudaError_t ue = cudaSuccess;
    if (!dev && buffk::upload_slices(bytes, c, 0u, s, &ue)) {
      CK(ue);  // slices read in place by the device, padding rows on the way
    } else {
      if (c->n)
        CK(cudaMemcpy2DAsync(c->slices, c->stride, bytes + 20, c->n, c->n, c->k,
                             cudaMemcpyDefault, s));
      if (c->stride > c->n)
        CK(cudaMemset2DAsync(c->slices + c->n, c->stride, 0x80, c->stride - c->n, c->k, s));
    }
    CK(cudaMemsetAsync(c->tail, 0, c->tail_alloc, s));
    if (!dev) CK(cudaStreamSynchronize(s));
  }
done:
  if (rc != BUFF_OK) {
    free_col(c);
    return rc;
  }
  *out = c;
  return BUFF_OK;
}

int buff_slice_decode(const buff_col *c, double *out, void *stream) {
  if (!c || (!out && c->n)) return BUFF_EINVAL;
  if (c->layout != 2) return BUFF_ENOTSUP;
  if (c->n == 0) return BUFF_OK;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  const bool stage = !is_device_ptr(out) || (reinterpret_cast<uintptr_t>(out) & 15);
  double *d = stage ? nullptr : out;
  if (stage) CK(scratch(&d, c->n, s));
  CK(buffk::launch_decode(c, c->fixed_len, 0, d, s));
  if (stage) {
    CK(cudaMemcpyAsync(out, d, (size_t)c->n * 8, cudaMemcpyDefault, s));
    CK(cudaStreamSynchronize(s));
  }
done:
  if (stage && d) cudaFreeAsync(d, s);
  return rc;
}

namespace {

// buff_slice_range_filter / buff_slice_equal_filter (buff_slice.rs:1348-1751):
// target byte per slice (`t >> (fl - 8(j+1))`, or `t << pad` for the padded
// last slice), at most 4 slices, rows of full 32-row blocks only; a target
// below the base prints n for both.  nosimd: the row-by-row forms
// buff_slice_range_filter_nosimd / _equal_filter_nosimd (:1753-1991), the
// same compare over every row.
int slice_filter_impl(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                      cudaStream_t s, bool is_range, bool nosimd = false) {
  if (!c || (!words && c->n > 0)) return BUFF_EINVAL;
  if (c->layout != 2) return BUFF_ENOTSUP;
  const uint32_t n = c->n, nw = (n + 31) / 32;
  const uint32_t fl = c->fixed_len - c->pad;
  int rc = BUFF_OK;
  uint32_t *dwords = words;
  unsigned long long *dcount = nullptr;
  const bool words_host = n > 0 && !is_device_ptr(words);
  const bool count_host = count && !is_device_ptr(count);
  const int64_t fp = fetch_fixed_host(pred, c->precision_exp, c->dlen);
  const bool early = fp < c->base;
  buffk::FilterArgs a;
  memset(&a, 0, sizeof(a));
  if (!early) {
    if (fl == 0) return BUFF_EREFPANIC;                // ceil(0, 8) underflows
    if (!nosimd && n < 32) return BUFF_EREFPANIC;  // `len - 32` underflows
    const uint64_t t = (uint64_t)(fp - c->base);
    a.slices = c->slices;
    a.stride = c->stride;
    a.tail = c->tail;
    a.n = n;
    a.is_range = is_range ? 1u : 0u;
    a.k_used = c->k < 4 ? c->k : 4u;
    a.r = 0;
    a.full_rows = nosimd ? n : n / 32 * 32;
    for (uint32_t j = 0; j < a.k_used; ++j)
      a.tbyte[j] = (fl >= 8 * (j + 1)) ? (uint8_t)(t >> (fl - 8 * (j + 1)))
                                       : (uint8_t)(t << ((8 * (j + 1) - fl) & 63));
  }
  if (n == 0) {
    if (count) {
      if (count_host)
        *count = 0;
      else
        return cuda_status(cudaMemsetAsync(count, 0, sizeof(uint64_t), s));
    }
    return BUFF_OK;
  }
  if (words_host) CK(scratch(&dwords, nw, s));
  if (count) {
    if (count_host)
      CK(scratch(&dcount, 1, s));
    else
      dcount = reinterpret_cast<unsigned long long *>(count);
    CK(buffk::zero_u64(dcount, 1, s));
  }
  if (early) {
    CK(buffk::launch_fill_words(dwords, n, 0xFFFFFFFFu, dcount, s));
  } else {
    a.words = dwords;
    a.count = dcount;
    CK(buffk::launch_filter(a, s));
  }
  if (words_host) CK(cudaMemcpyAsync(words, dwords, (size_t)nw * 4, cudaMemcpyDeviceToHost, s));
  if (count_host) CK(cudaMemcpyAsync(count, dcount, sizeof(uint64_t), cudaMemcpyDeviceToHost, s));
  if (words_host || count_host) CK(cudaStreamSynchronize(s));
done:
  if (words_host && dwords && dwords != words) cudaFreeAsync(dwords, s);
  if (count_host && dcount) cudaFreeAsync(dcount, s);
  return rc;
}

// True when every partial sum of the values and every value is an exact
// multiple of 2^-dlen below 2^53 of them: then the reference's sequential
// f64 sum and its f64 compares are exact, and so is ours.
bool slice_exact(const buff_col *c) {
  const uint32_t fl = c->fixed_len - c->pad;
  const long double top = (long double)c->base + ldexpl(1.0L, (int)fl);
  const long double lo = (long double)c->base;
  const long double m = fabsl(top) > fabsl(lo) ? fabsl(top) : fabsl(lo);
  return m * (long double)(c->n ? c->n : 1) < ldexpl(1.0L, 53);
}

int slice_sum_impl(const buff_col *c, double *sum, cudaStream_t s, bool any_width) {
  if (!c || !sum) return BUFF_EINVAL;
  if (c->layout != 2) return BUFF_ENOTSUP;
  const uint32_t fl = c->fixed_len - c->pad;
  if (!any_width && (fl == 0 || c->k > 4)) return BUFF_EREFPANIC;  // buff_slice.rs:1178
  if (!slice_exact(c)) return BUFF_ENOTSUP;  // the sequential f64 sum would round
  if (c->n == 0) {
    *sum = 0.0;
    return BUFF_OK;
  }
  int rc = BUFF_OK;
  unsigned long long *d = nullptr;
  uint64_t parts[9] = {0};
  CK(scratch(&d, 9, s));
  CK(buffk::zero_u64(d, 9, s));
  CK(buffk::launch_sum(c, c->k, 0, d, s));
  CK(cudaMemcpyAsync(parts, d, sizeof(parts), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  {
    // sum of padded codes, the padding shifted out (every padded code is a
    // multiple of 2^pad, so the division is exact)
    __int128 acc = 0;
    for (uint32_t j = 0; j < c->k; ++j) acc += (__int128)parts[j] << (8 * (c->k - 1 - j));
    acc >>= c->pad;
    acc += (__int128)c->n * (__int128)c->base;
    *sum = ldexp((double)(int64_t)acc, -(int)c->dlen);
  }
done:
  if (d) cudaFreeAsync(d, s);
  return rc;
}

int slice_max_impl(const buff_col *c, double *max_value, uint32_t *argmax_words,
                   uint64_t *argmax_count, cudaStream_t s, bool any_width) {
  if (!c) return BUFF_EINVAL;
  if (c->layout != 2) return BUFF_ENOTSUP;
  const uint32_t fl = c->fixed_len - c->pad;
  if (!any_width && (fl == 0 || c->k > 4)) return BUFF_EREFPANIC;
  if (!slice_exact(c)) return BUFF_ENOTSUP;  // f64 compares of rounded values
  const uint32_t nw = (c->n + 31) / 32;
  int rc = BUFF_OK;
  unsigned long long *d = nullptr;
  uint32_t *dwords = nullptr;
  uint64_t m = 0, cnt = 0;
  const bool words_dev = argmax_words && is_device_ptr(argmax_words);
  if (c->n == 0) {  // f64::min_value() and no rows
    if (max_value) *max_value = -1.7976931348623157e308;
    if (argmax_count) *argmax_count = 0;
    return BUFF_OK;
  }
  CK(scratch(&d, 2, s));
  CK(buffk::zero_u64(d, 2, s));
  CK(buffk::launch_max(c, d, s));
  if (argmax_words || argmax_count) {
    if (argmax_words && words_dev)
      dwords = argmax_words;
    else
      CK(scratch(&dwords, nw, s));
    CK(buffk::launch_argmax(c, d, dwords, d + 1, s));
    if (argmax_words && !words_dev)
      CK(cudaMemcpyAsync(argmax_words, dwords, (size_t)nw * 4, cudaMemcpyDeviceToHost, s));
  }
  CK(cudaMemcpyAsync(&m, d, sizeof(m), cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(&cnt, d + 1, sizeof(cnt), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (max_value)
    *max_value = (double)(int64_t)((uint64_t)c->base + (m >> c->pad)) / ldexp(1.0, (int)c->dlen);
  if (argmax_count) *argmax_count = cnt;
done:
  if (d) cudaFreeAsync(d, s);
  if (dwords && !words_dev) cudaFreeAsync(dwords, s);
  return rc;
}

}  // namespace

int buff_slice_range_filter(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                            void *stream) {
  return slice_filter_impl(c, pred, words, count, S(stream), true);
}

int buff_slice_equal_filter(const buff_col *c, double pred, uint32_t *words, uint64_t *count,
                            void *stream) {
  return slice_filter_impl(c, pred, words, count, S(stream), false);
}

int buff_slice_range_filter_nosimd(const buff_col *c, double pred, uint32_t *words,
                                   uint64_t *count, void *stream) {
  return slice_filter_impl(c, pred, words, count, S(stream), true, true);
}

int buff_slice_equal_filter_nosimd(const buff_col *c, double pred, uint32_t *words,
                                   uint64_t *count, void *stream) {
  return slice_filter_impl(c, pred, words, count, S(stream), false, true);
}

int buff_slice_decode_bs(const buff_col *c, double *out, void *stream) {
  if (!c || (!out && c->n)) return BUFF_EINVAL;
  if (c->layout != 2) return BUFF_ENOTSUP;
  // `match num { 1..=4 => ..., _ => panic!(..) }`: ceil(0, 8) underflows
  const uint32_t fl = c->fixed_len - c->pad;
  if (fl == 0 || c->k > 4) return BUFF_EREFPANIC;
  return buff_slice_decode(c, out, stream);
}

int buff_slice_sum(const buff_col *c, double *sum, void *stream) {
  return slice_sum_impl(c, sum, S(stream), false);
}

int buff_slice_buffsum(const buff_col *c, double *sum, void *stream) {
  return slice_sum_impl(c, sum, S(stream), true);
}

int buff_slice_max(const buff_col *c, double *max_value, uint32_t *argmax_words,
                   uint64_t *argmax_count, void *stream) {
  return slice_max_impl(c, max_value, argmax_words, argmax_count, S(stream), false);
}

int buff_slice_buffmax(const buff_col *c, double *max_value, uint32_t *argmax_words,
                       uint64_t *argmax_count, void *stream) {
  return slice_max_impl(c, max_value, argmax_words, argmax_count, S(stream), true);
}

int buff_slice_max_range(const buff_col *c, uint32_t start, uint32_t end, uint32_t window,
                         double *out, uint64_t *nout, void *stream) {
  if (!c || !nout) return BUFF_EINVAL;
  if (c->layout != 2) return BUFF_ENOTSUP;
  *nout = 0;
  const uint32_t fl = c->fixed_len - c->pad;
  const uint32_t n = c->n;
  uint32_t hi, nwin, empty_from = 0xFFFFFFFFu;
  // buff_slice.rs:930-1099: widths 1..32 bits only; rows [start, min(end, n))
  // read; then assert_eq!((cur_s - s) / window + 1, (e - s) / window) in u32
  if (fl == 0 || c->k > 4 || window == 0) return BUFF_EREFPANIC;
  hi = end < n ? end : n;
  if (hi > start) {
    nwin = (uint32_t)(((uint64_t)hi - start + window - 1) / window);
  } else {
    nwin = 1;  // no row read: the pushed maximum is f64::min_value()
    empty_from = 0;
    hi = start;
  }
  if (nwin != (uint32_t)(end - start) / window) return BUFF_EREFPANIC;
  if (!out) return BUFF_EINVAL;
  cudaStream_t s = S(stream);
  int rc = BUFF_OK;
  unsigned long long *codes = nullptr;
  double *d = nullptr;
  const bool stage = !is_device_ptr(out);
  CK(scratch(&codes, nwin, s));
  if (stage)
    CK(scratch(&d, nwin, s));
  else
    d = out;
  CK(buffk::max_range(c, start, hi, start, window, nwin, codes, d, s, c->pad, empty_from));
  if (stage) {
    CK(cudaMemcpyAsync(out, d, sizeof(double) * nwin, cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
  }
  *nout = nwin;
done:
  if (codes) cudaFreeAsync(codes, s);
  if (stage && d) cudaFreeAsync(d, s);
  return rc;
}

const char *buff_status_string(int st) {
  switch (st) {
    case BUFF_OK: return "ok";
    case BUFF_EINVAL: return "invalid argument";
    case BUFF_ENOMEM: return "out of memory";
    case BUFF_ECUDA: return "CUDA runtime error";
    case BUFF_EREFPANIC: return "input on which the reference implementation panics";
    case BUFF_ECORRUPT: return "serialized column is inconsistent with its header";
    case BUFF_ETIMEDOUT: return "bounded device wait expired";
    case BUFF_ENOTSUP: return "not supported for this column layout";
    case BUFF_EFULL: return "queue or memory budget exhausted";
    case BUFF_ESCRATCH: return "column larger than the fixed scratch of the allocation-free entry point";
    default: return "unknown status";
  }
}

int buff_last_cuda_error(void) { return g_last_cuda; }

int buff_copy(void *dst, const void *src, uint64_t nbytes, void *stream) {
  if (nbytes && (!dst || !src)) return BUFF_EINVAL;
  if (!nbytes) return BUFF_OK;
  cudaStream_t s = S(stream);
  cudaError_t e = cudaMemcpyAsync(dst, src, nbytes, cudaMemcpyDefault, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return cuda_status(e);
}

uint64_t buff_kernel_launches(void) { return buffk::launches(); }

}  // extern "C"

namespace buffh {
int cuda_status(cudaError_t e) { return ::cuda_status(e); }
bool is_device_ptr(const void *p) { return ::is_device_ptr(p); }
int64_t fetch_fixed(double v, int pexp, uint32_t dlen) { return fetch_fixed_host(v, pexp, dlen); }
void set_layout(buff_col *c, uint32_t fl) { ::set_layout(c, fl); }
buff_col *new_col(uint64_t scale, uint32_t flags) { return ::new_col(scale, flags); }
void free_col(buff_col *c) { ::free_col(c); }
int precision_bits(const buff_col *c, uint32_t precision, uint32_t *total) {
  return ::precision_bits(c, precision, total);
}
double combine_sum(const buff_col *c, uint32_t total, const uint64_t *parts, bool intended) {
  return ::combine_sum(c, total, parts, intended);
}
int plan_filter(const buff_col *c, double pred, int kind, buffk::FilterArgs *a, int *action) {
  return ::plan_filter(c, pred, kind, a, action);
}
int dlen_of_scale(uint64_t scale) { return dlen_of_prec(prec_of_scale(scale)); }
int encode_admitted(const void *values, int is_f32, uint64_t n, uint64_t scale, uint32_t flags,
                    cudaStream_t s, const EncodeAdmit *admit, buff_col **out) {
  if (is_f32)
    return encode_impl<float>(static_cast<const float *>(values), n, scale, flags, s, out, false,
                              admit);
  return encode_impl<double>(static_cast<const double *>(values), n, scale, flags, s, out, false,
                             admit);
}
}  // namespace buffh
