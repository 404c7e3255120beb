// Internal declarations shared by the C ABI (buff_capi.cu) and the kernels
// (buff_kernels.cu).  Not part of the public interface.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/buff_gpu.h"

// Device image of one column.  `slices` holds k byte slices, each `stride`
// bytes apart (stride >= n, a multiple of kRowChunk), bytes stored flipped
// (x ^ 0x80) exactly as the reference writes them (compress/buff_simd.rs:3181-3225).
// `tail` holds the r-bit packed remainder, LSB-first, byte-identical to
// BitPack::write_bits (methods/bit_packing.rs:106-135); for fixed_len < 8 it
// holds the whole packed code (k == 0, r == fixed_len).  Padding rows beyond
// n are zero in the tail and hold the flipped zero byte 0x80 in the slices.
// One device allocation shared by the columns of a batched encode; freed
// when the last of them is freed.
struct buff_arena {
  void *base;
  std::atomic<int> refs;
};

struct buff_col {
  int64_t base;
  uint32_t n;
  uint32_t ilen, dlen, fixed_len, k, r;
  uint64_t scale;
  int32_t prec, precision_exp;
  uint32_t flags;
  int device;
  uint8_t *slices;
  size_t stride;
  uint8_t *tail;
  size_t tail_bytes;  // bytes of the packed tail (ceil(n*r/8)), excluding padding
  size_t tail_alloc;
  // buff-major layout (compress/buff_simd.rs:317-630): the first m full bytes
  // are sparse columns (major byte + outlier rows + outlier bytes); `slices`
  // then holds only the k - m dense slices (still flipped on the device).
  uint32_t layout;      // 0: buff-simd, 1: buff-major, 2: buff-slice
  uint32_t pad;         // buff-slice: zero bits below the code in the last slice
  uint32_t m;           // sparse columns
  uint8_t majors[8];
  uint32_t nout[8];     // outliers per sparse column
  uint32_t olast[8];    // row of the last outlier per sparse column
  size_t nwp;           // bitmap words per sparse column (stride / 32)
  uint32_t *obits;      // m x nwp outlier bitmaps (BitVec<u32> words)
  uint32_t *orank;      // m x (nwp + 1) outliers before each word
  uint8_t *obytes;      // outlier bytes of all sparse columns, row order
  uint64_t oofs[9];     // start of each column's outlier bytes
  buff_arena *arena;    // non-null: slices and tail live in a shared arena
  // RAPG byte_residue layout (layout 3, compress/split_double.rs:624-955):
  // the sparse columns above hold the rows whose byte is nonzero (major 0).
  uint32_t rg_count_byte;  // the image carries the outlier-column count byte (ilen > 15)
  uint32_t rg_skip;        // bytes of `tail` before where the readers start reading it
  uint32_t rg_bad;         // the readers would take packed codes for a column directory
  // buff-major columns of the RAPG-major image (byte_residue_encode_outlieru8):
  // the outlier bitmaps are croaring portable images instead of snappy BitVecs
  uint32_t bm_roaring;
};

// Host helpers of the C ABI (buff_capi.cu) shared with the batched and
// serving code.
namespace buffh {
int cuda_status(cudaError_t e);
bool is_device_ptr(const void *p);
int64_t fetch_fixed(double v, int pexp, uint32_t dlen);
void set_layout(buff_col *c, uint32_t fl);
buff_col *new_col(uint64_t scale, uint32_t flags);
void free_col(buff_col *c);
int precision_bits(const buff_col *c, uint32_t precision, uint32_t *total);
double combine_sum(const buff_col *c, uint32_t total, const uint64_t *parts, bool intended);
int dlen_of_scale(uint64_t scale);  // -1: PRECISION_MAP has no entry
// buff_encode_f64 / _f32 with a hook that is given the column's device
// bytes before they are allocated (see encode_impl).
struct EncodeAdmit {
  int (*fn)(void *ctx, uint64_t bytes);
  void *ctx;
};
int encode_admitted(const void *values, int is_f32, uint64_t n, uint64_t scale, uint32_t flags,
                    cudaStream_t s, const EncodeAdmit *admit, buff_col **out);
}  // namespace buffh

namespace buffk {
namespace dev {
struct MajorSumArgs;
}

constexpr uint32_t kRowChunk = 512;  // rows one warp covers per step (32 lanes x 16 rows)

inline size_t round_up(size_t x, size_t m) { return (x + m - 1) / m * m; }

// Encode statistics gathered by the reduce pass.
struct EncStats {
  long long mn;     // min over all rows (quantized)
  long long mx1;    // max over rows >= from (quantized)
  long long mx0;    // max over all rows
  long long x0, x1; // first two quantized rows
  unsigned long long brk;  // first i >= 1 with x_i >= x_{i-1} (n if none)
  int ok;           // 0: a key-mode extreme was non-finite or out of range
  int pad;
};

struct FilterArgs {
  const uint8_t *slices;
  size_t stride;
  const uint8_t *tail;
  uint32_t n;          // rows
  uint32_t full_rows;  // rows that may be set (32*floor(n/32) for the reference's SIMD compare)
  uint32_t k_used;     // slices compared
  uint32_t r;          // packed tail bits compared (0 = no tail step)
  uint32_t is_range;   // 1: value > pred, 0: value == pred
  uint32_t tail_only_eq;  // equality result requires the tail step
  uint8_t tbyte[8];    // target byte per slice (unflipped)
  uint32_t ttail;      // target tail bits
  uint32_t *words;
  unsigned long long *count;  // may be null
};

// Per-stream launch helpers (buff_kernels.cu).  All return cudaError_t.
// min over all rows and max over rows >= from, quantized; keys = 1 reduces
// on order keys of the raw values (check EncStats::ok), keys = 0 on the
// quantized values.  find_brk also locates the end of the leading strictly
// decreasing run.
cudaError_t launch_encode_reduce_f64(const double *x, uint32_t n, uint32_t from, int32_t pexp,
                                     uint32_t dlen, int keys, int find_brk, EncStats *d_out,
                                     cudaStream_t s);
cudaError_t launch_encode_reduce_f32(const float *x, uint32_t n, uint32_t from, int32_t pexp,
                                     uint32_t dlen, int keys, int find_brk, EncStats *d_out,
                                     cudaStream_t s);
// Quantize and slice; the first `nlead` slices are written to `lead` (stride
// apart) instead of the column's slices (the sparse columns of buff-major).
cudaError_t launch_encode_scatter_f64(const double *x, const buff_col *c, cudaStream_t s,
                                      uint8_t *lead = nullptr, uint32_t nlead = 0);
cudaError_t launch_encode_scatter_f32(const float *x, const buff_col *c, cudaStream_t s,
                                      uint8_t *lead = nullptr, uint32_t nlead = 0);
cudaError_t launch_filter(const FilterArgs &a, cudaStream_t s);
// n u64 words at p and m at q (8-byte aligned device memory; q may be null)
// set to 0: by one kernel while s is being captured or when q is given, else
// by a memset (less host time per call).
cudaError_t zero_u64(unsigned long long *p, uint32_t n, cudaStream_t s,
                     unsigned long long *q = nullptr, uint32_t m = 0);
cudaError_t launch_fill_words(uint32_t *words, uint32_t n, uint32_t value,
                              unsigned long long *count, cudaStream_t s);
// Sums of the first k_used slices and of the packed tail read as `tail_bits`-bit
// fields (tail_bits == 0: no tail).  Slice padding must hold 0x80.
cudaError_t launch_sum(const buff_col *c, uint32_t k_used, uint32_t tail_bits,
                       unsigned long long *d_partials, cudaStream_t s);
// Range filter (REF plan in `a`, k >= 1) and the full-width sums in one pass.
cudaError_t launch_filter_sum(const FilterArgs &a, const buff_col *c,
                              unsigned long long *d_partials, cudaStream_t s);
cudaError_t launch_max(const buff_col *c, unsigned long long *d_max, cudaStream_t s);
cudaError_t launch_argmax(const buff_col *c, const unsigned long long *d_max, uint32_t *words,
                          unsigned long long *count, cudaStream_t s);
// Decode with `total` leading bits (REF) or masked to `total` bits (INTENDED);
// buff-slice columns shift their padding out (c->pad).
cudaError_t launch_decode(const buff_col *c, uint32_t total, int intended_mask, double *out,
                          cudaStream_t s);

// buff-major layout (buff_major.cu)
cudaError_t major_build_sparse(buff_col *c, const uint8_t *lead, cudaStream_t s);
cudaError_t major_index(buff_col *c, cudaStream_t s);
cudaError_t flip_bytes(uint8_t *p, size_t nbytes, cudaStream_t s);
// The k slices of a serialized image into c->slices (flipped; padding rows
// 0x80) read in place by the device; false when the device cannot reach the
// image (nothing launched).  flipx = 0x80808080 for the buff layout.
bool upload_slices(const uint8_t *image, buff_col *c, uint32_t flipx, cudaStream_t s,
                   cudaError_t *err);
// The first `nslices` slices of c (XOR flipx), then its packed tail, written
// by the device at dst where it lies (host memory the device can write: the
// body of a serialized image); false when the device cannot reach it
// (nothing launched).
bool download_body(const buff_col *c, uint8_t *dst, uint32_t nslices, uint32_t flipx,
                   cudaStream_t s, cudaError_t *err);
// The same body (body_bytes long) into host memory: in place when dst is
// pinned, else staged in device memory and copied by the copy engine.
bool body_to_host(const buff_col *c, uint8_t *dst, uint64_t body_bytes, uint32_t nslices,
                  uint32_t flipx, cudaStream_t s, cudaError_t *err);
// Filters of the buff-major layout; with m == 0 the same compare runs over a
// plain column's slices and tail.  cand (may be null) restricts the rows.
cudaError_t major_filter(const buff_col *c, int is_range, const uint8_t *tbyte, uint32_t ttail,
                         uint32_t *words, unsigned long long *count, cudaStream_t s,
                         const uint32_t *cand = nullptr);
// Exclusive scan of `count` u32 in place (data holds count + 1; data[count]
// receives the total), with exclusive_scan_tmp(count) u32 of device scratch.
size_t exclusive_scan_tmp(size_t count);
cudaError_t exclusive_scan(uint32_t *data, size_t count, uint32_t *tmp, cudaStream_t s);
// Selected rows before each 128-row step of a bitmap over n rows (bits of
// rows >= n ignored): rank holds ceil(n/128) + 1 u32, the last the total.
cudaError_t step_ranks(const uint32_t *words, uint32_t n, uint32_t *rank, cudaStream_t s);
cudaError_t major_bytesum(const uint8_t *p, size_t nbytes, unsigned long long *out,
                          cudaStream_t s);
// buff_sum_majority's sums in one launch after zeroing raw (24 u64): the
// sparse columns' outlier-byte sums at raw[0..m), the dense slices and the
// tail from raw[8]; with `sum` set, the last block also combines them into
// the f64 sum and, when parts is not null, the k (+1) partials.
cudaError_t major_sums(const buff_col *c, const dev::MajorSumArgs &a, unsigned long long *raw,
                       double *sum, unsigned long long *parts, cudaStream_t s);
// buff_max_majority's progressive max on the device: cand (nwp words) ends
// as the arg-max bitmap; state_dev (major_max_state_bytes(), device) holds
// the max code (u64 at major_max_state_mx_offset()) and, after it, the
// arg-max count (u64).
cudaError_t major_max(const buff_col *c, uint32_t *cand, void *state_dev, cudaStream_t s);
// One sparse column with rows outside it: the progressive max is the
// largest code, found in one launch (major1_max) into *out (device u64).
bool major1_max_applies(const buff_col *c);
cudaError_t major1_max(const buff_col *c, unsigned long long *out, cudaStream_t s);
size_t major_max_state_bytes();
size_t major_max_state_mx_offset();
cudaError_t popcount_words(const uint32_t *w, size_t nw, unsigned long long *out, cudaStream_t s);
cudaError_t major_decode(const buff_col *c, double *out, cudaStream_t s);
// RAPG decode of the top R bits: m sparse columns, ks slices (those past the
// k - m dense ones read from the bytes after them, as the reference's reader
// does), then ts-bit fields from bit `tbit0` of the tail buffer.
cudaError_t rapg_decode(const buff_col *c, uint32_t R, uint32_t ks, uint32_t ts, uint64_t tbit0,
                        double *out, cudaStream_t s);
// Sum of n `width`-bit fields packed LSB-first from bit `bit0` of `p`.
cudaError_t field_sum(const uint8_t *p, uint64_t bit0, uint32_t width, uint32_t n,
                      unsigned long long *out, cudaStream_t s);

// Row-conditioned decode (buff_cond.cu): rows from a list (rows != null,
// nrows entries) or from a bitmap with its step ranks (step_ranks).
// tail_shift: 1 ORs the packed tail shifted by r (buff_decode_condition).
cudaError_t decode_rows(const buff_col *c, const uint32_t *rows, uint64_t nrows,
                        const uint32_t *words, const uint32_t *rank, int tail_shift, double *out,
                        cudaStream_t s);
// Maxima of the codes of rows [lo, hi) per window of w rows from s (nwin
// windows) into codes[] and, as values, out[] (device).
cudaError_t max_range(const buff_col *c, uint32_t lo, uint32_t hi, uint32_t s, uint32_t w,
                      uint32_t nwin, unsigned long long *codes, double *out, cudaStream_t st,
                      uint32_t shift = 0, uint32_t empty_from = 0xFFFFFFFFu);
// Sets *bad (device) to 1 unless rows[] is strictly ascending and below n.
cudaError_t check_rows(const uint32_t *rows, uint64_t nrows, uint32_t n, uint32_t *bad,
                       cudaStream_t s);

// Batched queries (buff_batch.cu) for the serving loop: per-query device
// descriptors of batch_desc_size() bytes, accumulators of kBatchAcc u64.
constexpr int kBatchAcc = 12;
size_t batch_desc_size();
int batch_plan_query(const buff_query &q, unsigned long long *acc, void *desc);
// Per-class work lists of one batch (query indices and tile prefixes packed
// into one u32 buffer of batch_sched_words(nq) words).
struct BatchSched {
  uint32_t n[4], items[4], qidx_off[4], prefix_off[4];
  uint32_t words;  // used length of the buffer
};
size_t batch_sched_words(uint32_t nq);
void batch_schedule(const void *h_desc, uint32_t nq, uint32_t tile, uint32_t *buf,
                    BatchSched *sc);
// A batch's completion, written by its last launch: the last block to finish
// copies the nacc accumulator words to hacc (host memory the device writes)
// and then stores seq into *flag, so the host reads the results once the
// flag shows seq (no read-back copy, no event to ask).
struct BatchDone {
  unsigned int *ticket;  // a zeroed device word
  const unsigned long long *acc;
  unsigned long long *hacc;
  uint32_t nacc;
  uint32_t *flag;  // device address of the host flag
  uint32_t seq;
};
// Launches every class of a scheduled batch on s; counters: 4 zeroed u32.
// With `done`, the last class launch also writes the batch's completion.
cudaError_t batch_launch(const void *d_desc, const uint32_t *d_buf, const BatchSched &sc,
                         const buff_batch_tune &t, unsigned int *counters, cudaStream_t s,
                         const BatchDone *done = nullptr);
void batch_result(const buff_query &q, const unsigned long long *acc, buff_query_result *out);

int num_sms(int device);
void count_launch(uint64_t n = 1);
uint64_t launches();

}  // namespace buffk

namespace buffh {
// The filter plan of the buff-simd range/equality filters (kind: 0 range,
// 1 equality, 2 range _with_slice, 3 equality _with_slice): *action 0 = no
// row set, 1 = every row set, 2 = run the filter kernel with *a (device
// pointers left null).  BUFF_EREFPANIC where the reference panics.
int plan_filter(const buff_col *c, double pred, int kind, buffk::FilterArgs *a, int *action);
}  // namespace buffh
