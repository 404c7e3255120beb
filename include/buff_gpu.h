/*
 * buff_gpu.h — C ABI of the GB300 (sm_103a) BUFF column codec.
 *
 * BUFF ("decomposed bounded floats", Tranway1/buff) stores an f64/f32 column
 * as bounded fixed-point codes split most-significant byte first into byte
 * slices, plus a bit-packed tail, and answers queries directly on the slices.
 * This library keeps the column resident in HBM behind an opaque handle and
 * runs encode, filters, sum, max and (variable-precision) decode as CUDA
 * kernels.  Every entry point mirrors one method of the reference's
 * `SplitBDDoubleCompress` (database/src/compress/split_double.rs:29-39 and
 * database/src/compress/buff_simd.rs); the comment on each one names the
 * reference function it replaces.
 *
 * Conventions
 *  - Every function returns an int status (BUFF_OK == 0).  Nothing aborts:
 *    inputs on which the reference panics return BUFF_EREFPANIC.
 *  - `stream` is a cudaStream_t (NULL = the legacy default stream).
 *  - Pointers to values/outputs may be host (pageable or pinned) or device
 *    memory; the library detects which.  A call that writes any host memory
 *    synchronizes `stream` before returning; a call whose outputs are all
 *    device memory only enqueues work.
 *  - Handles are immutable after encode/deserialize: concurrent queries on
 *    one handle from several streams or threads are safe.
 *  - Bitmaps are BitVec<u32> words (bit-vec/src/lib.rs:213-218): row i is
 *    bit (i % 32) of word (i / 32); ceil(n/32) words; bits past n are zero.
 *  - By default every result is bit-identical to the reference, including
 *    its documented quirks.  BUFF_FLAG_INTENDED (given at encode or
 *    deserialize time) switches the column to the mathematically intended
 *    semantics instead.
 */
#ifndef BUFF_GPU_H
#define BUFF_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define BUFF_OK 0
#define BUFF_EINVAL 1     /* bad argument (NULL handle, n >= 2^32, short buffer, ...) */
#define BUFF_ENOMEM 2     /* device or host allocation failed */
#define BUFF_ECUDA 3      /* a CUDA runtime call failed (see buff_last_cuda_error) */
#define BUFF_EREFPANIC 4  /* the reference panics on this input */
#define BUFF_ECORRUPT 5   /* serialized bytes are inconsistent with their header */
#define BUFF_ETIMEDOUT 6  /* a bounded device-side wait expired */
#define BUFF_ENOTSUP 7    /* not supported for this column layout */
#define BUFF_EFULL 8      /* a queue or memory budget is exhausted */
#define BUFF_ESCRATCH 9   /* larger than the fixed scratch of an allocation-free entry point */

/* ---- flags ---- */
/* Intended semantics instead of the reference's quirks: exact min/max and
 * bit width at encode (constant columns allowed), filters cover the rows
 * after the last full 32-row block, targets above the code range compare
 * correctly, sum keeps the base term when the tail is empty, equality
 * answers columns without tail bits, variable-precision decode keeps the
 * retained bits in place. */
#define BUFF_FLAG_INTENDED 0x1u
/* buff-major columns: store (and expect) the outlier bitmaps as raw
 * BitVec::to_binary bytes instead of snappy-compressed ones. */
#define BUFF_FLAG_RAW_BITMAPS 0x2u
/* Plain columns: the byte image is the buff layout of byte_fixed_encode
 * (compress/split_double.rs:298-432), whose slice bytes are stored without
 * the ^0x80 flip of buff_simd256_encode.  Affects buff_serialize and
 * buff_deserialize only; every query returns the same results. */
#define BUFF_FLAG_BUFF_LAYOUT 0x4u
/* Largest row count a column may have: the header stores n as u32, and the
 * library rounds row counts up to whole 512-row steps in 32-bit arithmetic,
 * so the last 511 values of u32 are refused (encode: BUFF_EINVAL,
 * deserialize: BUFF_ENOTSUP). */
#define BUFF_MAX_ROWS 4294966784u

typedef struct buff_col buff_col;

/* Column metadata (the 20-byte reference header plus derived fields). */
typedef struct buff_col_info {
  int64_t base;          /* column minimum in fixed-point units */
  uint32_t n;            /* rows */
  uint32_t ilen;         /* integer bits as stored (wraps when fixed_len < dlen) */
  uint32_t dlen;         /* fractional bits = PRECISION_MAP[prec] */
  uint32_t fixed_len;    /* code width = ilen + dlen */
  uint32_t k;            /* full byte slices (0 when fixed_len < 8) */
  uint32_t r;            /* packed bits per row after the slices (fixed_len when < 8) */
  uint64_t scale;        /* the SplitBDDoubleCompress scale the column was built with */
  int32_t prec;          /* floor(log10(scale)) */
  int32_t precision_exp; /* exponent of the reference's precision bound */
  uint32_t flags;
  uint32_t outlier_cols;     /* sparse (majority) byte columns of a buff-major column */
  uint64_t serialized_bytes; /* size of the reference byte image (0 for buff-major: call
                                buff_serialize with out = NULL) */
  uint64_t device_bytes;     /* HBM held by the handle */
} buff_col_info;

/* Sum of a column. */
typedef struct buff_sum_result {
  double sum;            /* the reference's f64 accumulation, bit-exact */
  double exact;          /* exact_num / 2^dlen, rounded once */
  int64_t exact_num_lo;  /* exact numerator n*base + sum(code) as a 128-bit */
  int64_t exact_num_hi;  /*   two's-complement integer (lo, hi) */
  uint64_t partials[9];  /* per-slice byte sums (unflipped), then the tail sum */
  uint32_t n_partials;
  uint32_t reserved;
} buff_sum_result;

/* ---- encode / lifetime ---- */

/* SplitBDDoubleCompress::buff_simd256_encode (compress/buff_simd.rs:3116-3250).
 * Quantizes `n` values with scale `scale` (decimals = floor(log10(scale))),
 * and builds the byte-sliced column in HBM.  n < 2^32. */
int buff_encode_f64(const double *values, uint64_t n, uint64_t scale, uint32_t flags,
                    void *stream, buff_col **out);
/* The same for f32 input (T: Into<f64>, compress/buff_simd.rs:3117). */
int buff_encode_f32(const float *values, uint64_t n, uint64_t scale, uint32_t flags,
                    void *stream, buff_col **out);
/* Releases the handle and its device memory (drains the device first, so
 * queries still running on any stream are safe). */
int buff_col_free(buff_col *col);
/* Releases the handle; the memory returns to the pool in stream order on
 * `stream`, after the work already queued there. */
int buff_col_free_async(buff_col *col, void *stream);
int buff_col_get_info(const buff_col *col, buff_col_info *info);

/* The exact reference byte image (the Vec<u8> buff_simd256_encode returns):
 * 20-byte header, k flipped byte slices of n bytes, packed tail.  *len
 * receives the image size; out = NULL (or cap < *len) returns BUFF_EINVAL
 * after setting it.  out is device or host memory the caller may write; a
 * pinned host image has its slices and tail written there by the device
 * directly, a pageable one receives them in one copy.  Returns when the
 * image is complete. */
int buff_serialize(const buff_col *col, uint8_t *out, uint64_t cap, uint64_t *len,
                   void *stream);
/* Rebuilds a handle from a reference byte image.  The image does not carry
 * the scale, so the caller passes the SplitBDDoubleCompress scale. */
int buff_deserialize(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                     void *stream, buff_col **out);

/* ---- queries ---- */

/* SplitBDDoubleCompress::buff_simd256_decode (compress/buff_simd.rs:3252-3357):
 * out[i] = (base + code_i) / 2^dlen for all n rows. */
int buff_decode(const buff_col *col, double *out, void *stream);

/* SplitBDDoubleCompress::byte_residue_decode_with_precision
 * (compress/split_double.rs:1612-1893), applied to this layout: rebuilds only
 * the leading bits that `precision` decimals need (precision 0 = integer
 * part).  Unknown precision or one finer than the column: BUFF_EREFPANIC. */
int buff_decode_at_precision(const buff_col *col, uint32_t precision, double *out,
                             void *stream);

/* SplitBDDoubleCompress::buff_simd_range_filter (compress/buff_simd.rs:3361-3547):
 * rows with value > pred.  `words` receives ceil(n/32) bitmap words; `count`
 * (may be NULL) the number of set bits. */
int buff_range_filter(const buff_col *col, double pred, uint32_t *words, uint64_t *count,
                      void *stream);
/* SplitBDDoubleCompress::buff_simd_equal_filter (compress/buff_simd.rs:3549-3733). */
int buff_equal_filter(const buff_col *col, double pred, uint32_t *words, uint64_t *count,
                      void *stream);
/* SplitBDDoubleCompress::buff_range_filter (compress/buff_simd.rs:4507-4679),
 * the scalar filter of the `buff` profiler arm on byte_fixed_encode's
 * layout: the same target bytes as buff_range_filter above, but slice 0 is
 * read byte by byte for every row, so rows after the last full 32-row block
 * are set too.  (The layout affects only the byte image, not the result.) */
int buff_scalar_range_filter(const buff_col *col, double pred, uint32_t *words, uint64_t *count,
                             void *stream);
/* SplitBDDoubleCompress::buff_equal_filter (compress/buff_simd.rs:4925-5094):
 * rows equal to pred, set only in the tail step (no rows when r = 0), every
 * row compared; a target below the base gives no rows. */
int buff_scalar_equal_filter(const buff_col *col, double pred, uint32_t *words, uint64_t *count,
                             void *stream);
/* buff_simd_range_filter_with_slice (compress/buff_simd.rs:3736-3884): the
 * fused form that compares at most 4 leading slices. */
int buff_range_filter_with_slice(const buff_col *col, double pred, uint32_t *words,
                                 uint64_t *count, void *stream);
/* buff_simd_equal_filter_with_slice (compress/buff_simd.rs:3888-4025). */
int buff_equal_filter_with_slice(const buff_col *col, double pred, uint32_t *words,
                                 uint64_t *count, void *stream);

/* SplitBDDoubleCompress::byte_fixed_sum (compress/split_double.rs:2127-2208) on
 * the unflipped slice bytes; synchronizes. */
int buff_sum(const buff_col *col, buff_sum_result *out, void *stream);
/* byte_residue_sum_with_precision (compress/split_double.rs:2409-2630). */
int buff_sum_at_precision(const buff_col *col, uint32_t precision, double *out, void *stream);
/* Device-only half of buff_sum: enqueues the per-slice byte sums into
 * `dev_partials` (k+1 u64, device memory).  buff_sum_finish turns host copies
 * of those partials into the reference's f64 result. */
int buff_sum_partials_async(const buff_col *col, uint64_t *dev_partials, void *stream);
int buff_sum_finish(const buff_col *col, const uint64_t *host_partials, buff_sum_result *out);
/* No counterpart in the reference (it reads the column once per call): the
 * bitmap and count of buff_range_filter and the partial sums of
 * buff_sum_partials_async, from one pass over the slices.  partials: 9
 * u64 (device or host); buff_sum_finish turns them into the sum. */
int buff_range_filter_sum(const buff_col *col, double pred, uint32_t *words, uint64_t *count,
                          uint64_t *partials, void *stream);
/* buff_simd_range_filter (compress/buff_simd.rs:3361-3547) then byte_fixed_sum
 * (compress/split_double.rs:2127-2208) on the serialized image itself -- the
 * reference's calling pattern, where each query takes the encoded Vec<u8>.
 * No resident column is made: the kernel reads the image where it lies
 * (device memory, pinned host memory through its mapping, or pageable host
 * memory when the device shares the host's page tables) and answers both
 * queries in one pass, so each byte crosses the host link once.  scale and
 * flags as buff_deserialize.  words: ceil(n/32) u32 (host or device; written
 * in place when the device can reach them); count may be NULL; *sum (host)
 * receives what buff_sum returns.  Plans that are not a single pass (the
 * early return, fixed_len < 8, BUFF_FLAG_INTENDED) and buffers the device
 * cannot reach run as buff_deserialize + buff_range_filter_sum; the results
 * are the same either way.  Synchronizes the stream. */
int buff_range_filter_sum_image(const uint8_t *image, uint64_t len, uint64_t scale,
                                uint32_t flags, double pred, uint32_t *words, uint64_t *count,
                                buff_sum_result *sum, void *stream);
/* buff_simd_range_filter, buff_simd_equal_filter and their _with_slice forms
 * (compress/buff_simd.rs:3361-4025) on the serialized image itself, read
 * where it lies as in buff_range_filter_sum_image: slice 0 in full, later
 * slices and tail bytes only for the candidate rows, so about 1/k of the
 * image crosses the host link.  kind: BUFF_FILTER_*.  Results, panics
 * (BUFF_EREFPANIC) and the early return are those of the column calls;
 * fixed_len < 8 and buffers the device cannot reach run as
 * buff_deserialize + the column call.  Synchronizes the stream. */
#define BUFF_FILTER_RANGE 0
#define BUFF_FILTER_EQUAL 1
#define BUFF_FILTER_RANGE_WITH_SLICE 2
#define BUFF_FILTER_EQUAL_WITH_SLICE 3
int buff_filter_image(const uint8_t *image, uint64_t len, uint64_t scale, uint32_t flags,
                      int kind, double pred, uint32_t *words, uint64_t *count, void *stream);

/* SplitBDDoubleCompress::byte_fixed_max (compress/split_double.rs:3919-4105):
 * the column maximum, its code, and optionally the arg-max bitmap and its
 * cardinality (argmax_words/argmax_count may be NULL). */
int buff_max(const buff_col *col, double *max_value, uint64_t *max_code,
             uint32_t *argmax_words, uint64_t *argmax_count, void *stream);
/* Device-only max: enqueues the maximum code into *dev_max_code (device u64). */
int buff_max_async(const buff_col *col, uint64_t *dev_max_code, void *stream);

/* ---- buff-major (outlier) columns ---- */

/* SplitBDDoubleCompress::buff_encode_majority (compress/buff_simd.rs:317-630):
 * leading byte columns whose Boyer-Moore majority over the first 2000 rows
 * reaches 1200 are stored as (major byte, outlier-row bitmap, outlier bytes);
 * the remaining bytes as slices and the packed tail.  Needs n >= 2000 and
 * codes of at least 8 bits. */
int buff_encode_majority_f64(const double *values, uint64_t n, uint64_t scale, uint32_t flags,
                             void *stream, buff_col **out);
int buff_encode_majority_f32(const float *values, uint64_t n, uint64_t scale, uint32_t flags,
                             void *stream, buff_col **out);
/* Rebuilds a buff-major column from its reference byte image. */
int buff_deserialize_majority(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                              void *stream, buff_col **out);
/* buff_decode_majority (compress/buff_simd.rs:633-861). */
int buff_decode_majority(const buff_col *col, double *out, void *stream);
/* buff_range_filter_majority (compress/buff_simd.rs:863-1277). */
int buff_range_filter_majority(const buff_col *col, double pred, uint32_t *words, uint64_t *count,
                               void *stream);
/* buff_equal_filter_majority (compress/buff_simd.rs:1916-2292). */
int buff_equal_filter_majority(const buff_col *col, double pred, uint32_t *words, uint64_t *count,
                               void *stream);
/* buff_sum_majority (compress/buff_simd.rs:2294-2442); synchronizes. */
int buff_sum_majority(const buff_col *col, buff_sum_result *out, void *stream);
/* buff_max_majority (compress/buff_simd.rs:2444-2861): max, its code and the
 * arg-max rows of the tail step (argmax_words/argmax_count may be NULL). */
int buff_max_majority(const buff_col *col, double *max_value, uint64_t *max_code,
                      uint32_t *argmax_words, uint64_t *argmax_count, void *stream);
/* Device-only buff_sum_majority (compress/buff_simd.rs:2294-2442): enqueues
 * the reference's f64 sum into *dev_sum (device) and, when dev_partials is
 * not NULL, its k (+1 with a tail) per-byte partials (device u64) -- the
 * same bits as buff_sum_majority's `sum` and `partials`, combined on the
 * device; nothing waits for the stream. */
int buff_sum_majority_async(const buff_col *col, double *dev_sum, uint64_t *dev_partials,
                            void *stream);
/* Device-only buff_max_majority (compress/buff_simd.rs:2444-2861): enqueues
 * the maximum code into *dev_max_code (device u64). */
int buff_max_majority_async(const buff_col *col, uint64_t *dev_max_code, void *stream);

/* ---- row-conditioned reads ---- */

/* buff_decode_condition (compress/buff_simd.rs:1528-1712): the values of the
 * listed rows, in list order.  rows: strictly ascending row ids below n (host
 * or device), else BUFF_EINVAL.  As in the reference, a code with a packed
 * tail (fixed_len > 8, r > 0) gets its tail field ORed r bits too high, and an
 * empty list panics (BUFF_EREFPANIC); BUFF_FLAG_INTENDED decodes exactly. */
int buff_decode_condition(const buff_col *col, const uint32_t *rows, uint64_t nrows, double *out,
                          void *stream);
/* buff_major_decode_condition (compress/buff_simd.rs:1714-1914): exact values
 * of the listed rows of a buff-major column without sparse columns; with
 * sparse columns the reference returns an empty Vec (*nout = 0). */
int buff_major_decode_condition(const buff_col *col, const uint32_t *rows, uint64_t nrows,
                                double *out, uint64_t *nout, void *stream);
/* buff_decode_condition over the rows set in a BitVec<u32> bitmap (the order
 * BVIter yields them; bits at or past n are ignored).  *count = rows decoded;
 * out needs room for that many values.  An empty bitmap gives *count = 0. */
int buff_decode_selected(const buff_col *col, const uint32_t *words, double *out, uint64_t *count,
                         void *stream);
/* buff_range_filter_condition (compress/buff_simd.rs:4683-4921): the range
 * predicate on the candidate rows set in cand_words (the reference walks them
 * as a row iterator).  A target below the column's base gives no rows (the
 * reference returns its empty result); target bytes are truncated as in the
 * plain filter; every row may be set (no 32-row restriction). */
int buff_range_filter_condition(const buff_col *col, double pred, const uint32_t *cand_words,
                                uint32_t *words, uint64_t *count, void *stream);
/* buff_range_filter_majority_condition (compress/buff_simd.rs:1279-1526):
 * as above on a buff-major column without sparse columns; with sparse columns
 * the reference returns an empty result. */
int buff_range_filter_majority_condition(const buff_col *col, double pred,
                                         const uint32_t *cand_words, uint32_t *words,
                                         uint64_t *count, void *stream);
/* No counterpart in the reference (it has no caller chaining the two): the
 * bitmap of buff_range_filter, then buff_decode_selected on it, with the
 * selected values left on the device when out is device memory.  words may be
 * NULL; *count = rows selected. */
int buff_range_filter_decode(const buff_col *col, double pred, uint32_t *words, double *out,
                             uint64_t *count, void *stream);

/* buff_max_range (compress/buff_simd.rs:5096-5334): the maximum of every
 * window of `window` rows in [start, end), as values, into out (host or
 * device; room for (end - start) / window values); *nout = windows written.
 * As in the reference a ragged last window is dropped when the code fits one
 * byte and panics otherwise (BUFF_EREFPANIC), as do window = 0, end < start,
 * end > n and, for wider codes, a range shorter than one window.  With
 * BUFF_FLAG_INTENDED the ragged last window is kept and bad ranges return
 * BUFF_EINVAL. */
int buff_max_range(const buff_col *col, uint32_t start, uint32_t end, uint32_t window,
                   double *out, uint64_t *nout, void *stream);
/* buff_max_majority_range (compress/buff_simd.rs:2863-3115): buff_max_range
 * on a buff-major column; with sparse columns the reference returns no
 * windows (*nout = 0). */
int buff_max_majority_range(const buff_col *col, uint32_t start, uint32_t end, uint32_t window,
                            double *out, uint64_t *nout, void *stream);

/* ---- buff-slice layout (compress/buff_slice.rs) ----
 * ceil(fixed_len/8) flipped byte slices, the last one holding the low code
 * bits left-aligned (`code << padding`); no packed tail.  Handles made by
 * these calls answer only the buff_slice_* queries (and buff_serialize). */

/* buff_slice_encode (buff_slice.rs:298-437); a constant column is allowed. */
int buff_slice_encode_f64(const double *values, uint64_t n, uint64_t scale, uint32_t flags,
                          void *stream, buff_col **out);
int buff_slice_encode_f32(const float *values, uint64_t n, uint64_t scale, uint32_t flags,
                          void *stream, buff_col **out);
int buff_slice_deserialize(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                           void *stream, buff_col **out);
/* buff_slice_decode (:439-546). */
int buff_slice_decode(const buff_col *col, double *out, void *stream);
/* buff_slice_range_filter / buff_slice_equal_filter (:1348-1439, :1665-1751):
 * at most 4 slices compared, rows of full 32-row blocks only; a target below
 * the base prints n for both (every row set); fewer than 32 rows panic. */
int buff_slice_range_filter(const buff_col *col, double pred, uint32_t *words, uint64_t *count,
                            void *stream);
int buff_slice_equal_filter(const buff_col *col, double pred, uint32_t *words, uint64_t *count,
                            void *stream);
/* buff_slice_range_filter_nosimd / buff_slice_equal_filter_nosimd
 * (:1753-1871, :1873-1991), the filters of the `buff-slice-scalar` arm:
 * the same per-slice targets and at most 4 slices, compared row by row for
 * every row (no 32-row blocks, no panic below 32 rows); a target below the
 * base prints n for both (every row set); a constant column panics. */
int buff_slice_range_filter_nosimd(const buff_col *col, double pred, uint32_t *words,
                                   uint64_t *count, void *stream);
int buff_slice_equal_filter_nosimd(const buff_col *col, double pred, uint32_t *words,
                                   uint64_t *count, void *stream);
/* buff_slice_decode_bs (:1184-1262): buff_slice_decode for codes of 1 to 4
 * slices; wider codes and constant columns panic (BUFF_EREFPANIC). */
int buff_slice_decode_bs(const buff_col *col, double *out, void *stream);
/* buff_slice_sum (:1101-1182, at most 4 slices) and buff_slice_buffsum
 * (:702-814): the reference adds the decoded values in row order in f64;
 * the result here is that sum whenever it is exact (every value and partial
 * sum below 2^53 units of 2^-dlen), else BUFF_ENOTSUP. */
int buff_slice_sum(const buff_col *col, double *sum, void *stream);
int buff_slice_buffsum(const buff_col *col, double *sum, void *stream);
/* buff_slice_max (:816-928, at most 4 slices) and buff_slice_buffmax
 * (:548-700): the largest value and the rows that reach it. */
int buff_slice_max(const buff_col *col, double *max_value, uint32_t *argmax_words,
                   uint64_t *argmax_count, void *stream);
int buff_slice_buffmax(const buff_col *col, double *max_value, uint32_t *argmax_words,
                       uint64_t *argmax_count, void *stream);
/* buff_slice_max_range (:930-1099): the maximum of every window of `window`
 * rows in [start, end), as values, into out (host or device; room for
 * ceil((min(end, n) - start) / window) values, at least 1); *nout = windows
 * written.  As in the reference, rows past n are not read, and the call
 * panics (BUFF_EREFPANIC) unless the windows it started number
 * (end - start) / window (u32): a ragged last window panics unless end runs
 * past the rows; widths above 32 bits and window = 0 panic too.  When no row
 * is read the one window holds f64::min_value(). */
int buff_slice_max_range(const buff_col *col, uint32_t start, uint32_t end, uint32_t window,
                         double *out, uint64_t *nout, void *stream);

/* ---- RAPG byte_residue layout (compress/split_double.rs:624-2630) ----
 * The header, then -- when ilen > 15 -- a count of sparse leading bytes and
 * per sparse byte the rows where it is nonzero (a croaring bitmap, portable
 * format) and those bytes, then unflipped dense slices and the packed tail.
 * Handles made by these calls answer only the buff_rapg_* queries (and
 * buff_serialize, which writes the reference's image). */

/* byte_residue_encode (:624-955).  Reference panics (BUFF_EREFPANIC): no
 * PRECISION_MAP entry for the scale; ilen > 15 with fewer than 2000 rows;
 * four sparse bytes of a code at least 48 bits wide (bits_counter[32]). */
int buff_rapg_encode_f64(const double *values, uint64_t n, uint64_t scale, uint32_t flags,
                         void *stream, buff_col **out);
int buff_rapg_encode_f32(const float *values, uint64_t n, uint64_t scale, uint32_t flags,
                         void *stream, buff_col **out);
/* A byte_residue_encode image: BUFF_ECORRUPT when its length differs from
 * what the encoder writes for its directory, or a bitmap does not list
 * exactly its outlier rows (below n). */
int buff_rapg_deserialize(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                          void *stream, buff_col **out);
/* byte_residue_decode (:1353-1610): out (host or device, n values); *nout =
 * values written.  A sparse byte without outliers panics
 * (outlier_iter.next().unwrap()), as do reads past the image. */
int buff_rapg_decode(const buff_col *col, double *out, uint64_t *nout, void *stream);
/* byte_residue_decode_with_precision (:1612-1893): the top R bits of each
 * code (R from the precision as for buff_decode_at_precision), not shifted
 * back; *nout = 0 when R ends with the sparse bytes (the reference returns
 * an empty vector there). */
int buff_rapg_decode_at_precision(const buff_col *col, uint32_t precision, double *out,
                                  uint64_t *nout, void *stream);
/* byte_residue_sum (:2211-2407) and byte_residue_sum_with_precision
 * (:2409-2630): the reference's f64 steps; synchronizes. */
int buff_rapg_sum(const buff_col *col, double *sum, void *stream);
int buff_rapg_sum_at_precision(const buff_col *col, uint32_t precision, double *sum, void *stream);

/* ---- RAPG-major (compress/split_double.rs:957-4676, used by outlier_exp) ----
 * byte_residue_encode_outlieru8 writes the buff-major image with exactly one
 * sparse column -- the leading byte, major byte MAJOR = 69 (the vote it runs
 * is overwritten, :1049) -- and the outlier rows as a croaring bitmap.  With
 * one sparse column its queries are the buff-major ones (they differ from
 * buff_simd.rs only in branches for further sparse columns), so these
 * handles also answer buff_*_majority; the buff_rapg_* forms reject
 * buff-major handles (BUFF_ENOTSUP). */
/* byte_residue_encode_outlieru8 (:957-1240): fewer than 2000 rows or codes
 * narrower than a byte panic (BUFF_EREFPANIC). */
int buff_rapg_encode_outlieru8_f64(const double *values, uint64_t n, uint64_t scale, uint32_t flags,
                                   void *stream, buff_col **out);
int buff_rapg_encode_outlieru8_f32(const float *values, uint64_t n, uint64_t scale, uint32_t flags,
                                   void *stream, buff_col **out);
/* A byte_residue_encode_outlieru8 image; images with other than one sparse
 * column return BUFF_ENOTSUP, a bitmap that does not list exactly its
 * outlier rows BUFF_ECORRUPT. */
int buff_rapg_major_deserialize(const uint8_t *bytes, uint64_t len, uint64_t scale, uint32_t flags,
                                void *stream, buff_col **out);
/* byte_residue_decode_majority (:1897-2125). */
int buff_rapg_decode_majority(const buff_col *col, double *out, void *stream);
/* byte_residue_range_filter_majority (:2958-3370) / _equal_filter_majority
 * (:3541-3918): the reference prints the count. */
int buff_rapg_range_filter_majority(const buff_col *col, double pred, uint32_t *words,
                                    uint64_t *count, void *stream);
int buff_rapg_equal_filter_majority(const buff_col *col, double pred, uint32_t *words,
                                    uint64_t *count, void *stream);
/* byte_residue_sum_majority (:2632-2782). */
int buff_rapg_sum_majority(const buff_col *col, buff_sum_result *out, void *stream);
/* byte_residue_max_majority (:4107-4676): the reference prints the maximum. */
int buff_rapg_max_majority(const buff_col *col, double *value, uint64_t *code, uint32_t *argmax,
                           uint64_t *argmax_count, void *stream);

/* ---- batched form (no counterpart in the reference: it runs one column per
 *      call) ---- */

/* Work-queue parameters of the persistent batched kernels. */
typedef struct buff_batch_tune {
  uint32_t tile_rows;     /* rows per work item: a multiple of 1024 (encode uses 4x) */
  uint32_t blocks_per_sm; /* persistent 256-thread CTAs per SM, 1..8 */
  uint32_t stage;         /* row steps whose slice loads are issued together: 1, 2 or 4 */
  uint32_t reserved;
} buff_batch_tune;

/* Encodes ncols f64 columns as buff_simd256_encode does, each with its own
 * scale: one persistent launch takes every column's min/max, one more
 * quantizes and scatters every column into a shared device arena (freed with
 * its last column).  Columns given as host or unaligned pointers, with
 * non-finite extremes, or whose `else if` max needs a second scan go through
 * buff_encode_f64.  tune may be NULL.  out receives ncols handles. */
int buff_batch_encode_f64(const double *const *values, const uint64_t *lens,
                          const uint64_t *scales, uint32_t ncols, uint32_t flags,
                          const buff_batch_tune *tune, void *stream, buff_col **out);

#define BUFF_Q_RANGE 0x1u  /* buff_simd_range_filter bitmap */
#define BUFF_Q_EQUAL 0x2u  /* buff_simd_equal_filter bitmap */
#define BUFF_Q_SUM 0x4u    /* byte_fixed_sum */
#define BUFF_Q_MAX 0x8u    /* byte_fixed_max value (no arg-max bitmap) */
#define BUFF_Q_DECODE 0x10u /* buff_simd256_decode / byte_residue_decode_with_precision */
#define BUFF_Q_ENCODE 0x20u /* buff_simd256_encode into a new column (serving requests only) */

/* One query of a batch: ops is one of RANGE or EQUAL (optionally with SUM),
 * or any of SUM, MAX, DECODE.  Outputs are device memory. */
typedef struct buff_query {
  const buff_col *col; /* a plain (buff-simd) column */
  uint32_t ops;
  uint32_t precision;  /* DECODE: 0 = full precision, else decimals */
  double pred;         /* RANGE / EQUAL */
  uint32_t *words;     /* RANGE / EQUAL: ceil(n/32) words */
  double *values;      /* DECODE: n values */
} buff_query;

typedef struct buff_query_result {
  uint64_t count;       /* rows set by the filter */
  double sum;           /* the reference's f64 sum */
  double max_value;
  uint64_t max_code;
  uint64_t partials[9]; /* per-slice byte sums, then the tail sum */
  uint32_t n_partials;
  int32_t status;
} buff_query_result;

/* A batch of queries as one persistent launch over (query, row tile) items. */
typedef struct buff_plan buff_plan;
int buff_plan_create(const buff_query *queries, uint32_t nq, const buff_batch_tune *tune,
                     void *stream, buff_plan **out);
/* New predicates for the same queries (takes effect at the next launch or
 * replay; the caller orders it after the previous one finished). */
int buff_plan_set_preds(buff_plan *plan, const double *preds);
int buff_plan_launch(buff_plan *plan, void *stream);
/* Records the launch sequence of the plan into a CUDA graph (stream must
 * not be the legacy default stream); buff_plan_replay launches it. */
int buff_plan_capture(buff_plan *plan, void *stream);
int buff_plan_replay(buff_plan *plan, void *stream);
/* Waits for the stream and fills one result per query. */
int buff_plan_results(buff_plan *plan, buff_query_result *out, void *stream);
int buff_plan_free(buff_plan *plan);
/* Times the plan over a grid of tile sizes, CTAs per SM and stage depths
 * and returns the fastest (and its launch time in ms). */
int buff_batch_autotune(const buff_query *queries, uint32_t nq, void *stream,
                        buff_batch_tune *best, float *best_ms);

/* ---- serving (no counterpart in the reference) ---- */

/* A store of resident columns and a request loop on one host thread.  With
 * batched = 1 it batches the requests that are waiting whenever a batch slot
 * is free (continuous batching: up to max_inflight batches run at once, each
 * one persistent launch of up to max_batch queries); with batched = 0 every
 * request runs alone through the single-column calls (one query per launch).
 *
 * Memory.  The server's HBM is two budgets.  Transient device memory --
 * query outputs (bitmaps, decoded values) and the device copy of an encode
 * request's host input -- comes from one arena of output_budget_bytes,
 * allocated at create; requests are admitted into it in arrival order, and a
 * request whose memory does not fit now waits (and holds back the requests
 * behind it) until completions return memory, or fails with BUFF_EFULL when
 * it is larger than the whole arena.  Resident columns (added before start
 * or encoded by requests while serving) are charged to store_budget_bytes:
 * an encode request reserves its column's exact bytes once the column's code
 * width is known, before the column is allocated, and fails with BUFF_EFULL
 * when they exceed what is left (the store never shrinks while serving, so
 * it could never fit). */
typedef struct buff_server_config {
  uint64_t output_budget_bytes;
  uint64_t store_budget_bytes; /* 0: no limit on resident columns */
  uint32_t max_batch;
  uint32_t max_inflight;
  uint32_t batched;
  uint32_t auto_release; /* 1: outputs are freed when the request completes */
  buff_batch_tune tune;  /* tile_rows = 0: defaults */
} buff_server_config;

/* A request: a query on a store column (ops as in buff_query), or
 * ops = BUFF_Q_ENCODE: buff_simd256_encode (compress/buff_simd.rs:3116-3250)
 * of `values` into a new resident column, with `scale` and `flags` as in
 * buff_encode_f64.  The encode runs on the server's own encoder thread and
 * stream while queries keep running; its completion carries the new
 * column's store id (`column`) and its rows (result.count), after which
 * queries may name that id. */
typedef struct buff_request {
  uint32_t column;    /* store id (queries) */
  uint32_t ops;       /* BUFF_Q_* */
  uint32_t precision; /* DECODE: 0 = full precision */
  uint32_t reserved;
  double pred;
  uint64_t tag;       /* returned in the completion */
  /* ENCODE only: n values (f64, or f32 when is_f32) in host or device
   * memory, which must stay valid and unchanged until the completion */
  const void *values;
  uint64_t n;
  uint64_t scale;
  uint32_t flags;
  uint32_t is_f32;
} buff_request;

typedef struct buff_completion {
  uint64_t tag;
  int32_t status;
  uint32_t column;       /* the request's column; for ENCODE the new column's id */
  buff_query_result result;
  const uint32_t *words; /* device bitmap (auto_release = 0; NULL otherwise) */
  const double *values;  /* device values (auto_release = 0; NULL otherwise) */
  uint64_t submit_ns, done_ns; /* steady-clock times */
  uint64_t out_off[2];         /* opaque: for buff_server_release */
  int32_t out_cls[2];
} buff_completion;

typedef struct buff_server buff_server;
int buff_server_create(const buff_server_config *cfg, buff_server **out);
/* Adds a resident column (borrowed: it must outlive the server); BUFF_EFULL
 * beyond store_budget_bytes.  Only before buff_server_start. */
int buff_server_add_column(buff_server *srv, buff_col *col, uint32_t *id);
/* The handle of store column `id` (e.g. for buff_serialize); columns made by
 * ENCODE requests belong to the server and are freed with it. */
int buff_server_column(buff_server *srv, uint32_t id, const buff_col **col);
int buff_server_start(buff_server *srv);
/* Thread-safe. */
int buff_server_submit(buff_server *srv, const buff_request *reqs, uint32_t n);
/* Completed requests, oldest first. */
int buff_server_poll(buff_server *srv, buff_completion *out, uint32_t cap, uint32_t *n);
/* Returns a completion's outputs to the arena (auto_release = 0). */
int buff_server_release(buff_server *srv, const buff_completion *c);
int buff_server_stop(buff_server *srv);
int buff_server_free(buff_server *srv);
int buff_server_stats(buff_server *srv, uint64_t *batches, uint64_t *requests,
                      uint64_t *output_bytes_in_use);
/* Resident column bytes charged to store_budget_bytes, and the columns. */
int buff_server_store_stats(buff_server *srv, uint64_t *store_bytes, uint32_t *columns);
/* Load replay for measurement: submits reqs[i] at arrival_ns[i] after the
 * start (a feeder thread), waits for every completion and returns each
 * request's latency from its arrival time to its completion, its result
 * (results may be NULL) and the wall time from the first arrival to the last
 * completion. */
int buff_server_replay(buff_server *srv, const buff_request *reqs, const uint64_t *arrival_ns,
                       uint32_t n, uint64_t *latency_ns, buff_query_result *results,
                       double *wall_s);

/* ---- allocation-free query ---- */

/* Largest column (rows) that buff_range_filter_noalloc accepts. */
#define BUFF_NOALLOC_MAX_ROWS (1u << 26)

/* buff_range_filter for callers that cannot allocate device memory while
 * answering a query -- for example a server that has already reserved the
 * whole HBM budget for its resident columns, or a process whose device memory
 * belongs to another allocator.  No counterpart in the reference: it exists
 * only for this GPU library.  Same results as buff_range_filter; `words`
 * (ceil(n/32) u32) and `count` (may be NULL) may be host or device memory.
 * It calls no cudaMalloc/cudaFree or other allocating routine: the bitmap and
 * count are staged in a fixed scratch array of about 8 MiB that belongs to the
 * library's device code.  CUDA loads device code lazily, so a device reserves
 * the array the first time this call runs on it -- that first call returns
 * BUFF_ENOMEM if the device has no memory left, so make a warm-up call at
 * start-up, before any stream capture -- and holds it until the process
 * exits.  Columns with more than BUFF_NOALLOC_MAX_ROWS rows return
 * BUFF_ESCRATCH.  The first call on a device also looks up the scratch
 * address for that device; all calls share the array, so calls whose work
 * overlaps on the GPU race and must be ordered by the caller.  The call
 * synchronizes `stream`. */
int buff_range_filter_noalloc(const buff_col *col, double pred, uint32_t *words, uint64_t *count,
                              void *stream);

/* ---- diagnostics ---- */
const char *buff_status_string(int status);
/* Copies nbytes between any host and device addresses and waits for the
 * stream: lets a caller that does not link the CUDA runtime read device
 * outputs (bitmaps and values left on the device). */
int buff_copy(void *dst, const void *src, uint64_t nbytes, void *stream);
/* The last CUDA error code seen by this thread (0 if none). */
int buff_last_cuda_error(void);
/* Number of this library's kernels launched by this process so far. */
uint64_t buff_kernel_launches(void);

#ifdef __cplusplus
}
#endif
#endif /* BUFF_GPU_H */
