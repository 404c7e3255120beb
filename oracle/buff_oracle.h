/*
 * CPU oracle for the BUFF buff-simd hot path.  TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference algorithm (Tranway1/buff,
 * database/src/...), used by the test suite to check the CUDA path and by the
 * benchmark's CPU-baseline leg.  Nothing in the product library links or calls
 * it.  Every function names the reference lines it follows.
 *
 * Parity pinning: the BitPack bit order, BitVec word layout, BVIter order and
 * the movemask lane order are pinned to the reference's own known-answer tests
 * (tests/test_oracle_golden.py).  The codec outputs themselves (encoded bytes,
 * filter bitmaps, sum, max, precision decode) have no recorded outputs in the
 * reference: for those the oracle is parity-unpinned and is checked against an
 * independent numpy model plus the reference's documented quirks.
 */
#ifndef BUFF_ORACLE_H
#define BUFF_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  OR_PANIC marks inputs on which the reference panics
 * (unwrap on a missing PRECISION_MAP entry, slice index out of range, ...). */
#define OR_OK 0
#define OR_PANIC 1
#define OR_EINVAL 2
#define OR_ENOMEM 3

/* Behaviour switches.  0 = the reference's exact behaviour. */
#define OR_INTENDED 1u /* fix the documented quirks (exact min/max, width, ...) */

typedef struct or_header {
  int64_t base;
  uint32_t n;
  uint32_t ilen; /* as stored: wraps when fixed_len < dlen */
  uint32_t dlen;
  uint32_t fixed_len; /* ilen + dlen (u32 wrap), as the decoders compute it */
  uint32_t k;         /* full byte slices (0 when fixed_len < 8) */
  uint32_t r;         /* packed tail bits per row (fixed_len when < 8) */
  size_t slice_off;   /* byte offset of slice 0 */
  size_t tail_off;    /* byte offset of the packed tail / packed codes */
} or_header;

/* --- scalar helpers (prec_double.rs, compress/mod.rs) --- */
int or_prec_of_scale(uint64_t scale);
int or_dlen_of_prec(int prec); /* -1 when PRECISION_MAP has no entry */
int or_precision_exp(int prec);
int64_t or_fetch_fixed_aligned(double v, int32_t precision_exp, uint64_t dlen);
uint32_t or_fixed_len_of_delta(int64_t delta); /* ceil(log2(delta as f64)) as usize */

/* --- BitPack (methods/bit_packing.rs) exposed for known-answer tests --- */
typedef struct or_bw {
  uint8_t *buf;
  size_t len, cap, cursor;
  unsigned bits;
  int oom;
} or_bw;
void or_bw_init(or_bw *w);
void or_bw_free(or_bw *w);
int or_bw_write(or_bw *w, uint32_t value, unsigned bits);
int or_bw_write_bits(or_bw *w, uint32_t value, unsigned bits);
int or_bw_write_byte(or_bw *w, uint8_t v);
int or_bw_write_bytes(or_bw *w, const uint8_t *v, size_t n);
int or_bw_finish_write_byte(or_bw *w);

typedef struct or_br {
  const uint8_t *buf;
  size_t len, cursor;
  unsigned bits;
} or_br;
void or_br_init(or_br *r, const uint8_t *buf, size_t len);
int or_br_read(or_br *r, unsigned bits, uint32_t *out);
int or_br_read_bits(or_br *r, unsigned bits, uint8_t *out);
void or_br_finish_read_byte(or_br *r);
int or_br_read_byte(or_br *r, uint8_t *out);
int or_br_read_n_byte(or_br *r, size_t n, const uint8_t **out);
void or_br_skip_n_byte(or_br *r, size_t n);
int or_br_skip(or_br *r, size_t bits);

/* BitPack convenience for tests: write a sequence of (value,bits) pairs. */
int or_bitpack_write_seq(const uint32_t *values, const uint32_t *bits, size_t cnt,
                         uint8_t *out, size_t cap, size_t *len);
int or_bitpack_read_seq(const uint8_t *buf, size_t len, const uint32_t *bits, size_t cnt,
                        uint32_t *values);

/* BVIter (query/bit_vec_iter.rs:8-49): set positions in order. */
size_t or_bviter_positions(const uint32_t *words, size_t nwords, uint64_t *out, size_t cap);
/* BitVec::to_binary (bit-vec lib.rs:399-406). */
size_t or_bitvec_to_binary(const uint32_t *words, size_t nwords, uint64_t nbits, uint8_t *out);
/* movemask emulation used by the 32-byte compare (vectorize_query.rs:168-222). */
uint32_t or_movemask_gt(const uint8_t *bytes32, uint8_t pred);
uint32_t or_movemask_eq(const uint8_t *bytes32, uint8_t pred);

/* --- codec (compress/buff_simd.rs, compress/split_double.rs) --- */
/* flipped=1: buff-simd layout (slice bytes ^ 0x80); 0: buff layout.
 * Output buffer is malloc'd; free with or_free. */
int or_encode(const double *x, uint32_t n, uint64_t scale, int flipped, unsigned flags,
              uint8_t **out, size_t *out_len);
int or_encode_f32(const float *x, uint32_t n, uint64_t scale, int flipped, unsigned flags,
                  uint8_t **out, size_t *out_len);
void or_free(void *p);
int or_parse_header(const uint8_t *bytes, size_t len, or_header *h);

int or_decode(const uint8_t *bytes, size_t len, uint64_t scale, int flipped, double *out);

/* Filters.  words has ceil(n/32) entries.  *early = 1 when the reference takes
 * its "fixed(pred) < base" early return (the words then hold what the
 * reference's printed count implies: all rows for range, none for equal). */
int or_range_filter(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                    unsigned flags, uint32_t *words, uint64_t *count, int *early);
int or_equal_filter(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                    unsigned flags, uint32_t *words, uint64_t *count, int *early);
/* buff_range_filter (buff_simd.rs:4507-4679) / buff_equal_filter
 * (:4925-5094): the scalar filters of the `buff` profiler arm; flipped = 0
 * for the buff layout they run on. */
int or_scalar_range_filter(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                           int flipped, uint32_t *words, uint64_t *count, int *early);
int or_scalar_equal_filter(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                           int flipped, uint32_t *words, uint64_t *count, int *early);
int or_range_filter_with_slice(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                               uint32_t *words, uint64_t *count, int *early);
int or_equal_filter_with_slice(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                               uint32_t *words, uint64_t *count, int *early);

/* Sum: returns the reference's f64 and the per-slice unsigned byte sums
 * (partials[0..k-1], partials[k] = tail sum).  exact_num is the exact
 * numerator (n*base + sum of codes) as a 128-bit two's complement pair
 * (lo, hi); the exact value is exact_num / 2^dlen. */
int or_sum(const uint8_t *bytes, size_t len, uint64_t scale, int flipped, unsigned flags,
           double *sum, uint64_t *partials, int64_t exact_num[2]);
int or_max(const uint8_t *bytes, size_t len, uint64_t scale, int flipped, unsigned flags,
           double *maxv, uint64_t *max_code, uint32_t *argmax_words, uint64_t *argmax_count);
int or_decode_at_precision(const uint8_t *bytes, size_t len, uint64_t scale, int flipped,
                           uint32_t precision, unsigned flags, double *out);
int or_sum_at_precision(const uint8_t *bytes, size_t len, uint64_t scale, int flipped,
                        uint32_t precision, unsigned flags, double *sum);

/* Multi-threaded range filter + sum over row chunks, used only as the timed
 * CPU baseline (each thread runs the single-threaded reference algorithm on
 * a 32-row-aligned chunk).  Returns elapsed seconds. */
double or_bench_filter_sum(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                           int nthreads, int reps, uint64_t *count, double *sum);

/* --- buff-major (outlier) format: oracle/buff_oracle_major.c --- */
#define OR_BM_SNAPPY 0 /* outlier bitmaps snappy-compressed (the reference) */
#define OR_BM_RAW 1    /* outlier bitmaps stored as raw BitVec::to_binary bytes */
#define OR_BM_ROARING 2 /* outlier bitmaps as croaring portable images (RAPG-major) */
size_t or_snappy_max_compressed(size_t n);
int or_snappy_compress(const uint8_t *in, size_t n, uint8_t *out, size_t cap, size_t *outlen);
int or_snappy_decompress(const uint8_t *in, size_t n, uint8_t *out, size_t cap, size_t *outlen);
int or_encode_majority(const double *x, uint32_t n, uint64_t scale, int bm_mode, uint8_t **out,
                       size_t *out_len);
/* byte_residue_encode_outlieru8 (split_double.rs:957-1240): the majority
 * image with one sparse column whose major byte is MAJOR (69), roaring bitmap. */
int or_encode_outlieru8(const double *x, uint32_t n, uint64_t scale, uint8_t **out,
                        size_t *out_len);
int or_majority_layout(const uint8_t *bytes, size_t len, int bm_mode, uint32_t *ncols,
                       uint8_t *majors, uint32_t *nouts, size_t *dense_off);
int or_decode_majority(const uint8_t *bytes, size_t len, uint64_t scale, int bm_mode, double *out);
int or_range_filter_majority(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                             int bm_mode, uint32_t *words, uint64_t *count, int *early);
int or_equal_filter_majority(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                             int bm_mode, uint32_t *words, uint64_t *count, int *early);
int or_sum_majority(const uint8_t *bytes, size_t len, uint64_t scale, int bm_mode, double *sum,
                    uint64_t *partials);
int or_max_majority(const uint8_t *bytes, size_t len, uint64_t scale, int bm_mode, double *maxv,
                    uint64_t *max_code, uint32_t *argmax_words, uint64_t *argmax_count);

/* --- row-conditioned reads of the buff layout: oracle/buff_oracle_cond.c ---
 * rows: strictly ascending row ids below n (OR_EINVAL otherwise). */
int or_decode_condition(const uint8_t *bytes, size_t len, uint64_t scale, const uint64_t *rows,
                        size_t nrows, double *out);
int or_major_decode_condition(const uint8_t *bytes, size_t len, uint64_t scale,
                              const uint64_t *rows, size_t nrows, double *out, size_t *nout);
int or_range_filter_condition(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                              const uint64_t *rows, size_t nrows, uint32_t *words,
                              uint64_t *count);
int or_range_filter_majority_condition(const uint8_t *bytes, size_t len, uint64_t scale,
                                       double pred, const uint64_t *rows, size_t nrows,
                                       uint32_t *words, uint64_t *count);
/* buff_max_range: the maxima of the full windows of `window` rows in [s, e). */
int or_max_range(const uint8_t *bytes, size_t len, uint64_t scale, uint32_t s, uint32_t e,
                 uint32_t window, double *out, size_t *nout);
/* buff_max_majority_range: the same on a buff-major image (no windows when it
 * has sparse columns). */
int or_max_majority_range(const uint8_t *bytes, size_t len, uint64_t scale, uint32_t s, uint32_t e,
                          uint32_t window, double *out, size_t *nout);

/* --- buff-slice layout: oracle/buff_oracle_slice.c --- */
int or_slice_encode(const double *x, uint32_t n, uint64_t scale, uint8_t **out, size_t *out_len);
int or_slice_decode(const uint8_t *bytes, size_t len, uint64_t scale, double *out);
int or_slice_range_filter(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                          uint32_t *words, uint64_t *count, int *early);
int or_slice_equal_filter(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                          uint32_t *words, uint64_t *count, int *early);
int or_slice_range_filter_nosimd(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                                 uint32_t *words, uint64_t *count, int *early);
int or_slice_equal_filter_nosimd(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                                 uint32_t *words, uint64_t *count, int *early);
int or_slice_decode_bs(const uint8_t *bytes, size_t len, uint64_t scale, double *out);
int or_slice_sum(const uint8_t *bytes, size_t len, uint64_t scale, int any_width, double *sum);
int or_slice_max(const uint8_t *bytes, size_t len, uint64_t scale, int any_width, double *maxv,
                 uint32_t *words, uint64_t *count);
/* buff_slice_max_range: per-window maxima of rows [s, e); out has room for cap values. */
int or_slice_max_range(const uint8_t *b, size_t len, uint64_t scale, uint32_t s, uint32_t e,
                       uint32_t window, double *out, size_t cap, size_t *nout);

/* --- RAPG byte_residue formats (buff_oracle_rapg.c) --- */
/* croaring Bitmap (create + ascending add + run_optimize) in the portable format. */
int or_roaring_serialize(const uint32_t *rows, size_t cnt, uint8_t **out, size_t *out_len);
int or_roaring_parse(const uint8_t *b, size_t len, uint32_t **rows_out, size_t *cnt_out);
/* byte_residue_encode (split_double.rs:624-955). */
int or_rapg_encode(const double *x, uint32_t n, uint64_t scale, uint8_t **out, size_t *out_len);
/* byte_residue_decode (precision < 0) / _with_precision; *nout values (0 or n). */
int or_rapg_decode(const uint8_t *bytes, size_t len, uint64_t scale, int precision, double *out,
                   size_t *nout);
/* byte_residue_sum (precision < 0) / _with_precision. */
int or_rapg_sum(const uint8_t *bytes, size_t len, uint64_t scale, int precision, double *sum_out);
/* Outlier-column directory: count, and per column (up to 8) bitmap size,
 * outlier count, byte offset of the bitmap. */
int or_rapg_layout(const uint8_t *bytes, size_t len, uint32_t *ncols, uint32_t *bm_sizes,
                   uint32_t *nouts, uint64_t *bm_offs);

#ifdef __cplusplus
}
#endif
#endif
