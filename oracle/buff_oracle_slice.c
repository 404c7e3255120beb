/*
 * CPU oracle, part 4: the buff-slice layout (compress/buff_slice.rs).
 * TEST INFRASTRUCTURE ONLY (the product library never links it).
 *
 * buff_slice_encode (:298-437) writes ceil(fixed_len/8) byte slices, each
 * flipped (x ^ 0x80); the last one holds the low bits of the code
 * left-aligned (`code << padding`), so every slice is byte aligned and there
 * is no packed tail.  The header is the buff-simd header.
 *
 *   buff_slice_decode          :439-546
 *   buff_slice_range_filter    :1348-1439   (at most 4 slices, 32-row SIMD loop)
 *   buff_slice_equal_filter    :1665-1751
 *   buff_slice_sum             :1101-1182   (sequential f64 sum, at most 4 slices)
 *   buff_slice_buffsum         :702-814     (sequential f64 sum, any width)
 *   buff_slice_max             :816-928     (f64 max + arg-max rows, at most 4 slices)
 *   buff_slice_buffmax         :548-700     (f64 max + arg-max rows, any width)
 *   buff_slice_max_range       :930-1099    (per-window f64 maxima, at most 4 slices)
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "buff_oracle.h"

int or_slice_encode(const double *x, uint32_t n, uint64_t scale, uint8_t **out, size_t *out_len) {
  int prec = or_prec_of_scale(scale);
  int dl = or_dlen_of_prec(prec);
  if (dl < 0) return OR_PANIC;
  int pexp = or_precision_exp(prec);
  int64_t *fixed = (int64_t *)malloc((size_t)(n ? n : 1) * 8);
  if (!fixed) return OR_ENOMEM;
  int64_t mn = INT64_MAX, mx = INT64_MIN;
  for (uint32_t i = 0; i < n; i++) { /* :319-329, `else if` as buff-simd */
    int64_t f = or_fetch_fixed_aligned(x[i], pexp, (uint64_t)dl);
    if (f < mn)
      mn = f;
    else if (f > mx)
      mx = f;
    fixed[i] = f;
  }
  int64_t delta = (int64_t)((uint64_t)mx - (uint64_t)mn);
  /* `(delta as f64).log2().ceil() as usize`: a NaN or negative saturates to 0 */
  uint32_t fl = delta == 0 ? 0u : or_fixed_len_of_delta(delta);
  uint32_t ilen = (uint32_t)((uint64_t)fl - (uint64_t)dl);
  uint32_t num = fl < 8 ? 1u : (fl + 7) / 8;
  size_t len = 20 + (size_t)num * n;
  uint8_t *buf = (uint8_t *)malloc(len ? len : 1);
  if (!buf) {
    free(fixed);
    return OR_ENOMEM;
  }
  uint64_t ub = (uint64_t)mn;
  uint32_t hw[5] = {(uint32_t)ub, (uint32_t)(ub >> 32), n, ilen, (uint32_t)dl};
  for (int i = 0; i < 5; i++)
    for (int b = 0; b < 4; b++) buf[4 * i + b] = (uint8_t)(hw[i] >> (8 * b));
  for (uint32_t i = 0; i < n; i++) {
    uint64_t c = (uint64_t)(fixed[i] - mn);
    if (fl < 8) {
      buf[20 + i] = (uint8_t)(c << ((8 - fl) & 63)) ^ 0x80u; /* :362-369 */
      continue;
    }
    uint32_t remain = fl;
    for (uint32_t j = 0; j < num; j++) {
      uint8_t b;
      if (remain >= 8) {
        remain -= 8;
        b = (uint8_t)(c >> remain);
      } else {
        b = (uint8_t)(c << (8 - remain)); /* right padding of the last slice (:420-425) */
        remain = 0;
      }
      buf[20 + (size_t)j * n + i] = b ^ 0x80u;
    }
  }
  free(fixed);
  *out = buf;
  *out_len = len;
  return OR_OK;
}

typedef struct slice_hdr {
  int64_t base;
  uint32_t n, fl, dlen, num, pad;
} slice_hdr;

static int slice_header(const uint8_t *b, size_t len, slice_hdr *h) {
  if (len < 20) return OR_PANIC;
  uint32_t w[5];
  for (int i = 0; i < 5; i++)
    w[i] = (uint32_t)b[4 * i] | ((uint32_t)b[4 * i + 1] << 8) | ((uint32_t)b[4 * i + 2] << 16) |
           ((uint32_t)b[4 * i + 3] << 24);
  h->base = (int64_t)((uint64_t)w[0] | ((uint64_t)w[1] << 32));
  h->n = w[2];
  h->fl = w[3] + w[4]; /* ilen + dlen, u32 */
  h->dlen = w[4];
  h->num = h->fl ? (h->fl - 1) / 8 + 1 : 0; /* ceil(remain, 8); 0 stands for the underflow */
  h->pad = h->num ? h->num * 8 - h->fl : 0;
  if (h->fl < 8) {
    h->num = 1;
    h->pad = 8 - h->fl;
  }
  if ((size_t)20 + (size_t)h->num * h->n > len) return OR_PANIC;
  return OR_OK;
}

/* The code of row i: slices MSB-first, the padding shifted out. */
static uint64_t slice_code(const uint8_t *b, const slice_hdr *h, uint32_t i) {
  uint64_t c = 0;
  for (uint32_t j = 0; j < h->num; j++) c = (c << 8) | (uint8_t)(b[20 + (size_t)j * h->n + i] ^ 0x80u);
  return c >> (h->pad & 63);
}

static double slice_value(const slice_hdr *h, uint64_t code) {
  return (double)(int64_t)((uint64_t)h->base + code) / ldexp(1.0, (int)h->dlen);
}

int or_slice_decode(const uint8_t *b, size_t len, uint64_t scale, double *out) {
  (void)scale;
  slice_hdr h;
  if (slice_header(b, len, &h)) return OR_PANIC;
  for (uint32_t i = 0; i < h.n; i++) out[i] = slice_value(&h, slice_code(b, &h, i));
  return OR_OK;
}

/* Range (is_range) or equality filter: per 32-row block, the target byte of
 * every slice up to 4 (`remain - 8*cnt >= 8 ? t >> (remain - 8(cnt+1)) :
 * t << pad`), MSB-first refinement, movemask words for full blocks only. */
static int slice_filter(const uint8_t *b, size_t len, uint64_t scale, double pred, int is_range,
                        int nosimd, uint32_t *words, uint64_t *count, int *early) {
  slice_hdr h;
  if (slice_header(b, len, &h)) return OR_PANIC;
  const size_t nw = ((size_t)h.n + 31) / 32;
  memset(words, 0, nw * 4);
  *early = 0;
  int prec = or_prec_of_scale(scale);
  int64_t fp = or_fetch_fixed_aligned(pred, or_precision_exp(prec), h.dlen);
  if (fp < h.base) { /* both print len (:1375-1378, :1694-1697) */
    for (uint32_t i = 0; i < h.n; i++) words[i >> 5] |= 1u << (i & 31);
    *count = h.n;
    *early = 1;
    return OR_OK;
  }
  if (h.fl == 0) return OR_PANIC; /* ceil(0, 8) underflows: 2^29 slices */
  /* `while i <= len - BYTE_WORD` underflows (the SIMD forms only) */
  if (!nosimd && h.n < 32) return OR_PANIC;
  const uint64_t t = (uint64_t)(fp - h.base);
  uint32_t remain = h.fl, nsl = h.num;
  uint8_t tb[8];
  for (uint32_t cnt = 0; cnt < nsl && cnt < 8; cnt++) {
    if (remain - 8 * cnt >= 8 && remain >= 8 * (cnt + 1))
      tb[cnt] = (uint8_t)(t >> (remain - 8 * (1 + cnt)));
    else
      tb[cnt] = (uint8_t)(t << ((8 * (1 + cnt) - remain) & 63));
  }
  uint32_t used = nsl < 4 ? nsl : 4;
  uint64_t c = 0;
  /* SIMD forms: full 32-row blocks only; nosimd forms (:1753-1991): every
   * row, one at a time */
  const uint32_t nblk = nosimd ? (h.n + 31) / 32 : h.n / 32;
  for (uint32_t blk = 0; blk < nblk; blk++) {
    uint32_t gt = 0, eq = 0;
    for (uint32_t i = 0; i < 32; i++) {
      uint32_t row = blk * 32 + i;
      if (row >= h.n) break;
      int g = 0, e = 1;
      for (uint32_t j = 0; j < used && e; j++) {
        uint8_t v = b[20 + (size_t)j * h.n + row] ^ 0x80u;
        if (v > tb[j]) {
          g = 1;
          e = 0;
        } else if (v != tb[j]) {
          e = 0;
        }
      }
      gt |= (uint32_t)g << i;
      eq |= (uint32_t)e << i;
    }
    words[blk] = is_range ? gt : eq;
    c += (uint64_t)__builtin_popcount(words[blk]);
  }
  *count = c;
  return OR_OK;
}

int or_slice_range_filter(const uint8_t *b, size_t len, uint64_t scale, double pred,
                          uint32_t *words, uint64_t *count, int *early) {
  return slice_filter(b, len, scale, pred, 1, 0, words, count, early);
}

int or_slice_equal_filter(const uint8_t *b, size_t len, uint64_t scale, double pred,
                          uint32_t *words, uint64_t *count, int *early) {
  return slice_filter(b, len, scale, pred, 0, 0, words, count, early);
}

/* buff_slice_range_filter_nosimd / buff_slice_equal_filter_nosimd
 * (buff_slice.rs:1753-1871, :1873-1991): the same per-slice targets and at
 * most 4 slices, row by row over every row (the `buff-slice-scalar` arm). */
int or_slice_range_filter_nosimd(const uint8_t *b, size_t len, uint64_t scale, double pred,
                                 uint32_t *words, uint64_t *count, int *early) {
  return slice_filter(b, len, scale, pred, 1, 1, words, count, early);
}

int or_slice_equal_filter_nosimd(const uint8_t *b, size_t len, uint64_t scale, double pred,
                                 uint32_t *words, uint64_t *count, int *early) {
  return slice_filter(b, len, scale, pred, 0, 1, words, count, early);
}

/* buff_slice_decode_bs (buff_slice.rs:1184-1262): the full decode for codes
 * of 1 to 4 slices; `_ => panic!("bit length greater than 32 ...")` for the
 * rest, ceil(0, 8)'s underflow included. */
int or_slice_decode_bs(const uint8_t *b, size_t len, uint64_t scale, double *out) {
  slice_hdr h;
  if (slice_header(b, len, &h)) return OR_PANIC;
  if (h.fl == 0 || h.num > 4) return OR_PANIC;
  return or_slice_decode(b, len, scale, out);
}

/* Sequential f64 sum of the decoded values (`sum += f_cur`). */
int or_slice_sum(const uint8_t *b, size_t len, uint64_t scale, int any_width, double *sum) {
  (void)scale;
  slice_hdr h;
  if (slice_header(b, len, &h)) return OR_PANIC;
  if (!any_width && (h.fl == 0 || h.num > 4)) return OR_PANIC; /* "greater than 32 ..." */
  double s = 0.0;
  for (uint32_t i = 0; i < h.n; i++) s += slice_value(&h, slice_code(b, &h, i));
  *sum = s;
  return OR_OK;
}

/* f64 maximum of the decoded values and the rows that reach it. */
int or_slice_max(const uint8_t *b, size_t len, uint64_t scale, int any_width, double *maxv,
                 uint32_t *words, uint64_t *count) {
  (void)scale;
  slice_hdr h;
  if (slice_header(b, len, &h)) return OR_PANIC;
  if (!any_width && (h.fl == 0 || h.num > 4)) return OR_PANIC;
  const size_t nw = ((size_t)h.n + 31) / 32;
  memset(words, 0, nw * 4);
  double m = -DBL_MAX; /* f64::min_value() */
  for (uint32_t i = 0; i < h.n; i++) {
    double f = slice_value(&h, slice_code(b, &h, i));
    if (f > m) {
      m = f;
      memset(words, 0, nw * 4);
      words[i >> 5] |= 1u << (i & 31);
    } else if (f == m) {
      words[i >> 5] |= 1u << (i & 31);
    }
  }
  uint64_t c = 0;
  for (size_t w = 0; w < nw; w++) c += (uint64_t)__builtin_popcount(words[w]);
  *maxv = m;
  *count = c;
  return OR_OK;
}

/* Per-window maxima of the decoded values of rows [s, e), windows of
 * `window` rows starting at s (buff_slice.rs:930-1099).  The row loop runs
 * over all n rows and stops at e, so rows past n are never read; a window
 * closes when the row index reaches cur_s + window; the last window's
 * maximum is pushed after the loop (f64::min_value() if no row was read).
 * Then `assert_eq!((cur_s - s) / window + 1, (e - s) / window)` in u32:
 * a ragged last window panics unless e runs past the rows.  The arg-max
 * bitmap the reference keeps is never read, so it is not built here. */
int or_slice_max_range(const uint8_t *b, size_t len, uint64_t scale, uint32_t s, uint32_t e,
                       uint32_t window, double *out, size_t cap, size_t *nout) {
  (void)scale;
  slice_hdr h;
  *nout = 0;
  if (slice_header(b, len, &h)) return OR_PANIC;
  if (h.fl == 0 || h.num > 4) return OR_PANIC; /* `_ => panic!("bit length greater than 32 ...")` */
  if (window == 0) return OR_PANIC;             /* the final assert divides by the window */
  double m = -DBL_MAX;
  uint32_t cur_s = s;
  size_t k = 0;
  for (uint32_t i = 0; i < h.n; i++) {
    if (i < s) continue;
    if (i >= e) break;
    if ((uint64_t)i == (uint64_t)cur_s + window) {
      if (k < cap) out[k] = m;
      k++;
      m = -DBL_MAX;
      cur_s = i;
    }
    double f = slice_value(&h, slice_code(b, &h, i));
    if (f > m) m = f;
  }
  if ((cur_s - s) / window + 1 != (uint32_t)(e - s) / window) return OR_PANIC;
  if (k < cap) out[k] = m;
  k++;
  *nout = k;
  return k <= cap ? OR_OK : OR_EINVAL;
}
