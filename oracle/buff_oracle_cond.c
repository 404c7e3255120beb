/*
 * CPU oracle, part 3: the row-conditioned reads of the buff layout.
 * TEST INFRASTRUCTURE ONLY (the product library never links it).
 *
 *   buff_decode_condition              compress/buff_simd.rs:1528-1712
 *   buff_major_decode_condition        compress/buff_simd.rs:1714-1914
 *   buff_range_filter_condition        compress/buff_simd.rs:4683-4921
 *   buff_range_filter_majority_condition  compress/buff_simd.rs:1279-1526
 *   buff_max_range                     compress/buff_simd.rs:5096-5334
 *
 * Each walks the byte image with the BitPack reader in the reference's order:
 * per slice, skip to the next listed row, read its byte, skip to the end of
 * the slice; the packed tail last.  The row list must be strictly ascending
 * and below n (the reference subtracts consecutive entries as usize).  The
 * slices are read as stored, without undoing a flip: these functions belong
 * to the buff layout (compress/split_double.rs:298-432).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "buff_oracle.h"

typedef struct cond_hdr {
  int64_t base;
  uint32_t n, ilen, dlen;
  size_t remain; /* (dlen + ilen) as usize, u32 addition */
} cond_hdr;

static int cond_header(or_br *br, cond_hdr *h) {
  uint32_t lo, hi, n, ilen, dlen;
  if (or_br_read(br, 32, &lo) || or_br_read(br, 32, &hi) || or_br_read(br, 32, &n) ||
      or_br_read(br, 32, &ilen) || or_br_read(br, 32, &dlen))
    return OR_PANIC;
  h->base = (int64_t)((uint64_t)lo | ((uint64_t)hi << 32));
  h->n = n;
  h->ilen = ilen;
  h->dlen = dlen;
  h->remain = (size_t)(uint32_t)(dlen + ilen);
  return OR_OK;
}

static int rows_ok(const uint64_t *rows, size_t nrows, uint32_t n) {
  for (size_t i = 0; i < nrows; i++)
    if (rows[i] >= n || (i && rows[i] <= rows[i - 1])) return 0;
  return 1;
}

static inline double to_value(int64_t base, uint64_t v, double scl) {
  return (double)(int64_t)((uint64_t)base + v) / scl;
}

/* Per-slice pass shared by both decoders: for each listed row read one byte
 * (or `remain` bits when bits != 0) into cur[]. */
static int pass_bytes(or_br *br, const uint64_t *rows, size_t nrows, uint8_t *cur) {
  uint64_t pre = rows[0];
  or_br_skip_n_byte(br, (size_t)pre);
  if (or_br_read_byte(br, &cur[0])) return OR_PANIC;
  for (size_t i = 1; i < nrows; i++) {
    uint64_t delta = rows[i] - pre;
    if (delta != 1) or_br_skip_n_byte(br, (size_t)(delta - 1));
    if (or_br_read_byte(br, &cur[i])) return OR_PANIC;
    pre = rows[i];
  }
  return OR_OK;
}

static int pass_bits(or_br *br, const uint64_t *rows, size_t nrows, size_t bits, uint8_t *cur) {
  uint64_t pre = rows[0];
  if (pre) or_br_skip(br, (size_t)pre * bits);
  if (or_br_read_bits(br, (unsigned)bits, &cur[0])) return OR_PANIC;
  for (size_t i = 1; i < nrows; i++) {
    uint64_t delta = rows[i] - pre;
    if (delta != 1) or_br_skip(br, (size_t)(delta - 1) * bits);
    if (or_br_read_bits(br, (unsigned)bits, &cur[i])) return OR_PANIC;
    pre = rows[i];
  }
  return OR_OK;
}

static void skip_rest(or_br *br, uint32_t n, uint64_t last) {
  if ((uint64_t)n - last > 1) or_br_skip_n_byte(br, (size_t)((uint64_t)n - last - 1));
}

/* The decode of listed rows after the header (and the column-count byte of
 * a buff-major image).  tail_shift: 1 = buff_decode_condition, whose packed
 * tail is ORed as `cur << remain` (:1693, :1701); 0 = the plain OR of
 * buff_major_decode_condition (:1885, :1899). */
static int cond_decode(or_br *br, const cond_hdr *h, const uint64_t *rows, size_t nrows,
                       int tail_shift, double *out) {
  const double scl = ldexp(1.0, (int)h->dlen);
  size_t remain = h->remain;
  int rc = OR_OK;
  uint8_t *cur = (uint8_t *)malloc(nrows ? nrows : 1);
  uint64_t *fixed = (uint64_t *)calloc(nrows ? nrows : 1, 8);
  if (!cur || !fixed) {
    rc = OR_ENOMEM;
    goto done;
  }
  if (remain < 8) {
    if ((rc = pass_bits(br, rows, nrows, remain, cur))) goto done;
    for (size_t i = 0; i < nrows; i++) out[i] = to_value(h->base, cur[i], scl);
    goto done;
  }
  remain -= 8;
  if ((rc = pass_bytes(br, rows, nrows, cur))) goto done;
  if (remain == 0) {
    for (size_t i = 0; i < nrows; i++) out[i] = to_value(h->base, cur[i], scl);
    goto done;
  }
  for (size_t i = 0; i < nrows; i++) fixed[i] = (uint64_t)cur[i] << (remain & 63);
  skip_rest(br, h->n, rows[nrows - 1]);
  while (remain >= 8) {
    remain -= 8;
    if ((rc = pass_bytes(br, rows, nrows, cur))) goto done;
    if (remain == 0) { /* the last full byte emits the values (:1628-1645) */
      for (size_t i = 0; i < nrows; i++) out[i] = to_value(h->base, cur[i] | fixed[i], scl);
      goto done;
    }
    for (size_t i = 0; i < nrows; i++) fixed[i] |= (uint64_t)cur[i] << (remain & 63);
    skip_rest(br, h->n, rows[nrows - 1]);
  }
  or_br_finish_read_byte(br);
  if ((rc = pass_bits(br, rows, nrows, remain, cur))) goto done;
  for (size_t i = 0; i < nrows; i++) {
    uint64_t t = tail_shift ? ((uint64_t)cur[i] << (remain & 63)) : (uint64_t)cur[i];
    out[i] = to_value(h->base, fixed[i] | t, scl);
  }
done:
  free(cur);
  free(fixed);
  return rc;
}

int or_decode_condition(const uint8_t *bytes, size_t len, uint64_t scale, const uint64_t *rows,
                        size_t nrows, double *out) {
  (void)scale;
  or_br br;
  or_br_init(&br, bytes, len);
  cond_hdr h;
  if (cond_header(&br, &h)) return OR_PANIC;
  if (nrows == 0) return OR_PANIC; /* iter.next().unwrap() (:1559) */
  if (!rows_ok(rows, nrows, h.n)) return OR_EINVAL;
  return cond_decode(&br, &h, rows, nrows, 1, out);
}

int or_major_decode_condition(const uint8_t *bytes, size_t len, uint64_t scale,
                              const uint64_t *rows, size_t nrows, double *out, size_t *nout) {
  (void)scale;
  or_br br;
  or_br_init(&br, bytes, len);
  cond_hdr h;
  uint32_t cols;
  *nout = 0;
  if (cond_header(&br, &h) || or_br_read(&br, 8, &cols)) return OR_PANIC;
  if (cols > 0) return OR_OK; /* "not implemented yet": an empty Vec (:1741-1743) */
  if (nrows == 0) return OR_OK;
  if (!rows_ok(rows, nrows, h.n)) return OR_EINVAL;
  int rc = cond_decode(&br, &h, rows, nrows, 0, out);
  if (rc == OR_OK) *nout = nrows;
  return rc;
}

static inline void set_bit(uint32_t *w, uint64_t i) { w[i >> 5] |= 1u << (i & 31); }

/* Range filter over listed rows after the header (:4712-4917). */
static int cond_range(or_br *br, const cond_hdr *h, uint64_t scale, double pred,
                      const uint64_t *rows, size_t nrows, uint32_t *words) {
  const size_t nw = ((size_t)h->n + 31) / 32;
  size_t remain = h->remain;
  int prec = or_prec_of_scale(scale);
  int64_t fixed_part = or_fetch_fixed_aligned(pred, or_precision_exp(prec), h->dlen);
  memset(words, 0, nw * 4);
  if (fixed_part < h->base) return OR_OK; /* prints n, returns the empty res */
  const uint64_t t = (uint64_t)(fixed_part - h->base);
  if (nrows && !rows_ok(rows, nrows, h->n)) return OR_EINVAL;
  uint8_t *cur = (uint8_t *)malloc(nrows ? nrows : 1);
  uint64_t *cand = (uint64_t *)malloc((nrows ? nrows : 1) * 8), *next = NULL;
  size_t nc = 0;
  int rc = OR_OK;
  if (!cur || !cand) {
    rc = OR_ENOMEM;
    goto done;
  }
  if (remain < 8) {
    uint8_t tar = (uint8_t)t;
    if (nrows && (rc = pass_bits(br, rows, nrows, remain, cur))) goto done;
    for (size_t i = 0; i < nrows; i++)
      if (cur[i] > tar) set_bit(words, rows[i]);
    goto done;
  }
  remain -= 8;
  {
    uint8_t tar = (uint8_t)(t >> (remain & 63));
    if (nrows && (rc = pass_bytes(br, rows, nrows, cur))) goto done;
    for (size_t i = 0; i < nrows; i++) {
      if (cur[i] > tar)
        set_bit(words, rows[i]);
      else if (cur[i] == tar)
        cand[nc++] = rows[i];
    }
    if (nc == 0) goto done;
    skip_rest(br, h->n, rows[nrows - 1]);
  }
  next = (uint64_t *)malloc(nc * 8);
  if (!next) {
    rc = OR_ENOMEM;
    goto done;
  }
  while (remain > 0) {
    if (remain >= 8) {
      remain -= 8;
      if (nc == 0) break; /* the remaining slices are skipped */
      uint8_t tar = (uint8_t)(t >> (remain & 63));
      if ((rc = pass_bytes(br, cand, nc, cur))) goto done;
      size_t nn = 0;
      uint64_t last = cand[nc - 1];
      for (size_t i = 0; i < nc; i++) {
        if (cur[i] > tar)
          set_bit(words, cand[i]);
        else if (cur[i] == tar)
          next[nn++] = cand[i];
      }
      skip_rest(br, h->n, last);
      memcpy(cand, next, nn * 8);
      nc = nn;
    } else {
      uint8_t tar = (uint8_t)((uint8_t)((uint8_t)t << (8 - remain)) >> (8 - remain));
      or_br_finish_read_byte(br);
      if (nc == 0) break;
      if ((rc = pass_bits(br, cand, nc, remain, cur))) goto done;
      for (size_t i = 0; i < nc; i++)
        if (cur[i] > tar) set_bit(words, cand[i]);
      remain = 0;
    }
  }
done:
  free(cur);
  free(cand);
  free(next);
  return rc;
}

static uint64_t count_words(const uint32_t *w, size_t nw) {
  uint64_t c = 0;
  for (size_t i = 0; i < nw; i++) c += (uint64_t)__builtin_popcount(w[i]);
  return c;
}

int or_range_filter_condition(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                              const uint64_t *rows, size_t nrows, uint32_t *words,
                              uint64_t *count) {
  or_br br;
  or_br_init(&br, bytes, len);
  cond_hdr h;
  if (cond_header(&br, &h)) return OR_PANIC;
  int rc = cond_range(&br, &h, scale, pred, rows, nrows, words);
  if (count) *count = count_words(words, ((size_t)h.n + 31) / 32);
  return rc;
}

int or_range_filter_majority_condition(const uint8_t *bytes, size_t len, uint64_t scale,
                                       double pred, const uint64_t *rows, size_t nrows,
                                       uint32_t *words, uint64_t *count) {
  or_br br;
  or_br_init(&br, bytes, len);
  cond_hdr h;
  uint32_t cols;
  if (cond_header(&br, &h)) return OR_PANIC;
  const size_t nw = ((size_t)h.n + 31) / 32;
  memset(words, 0, nw * 4);
  if (count) *count = 0;
  {
    int prec = or_prec_of_scale(scale);
    int64_t fp = or_fetch_fixed_aligned(pred, or_precision_exp(prec), h.dlen);
    if (fp < h.base) return OR_OK; /* :1303-1306, before the column count is read */
  }
  if (or_br_read(&br, 8, &cols)) return OR_PANIC;
  if (cols > 0) return OR_OK; /* "not implemented yet": the empty res (:1313-1315) */
  int rc = cond_range(&br, &h, scale, pred, rows, nrows, words);
  if (count) *count = count_words(words, nw);
  return rc;
}

/* ------------------------------------------------------------------ */
/* buff_max_range (compress/buff_simd.rs:5096-5334): per-window maxima  */
/* of rows [s, e) in windows of `window` rows, on the buff layout.       */
/* ------------------------------------------------------------------ */

/* Candidate list with the roaring-style operations the reference uses
 * (add, remove_range, ascending iteration). */
typedef struct rows_t {
  uint32_t *v;
  size_t n, cap;
} rows_t;

static int rows_add(rows_t *r, uint32_t x) {
  if (r->n && r->v[r->n - 1] == x) return OR_OK;
  if (r->n == r->cap) {
    size_t nc = r->cap ? 2 * r->cap : 1024;
    uint32_t *nv = (uint32_t *)realloc(r->v, nc * 4);
    if (!nv) return OR_ENOMEM;
    r->v = nv;
    r->cap = nc;
  }
  r->v[r->n++] = x; /* callers add in ascending order */
  return OR_OK;
}

/* remove_range(lo .. hi): drops trailing entries in [lo, hi) (entries are
 * ascending and every later entry is >= hi when this is called). */
static void rows_remove_tail(rows_t *r, uint32_t lo, uint32_t hi) {
  while (r->n && r->v[r->n - 1] >= lo && r->v[r->n - 1] < hi) r->n--;
}

int or_max_range(const uint8_t *bytes, size_t len, uint64_t scale, uint32_t s, uint32_t e,
                 uint32_t window, double *out, size_t *nout) {
  (void)scale;
  or_br br;
  or_br_init(&br, bytes, len);
  cond_hdr h;
  *nout = 0;
  if (cond_header(&br, &h)) return OR_PANIC;
  if (window == 0) return OR_PANIC; /* (cur_s - s) / window */
  uint32_t remain = (uint32_t)h.remain;
  const double scl = ldexp(1.0, (int)h.dlen);
  const uint32_t nwin = e >= s ? (e - s) / window : 0;
  uint64_t *maxv = (uint64_t *)calloc(nwin + 1, 8);
  size_t nmax = 0;
  rows_t rb1 = {0, 0, 0}, cur = {0, 0, 0};
  int rc = OR_OK;
  if (!maxv) return OR_ENOMEM;
  if (e < s || e > h.n) { /* read_n_byte / read_bits past the data */
    rc = OR_PANIC;
    goto done;
  }
  if (remain < 8) {
    uint64_t mx = 0;
    uint32_t cur_s = s;
    if (or_br_skip(&br, (size_t)s * remain)) {
      rc = OR_PANIC;
      goto done;
    }
    for (uint32_t i = s; i < e; i++) {
      if (i == cur_s + window) {
        cur_s = i;
        maxv[nmax++] = mx;
        mx = 0;
      }
      uint8_t c;
      if (or_br_read_bits(&br, remain, &c)) {
        rc = OR_PANIC;
        goto done;
      }
      if (c > mx) mx = c;
    }
    if (e == cur_s + window) maxv[nmax++] = mx;
    goto emit;
  }
  remain -= 8;
  {
    uint8_t byte_max = 0;
    uint32_t cur_s = s, i = s;
    const uint8_t *chunk;
    or_br_skip_n_byte(&br, s);
    if (e > s) {
      if (or_br_read_n_byte(&br, e - s, &chunk)) {
        rc = OR_PANIC;
        goto done;
      }
    } else {
      chunk = NULL;
    }
    for (; i < e; i++) {
      uint8_t c = chunk[i - s];
      if (i == cur_s + window) {
        cur_s = i;
        maxv[nmax++] = (uint64_t)byte_max << remain;
        byte_max = 0;
      }
      if (c > byte_max) {
        byte_max = c;
        rows_remove_tail(&rb1, cur_s, i);
        if ((rc = rows_add(&rb1, i))) goto done;
      } else if (c == byte_max) {
        if ((rc = rows_add(&rb1, i))) goto done;
      }
    }
    if (i == cur_s + window) maxv[nmax++] = (uint64_t)byte_max << remain;
    or_br_skip_n_byte(&br, h.n - e);
  }
  while (remain > 0) {
    uint8_t byte_max = 0;
    uint32_t cur_s = s;
    const int bytewise = remain >= 8;
    uint32_t bits;
    if (bytewise) {
      remain -= 8;
      bits = 8;
    } else {
      or_br_finish_read_byte(&br);
      bits = remain;
    }
    cur.n = 0;
    uint32_t pre = 0;
    for (size_t t = 0; t < rb1.n; t++) {
      uint32_t dc = rb1.v[t];
      if (t > 0 && dc >= cur_s + window) {
        size_t wi = (cur_s - s) / window;
        if (wi >= nmax) {
          rc = OR_PANIC; /* max_vec.get_mut(..).unwrap() */
          goto done;
        }
        maxv[wi] |= (uint64_t)byte_max << (bytewise ? remain : 0);
        byte_max = 0;
        cur_s += window;
      }
      uint8_t d;
      if (bytewise) {
        if (t == 0) {
          if (dc) or_br_skip_n_byte(&br, dc);
        } else if (dc - pre != 1) {
          or_br_skip_n_byte(&br, dc - pre - 1);
        }
        if (or_br_read_byte(&br, &d)) {
          rc = OR_PANIC;
          goto done;
        }
      } else {
        if (t == 0) {
          if (dc && or_br_skip(&br, (size_t)dc * bits)) {
            rc = OR_PANIC;
            goto done;
          }
        } else if (dc - pre != 1 && or_br_skip(&br, (size_t)(dc - pre - 1) * bits)) {
          rc = OR_PANIC;
          goto done;
        }
        if (or_br_read_bits(&br, bits, &d)) {
          rc = OR_PANIC;
          goto done;
        }
      }
      if (d > byte_max) {
        byte_max = d;
        if (t > 0) rows_remove_tail(&cur, cur_s, dc);
        if ((rc = rows_add(&cur, dc))) goto done;
      } else if (d == byte_max) {
        if ((rc = rows_add(&cur, dc))) goto done;
      }
      pre = dc;
    }
    /* assert_eq!((cur_s-s)/window+1, (e-s)/window) */
    if ((cur_s - s) / window + 1 != nwin) {
      rc = OR_PANIC;
      goto done;
    }
    maxv[(cur_s - s) / window] |= (uint64_t)byte_max << (bytewise ? remain : 0);
    if (bytewise) {
      if (rb1.n && h.n - pre > 1) or_br_skip_n_byte(&br, h.n - pre - 1);
      rows_t tmp = rb1;
      rb1 = cur;
      cur = tmp;
    } else {
      remain = 0;
    }
  }
emit:
  for (size_t i = 0; i < nmax; i++) out[i] = (double)(int64_t)((uint64_t)h.base + maxv[i]) / scl;
  *nout = nmax;
done:
  free(maxv);
  free(rb1.v);
  free(cur.v);
  return rc;
}

/* buff_max_majority_range (compress/buff_simd.rs:2863-3115): the windowed
 * max of buff_max_range on a buff-major image.  It reads the column-count
 * byte after the header; with sparse columns it logs "not implemented" and
 * returns no windows; without, the rest of the image is the buff layout and
 * the steps are buff_max_range's (its BitVec remove_range clears the same
 * rows as croaring's in every call the loop makes).  Codes narrower than a
 * byte (packed over the count byte) are not restated: OR_EINVAL. */
int or_max_majority_range(const uint8_t *bytes, size_t len, uint64_t scale, uint32_t s, uint32_t e,
                          uint32_t window, double *out, size_t *nout) {
  *nout = 0;
  or_header h;
  if (len < 21 || or_parse_header(bytes, len, &h)) return OR_PANIC;
  if (h.fixed_len < 8) return OR_EINVAL;
  if (bytes[20] != 0) return OR_OK; /* error!("handle groupby for outlier is not implemented") */
  uint8_t *img = (uint8_t *)malloc(len - 1);
  if (!img) return OR_ENOMEM;
  memcpy(img, bytes, 20);
  memcpy(img + 20, bytes + 21, len - 21);
  const int rc = or_max_range(img, len - 1, scale, s, e, window, out, nout);
  free(img);
  return rc;
}
