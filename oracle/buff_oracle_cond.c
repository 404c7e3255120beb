/*
 * CPU oracle, part 3: the row-conditioned reads of the buff layout.
 * TEST INFRASTRUCTURE ONLY (the product library never links it).
 *
 *   buff_decode_condition              compress/buff_simd.rs:1528-1712
 *   buff_major_decode_condition        compress/buff_simd.rs:1714-1914
 *   buff_range_filter_condition        compress/buff_simd.rs:4683-4921
 *   buff_range_filter_majority_condition  compress/buff_simd.rs:1279-1526
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
