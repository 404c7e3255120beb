/*
 * CPU oracle, part 5: the RAPG "byte_residue" formats
 * (compress/split_double.rs).  TEST INFRASTRUCTURE ONLY (the product library
 * never links it).
 *
 *   byte_residue_encode                   :624-955
 *   byte_residue_decode                   :1353-1610
 *   byte_residue_decode_with_precision    :1612-1893
 *   byte_residue_sum                      :2211-2407
 *   byte_residue_sum_with_precision       :2409-2630
 *
 * Image: the 20-byte header, then -- only when ilen > 15 (u32, so also when
 * ilen wrapped because fixed_len < dlen) -- a u8 count of outlier columns and
 * per outlier column (a leading code byte that is nonzero in fewer than 200
 * of the first 2000 rows): u32 bitmap size, the row set as a croaring bitmap,
 * a pad byte, u32 outlier count, the nonzero bytes in row order, a pad byte;
 * then the remaining full bytes as unflipped slices and the packed tail.
 *
 * The row sets are croaring 0.5.0 bitmaps (Cargo.toml:49): `Bitmap::create`,
 * `add` in ascending row order, `run_optimize`, `serialize` (the portable
 * Roaring format).  croaring is not vendored with the reference, so the
 * bitmap bytes follow the published Roaring portable format specification
 * (container choice: array up to 4096 values, bitset above; run_optimize
 * turns a container into runs when 2 + 4*runs bytes beat its array
 * (2 + 2*card) or bitset (8192) size) -- parity unpinned.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "buff_oracle.h"

#define RG_SAMPLE 2000u        /* split_double.rs:25 */
#define RG_OUTLIER_R 0.1f      /* split_double.rs:26 */
#define RB_COOKIE_RUN 12347u   /* portable format, with run containers */
#define RB_COOKIE_NORUN 12346u /* portable format, no run containers */
#define RB_NO_OFFSET 4u        /* below this many containers a run image has no offsets */
#define RB_ARRAY_MAX 4096u     /* array containers hold at most this many values */

/* ------------------------------------------------------------------ */
/* Roaring portable format                                            */
/* ------------------------------------------------------------------ */

static void put16(uint8_t *p, uint32_t v) {
  p[0] = (uint8_t)v;
  p[1] = (uint8_t)(v >> 8);
}
static void put32(uint8_t *p, uint32_t v) {
  for (int i = 0; i < 4; i++) p[i] = (uint8_t)(v >> (8 * i));
}
static uint32_t get16(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
static uint32_t get32(const uint8_t *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

enum { RB_ARRAY = 0, RB_BITSET = 1, RB_RUN = 2 };

typedef struct rb_cont {
  uint32_t key, card, nruns, type;
  const uint32_t *v; /* the container's rows (full 32-bit values, ascending) */
} rb_cont;

static uint32_t rb_cont_bytes(const rb_cont *c) {
  if (c->type == RB_RUN) return 2 + 4 * c->nruns;
  if (c->type == RB_BITSET) return 8192;
  return 2 * c->card;
}

/* Bitmap of the ascending rows (no duplicates) after create + add +
 * run_optimize, serialized. */
int or_roaring_serialize(const uint32_t *rows, size_t cnt, uint8_t **out, size_t *out_len) {
  size_t ncont = 0;
  for (size_t i = 0; i < cnt; i++)
    if (i == 0 || (rows[i] >> 16) != (rows[i - 1] >> 16)) ncont++;
  rb_cont *cs = (rb_cont *)calloc(ncont ? ncont : 1, sizeof(rb_cont));
  if (!cs) return OR_ENOMEM;
  size_t ci = 0;
  for (size_t i = 0; i < cnt;) {
    size_t j = i;
    uint32_t runs = 0;
    while (j < cnt && (rows[j] >> 16) == (rows[i] >> 16)) {
      if (j == i || rows[j] != rows[j - 1] + 1) runs++;
      j++;
    }
    rb_cont *c = &cs[ci++];
    c->key = rows[i] >> 16;
    c->card = (uint32_t)(j - i);
    c->nruns = runs;
    c->v = rows + i;
    c->type = c->card > RB_ARRAY_MAX ? RB_BITSET : RB_ARRAY;
    /* run_optimize */
    const uint32_t as_run = 2 + 4 * runs;
    if (c->type == RB_ARRAY ? as_run < 2 + 2 * c->card : as_run < 8192) c->type = RB_RUN;
    i = j;
  }
  int hasrun = 0;
  for (size_t k = 0; k < ncont; k++) hasrun |= cs[k].type == RB_RUN;
  size_t len = 0, start;
  const size_t s = (ncont + 7) / 8;
  if (hasrun)
    start = ncont < RB_NO_OFFSET ? 4 + 4 * ncont + s : 4 + 8 * ncont + s;
  else
    start = 8 + 8 * ncont;
  len = start;
  for (size_t k = 0; k < ncont; k++) len += rb_cont_bytes(&cs[k]);
  uint8_t *b = (uint8_t *)calloc(len ? len : 1, 1);
  if (!b) {
    free(cs);
    return OR_ENOMEM;
  }
  size_t p = 0;
  if (hasrun) {
    put32(b, RB_COOKIE_RUN | ((uint32_t)(ncont - 1) << 16));
    p = 4;
    for (size_t k = 0; k < ncont; k++)
      if (cs[k].type == RB_RUN) b[p + k / 8] |= (uint8_t)(1u << (k % 8));
    p += s;
  } else {
    put32(b, RB_COOKIE_NORUN);
    put32(b + 4, (uint32_t)ncont);
    p = 8;
  }
  for (size_t k = 0; k < ncont; k++) {
    put16(b + p, cs[k].key);
    put16(b + p + 2, cs[k].card - 1);
    p += 4;
  }
  if (!hasrun || ncont >= RB_NO_OFFSET) {
    uint32_t off = (uint32_t)start;
    for (size_t k = 0; k < ncont; k++) {
      put32(b + p, off);
      p += 4;
      off += rb_cont_bytes(&cs[k]);
    }
  }
  for (size_t k = 0; k < ncont; k++) {
    const rb_cont *c = &cs[k];
    if (c->type == RB_ARRAY) {
      for (uint32_t i = 0; i < c->card; i++) put16(b + p + 2 * i, c->v[i] & 0xFFFFu);
    } else if (c->type == RB_BITSET) {
      for (uint32_t i = 0; i < c->card; i++) {
        const uint32_t lo = c->v[i] & 0xFFFFu;
        b[p + lo / 8] |= (uint8_t)(1u << (lo % 8)); /* u64 words, little-endian */
      }
    } else {
      put16(b + p, c->nruns);
      uint32_t r = 0, i = 0;
      while (i < c->card) {
        uint32_t j = i;
        while (j + 1 < c->card && c->v[j + 1] == c->v[j] + 1) j++;
        put16(b + p + 2 + 4 * r, c->v[i] & 0xFFFFu);
        put16(b + p + 4 + 4 * r, j - i); /* run length - 1 */
        r++;
        i = j + 1;
      }
    }
    p += rb_cont_bytes(c);
  }
  free(cs);
  *out = b;
  *out_len = len;
  return OR_OK;
}

/* `Bitmap::deserialize` then ascending iteration: the rows, or OR_PANIC for a
 * buffer that is not a portable Roaring image. */
int or_roaring_parse(const uint8_t *b, size_t len, uint32_t **rows_out, size_t *cnt_out) {
  *rows_out = NULL;
  *cnt_out = 0;
  if (len < 4) return OR_PANIC;
  const uint32_t cookie = get32(b);
  size_t p, size, s = 0;
  int hasrun;
  if ((cookie & 0xFFFFu) == RB_COOKIE_RUN) {
    hasrun = 1;
    size = (cookie >> 16) + 1;
    s = (size + 7) / 8;
    p = 4 + s;
  } else if (cookie == RB_COOKIE_NORUN) {
    hasrun = 0;
    if (len < 8) return OR_PANIC;
    size = get32(b + 4);
    p = 8;
  } else {
    return OR_PANIC;
  }
  if (size > 65536 || p + 4 * size > len) return OR_PANIC;
  const uint8_t *runflags = b + 4, *hdr = b + p;
  p += 4 * size;
  if (!hasrun || size >= RB_NO_OFFSET) p += 4 * size;
  if (p > len) return OR_PANIC;
  size_t total = 0;
  for (size_t k = 0; k < size; k++) total += get16(hdr + 4 * k + 2) + 1;
  uint32_t *rows = (uint32_t *)malloc((total ? total : 1) * 4);
  if (!rows) return OR_ENOMEM;
  size_t n = 0;
  int64_t prev = -1;
  for (size_t k = 0; k < size; k++) {
    const uint32_t key = get16(hdr + 4 * k), card = get16(hdr + 4 * k + 2) + 1;
    const int isrun = hasrun && ((runflags[k / 8] >> (k % 8)) & 1);
    size_t before = n;
    if (isrun) {
      if (p + 2 > len) goto bad;
      const uint32_t nr = get16(b + p);
      if (p + 2 + 4 * (size_t)nr > len) goto bad;
      for (uint32_t r = 0; r < nr; r++) {
        const uint32_t v0 = get16(b + p + 2 + 4 * r), l = get16(b + p + 4 + 4 * r);
        if (v0 + l > 0xFFFFu) goto bad;
        for (uint32_t v = v0; v <= v0 + l; v++) {
          if (n >= total) goto bad;
          rows[n++] = (key << 16) | v;
        }
      }
      p += 2 + 4 * (size_t)nr;
    } else if (card > RB_ARRAY_MAX) {
      if (p + 8192 > len) goto bad;
      for (uint32_t v = 0; v < 65536; v++)
        if ((b[p + v / 8] >> (v % 8)) & 1) {
          if (n >= total) goto bad;
          rows[n++] = (key << 16) | v;
        }
      p += 8192;
    } else {
      if (p + 2 * (size_t)card > len) goto bad;
      for (uint32_t i = 0; i < card; i++) rows[n++] = (key << 16) | get16(b + p + 2 * i);
      p += 2 * (size_t)card;
    }
    if (n - before != card) goto bad;
    for (size_t i = before; i < n; i++) {
      if ((int64_t)rows[i] <= prev) goto bad;
      prev = rows[i];
    }
  }
  *rows_out = rows;
  *cnt_out = n;
  return OR_OK;
bad:
  free(rows);
  return OR_PANIC;
}

/* ------------------------------------------------------------------ */
/* byte_residue_encode (split_double.rs:624-955)                       */
/* ------------------------------------------------------------------ */

static uint32_t clz64(uint64_t v) { return v ? (uint32_t)__builtin_clzll(v) : 64u; }

/* The shared tail of the encoder: every remaining full byte as a slice
 * (write_byte appends), then the packed low bits after a pad byte. */
static int write_dense(or_bw *w, const uint64_t *u, uint32_t n, uint32_t remain) {
  int rc = 0;
  while (remain >= 8) {
    remain -= 8;
    for (uint32_t i = 0; i < n; i++)
      rc |= or_bw_write_byte(w, remain > 0 ? (uint8_t)(u[i] >> remain) : (uint8_t)u[i]);
  }
  if (remain > 0) {
    rc |= or_bw_finish_write_byte(w);
    for (uint32_t i = 0; i < n && !rc; i++) rc |= or_bw_write_bits(w, (uint32_t)u[i], remain);
  }
  return rc;
}

int or_rapg_encode(const double *x, uint32_t n, uint64_t scale, uint8_t **out, size_t *out_len) {
  int prec = or_prec_of_scale(scale);
  int dl = or_dlen_of_prec(prec);
  if (dl < 0) return OR_PANIC; /* PRECISION_MAP.get(&prec).unwrap() */
  const int pexp = or_precision_exp(prec);
  const uint64_t dec_len = (uint64_t)dl;
  int64_t *fixed = (int64_t *)malloc((size_t)(n ? n : 1) * 8);
  uint64_t *u = (uint64_t *)malloc((size_t)(n ? n : 1) * 8);
  uint32_t *rows = (uint32_t *)malloc((size_t)(n ? n : 1) * 4);
  uint8_t *obytes = (uint8_t *)malloc(n ? n : 1);
  or_bw w;
  or_bw_init(&w);
  int rc = OR_OK;
  if (!fixed || !u || !rows || !obytes) {
    rc = OR_ENOMEM;
    goto done;
  }
  int64_t mn = INT64_MAX, mx = INT64_MIN;
  for (uint32_t i = 0; i < n; i++) { /* two ifs: the exact min and max (:643-652) */
    int64_t f = or_fetch_fixed_aligned(x[i], pexp, dec_len);
    if (f < mn) mn = f;
    if (f > mx) mx = f;
    fixed[i] = f;
  }
  const int64_t delta = (int64_t)((uint64_t)mx - (uint64_t)mn), base = mn;
  const uint32_t fl = delta == 0 ? 0u : or_fixed_len_of_delta(delta);
  const uint64_t ilen = (uint64_t)fl - dec_len; /* usize, wraps when fixed_len < dlen */
  for (uint32_t i = 0; i < n; i++) u[i] = (uint64_t)(fixed[i] - base);
  const uint64_t ub = (uint64_t)base;
  rc |= or_bw_write(&w, (uint32_t)ub, 32);
  rc |= or_bw_write(&w, (uint32_t)(ub >> 32), 32);
  rc |= or_bw_write(&w, n, 32);
  rc |= or_bw_write(&w, (uint32_t)ilen, 32);
  rc |= or_bw_write(&w, (uint32_t)dec_len, 32);
  if (rc) goto done;
  uint32_t remain = fl;
  if (ilen > 15) {
    if (n < RG_SAMPLE) { /* fixed_vec[0..SAMPLE] */
      rc = OR_PANIC;
      goto done;
    }
    /* leading-zero histogram of the first 2000 codes within fixed_len bits */
    const uint64_t head_len = 64u - fl;
    uint32_t bits_counter[32] = {0};
    for (uint32_t i = 0; i < RG_SAMPLE; i++) {
      const uint64_t lz = (uint64_t)clz64(u[i]) - head_len; /* usize, wraps */
      if (lz < 32) bits_counter[lz]++;
    }
    /* a leading byte is an outlier column while fewer than 200 sample codes
     * have a set bit in it or above (cumulative count, :703-716) */
    const uint32_t ol = (uint32_t)((float)RG_SAMPLE * RG_OUTLIER_R);
    const uint64_t adjusted = ilen / 8 * 8;
    uint32_t sum = 0, cols = 0;
    for (uint64_t i = 0; i < adjusted; i++) {
      if (i >= 32) { /* bits_counter[i]: index out of bounds */
        rc = OR_PANIC;
        goto done;
      }
      sum += bits_counter[i];
      if (i % 8 == 7) {
        if (sum < ol)
          cols++;
        else
          break;
      }
    }
    if (cols > 0) {
      rc |= or_bw_write(&w, cols, 8);
      for (uint32_t c = 0; c < cols && !rc; c++) {
        remain -= 8;
        uint32_t no = 0;
        for (uint32_t i = 0; i < n; i++) {
          const uint8_t b = (uint8_t)(u[i] >> remain);
          if (b != 0) {
            obytes[no] = b;
            rows[no++] = i;
          }
        }
        uint8_t *bm = NULL;
        size_t bm_len = 0;
        if ((rc = or_roaring_serialize(rows, no, &bm, &bm_len))) goto done;
        rc |= or_bw_write(&w, (uint32_t)bm_len, 32);
        rc |= or_bw_write_bytes(&w, bm, bm_len);
        rc |= or_bw_finish_write_byte(&w);
        rc |= or_bw_write(&w, no, 32);
        rc |= or_bw_write_bytes(&w, obytes, no);
        rc |= or_bw_finish_write_byte(&w);
        free(bm);
      }
      rc |= write_dense(&w, u, n, remain);
      goto done;
    }
    rc |= or_bw_write_byte(&w, 0); /* appended; the cursor stays before it */
  }
  if (remain < 8) {
    for (uint32_t i = 0; i < n && !rc; i++) rc |= or_bw_write_bits(&w, (uint32_t)u[i], remain);
  } else {
    rc |= write_dense(&w, u, n, remain);
  }
done:
  free(fixed);
  free(u);
  free(rows);
  free(obytes);
  if (rc) {
    or_bw_free(&w);
    return rc == OR_ENOMEM ? OR_ENOMEM : OR_PANIC;
  }
  *out = w.buf;
  *out_len = w.len;
  return OR_OK;
}

/* ------------------------------------------------------------------ */
/* decoders                                                            */
/* ------------------------------------------------------------------ */

typedef struct rg_head {
  int64_t base;
  uint32_t n, ilen, dlen, remain;
} rg_head;

/* Header and the number of bits to rebuild: all of them (precision < 0), or
 * the precision-limited count of :1642-1664 / :2439-2459. */
static int rg_header(or_br *br, int precision, rg_head *h) {
  uint32_t lo, hi;
  if (or_br_read(br, 32, &lo) || or_br_read(br, 32, &hi) || or_br_read(br, 32, &h->n) ||
      or_br_read(br, 32, &h->ilen) || or_br_read(br, 32, &h->dlen))
    return OR_PANIC;
  h->base = (int64_t)((uint64_t)lo | ((uint64_t)hi << 32));
  const uint32_t ilen = h->ilen, dlen = h->dlen;
  h->remain = dlen + ilen;
  if (precision == 0) {
    uint32_t bn = ilen / 8;
    h->remain = ilen;
    if (ilen % 8 > 0) {
      bn += 1;
      h->remain = bn * 8;
    }
  } else if (precision > 0) {
    const int need = or_dlen_of_prec(precision);
    if (need < 0) return OR_PANIC;               /* PRECISION_MAP unwrap */
    if (dlen < (uint32_t)need) return OR_PANIC;  /* assert!(dlen >= bits_needed) */
    h->remain = ilen + (uint32_t)need;
    const uint32_t fixed_byte = (dlen + ilen) / 8;
    uint32_t bn = (ilen + (uint32_t)need) / 8;
    const uint32_t extra = (ilen + (uint32_t)need) % 8;
    if (bn < fixed_byte && extra > 0) {
      bn += 1;
      h->remain = bn * 8;
    }
  }
  return OR_OK;
}

static double rg_value(int64_t base, uint64_t v, double scl) {
  return (double)(int64_t)((uint64_t)base + v) / scl;
}

/* 2.0f64.powi(e) */
static double rg_powi2(int32_t e) {
  if (e >= 1024) return INFINITY;
  if (e <= -1024) return 0.0;
  return ldexp(1.0, e);
}

/* The dense part of a decode (:1427-1460 and :1497-1545): slices while
 * remain >= 8, values emitted at the slice that ends the code, else the
 * packed low `remain` bits after a pad byte.  `fixed` may be NULL (no
 * outlier columns: the codes start at the first slice). */
static int rg_decode_dense(or_br *br, const rg_head *h, uint32_t remain, uint64_t *fixed,
                           double *out, size_t *k) {
  const double scl = ldexp(1.0, (int)h->dlen);
  const uint32_t n = h->n;
  while (remain >= 8) {
    remain -= 8;
    const uint8_t *chunk;
    if (or_br_read_n_byte(br, n, &chunk)) return OR_PANIC;
    if (remain == 0) {
      for (uint32_t i = 0; i < n; i++) out[(*k)++] = rg_value(h->base, fixed[i] | chunk[i], scl);
    } else {
      for (uint32_t i = 0; i < n; i++) fixed[i] |= (uint64_t)chunk[i] << (remain & 63);
    }
  }
  if (remain > 0) {
    or_br_finish_read_byte(br);
    for (uint32_t i = 0; i < n; i++) {
      uint8_t t;
      if (or_br_read_bits(br, remain, &t)) return OR_PANIC;
      out[(*k)++] = rg_value(h->base, fixed[i] | t, scl);
    }
  }
  return OR_OK;
}

int or_rapg_decode(const uint8_t *bytes, size_t len, uint64_t scale, int precision, double *out,
                   size_t *nout) {
  (void)scale;
  or_br br;
  or_br_init(&br, bytes, len);
  rg_head h;
  *nout = 0;
  if (rg_header(&br, precision, &h)) return OR_PANIC;
  const double scl = ldexp(1.0, (int)h.dlen);
  uint32_t remain = h.remain;
  size_t k = 0;
  int rc = OR_OK;
  uint64_t *fixed = (uint64_t *)calloc(h.n ? h.n : 1, 8);
  if (!fixed) return OR_ENOMEM;
  if (h.ilen > 15) {
    uint32_t cols;
    if (or_br_read(&br, 8, &cols)) {
      rc = OR_PANIC;
      goto done;
    }
    if (cols > 0) {
      for (uint32_t c = 0; c < cols; c++) {
        remain -= 8;
        uint32_t bm_len, no;
        const uint8_t *bm, *outs;
        uint32_t *rows = NULL;
        size_t nrows = 0;
        if (or_br_read(&br, 32, &bm_len) || or_br_read_n_byte(&br, bm_len, &bm) ||
            or_roaring_parse(bm, bm_len, &rows, &nrows)) {
          rc = OR_PANIC;
          goto done;
        }
        or_br_finish_read_byte(&br);
        if (or_br_read(&br, 32, &no) || or_br_read_n_byte(&br, no, &outs) || no == 0 ||
            nrows == 0) { /* outlier_iter / bm_iterator .next().unwrap() */
          free(rows);
          rc = OR_PANIC;
          goto done;
        }
        size_t ri = 0, oi = 0, counter = 0;
        for (uint32_t i = 0; i < h.n; i++) {
          if (i == rows[ri]) {
            fixed[i] |= (uint64_t)outs[oi] << (remain & 63);
            if (++counter == no) break;
            if (++ri >= nrows || ++oi >= no) {
              free(rows);
              rc = OR_PANIC;
              goto done;
            }
          }
        }
        free(rows);
        or_br_finish_read_byte(&br);
      }
      rc = rg_decode_dense(&br, &h, remain, fixed, out, &k);
      goto done;
    }
  }
  if (remain < 8) {
    for (uint32_t i = 0; i < h.n; i++) {
      uint8_t t;
      if (or_br_read_bits(&br, remain, &t)) {
        rc = OR_PANIC;
        goto done;
      }
      out[k++] = rg_value(h.base, t, scl);
    }
  } else {
    rc = rg_decode_dense(&br, &h, remain, fixed, out, &k);
  }
done:
  free(fixed);
  if (rc) return rc;
  *nout = k;
  return OR_OK;
}

int or_rapg_sum(const uint8_t *bytes, size_t len, uint64_t scale, int precision, double *sum_out) {
  (void)scale;
  or_br br;
  or_br_init(&br, bytes, len);
  rg_head h;
  if (rg_header(&br, precision, &h)) return OR_PANIC;
  uint32_t remain = h.remain;
  int32_t processed = 0;
  const int32_t ilen = (int32_t)h.ilen;
  const double sum_base = ((double)h.n * (double)h.base) / ldexp(1.0, (int)h.dlen);
  double sum = 0.0;
  if (h.ilen > 15) {
    uint32_t cols;
    if (or_br_read(&br, 8, &cols)) return OR_PANIC;
    for (uint32_t c = 0; c < cols; c++) {
      remain -= 8;
      processed += 8;
      uint32_t bm_len, no;
      const uint8_t *bm, *outs;
      if (or_br_read(&br, 32, &bm_len) || or_br_read_n_byte(&br, bm_len, &bm)) return OR_PANIC;
      or_br_finish_read_byte(&br);
      if (or_br_read(&br, 32, &no) || or_br_read_n_byte(&br, no, &outs)) return OR_PANIC;
      uint64_t sf = 0;
      for (uint32_t i = 0; i < no; i++) sf += outs[i];
      sum = sum + (double)sf / rg_powi2(processed - ilen);
      or_br_finish_read_byte(&br);
    }
  }
  while (remain >= 8) {
    remain -= 8;
    processed += 8;
    const uint8_t *chunk;
    if (or_br_read_n_byte(&br, h.n, &chunk)) return OR_PANIC;
    uint64_t sf = 0;
    for (uint32_t i = 0; i < h.n; i++) sf += chunk[i];
    sum = sum + (double)sf / rg_powi2(processed - ilen);
    if (remain == 0) { /* returns before the base term */
      *sum_out = sum;
      return OR_OK;
    }
  }
  if (remain > 0) {
    if (processed >= 8) or_br_finish_read_byte(&br);
    processed += (int32_t)remain;
    uint64_t sf = 0;
    for (uint32_t i = 0; i < h.n; i++) {
      uint8_t t;
      if (or_br_read_bits(&br, remain, &t)) return OR_PANIC;
      sf += t;
    }
    sum = sum + (double)sf / rg_powi2(processed - ilen);
  }
  sum += sum_base;
  *sum_out = sum;
  return OR_OK;
}

/* The outlier-column directory of an image: column count (0 when the image
 * has none or no count byte), and per column the bitmap size, the outlier
 * count and the byte offset of the bitmap. */
int or_rapg_layout(const uint8_t *bytes, size_t len, uint32_t *ncols, uint32_t *bm_sizes,
                   uint32_t *nouts, uint64_t *bm_offs) {
  or_br br;
  or_br_init(&br, bytes, len);
  rg_head h;
  *ncols = 0;
  if (rg_header(&br, -1, &h)) return OR_PANIC;
  if (h.ilen <= 15) return OR_OK;
  uint32_t cols;
  if (or_br_read(&br, 8, &cols)) return OR_PANIC;
  for (uint32_t c = 0; c < cols; c++) {
    uint32_t bm_len, no;
    const uint8_t *bm, *outs;
    if (or_br_read(&br, 32, &bm_len) || or_br_read_n_byte(&br, bm_len, &bm)) return OR_PANIC;
    or_br_finish_read_byte(&br);
    if (or_br_read(&br, 32, &no) || or_br_read_n_byte(&br, no, &outs)) return OR_PANIC;
    or_br_finish_read_byte(&br);
    if (c < 8) {
      bm_sizes[c] = bm_len;
      nouts[c] = no;
      bm_offs[c] = (uint64_t)(bm - bytes);
    }
  }
  *ncols = cols;
  return OR_OK;
}
