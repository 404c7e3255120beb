/*
 * CPU oracle for the BUFF buff-simd hot path.  TEST INFRASTRUCTURE ONLY:
 * only tests/, the smoke check and the benchmark's CPU-baseline leg load it.
 *
 * A plain-C restatement of the reference algorithm (Tranway1/buff); each
 * function cites the reference file:line it follows.  Integer behaviour of the
 * reference's release build is kept: i64/u32 arithmetic wraps, shift amounts
 * are masked to the operand width, f64->int casts saturate.
 *
 * Pinning: checked against every known-answer test the reference carries for
 * this path (BitPack, BitVec serialization, BVIter order, the movemask lane
 * order; tests/test_oracle_golden.py).  The codec outputs themselves (encoded
 * bytes, bitmaps, sums, maxima, precision decodes) are parity unpinned: no
 * reference test or recorded output asserts them, and the reference (a Rust
 * crate) cannot be built here; they are cross-checked against an independent
 * numpy statement (tests/model.py).
 */
#include "buff_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define EXP_MASK 0x7FF0000000000000ull
#define FIRST_ONE 0x8000000000000000ull
#define SIMD_THRESHOLD 0.06 /* compress/buff_simd.rs:26 */

/* ------------------------------------------------------------------ */
/* scalar helpers                                                      */
/* ------------------------------------------------------------------ */

/* `(scale as f32).log10() as i32` (compress/buff_simd.rs:3127). */
int or_prec_of_scale(uint64_t scale) {
  if (scale == 0) return 0; /* buff_simd.rs:3123-3125 */
  float f = (float)scale;
  float l = log10f(f);
  if (isnan(l)) return 0;
  if (l >= 2147483647.0f) return 2147483647;
  if (l <= -2147483648.0f) return (-2147483647 - 1);
  return (int)l; /* truncation toward zero, like `as i32` */
}

/* PRECISION_MAP (compress/mod.rs:29-46). */
int or_dlen_of_prec(int prec) {
  static const int map[16] = {-1, 5, 8, 11, 15, 18, 21, 25, 28, 31, 35, 38, 50, 10, 10, 10};
  if (prec < 1 || prec > 15) return -1;
  return map[prec];
}

/* get_precision_bound (methods/prec_double.rs:273-281) parsed to f64, then
 * PrecisionBound::new (prec_double.rs:28-33) keeps its unbiased exponent. */
int or_precision_exp(int prec) {
  char buf[64];
  int p = 0;
  buf[p++] = '0';
  buf[p++] = '.';
  for (int i = 0; i < prec && p < 60; i++) buf[p++] = '0';
  buf[p++] = '4';
  buf[p++] = '9';
  buf[p] = 0;
  double d = strtod(buf, NULL);
  uint64_t u;
  memcpy(&u, &d, 8);
  return (int)((u & EXP_MASK) >> 52) - 1023;
}

/* PrecisionBound::fetch_fixed_aligned (methods/prec_double.rs:190-205). */
int64_t or_fetch_fixed_aligned(double v, int32_t precision_exp, uint64_t dlen) {
  uint64_t bdu;
  memcpy(&bdu, &v, 8);
  int32_t exp = (int32_t)((bdu & EXP_MASK) >> 52) - 1023;
  uint64_t sign = bdu & FIRST_ONE;
  uint64_t fixed;
  if (exp < precision_exp) {
    fixed = 0;
  } else {
    int32_t sh = 63 - exp - (int32_t)dlen;
    fixed = ((bdu << 11) | FIRST_ONE) >> ((uint64_t)(int64_t)sh & 63u);
    if (sign) fixed = ~(fixed - 1u);
  }
  return (int64_t)fixed;
}

/* `(delta as f64).log2().ceil() as usize` (compress/buff_simd.rs:3156-3161). */
uint32_t or_fixed_len_of_delta(int64_t delta) {
  double c = ceil(log2((double)delta));
  if (isnan(c) || c <= 0.0) return 0;
  if (c >= 4294967295.0) return 0xFFFFFFFFu;
  return (uint32_t)c;
}

static inline uint8_t flip(uint8_t x) { return x ^ 0x80u; } /* buff_slice.rs:174-177 */

/* ------------------------------------------------------------------ */
/* BitPack writer (methods/bit_packing.rs:56-139, 286-388)             */
/* ------------------------------------------------------------------ */

void or_bw_init(or_bw *w) { memset(w, 0, sizeof(*w)); }
void or_bw_free(or_bw *w) {
  free(w->buf);
  memset(w, 0, sizeof(*w));
}

static int bw_resize(or_bw *w, size_t nlen) {
  if (nlen > w->cap) {
    size_t ncap = w->cap ? w->cap : 64;
    while (ncap < nlen) ncap *= 2;
    uint8_t *nb = (uint8_t *)realloc(w->buf, ncap);
    if (!nb) {
      w->oom = 1;
      return OR_ENOMEM;
    }
    w->buf = nb;
    w->cap = ncap;
  }
  if (nlen > w->len) memset(w->buf + w->len, 0, nlen - w->len);
  w->len = nlen;
  return OR_OK;
}

/* Vec-backed write/write_bits grow the buffer, then run the slice writer
 * (bit_packing.rs:316-338, 343-365 wrapping :72-101, :106-135). */
static int bw_write_impl(or_bw *w, uint32_t value, unsigned bits, int is_write) {
  size_t need = w->cursor * 8 + w->bits + bits;
  if (need > w->len * 8) {
    size_t extra = need - w->len * 8;
    if (bw_resize(w, w->len + (extra + 7) / 8)) return OR_ENOMEM;
  }
  if (is_write && bits > 32) return OR_PANIC;
  if (w->len * 8 < w->cursor * 8 + w->bits + bits) return OR_PANIC;
  if (is_write) {
    if (bits < 32) value &= (uint32_t)((1ull << bits) - 1);
  } else {
    value &= (uint32_t)((1ull << bits) - 1);
  }
  for (;;) {
    unsigned bits_left = 8 - w->bits;
    if (bits <= bits_left) {
      if (w->cursor >= w->len) return OR_PANIC; /* index out of bounds */
      w->buf[w->cursor] |= (uint8_t)((uint8_t)value << w->bits);
      w->bits += bits;
      if (w->bits >= 8) {
        w->cursor += 1;
        w->bits = 0;
      }
      break;
    }
    uint32_t bb = value & (uint32_t)((1u << bits_left) - 1);
    if (w->cursor >= w->len) return OR_PANIC;
    w->buf[w->cursor] |= (uint8_t)((uint8_t)bb << w->bits);
    w->cursor += 1;
    w->bits = 0;
    value >>= bits_left;
    bits -= bits_left;
  }
  return OR_OK;
}

int or_bw_write(or_bw *w, uint32_t value, unsigned bits) { return bw_write_impl(w, value, bits, 1); }
int or_bw_write_bits(or_bw *w, uint32_t value, unsigned bits) {
  return bw_write_impl(w, value, bits, 0);
}
/* write_byte appends without moving the cursor (bit_packing.rs:374-377). */
int or_bw_write_byte(or_bw *w, uint8_t v) {
  size_t l = w->len;
  if (bw_resize(w, l + 1)) return OR_ENOMEM;
  w->buf[l] = v;
  return OR_OK;
}
int or_bw_write_bytes(or_bw *w, const uint8_t *v, size_t n) {
  size_t l = w->len;
  if (bw_resize(w, l + n)) return OR_ENOMEM;
  if (n) memcpy(w->buf + l, v, n);
  return OR_OK;
}
/* finish_write_byte appends one zero byte and moves the cursor onto it
 * (bit_packing.rs:380-386). */
int or_bw_finish_write_byte(or_bw *w) {
  size_t l = w->len;
  if (bw_resize(w, l + 1)) return OR_ENOMEM;
  w->bits = 0;
  w->cursor = l;
  return OR_OK;
}

/* ------------------------------------------------------------------ */
/* BitPack reader (methods/bit_packing.rs:142-284)                     */
/* The cursor points at the last consumed byte once a byte is finished. */
/* ------------------------------------------------------------------ */

void or_br_init(or_br *r, const uint8_t *buf, size_t len) {
  r->buf = buf;
  r->len = len;
  r->cursor = 0;
  r->bits = 0;
}

static int br_read_impl(or_br *r, unsigned bits, uint32_t *out, int is_read) {
  if ((is_read && bits > 32) || r->len * 8 < r->cursor * 8 + r->bits + bits) return OR_PANIC;
  uint32_t bits_left = 0, output = 0;
  for (;;) {
    unsigned byte_left = 8 - r->bits;
    if (bits <= byte_left) {
      if (r->cursor >= r->len) return OR_PANIC;
      uint32_t bb = r->buf[r->cursor];
      bb >>= r->bits;
      bb &= (uint32_t)((1u << bits) - 1);
      output |= bb << bits_left;
      r->bits += bits;
      break;
    }
    if (r->cursor >= r->len) return OR_PANIC;
    uint32_t bb = r->buf[r->cursor];
    bb >>= r->bits;
    bb &= (uint32_t)((1u << byte_left) - 1);
    output |= bb << bits_left;
    r->bits += byte_left;
    bits_left += byte_left;
    bits -= byte_left;
    if (r->bits >= 8) {
      r->cursor += 1;
      r->bits -= 8;
    }
  }
  *out = output;
  return OR_OK;
}

int or_br_read(or_br *r, unsigned bits, uint32_t *out) { return br_read_impl(r, bits, out, 1); }
int or_br_read_bits(or_br *r, unsigned bits, uint8_t *out) {
  uint32_t v = 0;
  int rc = br_read_impl(r, bits, &v, 0);
  *out = (uint8_t)v;
  return rc;
}
void or_br_finish_read_byte(or_br *r) {
  r->cursor += 1;
  r->bits = 0;
}
int or_br_read_byte(or_br *r, uint8_t *out) {
  r->cursor += 1;
  if (r->cursor >= r->len) return OR_PANIC;
  *out = r->buf[r->cursor];
  return OR_OK;
}
int or_br_read_n_byte(or_br *r, size_t n, const uint8_t **out) {
  r->cursor += 1;
  size_t end = r->cursor + n;
  if (end > r->len || end < r->cursor) return OR_PANIC;
  *out = r->buf + r->cursor;
  r->cursor += n - 1; /* wraps for n == 0 exactly as the release build */
  return OR_OK;
}
void or_br_skip_n_byte(or_br *r, size_t n) { r->cursor += n; }
int or_br_skip(or_br *r, size_t bits) {
  if (r->len * 8 < r->cursor * 8 + r->bits + bits) return OR_PANIC; /* Err: cursor unchanged */
  size_t bytes = bits / 8, left = bits % 8;
  size_t cur_bits = r->bits + left;
  r->cursor = r->cursor + bytes + cur_bits / 8;
  r->bits = (unsigned)(cur_bits % 8);
  return OR_OK;
}

int or_bitpack_write_seq(const uint32_t *values, const uint32_t *bits, size_t cnt, uint8_t *out,
                         size_t cap, size_t *len) {
  or_bw w;
  or_bw_init(&w);
  for (size_t i = 0; i < cnt; i++) {
    int rc = or_bw_write(&w, values[i], bits[i]);
    if (rc) {
      or_bw_free(&w);
      return rc;
    }
  }
  *len = w.len;
  if (w.len > cap) {
    or_bw_free(&w);
    return OR_EINVAL;
  }
  if (w.len) memcpy(out, w.buf, w.len);
  or_bw_free(&w);
  return OR_OK;
}

int or_bitpack_read_seq(const uint8_t *buf, size_t len, const uint32_t *bits, size_t cnt,
                        uint32_t *values) {
  or_br r;
  or_br_init(&r, buf, len);
  for (size_t i = 0; i < cnt; i++) {
    int rc = or_br_read(&r, bits[i], &values[i]);
    if (rc) return rc;
  }
  return OR_OK;
}

/* ------------------------------------------------------------------ */
/* BitVec<u32> helpers (bit-vec/src/lib.rs) and BVIter                 */
/* ------------------------------------------------------------------ */

static inline size_t nwords_for(uint64_t nbits) { return (size_t)((nbits + 31) / 32); }
static inline void bv_set(uint32_t *w, size_t i) { w[i >> 5] |= 1u << (i & 31); }
static uint64_t bv_card(const uint32_t *w, size_t nw) {
  uint64_t c = 0;
  for (size_t i = 0; i < nw; i++) c += (uint64_t)__builtin_popcount(w[i]);
  return c;
}
static void bv_fix_last(uint32_t *w, uint64_t nbits) { /* fix_last_block lib.rs:537-543 */
  size_t nw = nwords_for(nbits);
  if (nw && (nbits & 31)) w[nw - 1] &= (1u << (nbits & 31)) - 1u;
}

size_t or_bviter_positions(const uint32_t *words, size_t nwords, uint64_t *out, size_t cap) {
  /* BVIter::next (query/bit_vec_iter.rs:35-47) */
  size_t cnt = 0;
  if (nwords == 0) return 0;
  size_t pointer = 0;
  uint32_t cached = words[0];
  for (;;) {
    while (cached == 0) {
      if (pointer == nwords - 1) return cnt;
      pointer += 1;
      cached = words[pointer];
    }
    uint32_t t = cached & ~(cached - 1u);
    cached ^= t;
    uint64_t res = ((uint64_t)pointer << 5) + (uint64_t)__builtin_popcount(t - 1u);
    if (cnt < cap) out[cnt] = res;
    cnt++;
  }
}

size_t or_bitvec_to_binary(const uint32_t *words, size_t nwords, uint64_t nbits, uint8_t *out) {
  /* to_binary: u64 LE nbits then u32 LE words (bit-vec lib.rs:399-406) */
  for (int i = 0; i < 8; i++) out[i] = (uint8_t)(nbits >> (8 * i));
  for (size_t j = 0; j < nwords; j++)
    for (int i = 0; i < 4; i++) out[8 + 4 * j + i] = (uint8_t)(words[j] >> (8 * i));
  return 8 + 4 * nwords;
}

/* 32-byte signed compare + movemask, the AVX2 block of range_simd_mybitvec /
 * equal_simd_mybitvec (simd/vectorize_query.rs:168-222), written with
 * portable 32-byte vectors.  Bit b of the mask is lane b. */
typedef int8_t v32i8 __attribute__((vector_size(32)));
static inline uint32_t mm8(uint64_t x) {
  return (uint32_t)(((x & 0x8080808080808080ull) * 0x0002040810204081ull) >> 56);
}
static inline void cmp32(const uint8_t *p, int8_t predicate, uint32_t *gt, uint32_t *eq) {
  v32i8 w, pv;
  memcpy(&w, p, 32);
  for (int i = 0; i < 32; i++) pv[i] = predicate;
  v32i8 g = (v32i8)(w > pv);
  v32i8 e = (v32i8)(w == pv);
  uint64_t gw[4], ew[4];
  memcpy(gw, &g, 32);
  memcpy(ew, &e, 32);
  if (gt) *gt = mm8(gw[0]) | (mm8(gw[1]) << 8) | (mm8(gw[2]) << 16) | (mm8(gw[3]) << 24);
  if (eq) *eq = mm8(ew[0]) | (mm8(ew[1]) << 8) | (mm8(ew[2]) << 16) | (mm8(ew[3]) << 24);
}
uint32_t or_movemask_gt(const uint8_t *bytes32, uint8_t pred) {
  uint32_t g;
  cmp32(bytes32, (int8_t)flip(pred), &g, NULL);
  return g;
}
uint32_t or_movemask_eq(const uint8_t *bytes32, uint8_t pred) {
  uint32_t e;
  cmp32(bytes32, (int8_t)flip(pred), NULL, &e);
  return e;
}

/* range_simd_mybitvec (vectorize_query.rs:168-195): gt words go to res via
 * set_storage (only the first floor(n/32) words); returns eq words padded
 * with zero words (BitVec::from_vec, lib.rs:362-373). */
static void range_simd(const uint8_t *x, size_t len, uint32_t *res, uint32_t *eqw, uint8_t pred) {
  int8_t predicate = (int8_t)flip(pred);
  size_t nblk = len / 32, nw = nwords_for(len);
  for (size_t b = 0; b < nblk; b++) cmp32(x + 32 * b, predicate, &res[b], &eqw[b]);
  for (size_t b = nblk; b < nw; b++) eqw[b] = 0;
}
static void equal_simd(const uint8_t *x, size_t len, uint32_t *eqw, uint8_t pred) {
  int8_t predicate = (int8_t)flip(pred);
  size_t nblk = len / 32, nw = nwords_for(len);
  for (size_t b = 0; b < nblk; b++) cmp32(x + 32 * b, predicate, NULL, &eqw[b]);
  for (size_t b = nblk; b < nw; b++) eqw[b] = 0;
}

/* ------------------------------------------------------------------ */
/* encode: buff_simd256_encode (compress/buff_simd.rs:3116-3250) and    */
/* byte_fixed_encode (compress/split_double.rs:298-432)                 */
/* ------------------------------------------------------------------ */

void or_free(void *p) { free(p); }

int or_encode(const double *x, uint32_t n, uint64_t scale, int flipped, unsigned flags,
              uint8_t **out, size_t *out_len) {
  int prec = or_prec_of_scale(scale);
  int dl = or_dlen_of_prec(prec);
  if (dl < 0) return OR_PANIC; /* PRECISION_MAP.get(&prec).unwrap() */
  int pexp = or_precision_exp(prec);
  uint64_t dec_len = (uint64_t)dl;
  int64_t *fixed = (int64_t *)malloc((size_t)(n ? n : 1) * sizeof(int64_t));
  if (!fixed) return OR_ENOMEM;
  int64_t mn = INT64_MAX, mx = INT64_MIN;
  for (uint32_t i = 0; i < n; i++) {
    int64_t f = or_fetch_fixed_aligned(x[i], pexp, dec_len);
    if (flags & OR_INTENDED) {
      if (f < mn) mn = f;
      if (f > mx) mx = f;
    } else {
      /* buff_simd.rs:3139-3148: `else if` -- the first row never updates max */
      if (f < mn)
        mn = f;
      else if (f > mx)
        mx = f;
    }
    fixed[i] = f;
  }
  int64_t delta = (int64_t)((uint64_t)mx - (uint64_t)mn);
  int64_t base = mn;
  uint32_t fixed_len;
  if (flags & OR_INTENDED) {
    fixed_len = (n == 0 || delta == 0) ? 0u : (uint32_t)(64 - __builtin_clzll((uint64_t)delta));
  } else {
    fixed_len = delta == 0 ? 0u : or_fixed_len_of_delta(delta);
  }
  uint64_t ilen = (uint64_t)fixed_len - dec_len; /* usize wrap */
  or_bw w;
  or_bw_init(&w);
  uint64_t ub = (uint64_t)base;
  int rc = 0;
  rc |= or_bw_write(&w, (uint32_t)ub, 32);
  rc |= or_bw_write(&w, (uint32_t)(ub >> 32), 32);
  rc |= or_bw_write(&w, n, 32);
  rc |= or_bw_write(&w, (uint32_t)ilen, 32);
  rc |= or_bw_write(&w, (uint32_t)dec_len, 32);
  if (rc) goto fail;
  uint32_t remain = fixed_len;
  if (remain < 8) {
    if (!(remain == 0 && (flags & OR_INTENDED))) {
      for (uint32_t i = 0; i < n; i++) {
        rc = or_bw_write_bits(&w, (uint32_t)(uint64_t)(fixed[i] - base), remain);
        if (rc) goto fail;
      }
    }
  } else {
    uint8_t fx = flipped ? 0x80u : 0u;
    remain -= 8;
    /* first slice (:3181-3199) */
    size_t l0 = w.len;
    if (bw_resize(&w, l0 + n)) {
      rc = OR_ENOMEM;
      goto fail;
    }
    for (uint32_t i = 0; i < n; i++) {
      uint64_t c = (uint64_t)(fixed[i] - base);
      w.buf[l0 + i] = (uint8_t)(c >> remain) ^ fx;
    }
    while (remain >= 8) { /* :3202-3219 */
      remain -= 8;
      size_t l = w.len;
      if (bw_resize(&w, l + n)) {
        rc = OR_ENOMEM;
        goto fail;
      }
      for (uint32_t i = 0; i < n; i++) {
        uint64_t c = (uint64_t)(fixed[i] - base);
        w.buf[l + i] = (uint8_t)(c >> remain) ^ fx;
      }
    }
    if (remain > 0) { /* :3220-3226 */
      if ((rc = or_bw_finish_write_byte(&w))) goto fail;
      for (uint32_t i = 0; i < n; i++) {
        rc = or_bw_write_bits(&w, (uint32_t)(uint64_t)(fixed[i] - base), remain);
        if (rc) goto fail;
      }
    }
  }
  free(fixed);
  *out = w.buf;
  *out_len = w.len;
  return OR_OK;
fail:
  free(fixed);
  or_bw_free(&w);
  return rc;
}

int or_encode_f32(const float *x, uint32_t n, uint64_t scale, int flipped, unsigned flags,
                  uint8_t **out, size_t *out_len) {
  /* T: Into<f64> widens exactly (buff_simd.rs:3117) */
  double *d = (double *)malloc((size_t)(n ? n : 1) * sizeof(double));
  if (!d) return OR_ENOMEM;
  for (uint32_t i = 0; i < n; i++) d[i] = (double)x[i];
  int rc = or_encode(d, n, scale, flipped, flags, out, out_len);
  free(d);
  return rc;
}

/* Header parse (buff_simd.rs:3257-3268): 5 x read(32). */
static int parse_header_r(or_br *br, or_header *h) {
  uint32_t lo, hi, len, ilen, dlen;
  if (or_br_read(br, 32, &lo) || or_br_read(br, 32, &hi) || or_br_read(br, 32, &len) ||
      or_br_read(br, 32, &ilen) || or_br_read(br, 32, &dlen))
    return OR_PANIC;
  h->base = (int64_t)((uint64_t)lo | ((uint64_t)hi << 32));
  h->n = len;
  h->ilen = ilen;
  h->dlen = dlen;
  h->fixed_len = dlen + ilen;
  if (h->fixed_len < 8) {
    h->k = 0;
    h->r = h->fixed_len;
    h->slice_off = 20;
    h->tail_off = 20;
  } else {
    h->k = h->fixed_len / 8;
    h->r = h->fixed_len % 8;
    h->slice_off = 20;
    h->tail_off = 20 + (size_t)h->k * h->n;
  }
  return OR_OK;
}

int or_parse_header(const uint8_t *bytes, size_t len, or_header *h) {
  or_br br;
  or_br_init(&br, bytes, len);
  return parse_header_r(&br, h);
}

static inline int64_t wadd(int64_t a, uint64_t b) { return (int64_t)((uint64_t)a + b); }

/* Stored code of every row, rebuilt from the slice/tail offsets of the
 * serialized layout (buff_simd.rs:3181-3232). */
static int codes_of(const uint8_t *bytes, size_t len, const or_header *h, int flipped,
                    uint64_t *codes) {
  uint8_t fx = flipped ? 0x80u : 0u;
  if (h->tail_off + ((uint64_t)h->n * h->r + 7) / 8 > len) return OR_PANIC;
  for (uint32_t i = 0; i < h->n; i++) {
    uint64_t c = 0;
    for (uint32_t j = 0; j < h->k; j++)
      c = (c << 8) | (uint8_t)(bytes[h->slice_off + (size_t)j * h->n + i] ^ fx);
    if (h->r) {
      uint64_t bit = (uint64_t)i * h->r;
      uint32_t v = 0;
      for (uint32_t b = 0; b < h->r; b++) {
        uint64_t p = bit + b;
        v |= (uint32_t)((bytes[h->tail_off + p / 8] >> (p % 8)) & 1u) << b;
      }
      c = (c << h->r) | v;
    }
    codes[i] = c;
  }
  return OR_OK;
}

/* ------------------------------------------------------------------ */
/* decode: buff_simd256_decode (buff_simd.rs:3252-3357) and             */
/* byte_fixed_decode (split_double.rs:1243-1350)                        */
/* ------------------------------------------------------------------ */

/* Shared slice walk of the decoders with `total` bits to rebuild
 * (split_double.rs:1700-1744 / 1818-1887): leading byte slices, then
 * `total % 8` packed bits per row read right after them. */
static int decode_bits(or_br *br, const or_header *h, uint32_t total, int flipped, double *out) {
  double dec_scl = ldexp(1.0, (int)h->dlen); /* 2.0f64.powi(dlen as i32) */
  uint32_t n = h->n, remain = total;
  uint8_t fx = flipped ? 0x80u : 0u;
  if (remain < 8) {
    for (uint32_t i = 0; i < n; i++) {
      uint8_t cur;
      if (or_br_read_bits(br, remain, &cur)) return OR_PANIC;
      out[i] = (double)wadd(h->base, (uint64_t)cur) / dec_scl;
    }
    return OR_OK;
  }
  uint64_t *fv = (uint64_t *)calloc(n ? n : 1, sizeof(uint64_t));
  if (!fv) return OR_ENOMEM;
  const uint8_t *chunk;
  remain -= 8;
  if (or_br_read_n_byte(br, n, &chunk)) goto panic;
  if (remain == 0) {
    for (uint32_t i = 0; i < n; i++) out[i] = (double)wadd(h->base, (uint64_t)(chunk[i] ^ fx)) / dec_scl;
    free(fv);
    return OR_OK;
  }
  for (uint32_t i = 0; i < n; i++) fv[i] = (uint64_t)(chunk[i] ^ fx) << remain;
  while (remain >= 8) {
    remain -= 8;
    if (or_br_read_n_byte(br, n, &chunk)) goto panic;
    if (remain == 0) {
      for (uint32_t i = 0; i < n; i++)
        out[i] = (double)wadd(h->base, fv[i] | (uint64_t)(chunk[i] ^ fx)) / dec_scl;
      free(fv);
      return OR_OK;
    }
    for (uint32_t i = 0; i < n; i++) fv[i] |= (uint64_t)(chunk[i] ^ fx) << remain;
  }
  if (remain > 0) {
    or_br_finish_read_byte(br);
    for (uint32_t i = 0; i < n; i++) {
      uint8_t b;
      if (or_br_read_bits(br, remain, &b)) goto panic;
      out[i] = (double)wadd(h->base, fv[i] | (uint64_t)b) / dec_scl;
    }
  }
  free(fv);
  return OR_OK;
panic:
  free(fv);
  return OR_PANIC;
}

int or_decode(const uint8_t *bytes, size_t len, uint64_t scale, int flipped, double *out) {
  (void)scale; /* the bound is built but unused by the decoder */
  or_br br;
  or_br_init(&br, bytes, len);
  or_header h;
  if (parse_header_r(&br, &h)) return OR_PANIC;
  return decode_bits(&br, &h, h.fixed_len, flipped, out);
}

/* ------------------------------------------------------------------ */
/* filters: buff_simd_range_filter (buff_simd.rs:3361-3547) and         */
/* buff_simd_equal_filter (buff_simd.rs:3549-3733)                      */
/* ------------------------------------------------------------------ */

/* Predicate target in code space; returns 1 for the early return
 * `fixed_part < base_int` (:3384-3389 / :3572-3577). */
static int filter_target(const or_header *h, uint64_t scale, double pred, uint64_t *t) {
  int prec = or_prec_of_scale(scale);
  int pexp = or_precision_exp(prec);
  int64_t fixed_part = or_fetch_fixed_aligned(pred, pexp, h->dlen);
  if (fixed_part < h->base) return 1;
  *t = (uint64_t)(fixed_part - h->base);
  return 0;
}

/* INTENDED semantics of both filters: direct compare of the stored code
 * against the full target on every row. */
static int filter_intended(const uint8_t *bytes, size_t len, const or_header *h, uint64_t t,
                           int is_range, uint32_t *words) {
  double *tmp = NULL;
  (void)tmp;
  size_t nw = nwords_for(h->n);
  memset(words, 0, nw * 4);
  uint32_t fl = h->fixed_len;
  if ((uint64_t)h->tail_off + ((uint64_t)h->n * h->r + 7) / 8 > len) return OR_PANIC;
  for (uint32_t i = 0; i < h->n; i++) {
    uint64_t c = 0;
    for (uint32_t j = 0; j < h->k; j++) c = (c << 8) | (uint8_t)(bytes[h->slice_off + (size_t)j * h->n + i] ^ 0x80u);
    if (h->r) {
      uint64_t bit = (uint64_t)i * h->r;
      uint32_t v = 0;
      for (uint32_t b = 0; b < h->r; b++) {
        uint64_t p = bit + b;
        v |= (uint32_t)((bytes[h->tail_off + p / 8] >> (p % 8)) & 1u) << b;
      }
      c = (c << h->r) | v;
    }
    (void)fl;
    int hit = is_range ? (c > t) : (c == t);
    if (hit) bv_set(words, i);
  }
  return OR_OK;
}

int or_range_filter(const uint8_t *bytes, size_t blen, uint64_t scale, double pred, unsigned flags,
                    uint32_t *words, uint64_t *count, int *early) {
  or_br br;
  or_br_init(&br, bytes, blen);
  or_header h;
  if (parse_header_r(&br, &h)) return OR_PANIC;
  size_t len = h.n, nw = nwords_for(len);
  uint64_t ft;
  *early = 0;
  if (filter_target(&h, scale, pred, &ft)) {
    *early = 1; /* prints len and returns (:3385-3388) */
    for (size_t i = 0; i < nw; i++) words[i] = 0xFFFFFFFFu;
    bv_fix_last(words, len);
    *count = len;
    return OR_OK;
  }
  if (flags & OR_INTENDED) {
    int rc = filter_intended(bytes, blen, &h, ft, 1, words);
    *count = bv_card(words, nw);
    return rc;
  }
  uint32_t remain = h.fixed_len;
  uint32_t *res = words;
  memset(res, 0, nw * 4);
  uint32_t *rb1 = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t *tmp = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t *eqb = (uint32_t *)calloc(nw ? nw : 1, 4);
  int rc = OR_OK;
  if (!rb1 || !tmp || !eqb) {
    rc = OR_ENOMEM;
    goto done;
  }
  double check_ratio = 0.0;
  if (remain < 8) {
    for (size_t i = 0; i < len; i++) {
      uint8_t cur;
      if (or_br_read_bits(&br, remain, &cur)) {
        rc = OR_PANIC;
        goto done;
      }
      if ((uint64_t)cur > ft) bv_set(res, i);
    }
    remain = 0;
  } else {
    remain -= 8;
    const uint8_t *chunk;
    if (or_br_read_n_byte(&br, len, &chunk)) {
      rc = OR_PANIC;
      goto done;
    }
    uint8_t cur_tar = (uint8_t)(ft >> remain);
    range_simd(chunk, len, res, rb1, cur_tar);
    check_ratio = (double)bv_card(rb1, nw) / (double)len;
  }
  while (remain > 0) {
    if (remain >= 8) {
      remain -= 8;
      if (check_ratio > SIMD_THRESHOLD) { /* :3422-3435 */
        const uint8_t *chunk;
        if (or_br_read_n_byte(&br, len, &chunk)) {
          rc = OR_PANIC;
          goto done;
        }
        uint8_t cur_tar = (uint8_t)(ft >> remain);
        memset(tmp, 0, nw * 4);
        range_simd(chunk, len, tmp, eqb, cur_tar);
        for (size_t i = 0; i < nw; i++) {
          tmp[i] &= rb1[i];
          res[i] |= tmp[i];
          rb1[i] &= eqb[i];
        }
        check_ratio = (double)bv_card(rb1, nw) / (double)len;
      } else { /* progressive gather over BVIter (:3436-3493) */
        uint32_t *cur_rb = tmp;
        memset(cur_rb, 0, nw * 4);
        if (bv_card(rb1, nw) != 0) {
          uint8_t cur_tar = (uint8_t)(ft >> remain);
          size_t dec_pre = 0;
          int first = 1;
          for (size_t wi = 0; wi < nw; wi++) {
            uint32_t c = rb1[wi];
            while (c) {
              size_t dec_cur = (wi << 5) + (size_t)__builtin_ctz(c);
              c &= c - 1;
              if (first) {
                if (dec_cur != 0) or_br_skip_n_byte(&br, dec_cur);
                first = 0;
              } else {
                size_t delta = dec_cur - dec_pre;
                if (delta != 1) or_br_skip_n_byte(&br, delta - 1);
              }
              uint8_t b;
              if (or_br_read_byte(&br, &b)) {
                rc = OR_PANIC;
                goto done;
              }
              uint8_t dec = flip(b);
              if (dec > cur_tar)
                bv_set(res, dec_cur);
              else if (dec == cur_tar)
                bv_set(cur_rb, dec_cur);
              dec_pre = dec_cur;
            }
          }
          if (len - dec_pre > 1) or_br_skip_n_byte(&br, len - dec_pre - 1);
        } else {
          or_br_skip_n_byte(&br, len);
          break;
        }
        uint32_t *sw = rb1;
        rb1 = cur_rb;
        tmp = sw;
      }
    } else { /* packed tail (:3496-3543) */
      uint8_t cur_tar = (uint8_t)((uint8_t)((uint8_t)ft << (8 - remain)) >> (8 - remain));
      or_br_finish_read_byte(&br);
      if (bv_card(rb1, nw) != 0) {
        size_t dec_pre = 0;
        int first = 1;
        for (size_t wi = 0; wi < nw; wi++) {
          uint32_t c = rb1[wi];
          while (c) {
            size_t dec_cur = (wi << 5) + (size_t)__builtin_ctz(c);
            c &= c - 1;
            if (first) {
              if (dec_cur != 0) or_br_skip(&br, dec_cur * remain);
              first = 0;
            } else {
              size_t delta = dec_cur - dec_pre;
              if (delta != 1) or_br_skip(&br, (delta - 1) * remain);
            }
            uint8_t dec;
            if (or_br_read_bits(&br, remain, &dec)) {
              rc = OR_PANIC;
              goto done;
            }
            if (dec > cur_tar) bv_set(res, dec_cur);
            dec_pre = dec_cur;
          }
        }
        remain = 0;
      } else {
        break;
      }
    }
  }
done:
  if (rc == OR_OK) *count = bv_card(res, nw);
  free(rb1);
  free(tmp);
  free(eqb);
  return rc;
}

int or_equal_filter(const uint8_t *bytes, size_t blen, uint64_t scale, double pred, unsigned flags,
                    uint32_t *words, uint64_t *count, int *early) {
  or_br br;
  or_br_init(&br, bytes, blen);
  or_header h;
  if (parse_header_r(&br, &h)) return OR_PANIC;
  size_t len = h.n, nw = nwords_for(len);
  uint64_t ft;
  *early = 0;
  memset(words, 0, nw * 4);
  if (filter_target(&h, scale, pred, &ft)) {
    *early = 1; /* prints 0 and returns (:3573-3576) */
    *count = 0;
    return OR_OK;
  }
  if (flags & OR_INTENDED) {
    int rc = filter_intended(bytes, blen, &h, ft, 0, words);
    *count = bv_card(words, nw);
    return rc;
  }
  uint32_t remain = h.fixed_len;
  uint32_t *res = words;
  uint32_t *rb1 = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t *tmp = (uint32_t *)calloc(nw ? nw : 1, 4);
  int rc = OR_OK;
  if (!rb1 || !tmp) {
    rc = OR_ENOMEM;
    goto done;
  }
  double check_ratio = 0.0;
  if (remain < 8) {
    for (size_t i = 0; i < len; i++) {
      uint8_t cur;
      if (or_br_read_bits(&br, remain, &cur)) {
        rc = OR_PANIC;
        goto done;
      }
      if ((uint64_t)cur == ft) bv_set(res, i);
    }
    remain = 0;
  } else {
    remain -= 8;
    const uint8_t *chunk;
    if (or_br_read_n_byte(&br, len, &chunk)) {
      rc = OR_PANIC;
      goto done;
    }
    equal_simd(chunk, len, rb1, (uint8_t)(ft >> remain));
    check_ratio = (double)bv_card(rb1, nw) / (double)len;
  }
  while (remain > 0) {
    if (remain >= 8) {
      remain -= 8;
      if (check_ratio > SIMD_THRESHOLD) { /* :3617-3628 */
        const uint8_t *chunk;
        if (or_br_read_n_byte(&br, len, &chunk)) {
          rc = OR_PANIC;
          goto done;
        }
        equal_simd(chunk, len, tmp, (uint8_t)(ft >> remain));
        for (size_t i = 0; i < nw; i++) rb1[i] &= tmp[i];
        check_ratio = (double)bv_card(rb1, nw) / (double)len;
      } else { /* :3629-3677 */
        uint32_t *cur_rb = tmp;
        memset(cur_rb, 0, nw * 4);
        if (bv_card(rb1, nw) != 0) {
          uint8_t dec_byte = (uint8_t)(ft >> remain);
          size_t dec_pre = 0;
          int first = 1;
          for (size_t wi = 0; wi < nw; wi++) {
            uint32_t c = rb1[wi];
            while (c) {
              size_t dec_cur = (wi << 5) + (size_t)__builtin_ctz(c);
              c &= c - 1;
              if (first) {
                if (dec_cur != 0) or_br_skip_n_byte(&br, dec_cur);
                first = 0;
              } else {
                size_t delta = dec_cur - dec_pre;
                if (delta != 1) or_br_skip_n_byte(&br, delta - 1);
              }
              uint8_t b;
              if (or_br_read_byte(&br, &b)) {
                rc = OR_PANIC;
                goto done;
              }
              if (flip(b) == dec_byte) bv_set(cur_rb, dec_cur);
              dec_pre = dec_cur;
            }
          }
          if (len - dec_pre > 1) or_br_skip_n_byte(&br, len - dec_pre - 1);
        } else {
          or_br_skip_n_byte(&br, len);
          break;
        }
        uint32_t *sw = rb1;
        rb1 = cur_rb;
        tmp = sw;
      }
    } else { /* :3684-3729: only this step writes res */
      uint8_t dec_byte = (uint8_t)((uint8_t)((uint8_t)ft << (8 - remain)) >> (8 - remain));
      or_br_finish_read_byte(&br);
      if (bv_card(rb1, nw) != 0) {
        size_t dec_pre = 0;
        int first = 1;
        for (size_t wi = 0; wi < nw; wi++) {
          uint32_t c = rb1[wi];
          while (c) {
            size_t dec_cur = (wi << 5) + (size_t)__builtin_ctz(c);
            c &= c - 1;
            if (first) {
              if (dec_cur != 0) or_br_skip(&br, dec_cur * remain);
              first = 0;
            } else {
              size_t delta = dec_cur - dec_pre;
              if (delta != 1) or_br_skip(&br, (delta - 1) * remain);
            }
            uint8_t dec;
            if (or_br_read_bits(&br, remain, &dec)) {
              rc = OR_PANIC;
              goto done;
            }
            if (dec == dec_byte) bv_set(res, dec_cur);
            dec_pre = dec_cur;
          }
        }
        remain = 0;
      } else {
        break;
      }
    }
  }
done:
  if (rc == OR_OK) *count = bv_card(res, nw);
  free(rb1);
  free(tmp);
  return rc;
}

/* ------------------------------------------------------------------ */
/* scalar filters of the buff layout: buff_range_filter                 */
/* (buff_simd.rs:4507-4679) and buff_equal_filter (:4925-5094), the     */
/* `buff` arm of comp_profiler (buff_simd.rs:167-245)                   */
/* ------------------------------------------------------------------ */

/* Both filters read slice 0 for every row (no 32-row SIMD blocks), then
 * refine the rows still equal to the target byte by byte through BVIter
 * gathers, then the packed tail bits.  The range filter sets a row when a
 * byte exceeds the target byte; the equality filter sets rows only in its
 * tail step.  `flipped` = 0 reads the buff layout (byte_fixed_encode,
 * unflipped slices), 1 the buff-simd layout. */
static int scalar_filter(const uint8_t *bytes, size_t blen, uint64_t scale, double pred,
                         int is_range, int flipped, uint32_t *words, uint64_t *count,
                         int *early) {
  or_br br;
  or_br_init(&br, bytes, blen);
  or_header h;
  if (parse_header_r(&br, &h)) return OR_PANIC;
  size_t len = h.n, nw = nwords_for(len);
  uint64_t ft;
  *early = 0;
  memset(words, 0, (nw ? nw : 1) * 4);
  if (filter_target(&h, scale, pred, &ft)) {
    /* :4528-4531 prints len; :4948-4951 prints 0 */
    *early = 1;
    if (is_range) {
      for (size_t i = 0; i < nw; i++) words[i] = 0xFFFFFFFFu;
      bv_fix_last(words, len);
      *count = len;
    } else {
      *count = 0;
    }
    return OR_OK;
  }
  uint32_t remain = h.ilen + h.dlen; /* u32 add, wrapping as `dlen+ilen` */
  uint32_t *res = words;
  uint32_t *rb1 = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t *cur_rb = (uint32_t *)calloc(nw ? nw : 1, 4);
  int rc = OR_OK;
  if (!rb1 || !cur_rb) {
    rc = OR_ENOMEM;
    goto done;
  }
  if (remain < 8) { /* :4535-4543 / :4959-4967: every row against the full target */
    for (size_t i = 0; i < len; i++) {
      uint8_t cur;
      if (or_br_read_bits(&br, remain, &cur)) {
        rc = OR_PANIC;
        goto done;
      }
      if (is_range ? ((uint64_t)cur > ft) : ((uint64_t)cur == ft)) bv_set(res, i);
    }
    remain = 0;
  } else { /* :4544-4558 / :4968-4979 */
    remain -= 8;
    const uint8_t *chunk;
    if (or_br_read_n_byte(&br, len, &chunk)) {
      rc = OR_PANIC;
      goto done;
    }
    uint8_t cur_tar = (uint8_t)(ft >> remain);
    for (size_t i = 0; i < len; i++) {
      uint8_t c = flipped ? flip(chunk[i]) : chunk[i];
      if (is_range && c > cur_tar)
        bv_set(res, i);
      else if (c == cur_tar)
        bv_set(rb1, i);
    }
  }
  while (remain > 0) {
    if (remain >= 8) { /* :4565-4622 / :4987-5039 */
      remain -= 8;
      memset(cur_rb, 0, (nw ? nw : 1) * 4);
      if (bv_card(rb1, nw) != 0) {
        uint8_t cur_tar = (uint8_t)(ft >> remain);
        size_t dec_pre = 0;
        int first = 1;
        for (size_t wi = 0; wi < nw; wi++) {
          uint32_t c = rb1[wi];
          while (c) {
            size_t dec_cur = (wi << 5) + (size_t)__builtin_ctz(c);
            c &= c - 1;
            if (first) {
              if (dec_cur != 0) or_br_skip_n_byte(&br, dec_cur);
              first = 0;
            } else {
              size_t delta = dec_cur - dec_pre;
              if (delta != 1) or_br_skip_n_byte(&br, delta - 1);
            }
            uint8_t b;
            if (or_br_read_byte(&br, &b)) {
              rc = OR_PANIC;
              goto done;
            }
            uint8_t dec = flipped ? flip(b) : b;
            if (is_range && dec > cur_tar)
              bv_set(res, dec_cur);
            else if (dec == cur_tar)
              bv_set(cur_rb, dec_cur);
            dec_pre = dec_cur;
          }
        }
        if (len - dec_pre > 1) or_br_skip_n_byte(&br, len - dec_pre - 1);
      } else {
        or_br_skip_n_byte(&br, len);
        break;
      }
      uint32_t *sw = rb1;
      rb1 = cur_rb;
      cur_rb = sw;
    } else { /* packed tail, :4625-4673 / :5042-5090 */
      uint8_t cur_tar = (uint8_t)((uint8_t)((uint8_t)ft << (8 - remain)) >> (8 - remain));
      or_br_finish_read_byte(&br);
      if (bv_card(rb1, nw) != 0) {
        size_t dec_pre = 0;
        int first = 1;
        for (size_t wi = 0; wi < nw; wi++) {
          uint32_t c = rb1[wi];
          while (c) {
            size_t dec_cur = (wi << 5) + (size_t)__builtin_ctz(c);
            c &= c - 1;
            if (first) {
              if (dec_cur != 0) or_br_skip(&br, dec_cur * remain);
              first = 0;
            } else {
              size_t delta = dec_cur - dec_pre;
              if (delta != 1) or_br_skip(&br, (delta - 1) * remain);
            }
            uint8_t dec;
            if (or_br_read_bits(&br, remain, &dec)) {
              rc = OR_PANIC;
              goto done;
            }
            if (is_range ? (dec > cur_tar) : (dec == cur_tar)) bv_set(res, dec_cur);
            dec_pre = dec_cur;
          }
        }
        remain = 0;
      } else {
        break;
      }
    }
  }
done:
  if (rc == OR_OK) *count = bv_card(res, nw);
  free(rb1);
  free(cur_rb);
  return rc;
}

int or_scalar_range_filter(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                           int flipped, uint32_t *words, uint64_t *count, int *early) {
  return scalar_filter(bytes, len, scale, pred, 1, flipped, words, count, early);
}
int or_scalar_equal_filter(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                           int flipped, uint32_t *words, uint64_t *count, int *early) {
  return scalar_filter(bytes, len, scale, pred, 0, flipped, words, count, early);
}

/* buff_simd_range_filter_with_slice / buff_simd_equal_filter_with_slice
 * (buff_simd.rs:3736-3884, 3888-4025): fused compare of up to 4 leading
 * slices per 32 rows, then the packed tail for the surviving rows. */
static int filter_with_slice(const uint8_t *bytes, size_t blen, uint64_t scale, double pred,
                             int is_range, uint32_t *words, uint64_t *count, int *early) {
  or_br br;
  or_br_init(&br, bytes, blen);
  or_header h;
  if (parse_header_r(&br, &h)) return OR_PANIC;
  uint32_t len = h.n;
  size_t nw = nwords_for(len);
  uint64_t ft;
  *early = 0;
  memset(words, 0, nw * 4);
  uint32_t remain = h.fixed_len;
  uint32_t num_slice = remain / 8; /* floor (buff_slice.rs:185-187) */
  if (filter_target(&h, scale, pred, &ft)) {
    *early = 1; /* both variants print len (:3769-3772, :3919-3922) */
    for (size_t i = 0; i < nw; i++) words[i] = 0xFFFFFFFFu;
    bv_fix_last(words, len);
    *count = len;
    return OR_OK;
  }
  /* slice_ptr.get(0).unwrap() panics with no slice; `len - BYTE_WORD`
   * underflows (u32) for len < 32 and the loop reads past the buffer. */
  if (num_slice == 0 || len < 32) return OR_PANIC;
  if ((size_t)20 + (size_t)num_slice * len > blen) return OR_PANIC;
  int8_t tw[4] = {0, 0, 0, 0};
  const uint8_t *sp[4] = {0, 0, 0, 0};
  for (uint32_t cnt = 0; cnt < num_slice && cnt < 4; cnt++) {
    sp[cnt] = bytes + 20 + (size_t)cnt * len; /* read_n_byte_unmut(cnt*len, len) */
    tw[cnt] = (int8_t)flip((uint8_t)(ft >> (remain - 8 * (1 + cnt))));
  }
  uint32_t *rb1 = (uint32_t *)calloc(nw, 4);
  if (!rb1) return OR_ENOMEM;
  for (uint32_t i = 0, b = 0; i <= len - 32; i += 32, b++) {
    uint32_t g, e, gj, ej;
    cmp32(sp[0] + i, tw[0], &g, &e);
    if (num_slice > 1 && e) {
      cmp32(sp[1] + i, tw[1], &gj, &ej);
      g |= e & gj;
      e &= ej;
      if (num_slice > 2 && e) {
        cmp32(sp[2] + i, tw[2], &gj, &ej);
        g |= e & gj;
        e &= ej;
        if (num_slice > 3 && e) {
          cmp32(sp[3] + i, tw[3], &gj, &ej);
          g |= e & gj;
          e &= ej;
        }
      }
    }
    rb1[b] = e;
    if (is_range) words[b] = g;
  }
  uint64_t card = bv_card(rb1, nw);
  remain = remain - 8 * num_slice;
  int rc = OR_OK;
  if (remain > 0 && card != 0) {
    or_br_skip_n_byte(&br, (size_t)num_slice * len);
    uint8_t dec_byte = (uint8_t)((uint8_t)((uint8_t)ft << (8 - remain)) >> (8 - remain));
    or_br_finish_read_byte(&br);
    size_t dec_pre = 0;
    int first = 1;
    for (size_t wi = 0; wi < nw; wi++) {
      uint32_t c = rb1[wi];
      while (c) {
        size_t dec_cur = (wi << 5) + (size_t)__builtin_ctz(c);
        c &= c - 1;
        if (first) {
          if (dec_cur != 0) or_br_skip(&br, dec_cur * remain);
          first = 0;
        } else {
          size_t delta = dec_cur - dec_pre;
          if (delta != 1) or_br_skip(&br, (delta - 1) * remain);
        }
        uint8_t dec;
        if (or_br_read_bits(&br, remain, &dec)) {
          rc = OR_PANIC;
          goto out;
        }
        if (is_range ? (dec > dec_byte) : (dec == dec_byte)) bv_set(words, dec_cur);
        dec_pre = dec_cur;
      }
    }
  }
out:
  free(rb1);
  if (rc == OR_OK) *count = bv_card(words, nw);
  return rc;
}

int or_range_filter_with_slice(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                               uint32_t *words, uint64_t *count, int *early) {
  return filter_with_slice(bytes, len, scale, pred, 1, words, count, early);
}
int or_equal_filter_with_slice(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                               uint32_t *words, uint64_t *count, int *early) {
  return filter_with_slice(bytes, len, scale, pred, 0, words, count, early);
}

/* ------------------------------------------------------------------ */
/* sum: byte_fixed_sum (split_double.rs:2127-2208) and                 */
/* byte_residue_sum_with_precision (split_double.rs:2409-2630)          */
/* ------------------------------------------------------------------ */

/* The number of bits a precision-limited read rebuilds
 * (split_double.rs:1642-1664 / 2439-2459).  Returns OR_PANIC on the
 * reference's unwrap/assert failures. */
static int precision_bits(const or_header *h, uint32_t precision, uint32_t *remain) {
  uint32_t ilen = h->ilen, dlen = h->dlen;
  if (precision == 0) {
    uint32_t rm = ilen;
    uint32_t byte_needed = ilen / 8;
    if (ilen % 8 > 0) {
      byte_needed += 1;
      rm = byte_needed * 8;
    }
    *remain = rm;
  } else {
    int bn = or_dlen_of_prec((int)precision);
    if (precision > 0x7FFFFFFFu || bn < 0) return OR_PANIC;
    uint32_t bits_needed = (uint32_t)bn;
    if (!(dlen >= bits_needed)) return OR_PANIC;
    uint32_t rm = ilen + bits_needed;
    uint32_t fixed_byte = (dlen + ilen) / 8;
    uint32_t byte_needed = (ilen + bits_needed) / 8;
    uint32_t extra_bits = (ilen + bits_needed) % 8;
    if (byte_needed < fixed_byte) {
      if (extra_bits > 0) {
        byte_needed += 1;
        rm = byte_needed * 8;
      }
    }
    *remain = rm;
  }
  return OR_OK;
}

static int sum_bits(or_br *br, const or_header *h, uint32_t total, int flipped, unsigned flags,
                    double *sum_out, uint64_t *partials) {
  uint32_t remain = total;
  int32_t processed = 0;
  int32_t ilen_i = (int32_t)h->ilen;
  double sum_base = (double)h->n * (double)h->base;
  double dec_scl = ldexp(1.0, (int)h->dlen);
  sum_base = sum_base / dec_scl;
  double sum = 0.0;
  uint8_t fx = flipped ? 0x80u : 0u;
  uint32_t slot = 0;
  while (remain >= 8) { /* :2151-2191 */
    remain -= 8;
    processed += 8;
    dec_scl = ldexp(1.0, processed - ilen_i);
    const uint8_t *chunk;
    if (or_br_read_n_byte(br, h->n, &chunk)) return OR_PANIC;
    uint64_t sf = 0;
    for (uint32_t i = 0; i < h->n; i++) sf += (uint64_t)(chunk[i] ^ fx);
    if (partials) partials[slot] = sf;
    slot++;
    sum = sum + (double)sf / dec_scl;
    if (remain == 0) {
      if (flags & OR_INTENDED) break;
      *sum_out = sum; /* returns without the base term (:2171-2173, 2188-2190) */
      return OR_OK;
    }
  }
  if (remain > 0) { /* :2192-2203 */
    if (processed >= 8) or_br_finish_read_byte(br);
    processed += (int32_t)remain;
    dec_scl = ldexp(1.0, processed - ilen_i);
    uint64_t sf = 0;
    for (uint32_t i = 0; i < h->n; i++) {
      uint8_t b;
      if (or_br_read_bits(br, remain, &b)) return OR_PANIC;
      sf += b;
    }
    if (partials) partials[slot] = sf;
    sum = sum + (double)sf / dec_scl;
  }
  sum += sum_base;
  *sum_out = sum;
  return OR_OK;
}

int or_sum(const uint8_t *bytes, size_t len, uint64_t scale, int flipped, unsigned flags,
           double *sum, uint64_t *partials, int64_t exact_num[2]) {
  (void)scale;
  or_br br;
  or_br_init(&br, bytes, len);
  or_header h;
  if (parse_header_r(&br, &h)) return OR_PANIC;
  uint64_t parts[16] = {0};
  int rc = sum_bits(&br, &h, h.fixed_len, flipped, flags, sum, parts);
  if (rc) return rc;
  if (partials)
    for (uint32_t j = 0; j <= h.k && j < 16; j++) partials[j] = parts[j];
  if (exact_num) {
    /* n*base + sum_j S_j * 2^(fl - 8(j+1)) + S_tail as a 128-bit integer */
    __int128 acc = (__int128)h.n * (__int128)h.base;
    for (uint32_t j = 0; j < h.k; j++) acc += (__int128)parts[j] << (h.fixed_len - 8 * (j + 1));
    if (h.r) acc += (__int128)parts[h.k];
    exact_num[0] = (int64_t)(uint64_t)acc;
    exact_num[1] = (int64_t)(acc >> 64);
  }
  return OR_OK;
}

int or_sum_at_precision(const uint8_t *bytes, size_t len, uint64_t scale, int flipped,
                        uint32_t precision, unsigned flags, double *sum) {
  (void)scale;
  or_br br;
  or_br_init(&br, bytes, len);
  or_header h;
  if (parse_header_r(&br, &h)) return OR_PANIC;
  uint32_t total;
  if (precision_bits(&h, precision, &total)) return OR_PANIC;
  return sum_bits(&br, &h, total, flipped, flags, sum, NULL);
}

/* ------------------------------------------------------------------ */
/* max: byte_fixed_max (split_double.rs:3919-4105)                      */
/* ------------------------------------------------------------------ */

int or_max(const uint8_t *bytes, size_t blen, uint64_t scale, int flipped, unsigned flags,
           double *maxv, uint64_t *max_code, uint32_t *argmax_words, uint64_t *argmax_count) {
  (void)scale;
  or_br br;
  or_br_init(&br, bytes, blen);
  or_header h;
  if (parse_header_r(&br, &h)) return OR_PANIC;
  uint32_t len = h.n, remain = h.fixed_len;
  size_t nw = nwords_for(len);
  uint8_t fx = flipped ? 0x80u : 0u;
  uint32_t *res = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t *rb1 = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t *cur = (uint32_t *)calloc(nw ? nw : 1, 4);
  int rc = OR_OK;
  uint64_t mx = 0;
  if (!res || !rb1 || !cur) {
    rc = OR_ENOMEM;
    goto done;
  }
  if (remain < 8) {
    for (uint32_t i = 0; i < len; i++) {
      uint8_t c;
      if (or_br_read_bits(&br, remain, &c)) {
        rc = OR_PANIC;
        goto done;
      }
      if ((uint64_t)c > mx) {
        mx = c;
        memset(res, 0, nw * 4);
        bv_set(res, i);
      } else if ((uint64_t)c == mx) {
        bv_set(res, i);
      }
    }
    remain = 0;
  } else {
    remain -= 8;
    const uint8_t *chunk;
    if (or_br_read_n_byte(&br, len, &chunk)) {
      rc = OR_PANIC;
      goto done;
    }
    uint8_t byte_max = 0;
    for (uint32_t i = 0; i < len; i++) {
      uint8_t c = chunk[i] ^ fx;
      if (c > byte_max) {
        byte_max = c;
        memset(rb1, 0, nw * 4);
        bv_set(rb1, i);
      } else if (c == byte_max) {
        bv_set(rb1, i);
      }
    }
    mx = (uint64_t)byte_max << remain;
  }
  while (remain > 0) {
    uint8_t byte_max = 0;
    if (remain >= 8) {
      remain -= 8;
      memset(cur, 0, nw * 4);
      uint32_t dec_pre = 0;
      int first = 1;
      for (size_t wi = 0; wi < nw; wi++) {
        uint32_t c = rb1[wi];
        while (c) {
          uint32_t dec_cur = (uint32_t)((wi << 5) + (size_t)__builtin_ctz(c));
          c &= c - 1;
          if (first) {
            if (dec_cur != 0) or_br_skip_n_byte(&br, dec_cur);
          } else {
            uint32_t delta = dec_cur - dec_pre;
            if (delta != 1) or_br_skip_n_byte(&br, delta - 1);
          }
          uint8_t b;
          if (or_br_read_byte(&br, &b)) {
            rc = OR_PANIC;
            goto done;
          }
          uint8_t dec = b ^ fx;
          if (first) {
            if (dec > byte_max) byte_max = dec;
            bv_set(cur, dec_cur);
            first = 0;
          } else if (dec > byte_max) {
            byte_max = dec;
            memset(cur, 0, nw * 4);
            bv_set(cur, dec_cur);
          } else if (dec == byte_max) {
            bv_set(cur, dec_cur);
          }
          dec_pre = dec_cur;
        }
      }
      if (len - dec_pre > 1) or_br_skip_n_byte(&br, (size_t)(len - dec_pre - 1));
      mx |= (uint64_t)byte_max << remain;
      uint32_t *sw = rb1;
      rb1 = cur;
      cur = sw;
    } else {
      or_br_finish_read_byte(&br);
      uint32_t dec_pre = 0;
      int first = 1;
      for (size_t wi = 0; wi < nw; wi++) {
        uint32_t c = rb1[wi];
        while (c) {
          uint32_t dec_cur = (uint32_t)((wi << 5) + (size_t)__builtin_ctz(c));
          c &= c - 1;
          if (first) {
            if (dec_cur != 0) or_br_skip(&br, (size_t)(dec_cur * remain));
          } else {
            uint32_t delta = dec_cur - dec_pre;
            if (delta != 1) or_br_skip(&br, (size_t)((delta - 1) * remain));
          }
          uint8_t dec;
          if (or_br_read_bits(&br, remain, &dec)) {
            rc = OR_PANIC;
            goto done;
          }
          if (dec > byte_max) {
            byte_max = dec;
            if (!first) memset(res, 0, nw * 4);
            bv_set(res, dec_cur);
          } else if (dec == byte_max) {
            bv_set(res, dec_cur);
          }
          first = 0;
          dec_pre = dec_cur;
        }
      }
      remain = 0;
      mx |= (uint64_t)byte_max;
    }
  }
  if ((flags & OR_INTENDED) && h.fixed_len >= 8 && h.r == 0) memcpy(res, rb1, nw * 4);
  *max_code = mx;
  *maxv = (double)wadd(h.base, mx) / ldexp(1.0, (int)h.dlen);
  if (argmax_words) memcpy(argmax_words, res, nw * 4);
  if (argmax_count) *argmax_count = bv_card(res, nw);
done:
  free(res);
  free(rb1);
  free(cur);
  return rc;
}

/* ------------------------------------------------------------------ */
/* variable precision: byte_residue_decode_with_precision               */
/* (split_double.rs:1612-1893), layout without outlier columns          */
/* ------------------------------------------------------------------ */

int or_decode_at_precision(const uint8_t *bytes, size_t len, uint64_t scale, int flipped,
                           uint32_t precision, unsigned flags, double *out) {
  (void)scale;
  or_br br;
  or_br_init(&br, bytes, len);
  or_header h;
  if (parse_header_r(&br, &h)) return OR_PANIC;
  uint32_t total;
  if (precision_bits(&h, precision, &total)) return OR_PANIC;
  if (!(flags & OR_INTENDED)) return decode_bits(&br, &h, total, flipped, out);
  /* INTENDED: keep the top `total` bits of the code in place. */
  if (total > h.fixed_len) return OR_PANIC;
  uint64_t *codes = (uint64_t *)malloc((size_t)(h.n ? h.n : 1) * 8);
  if (!codes) return OR_ENOMEM;
  int rc = codes_of(bytes, len, &h, flipped, codes);
  if (rc) {
    free(codes);
    return rc;
  }
  double dec_scl = ldexp(1.0, (int)h.dlen);
  uint32_t drop = h.fixed_len - total;
  uint64_t m = drop >= 64 ? 0 : (~0ull << drop);
  for (uint32_t i = 0; i < h.n; i++) out[i] = (double)wadd(h.base, codes[i] & m) / dec_scl;
  free(codes);
  return OR_OK;
}

/* ------------------------------------------------------------------ */
/* multi-threaded CPU baseline (filter + sum per 32-row-aligned chunk)  */
/* ------------------------------------------------------------------ */

typedef struct bench_job {
  const uint8_t *bytes;
  or_header h;
  uint64_t ft;
  uint32_t row0, row1;
  size_t tail_len;
  uint32_t *words;
  uint64_t count;
  uint64_t partials[16];
} bench_job;

/* One chunk of rows: the reference's slice-0 compare, progressive refinement
 * of later slices over the candidate bits, then the packed tail; plus the
 * per-slice byte sums of byte_fixed_sum. */
static void *bench_worker(void *arg) {
  bench_job *j = (bench_job *)arg;
  const or_header *h = &j->h;
  uint32_t r0 = j->row0, r1 = j->row1, len = r1 - r0;
  size_t nw = nwords_for(len);
  uint32_t *res = j->words + r0 / 32;
  uint32_t *rb1 = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t *cur = (uint32_t *)calloc(nw ? nw : 1, 4);
  memset(res, 0, nw * 4);
  uint32_t remain = h->fixed_len - 8;
  const uint8_t *s0 = j->bytes + h->slice_off + r0;
  range_simd(s0, len, res, rb1, (uint8_t)(j->ft >> remain));
  for (uint32_t s = 1; s < h->k; s++) {
    remain -= 8;
    uint8_t tar = (uint8_t)(j->ft >> remain);
    const uint8_t *sl = j->bytes + h->slice_off + (size_t)s * h->n + r0;
    memset(cur, 0, nw * 4);
    for (size_t wi = 0; wi < nw; wi++) {
      uint32_t c = rb1[wi];
      while (c) {
        size_t i = (wi << 5) + (size_t)__builtin_ctz(c);
        c &= c - 1;
        uint8_t dec = flip(sl[i]);
        if (dec > tar)
          res[i >> 5] |= 1u << (i & 31);
        else if (dec == tar)
          cur[i >> 5] |= 1u << (i & 31);
      }
    }
    uint32_t *sw = rb1;
    rb1 = cur;
    cur = sw;
  }
  if (h->r) {
    uint32_t rr = h->r;
    uint8_t tar = (uint8_t)(j->ft & ((1u << rr) - 1));
    const uint8_t *tl = j->bytes + h->tail_off;
    for (size_t wi = 0; wi < nw; wi++) {
      uint32_t c = rb1[wi];
      while (c) {
        size_t i = (wi << 5) + (size_t)__builtin_ctz(c);
        c &= c - 1;
        uint64_t bit = (uint64_t)(r0 + i) * rr;
        uint32_t v = (uint32_t)tl[bit / 8];
        if (bit / 8 + 1 < j->tail_len) v |= (uint32_t)tl[bit / 8 + 1] << 8;
        uint8_t dec = (uint8_t)((v >> (bit % 8)) & ((1u << rr) - 1));
        if (dec > tar) res[i >> 5] |= 1u << (i & 31);
      }
    }
  }
  j->count = bv_card(res, nw);
  /* sum partials */
  for (uint32_t s = 0; s < h->k; s++) {
    const uint8_t *sl = j->bytes + h->slice_off + (size_t)s * h->n + r0;
    uint64_t acc = 0;
    for (uint32_t i = 0; i < len; i++) acc += (uint8_t)(sl[i] ^ 0x80u);
    j->partials[s] = acc;
  }
  if (h->r) {
    uint32_t rr = h->r;
    const uint8_t *tl = j->bytes + h->tail_off;
    uint64_t acc = 0;
    for (uint32_t i = r0; i < r1; i++) {
      uint64_t bit = (uint64_t)i * rr;
      uint32_t v = (uint32_t)tl[bit / 8];
      if (bit / 8 + 1 < j->tail_len) v |= (uint32_t)tl[bit / 8 + 1] << 8;
      acc += (v >> (bit % 8)) & ((1u << rr) - 1);
    }
    j->partials[h->k] = acc;
  }
  free(rb1);
  free(cur);
  return NULL;
}

double or_bench_filter_sum(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                           int nthreads, int reps, uint64_t *count, double *sum) {
  or_header h;
  if (or_parse_header(bytes, len, &h) || h.k == 0 || nthreads < 1) return -1.0;
  uint64_t ft;
  if (filter_target(&h, scale, pred, &ft)) return -1.0;
  size_t nw = nwords_for(h.n);
  uint32_t *words = (uint32_t *)calloc(nw + 1, 4);
  bench_job *jobs = (bench_job *)calloc((size_t)nthreads, sizeof(bench_job));
  pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
  uint32_t full = h.n / 32 * 32;
  uint32_t per = (full / 32 + (uint32_t)nthreads - 1) / (uint32_t)nthreads * 32;
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int rep = 0; rep < reps; rep++) {
    for (int t = 0; t < nthreads; t++) {
      jobs[t].bytes = bytes;
      jobs[t].h = h;
      jobs[t].ft = ft;
      uint32_t a = (uint32_t)t * per, b = a + per;
      if (a > h.n) a = h.n;
      if (t == nthreads - 1 || b > h.n) b = h.n;
      jobs[t].row0 = a;
      jobs[t].row1 = b;
      jobs[t].words = words;
      jobs[t].tail_len = len - h.tail_off;
      if (nthreads == 1)
        bench_worker(&jobs[t]);
      else
        pthread_create(&th[t], NULL, bench_worker, &jobs[t]);
    }
    if (nthreads > 1)
      for (int t = 0; t < nthreads; t++) pthread_join(th[t], NULL);
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  uint64_t c = 0, parts[16] = {0};
  for (int t = 0; t < nthreads; t++) {
    c += jobs[t].count;
    for (uint32_t s = 0; s <= h.k; s++) parts[s] += jobs[t].partials[s];
  }
  /* the reference's f64 combine (split_double.rs:2141-2205) */
  int32_t ilen_i = (int32_t)h.ilen, processed = 0;
  double sum_base = (double)h.n * (double)h.base / ldexp(1.0, (int)h.dlen);
  double s = 0.0;
  for (uint32_t j = 0; j < h.k; j++) {
    processed += 8;
    s = s + (double)parts[j] / ldexp(1.0, processed - ilen_i);
  }
  if (h.r) {
    processed += (int32_t)h.r;
    s = s + (double)parts[h.k] / ldexp(1.0, processed - ilen_i);
    s += sum_base;
  }
  *count = c;
  *sum = s;
  free(words);
  free(jobs);
  free(th);
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
