/*
 * CPU oracle, part 2: the buff-major (outlier) format and the snappy codec of
 * its outlier bitmaps.  TEST INFRASTRUCTURE ONLY (see buff_oracle.c).
 *
 * buff_encode_majority (compress/buff_simd.rs:317-630) stores leading byte
 * columns whose first-2000-row Boyer-Moore majority is strong as
 * (major byte, snappy(BitVec::to_binary(outlier rows)), outlier bytes); the
 * queries (:633-2861) merge those side tables with the dense slices.  The
 * compressed bitmap uses parity-snappy 0.1.0 (Cargo.toml:45), which is not
 * vendored here: the compressor below restates the published snappy
 * algorithm, so the compressed bytes are parity-unpinned; the raw variant
 * (OR_BM_RAW) stores the to_binary bytes uncompressed and is what the
 * byte-exact tests compare.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "buff_oracle.h"

#define SAMPLE 2000 /* split_double.rs:25 */

/* ------------------------------------------------------------------ */
/* snappy raw format (varint length, literal / copy elements)          */
/* ------------------------------------------------------------------ */

size_t or_snappy_max_compressed(size_t n) { return 32 + n + n / 6; }

static inline uint32_t ld32(const uint8_t *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

static uint8_t *emit_literal(uint8_t *op, const uint8_t *lit, size_t len) {
  size_t n = len - 1;
  if (n < 60) {
    *op++ = (uint8_t)(n << 2);
  } else {
    int cnt = 0;
    uint8_t tmp[4];
    while (n > 0) {
      tmp[cnt++] = (uint8_t)n;
      n >>= 8;
    }
    *op++ = (uint8_t)((59 + cnt) << 2);
    for (int i = 0; i < cnt; i++) *op++ = tmp[i];
  }
  memcpy(op, lit, len);
  return op + len;
}

static uint8_t *emit_copy_upto64(uint8_t *op, size_t offset, size_t len) {
  if (len < 12 && offset < 2048) {
    *op++ = (uint8_t)(1 | ((len - 4) << 2) | ((offset >> 8) << 5));
    *op++ = (uint8_t)offset;
  } else {
    *op++ = (uint8_t)(2 | ((len - 1) << 2));
    *op++ = (uint8_t)offset;
    *op++ = (uint8_t)(offset >> 8);
  }
  return op;
}

static uint8_t *emit_copy(uint8_t *op, size_t offset, size_t len) {
  while (len >= 68) {
    op = emit_copy_upto64(op, offset, 64);
    len -= 64;
  }
  if (len > 64) {
    op = emit_copy_upto64(op, offset, 60);
    len -= 60;
  }
  return emit_copy_upto64(op, offset, len);
}

/* One block of at most 64 KiB: hash 4-byte sequences, extend matches,
 * literal runs between them, with the usual growing skip on misses. */
static uint8_t *compress_block(const uint8_t *in, size_t n, uint8_t *op, uint16_t *table,
                               int table_bits) {
  const uint8_t *ip = in, *ip_end = in + n, *next_emit = in;
  const int shift = 32 - table_bits;
  memset(table, 0, sizeof(uint16_t) << table_bits);
  if (n >= 15) {
    const uint8_t *ip_limit = in + n - 15;
    uint32_t next_hash = (ld32(++ip) * 0x1e35a7bdu) >> shift;
    for (;;) {
      uint32_t skip = 32;
      const uint8_t *next_ip = ip, *cand;
      do {
        ip = next_ip;
        uint32_t h = next_hash;
        uint32_t step = skip >> 5;
        skip += step;
        next_ip = ip + step;
        if (next_ip > ip_limit) goto remainder;
        next_hash = (ld32(next_ip) * 0x1e35a7bdu) >> shift;
        cand = in + table[h];
        table[h] = (uint16_t)(ip - in);
      } while (ld32(ip) != ld32(cand));
      op = emit_literal(op, next_emit, (size_t)(ip - next_emit));
      do {
        const uint8_t *base = ip;
        size_t matched = 4;
        while (ip + matched < ip_end && cand[matched] == ip[matched]) matched++;
        ip += matched;
        op = emit_copy(op, (size_t)(base - cand), matched);
        next_emit = ip;
        if (ip >= ip_limit) goto remainder;
        table[(ld32(ip - 1) * 0x1e35a7bdu) >> shift] = (uint16_t)(ip - 1 - in);
        uint32_t h = (ld32(ip) * 0x1e35a7bdu) >> shift;
        cand = in + table[h];
        table[h] = (uint16_t)(ip - in);
      } while (ld32(ip) == ld32(cand));
      next_hash = (ld32(++ip) * 0x1e35a7bdu) >> shift;
    }
  }
remainder:
  if (next_emit < ip_end) op = emit_literal(op, next_emit, (size_t)(ip_end - next_emit));
  return op;
}

int or_snappy_compress(const uint8_t *in, size_t n, uint8_t *out, size_t cap, size_t *outlen) {
  if (cap < or_snappy_max_compressed(n)) return OR_EINVAL;
  uint8_t *op = out;
  size_t v = n;
  while (v >= 0x80) {
    *op++ = (uint8_t)(v | 0x80);
    v >>= 7;
  }
  *op++ = (uint8_t)v;
  uint16_t *table = (uint16_t *)malloc(sizeof(uint16_t) << 14);
  if (!table) return OR_ENOMEM;
  for (size_t off = 0; off < n; off += 65536) {
    size_t blk = n - off < 65536 ? n - off : 65536;
    int bits = 8;
    while (bits < 14 && ((size_t)1 << bits) < blk) bits++;
    op = compress_block(in + off, blk, op, table, bits);
  }
  free(table);
  *outlen = (size_t)(op - out);
  return OR_OK;
}

int or_snappy_decompress(const uint8_t *in, size_t n, uint8_t *out, size_t cap, size_t *outlen) {
  size_t ulen = 0, i = 0;
  int sh = 0;
  for (;;) {
    if (i >= n || sh > 35) return OR_PANIC;
    uint8_t b = in[i++];
    ulen |= (size_t)(b & 0x7F) << sh;
    if (!(b & 0x80)) break;
    sh += 7;
  }
  *outlen = ulen;
  if (!out) return OR_OK;
  if (cap < ulen) return OR_EINVAL;
  size_t o = 0;
  while (i < n) {
    uint8_t tag = in[i++];
    size_t len, off;
    switch (tag & 3) {
      case 0:
        len = (size_t)(tag >> 2) + 1;
        if (len > 60) {
          size_t nb = len - 60, v = 0;
          if (i + nb > n) return OR_PANIC;
          for (size_t k = 0; k < nb; k++) v |= (size_t)in[i + k] << (8 * k);
          i += nb;
          len = v + 1;
        }
        if (i + len > n || o + len > ulen) return OR_PANIC;
        memcpy(out + o, in + i, len);
        i += len;
        o += len;
        continue;
      case 1:
        if (i + 1 > n) return OR_PANIC;
        len = 4 + ((tag >> 2) & 7);
        off = ((size_t)(tag >> 5) << 8) | in[i];
        i += 1;
        break;
      case 2:
        if (i + 2 > n) return OR_PANIC;
        len = (size_t)(tag >> 2) + 1;
        off = (size_t)in[i] | ((size_t)in[i + 1] << 8);
        i += 2;
        break;
      default:
        if (i + 4 > n) return OR_PANIC;
        len = (size_t)(tag >> 2) + 1;
        off = ld32(in + i);
        i += 4;
        break;
    }
    if (off == 0 || off > o || o + len > ulen) return OR_PANIC;
    for (size_t k = 0; k < len; k++, o++) out[o] = out[o - off];
  }
  return o == ulen ? OR_OK : OR_PANIC;
}

/* bit_vec_compress (query/bit_vec_iter.rs:61-63) of BitVec::to_binary. */
static int bm_serialize(const uint32_t *words, size_t nw, uint64_t nbits, int mode, uint8_t **out,
                        size_t *len) {
  if (mode == OR_BM_ROARING) { /* Bitmap::create + add + run_optimize + serialize */
    uint32_t *rows = (uint32_t *)malloc((nbits ? nbits : 1) * 4);
    if (!rows) return OR_ENOMEM;
    size_t cnt = 0;
    for (uint64_t i = 0; i < nbits; i++)
      if ((words[i >> 5] >> (i & 31)) & 1u) rows[cnt++] = (uint32_t)i;
    int rc = or_roaring_serialize(rows, cnt, out, len);
    free(rows);
    return rc;
  }
  size_t blen = 8 + 4 * nw;
  uint8_t *bin = (uint8_t *)malloc(blen);
  if (!bin) return OR_ENOMEM;
  or_bitvec_to_binary(words, nw, nbits, bin);
  if (mode == OR_BM_RAW) {
    *out = bin;
    *len = blen;
    return OR_OK;
  }
  size_t cap = or_snappy_max_compressed(blen);
  uint8_t *c = (uint8_t *)malloc(cap);
  if (!c) {
    free(bin);
    return OR_ENOMEM;
  }
  int rc = or_snappy_compress(bin, blen, c, cap, len);
  free(bin);
  if (rc) {
    free(c);
    return rc;
  }
  *out = c;
  return OR_OK;
}

/* bit_vec_decompress + BitVec::from_binary (bit-vec lib.rs:409-428) into
 * nw words (zero padded); returns the number of words found. */
static int bm_parse(const uint8_t *bm, size_t bm_len, int mode, uint32_t *words, size_t nw) {
  uint8_t *bin = NULL;
  size_t blen = 0;
  if (mode == OR_BM_ROARING) { /* Bitmap::deserialize; rows past the words are not kept */
    uint32_t *rows = NULL;
    size_t cnt = 0;
    int rc = or_roaring_parse(bm, bm_len, &rows, &cnt);
    if (rc) return rc;
    memset(words, 0, nw * 4);
    for (size_t i = 0; i < cnt; i++)
      if ((rows[i] >> 5) < nw) words[rows[i] >> 5] |= 1u << (rows[i] & 31);
    free(rows);
    return OR_OK;
  }
  if (mode == OR_BM_RAW) {
    bin = (uint8_t *)bm;
    blen = bm_len;
  } else {
    if (or_snappy_decompress(bm, bm_len, NULL, 0, &blen)) return OR_PANIC;
    bin = (uint8_t *)malloc(blen ? blen : 1);
    if (!bin) return OR_ENOMEM;
    if (or_snappy_decompress(bm, bm_len, bin, blen, &blen)) {
      free(bin);
      return OR_PANIC;
    }
  }
  memset(words, 0, nw * 4);
  if (blen < 8) {
    if (mode != OR_BM_RAW) free(bin);
    return OR_PANIC;
  }
  uint64_t nbits = 0;
  for (int i = 0; i < 8; i++) nbits |= (uint64_t)bin[i] << (8 * i);
  size_t cnt = 8, lim = blen - 4, j = 0;
  while (cnt <= lim && j < nw) {
    words[j++] = ld32(bin + cnt);
    cnt += 4;
  }
  if (nw && (nbits & 31) && (nbits + 31) / 32 <= nw) words[(nbits + 31) / 32 - 1] &= (1u << (nbits & 31)) - 1u;
  if (mode != OR_BM_RAW) free(bin);
  return OR_OK;
}

static inline size_t nwords_of(uint64_t n) { return (size_t)((n + 31) / 32); }
static inline int bit_of(const uint32_t *w, size_t i) { return (w[i >> 5] >> (i & 31)) & 1u; }
static inline void set_bit(uint32_t *w, size_t i) { w[i >> 5] |= 1u << (i & 31); }
static uint64_t card(const uint32_t *w, size_t nw) {
  uint64_t c = 0;
  for (size_t i = 0; i < nw; i++) c += (uint64_t)__builtin_popcount(w[i]);
  return c;
}
static void negate(uint32_t *w, size_t nw, uint64_t nbits) { /* BitVec::negate */
  for (size_t i = 0; i < nw; i++) w[i] = ~w[i];
  if (nw && (nbits & 31)) w[nw - 1] &= (1u << (nbits & 31)) - 1u;
}

/* ------------------------------------------------------------------ */
/* buff_encode_majority (compress/buff_simd.rs:317-630)                */
/* ------------------------------------------------------------------ */

static int encode_major(const double *x, uint32_t n, uint64_t scale, int bm_mode, int forced,
                        uint8_t **out, size_t *out_len);

int or_encode_majority(const double *x, uint32_t n, uint64_t scale, int bm_mode, uint8_t **out,
                       size_t *out_len) {
  return encode_major(x, n, scale, bm_mode, -1, out, out_len);
}

/* byte_residue_encode_outlieru8 (split_double.rs:957-1240) runs the same
 * Boyer-Moore vote over the leading byte of the first 2000 codes, then
 * overwrites its result with MAJOR = 69 (:1049, outlier/mod.rs:11); the
 * vote's count is never negative, so the leading byte is always the one
 * sparse column (:1051-1054).  The image is the buff-major image with a
 * croaring bitmap per column. */
int or_encode_outlieru8(const double *x, uint32_t n, uint64_t scale, uint8_t **out,
                        size_t *out_len) {
  return encode_major(x, n, scale, OR_BM_ROARING, 69, out, out_len);
}

static int encode_major(const double *x, uint32_t n, uint64_t scale, int bm_mode, int forced,
                        uint8_t **out, size_t *out_len) {
  int prec = or_prec_of_scale(scale);
  int dl = or_dlen_of_prec(prec);
  if (dl < 0) return OR_PANIC;
  int pexp = or_precision_exp(prec);
  uint64_t dec_len = (uint64_t)dl;
  int64_t *fixed = (int64_t *)malloc((size_t)(n ? n : 1) * 8);
  if (!fixed) return OR_ENOMEM;
  int64_t mn = INT64_MAX, mx = INT64_MIN;
  for (uint32_t i = 0; i < n; i++) { /* two ifs here (:340-347) */
    int64_t f = or_fetch_fixed_aligned(x[i], pexp, dec_len);
    if (f < mn) mn = f;
    if (f > mx) mx = f;
    fixed[i] = f;
  }
  int64_t delta = (int64_t)((uint64_t)mx - (uint64_t)mn), base = mn;
  uint32_t fl = delta == 0 ? 0u : or_fixed_len_of_delta(delta);
  uint64_t ilen = (uint64_t)fl - dec_len;
  or_bw w;
  or_bw_init(&w);
  uint64_t ub = (uint64_t)base;
  int rc = 0;
  uint32_t *bm = NULL;
  uint8_t *outl = NULL;
  rc |= or_bw_write(&w, (uint32_t)ub, 32);
  rc |= or_bw_write(&w, (uint32_t)(ub >> 32), 32);
  rc |= or_bw_write(&w, n, 32);
  rc |= or_bw_write(&w, (uint32_t)ilen, 32);
  rc |= or_bw_write(&w, (uint32_t)dec_len, 32);
  if (rc) goto fail;
  uint32_t remain = fl;
  if (n < SAMPLE) { /* fixed_vec[0..SAMPLE] */
    rc = OR_PANIC;
    goto fail;
  }
  /* Boyer-Moore majority of the leading byte over the first SAMPLE rows,
   * then of each following byte while it stays a majority (:382-446). */
  uint32_t rsf = fl >= 8 ? fl - 8 : 0;
  const int32_t m_limit = (int32_t)((float)SAMPLE * 0.6f);
  uint8_t majors[8];
  int ncols = 0;
  {
    int32_t freq = 0;
    uint8_t major = 0;
    for (int i = 0; i < SAMPLE; i++) {
      uint8_t b = (uint8_t)((uint64_t)(fixed[i] - base) >> rsf);
      if (freq == 0) {
        major = b;
        freq = 1;
      } else if (major == b)
        freq++;
      else
        freq--;
    }
    if (forced >= 0) {
      majors[ncols++] = (uint8_t)forced;
    } else if (freq > m_limit) {
      majors[ncols++] = major;
      while (rsf > 7 && ncols < 8) {
        rsf -= 8;
        freq = 0;
        major = 0;
        for (int i = 0; i < SAMPLE; i++) {
          uint8_t b = (uint8_t)((uint64_t)(fixed[i] - base) >> rsf);
          if (freq == 0) {
            major = b;
            freq = 1;
          } else if (major == b)
            freq++;
          else
            freq--;
        }
        if (freq > m_limit)
          majors[ncols++] = major;
        else
          break;
      }
    }
  }
  size_t nw = nwords_of(n);
  if (ncols > 0) {
    if (remain < 8) { /* `remain -= 8` underflows */
      rc = OR_PANIC;
      goto fail;
    }
    if ((rc = or_bw_write(&w, (uint32_t)ncols, 8))) goto fail;
    bm = (uint32_t *)malloc(nw * 4);
    outl = (uint8_t *)malloc(n);
    if (!bm || !outl) {
      rc = OR_ENOMEM;
      goto fail;
    }
    for (int c = 0; c < ncols; c++) {
      remain -= 8;
      memset(bm, 0, nw * 4);
      uint32_t nout = 0;
      for (uint32_t i = 0; i < n; i++) {
        uint8_t b = (uint8_t)((uint64_t)(fixed[i] - base) >> remain);
        if (b != majors[c]) {
          outl[nout++] = b;
          set_bit(bm, i);
        }
      }
      uint8_t *bmb = NULL;
      size_t bml = 0;
      if ((rc = bm_serialize(bm, nw, n, bm_mode, &bmb, &bml))) goto fail;
      rc |= or_bw_write(&w, majors[c], 8);
      rc |= or_bw_write(&w, (uint32_t)bml, 32);
      rc |= or_bw_write_bytes(&w, bmb, bml);
      free(bmb);
      rc |= or_bw_finish_write_byte(&w);
      rc |= or_bw_write(&w, nout, 32);
      rc |= or_bw_write_bytes(&w, outl, nout);
      rc |= or_bw_finish_write_byte(&w);
      if (rc) goto fail;
    }
    while (remain >= 8) {
      remain -= 8;
      size_t l = w.len;
      for (uint32_t i = 0; i < n; i++)
        if ((rc = or_bw_write_byte(&w, (uint8_t)((uint64_t)(fixed[i] - base) >> remain)))) goto fail;
      (void)l;
    }
    if (remain > 0) {
      if ((rc = or_bw_finish_write_byte(&w))) goto fail;
      for (uint32_t i = 0; i < n; i++)
        if ((rc = or_bw_write_bits(&w, (uint32_t)(uint64_t)(fixed[i] - base), remain))) goto fail;
    }
  } else {
    if ((rc = or_bw_write_byte(&w, 0))) goto fail;
    if (remain < 8) {
      for (uint32_t i = 0; i < n; i++)
        if ((rc = or_bw_write_bits(&w, (uint32_t)(uint64_t)(fixed[i] - base), remain))) goto fail;
    } else {
      remain -= 8;
      for (uint32_t i = 0; i < n; i++)
        if ((rc = or_bw_write_byte(&w, (uint8_t)((uint64_t)(fixed[i] - base) >> remain)))) goto fail;
      while (remain >= 8) {
        remain -= 8;
        for (uint32_t i = 0; i < n; i++)
          if ((rc = or_bw_write_byte(&w, (uint8_t)((uint64_t)(fixed[i] - base) >> remain)))) goto fail;
      }
      if (remain > 0) {
        if ((rc = or_bw_finish_write_byte(&w))) goto fail;
        for (uint32_t i = 0; i < n; i++)
          if ((rc = or_bw_write_bits(&w, (uint32_t)(uint64_t)(fixed[i] - base), remain))) goto fail;
      }
    }
  }
  free(fixed);
  free(bm);
  free(outl);
  *out = w.buf;
  *out_len = w.len;
  return OR_OK;
fail:
  free(fixed);
  free(bm);
  free(outl);
  or_bw_free(&w);
  return rc;
}

/* ------------------------------------------------------------------ */
/* shared walk of the sparse columns                                    */
/* ------------------------------------------------------------------ */

typedef struct maj_col {
  uint8_t major;
  uint32_t nout;
  const uint8_t *outl;
  uint32_t *bm; /* decompressed outlier rows */
} maj_col;

typedef struct maj_view {
  or_header h;
  uint32_t ncols;
  maj_col col[8];
  uint32_t remain; /* bits left after the sparse columns */
} maj_view;

static void maj_free(maj_view *v) {
  for (uint32_t c = 0; c < v->ncols && c < 8; c++) free(v->col[c].bm);
}

/* Reads the header, the column count and every sparse column the way the
 * queries do (read(8) major, read(32) size, read_n_byte(bitmap),
 * finish_read_byte, read(32) count, read_n_byte(outliers),
 * finish_read_byte); leaves `br` where the dense slices start. */
static int maj_open(or_br *br, const uint8_t *bytes, size_t len, int bm_mode, maj_view *v) {
  memset(v, 0, sizeof(*v));
  or_br_init(br, bytes, len);
  uint32_t lo, hi, n, ilen, dlen, cols;
  if (or_br_read(br, 32, &lo) || or_br_read(br, 32, &hi) || or_br_read(br, 32, &n) ||
      or_br_read(br, 32, &ilen) || or_br_read(br, 32, &dlen))
    return OR_PANIC;
  v->h.base = (int64_t)((uint64_t)lo | ((uint64_t)hi << 32));
  v->h.n = n;
  v->h.ilen = ilen;
  v->h.dlen = dlen;
  v->h.fixed_len = ilen + dlen;
  if (or_br_read(br, 8, &cols)) return OR_PANIC;
  if (cols > 8) return OR_PANIC;
  v->ncols = cols;
  v->remain = v->h.fixed_len;
  size_t nw = nwords_of(n);
  for (uint32_t c = 0; c < cols; c++) {
    uint32_t major, bml, nout;
    const uint8_t *bmp, *outl;
    if (v->remain < 8) return OR_PANIC;
    v->remain -= 8;
    if (or_br_read(br, 8, &major) || or_br_read(br, 32, &bml)) return OR_PANIC;
    if (or_br_read_n_byte(br, bml, &bmp)) return OR_PANIC;
    v->col[c].bm = (uint32_t *)calloc(nw ? nw : 1, 4);
    if (!v->col[c].bm) return OR_ENOMEM;
    if (bm_parse(bmp, bml, bm_mode, v->col[c].bm, nw)) return OR_PANIC;
    or_br_finish_read_byte(br);
    if (or_br_read(br, 32, &nout)) return OR_PANIC;
    if (or_br_read_n_byte(br, nout, &outl)) return OR_PANIC;
    or_br_finish_read_byte(br);
    v->col[c].major = (uint8_t)major;
    v->col[c].nout = nout;
    v->col[c].outl = outl;
  }
  return OR_OK;
}

int or_majority_layout(const uint8_t *bytes, size_t len, int bm_mode, uint32_t *ncols,
                       uint8_t *majors, uint32_t *nouts, size_t *dense_off) {
  or_br br;
  maj_view v;
  int rc = maj_open(&br, bytes, len, bm_mode, &v);
  if (!rc) {
    *ncols = v.ncols;
    for (uint32_t c = 0; c < v.ncols; c++) {
      majors[c] = v.col[c].major;
      nouts[c] = v.col[c].nout;
    }
    *dense_off = br.cursor + 1; /* read_n_byte pre-increments */
  }
  maj_free(&v);
  return rc;
}

/* ------------------------------------------------------------------ */
/* buff_decode_majority (compress/buff_simd.rs:633-861)                 */
/* ------------------------------------------------------------------ */

int or_decode_majority(const uint8_t *bytes, size_t len, uint64_t scale, int bm_mode, double *out) {
  (void)scale;
  or_br br;
  maj_view v;
  int rc = maj_open(&br, bytes, len, bm_mode, &v);
  if (rc) {
    maj_free(&v);
    return rc;
  }
  uint32_t n = v.h.n;
  double dec_scl = ldexp(1.0, (int)v.h.dlen);
  uint64_t *fv = (uint64_t *)calloc(n ? n : 1, 8);
  if (!fv) {
    maj_free(&v);
    return OR_ENOMEM;
  }
  uint32_t remain = v.h.fixed_len;
  if (v.ncols == 0) {
    maj_free(&v);
    free(fv);
    /* no sparse column: the buff layout one byte later */
    or_br br2;
    or_br_init(&br2, bytes, len);
    or_header h;
    uint32_t t;
    or_br_read(&br2, 32, &t);
    or_br_read(&br2, 32, &t);
    or_br_read(&br2, 32, &t);
    or_br_read(&br2, 32, &t);
    or_br_read(&br2, 32, &t);
    or_br_read(&br2, 8, &t);
    (void)h;
    /* reuse the generic walk via a re-based header */
    or_header hh;
    hh.base = v.h.base;
    hh.n = v.h.n;
    hh.ilen = v.h.ilen;
    hh.dlen = v.h.dlen;
    hh.fixed_len = v.h.fixed_len;
    remain = hh.fixed_len;
    double scl = ldexp(1.0, (int)hh.dlen);
    if (remain < 8) {
      for (uint32_t i = 0; i < n; i++) {
        uint8_t cur;
        if (or_br_read_bits(&br2, remain, &cur)) return OR_PANIC;
        out[i] = (double)(int64_t)((uint64_t)hh.base + cur) / scl;
      }
      return OR_OK;
    }
    uint64_t *f2 = (uint64_t *)calloc(n ? n : 1, 8);
    const uint8_t *chunk;
    while (remain >= 8) {
      remain -= 8;
      if (or_br_read_n_byte(&br2, n, &chunk)) {
        free(f2);
        return OR_PANIC;
      }
      for (uint32_t i = 0; i < n; i++) f2[i] |= (uint64_t)chunk[i] << remain;
    }
    if (remain > 0) {
      or_br_finish_read_byte(&br2);
      for (uint32_t i = 0; i < n; i++) {
        uint8_t b;
        if (or_br_read_bits(&br2, remain, &b)) {
          free(f2);
          return OR_PANIC;
        }
        f2[i] |= b;
      }
    }
    for (uint32_t i = 0; i < n; i++) out[i] = (double)(int64_t)((uint64_t)hh.base + f2[i]) / scl;
    free(f2);
    return OR_OK;
  }
  /* first sparse column */
  remain -= 8;
  uint64_t first_major = (uint64_t)v.col[0].major << remain;
  for (uint32_t i = 0; i < n; i++) fv[i] = first_major;
  if (v.col[0].nout == 0 || card(v.col[0].bm, nwords_of(n)) == 0) {
    rc = OR_PANIC; /* outlier_iter.next().unwrap() / bm_iterator.next().unwrap() */
    goto done;
  }
  {
    uint32_t counter = 0;
    for (uint32_t i = 0; i < n && counter < v.col[0].nout; i++)
      if (bit_of(v.col[0].bm, i)) fv[i] = (uint64_t)v.col[0].outl[counter++] << remain;
  }
  for (uint32_t c = 1; c < v.ncols; c++) {
    remain -= 8;
    uint64_t major_u64 = (uint64_t)v.col[c].major << remain;
    if (v.col[c].nout == 0 || card(v.col[c].bm, nwords_of(n)) == 0) {
      rc = OR_PANIC;
      goto done;
    }
    uint32_t counter = 0;
    for (uint32_t i = 0; i < n; i++) {
      if (bit_of(v.col[c].bm, i)) {
        fv[i] |= (uint64_t)v.col[c].outl[counter] << remain;
        counter++;
        if (counter == v.col[c].nout) break; /* rows after the last outlier get nothing */
      } else {
        fv[i] |= major_u64 << remain; /* shifted twice (:711, :739) */
      }
    }
  }
  {
    const uint8_t *chunk;
    while (remain >= 8) {
      remain -= 8;
      if (or_br_read_n_byte(&br, n, &chunk)) {
        rc = OR_PANIC;
        goto done;
      }
      for (uint32_t i = 0; i < n; i++) fv[i] |= (uint64_t)chunk[i] << remain;
    }
    if (remain > 0) {
      or_br_finish_read_byte(&br);
      for (uint32_t i = 0; i < n; i++) {
        uint8_t b;
        if (or_br_read_bits(&br, remain, &b)) {
          rc = OR_PANIC;
          goto done;
        }
        fv[i] |= b;
      }
    }
    for (uint32_t i = 0; i < n; i++) out[i] = (double)(int64_t)((uint64_t)v.h.base + fv[i]) / dec_scl;
  }
done:
  free(fv);
  maj_free(&v);
  return rc;
}

/* Progressive refinement over dense byte slices (unflipped) and the packed
 * tail, the shared loop of the majority filters (buff_simd.rs:1002-1131). */
static int dense_refine(or_br *br, uint32_t n, uint32_t remain, uint64_t ft, uint32_t *rb1,
                        uint32_t *res, int is_range) {
  size_t nw = nwords_of(n);
  uint32_t *cur = (uint32_t *)calloc(nw ? nw : 1, 4);
  if (!cur) return OR_ENOMEM;
  int rc = OR_OK;
  while (remain > 0) {
    if (remain >= 8) {
      remain -= 8;
      memset(cur, 0, nw * 4);
      if (card(rb1, nw) != 0) {
        uint8_t tar = (uint8_t)(ft >> remain);
        size_t pre = 0;
        int first = 1;
        for (size_t i = 0; i < n; i++) {
          if (!bit_of(rb1, i)) continue;
          if (first) {
            if (i != 0) or_br_skip_n_byte(br, i);
            first = 0;
          } else if (i - pre != 1) {
            or_br_skip_n_byte(br, i - pre - 1);
          }
          uint8_t d;
          if (or_br_read_byte(br, &d)) {
            rc = OR_PANIC;
            goto out;
          }
          if (is_range && d > tar)
            set_bit(res, i);
          else if (d == tar)
            set_bit(cur, i);
          pre = i;
        }
        if (n - pre > 1) or_br_skip_n_byte(br, n - pre - 1);
      } else {
        or_br_skip_n_byte(br, n);
        break;
      }
      memcpy(rb1, cur, nw * 4);
    } else {
      uint8_t tar = (uint8_t)((uint8_t)((uint8_t)ft << (8 - remain)) >> (8 - remain));
      or_br_finish_read_byte(br);
      if (card(rb1, nw) != 0) {
        size_t pre = 0;
        int first = 1;
        for (size_t i = 0; i < n; i++) {
          if (!bit_of(rb1, i)) continue;
          if (first) {
            if (i != 0) or_br_skip(br, i * remain);
            first = 0;
          } else if (i - pre != 1) {
            or_br_skip(br, (i - pre - 1) * remain);
          }
          uint8_t d;
          if (or_br_read_bits(br, remain, &d)) {
            rc = OR_PANIC;
            goto out;
          }
          if (is_range ? (d > tar) : (d == tar)) set_bit(res, i);
          pre = i;
        }
        remain = 0;
      } else {
        break;
      }
    }
  }
out:
  free(cur);
  return rc;
}

/* ------------------------------------------------------------------ */
/* buff_range_filter_majority (compress/buff_simd.rs:863-1277) and      */
/* buff_equal_filter_majority (:1916-2292)                               */
/* ------------------------------------------------------------------ */

static int filter_majority(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                           int bm_mode, int is_range, uint32_t *words, uint64_t *count, int *early) {
  or_br br;
  maj_view v;
  int rc = maj_open(&br, bytes, len, bm_mode, &v);
  if (rc) {
    maj_free(&v);
    return rc;
  }
  uint32_t n = v.h.n;
  size_t nw = nwords_of(n);
  memset(words, 0, nw * 4);
  *early = 0;
  int pexp = or_precision_exp(or_prec_of_scale(scale));
  int64_t fp = or_fetch_fixed_aligned(pred, pexp, v.h.dlen);
  if (fp < v.h.base) {
    *early = 1;
    if (is_range) {
      for (size_t i = 0; i < nw; i++) words[i] = 0xFFFFFFFFu;
      if (n & 31) words[nw - 1] &= (1u << (n & 31)) - 1u;
      *count = n;
    } else {
      *count = 0;
    }
    maj_free(&v);
    return OR_OK;
  }
  uint64_t ft = (uint64_t)(fp - v.h.base);
  uint32_t *res = words;
  uint32_t *rb1 = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t *tmp = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t remain = v.h.fixed_len;
  if (!rb1 || !tmp) {
    rc = OR_ENOMEM;
    goto done;
  }
  if (v.ncols > 0) {
    for (uint32_t c = 0; c < v.ncols; c++) {
      remain -= 8;
      uint8_t tar = (uint8_t)(ft >> remain);
      const maj_col *col = &v.col[c];
      if (!is_range) {
        /* equality (:1956-2033) */
        if (tar == col->major) {
          memcpy(tmp, col->bm, nw * 4);
          negate(tmp, nw, n);
          if (c == 0)
            for (size_t i = 0; i < nw; i++) rb1[i] |= tmp[i];
          else
            for (size_t i = 0; i < nw; i++) rb1[i] &= tmp[i];
        } else {
          memset(tmp, 0, nw * 4);
          uint32_t k = 0;
          for (size_t i = 0; i < n && k < col->nout; i++)
            if (bit_of(col->bm, i)) {
              if (col->outl[k] == tar) set_bit(tmp, i);
              k++;
            }
          if (c == 0)
            memcpy(rb1, tmp, nw * 4);
          else
            for (size_t i = 0; i < nw; i++) rb1[i] &= tmp[i];
        }
        continue;
      }
      if (c == 0) { /* :899-951 */
        if (tar == 0 && col->major == 0) {
          for (size_t i = 0; i < nw; i++) res[i] |= col->bm[i];
          memcpy(tmp, col->bm, nw * 4);
          negate(tmp, nw, n);
          for (size_t i = 0; i < nw; i++) rb1[i] |= tmp[i];
        } else {
          uint32_t k = 0;
          for (size_t i = 0; i < n && k < col->nout; i++)
            if (bit_of(col->bm, i)) {
              uint8_t val = col->outl[k++];
              if (val == tar)
                set_bit(rb1, i);
              else if (val > tar)
                set_bit(res, i);
            }
          memcpy(tmp, col->bm, nw * 4);
          negate(tmp, nw, n);
          if (tar < col->major)
            for (size_t i = 0; i < nw; i++) res[i] |= tmp[i];
          else if (tar == col->major)
            for (size_t i = 0; i < nw; i++) rb1[i] |= tmp[i];
        }
      } else { /* :955-1001 */
        if (tar == 0 && col->major == 0) {
          for (size_t i = 0; i < nw; i++) rb1[i] &= col->bm[i];
          for (size_t i = 0; i < nw; i++) res[i] |= rb1[i];
          memcpy(tmp, col->bm, nw * 4);
          negate(tmp, nw, n);
          for (size_t i = 0; i < nw; i++) rb1[i] &= tmp[i]; /* leaves rb1 empty */
        } else {
          uint32_t *cur_rb = (uint32_t *)calloc(nw ? nw : 1, 4);
          if (!cur_rb) {
            rc = OR_ENOMEM;
            goto done;
          }
          uint32_t k = 0;
          for (size_t i = 0; i < n && k < col->nout; i++)
            if (bit_of(col->bm, i)) {
              uint8_t val = col->outl[k++];
              if (val == tar)
                set_bit(cur_rb, i);
              else if (val > tar)
                set_bit(res, i); /* not restricted to the candidates */
            }
          memcpy(tmp, col->bm, nw * 4);
          negate(tmp, nw, n);
          if (tar < col->major) {
            for (size_t i = 0; i < nw; i++) res[i] |= tmp[i] & rb1[i];
          } else if (tar == col->major) {
            for (size_t i = 0; i < nw; i++) cur_rb[i] |= tmp[i];
          }
          for (size_t i = 0; i < nw; i++) rb1[i] &= cur_rb[i];
          free(cur_rb);
        }
      }
    }
  } else {
    /* no sparse column: full compare of the first slice (:1134-1152) */
    if (remain < 8) {
      for (uint32_t i = 0; i < n; i++) {
        uint8_t cur;
        if (or_br_read_bits(&br, remain, &cur)) {
          rc = OR_PANIC;
          goto done;
        }
        if (is_range ? ((uint64_t)cur > ft) : ((uint64_t)cur == ft)) set_bit(res, i);
      }
      remain = 0;
    } else {
      remain -= 8;
      const uint8_t *chunk;
      if (or_br_read_n_byte(&br, n, &chunk)) {
        rc = OR_PANIC;
        goto done;
      }
      uint8_t tar = (uint8_t)(ft >> remain);
      for (uint32_t i = 0; i < n; i++) {
        if (is_range && chunk[i] > tar)
          set_bit(res, i);
        else if (chunk[i] == tar)
          set_bit(rb1, i);
      }
    }
  }
  rc = dense_refine(&br, n, remain, ft, rb1, res, is_range);
done:
  if (rc == OR_OK) *count = card(res, nw);
  free(rb1);
  free(tmp);
  maj_free(&v);
  return rc;
}

int or_range_filter_majority(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                             int bm_mode, uint32_t *words, uint64_t *count, int *early) {
  return filter_majority(bytes, len, scale, pred, bm_mode, 1, words, count, early);
}
int or_equal_filter_majority(const uint8_t *bytes, size_t len, uint64_t scale, double pred,
                             int bm_mode, uint32_t *words, uint64_t *count, int *early) {
  return filter_majority(bytes, len, scale, pred, bm_mode, 0, words, count, early);
}

/* ------------------------------------------------------------------ */
/* buff_sum_majority (compress/buff_simd.rs:2294-2442)                  */
/* ------------------------------------------------------------------ */

int or_sum_majority(const uint8_t *bytes, size_t len, uint64_t scale, int bm_mode, double *sum_out,
                    uint64_t *partials) {
  (void)scale;
  or_br br;
  maj_view v;
  int rc = maj_open(&br, bytes, len, bm_mode, &v);
  if (rc) {
    maj_free(&v);
    return rc;
  }
  uint32_t n = v.h.n, remain = v.h.fixed_len, slot = 0;
  int32_t processed = 0, ilen_i = (int32_t)v.h.ilen;
  double sum_base = (double)n * (double)v.h.base;
  sum_base = sum_base / ldexp(1.0, (int)v.h.dlen);
  double sum = 0.0;
  for (uint32_t c = 0; c < v.ncols; c++) {
    remain -= 8;
    processed += 8;
    uint64_t sf = 0;
    for (uint32_t k = 0; k < v.col[c].nout; k++) sf += v.col[c].outl[k];
    sf += (uint64_t)v.col[c].major * ((uint64_t)n - v.col[c].nout);
    if (partials) partials[slot] = sf;
    slot++;
    sum = sum + (double)sf / ldexp(1.0, processed - ilen_i);
  }
  while (remain >= 8) {
    remain -= 8;
    processed += 8;
    const uint8_t *chunk;
    if (or_br_read_n_byte(&br, n, &chunk)) {
      rc = OR_PANIC;
      goto done;
    }
    uint64_t sf = 0;
    for (uint32_t i = 0; i < n; i++) sf += chunk[i];
    if (partials) partials[slot] = sf;
    slot++;
    sum = sum + (double)sf / ldexp(1.0, processed - ilen_i);
    if (remain == 0) {
      *sum_out = sum;
      goto done;
    }
  }
  if (remain > 0) {
    if (processed >= 8) or_br_finish_read_byte(&br);
    processed += (int32_t)remain;
    uint64_t sf = 0;
    for (uint32_t i = 0; i < n; i++) {
      uint8_t b;
      if (or_br_read_bits(&br, remain, &b)) {
        rc = OR_PANIC;
        goto done;
      }
      sf += b;
    }
    if (partials) partials[slot] = sf;
    sum = sum + (double)sf / ldexp(1.0, processed - ilen_i);
  }
  sum += sum_base;
  *sum_out = sum;
done:
  maj_free(&v);
  return rc;
}

/* ------------------------------------------------------------------ */
/* buff_max_majority (compress/buff_simd.rs:2444-2861)                  */
/* ------------------------------------------------------------------ */

int or_max_majority(const uint8_t *bytes, size_t len, uint64_t scale, int bm_mode, double *maxv,
                    uint64_t *max_code, uint32_t *argmax_words, uint64_t *argmax_count) {
  (void)scale;
  or_br br;
  maj_view v;
  int rc = maj_open(&br, bytes, len, bm_mode, &v);
  if (rc) {
    maj_free(&v);
    return rc;
  }
  uint32_t n = v.h.n, remain = v.h.fixed_len;
  size_t nw = nwords_of(n);
  uint32_t *rb1 = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t *cur = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint32_t *res = (uint32_t *)calloc(nw ? nw : 1, 4);
  uint64_t mx = 0;
  if (!rb1 || !cur || !res) {
    rc = OR_ENOMEM;
    goto done;
  }
  if (v.ncols > 0) {
    /* first sparse column (:2468-2497) */
    uint8_t byte_max = v.col[0].major;
    remain -= 8;
    memcpy(rb1, v.col[0].bm, nw * 4);
    negate(rb1, nw, n);
    uint32_t k = 0;
    for (size_t i = 0; i < n && k < v.col[0].nout; i++)
      if (bit_of(v.col[0].bm, i)) {
        uint8_t val = v.col[0].outl[k++];
        if (val > byte_max) {
          byte_max = val;
          memset(rb1, 0, nw * 4);
          set_bit(rb1, i);
        } else if (val == byte_max) {
          set_bit(rb1, i);
        }
      }
    mx |= (uint64_t)byte_max << remain;
    for (uint32_t c = 1; c < v.ncols; c++) { /* :2499-2557 */
      byte_max = v.col[c].major;
      remain -= 8;
      memcpy(cur, v.col[c].bm, nw * 4);
      negate(cur, nw, n);
      for (size_t i = 0; i < nw; i++) cur[i] &= rb1[i];
      for (size_t i = 0; i < nw; i++) rb1[i] &= v.col[c].bm[i];
      if (card(rb1, nw) == 0) {
        memcpy(rb1, cur, nw * 4);
        continue; /* the major byte is never added to max */
      }
      k = 0;
      for (size_t i = 0; i < n && k < v.col[c].nout; i++)
        if (bit_of(v.col[c].bm, i)) {
          uint8_t val = v.col[c].outl[k++];
          if (!bit_of(rb1, i)) continue;
          if (val > byte_max) {
            byte_max = val;
            memset(cur, 0, nw * 4);
            set_bit(cur, i);
          } else if (val == byte_max) {
            set_bit(cur, i);
          }
        }
      memcpy(rb1, cur, nw * 4);
      mx |= (uint64_t)byte_max << remain;
    }
  } else {
    if (remain < 8) {
      for (uint32_t i = 0; i < n; i++) {
        uint8_t c;
        if (or_br_read_bits(&br, remain, &c)) {
          rc = OR_PANIC;
          goto done;
        }
        if ((uint64_t)c > mx) {
          mx = c;
          memset(res, 0, nw * 4);
          set_bit(res, i);
        } else if ((uint64_t)c == mx) {
          set_bit(res, i);
        }
      }
      remain = 0;
    } else {
      remain -= 8;
      const uint8_t *chunk;
      if (or_br_read_n_byte(&br, n, &chunk)) {
        rc = OR_PANIC;
        goto done;
      }
      uint8_t byte_max = 0;
      for (uint32_t i = 0; i < n; i++) {
        if (chunk[i] > byte_max) {
          byte_max = chunk[i];
          memset(rb1, 0, nw * 4);
          set_bit(rb1, i);
        } else if (chunk[i] == byte_max) {
          set_bit(rb1, i);
        }
      }
      mx = (uint64_t)byte_max << remain;
    }
  }
  while (remain > 0) { /* dense slices and tail (:2560-2651) */
    uint8_t byte_max = 0;
    if (remain >= 8) {
      remain -= 8;
      memset(cur, 0, nw * 4);
      size_t pre = 0;
      int first = 1;
      for (size_t i = 0; i < n; i++) {
        if (!bit_of(rb1, i)) continue;
        if (first) {
          if (i != 0) or_br_skip_n_byte(&br, i);
        } else if (i - pre != 1) {
          or_br_skip_n_byte(&br, i - pre - 1);
        }
        uint8_t d;
        if (or_br_read_byte(&br, &d)) {
          rc = OR_PANIC;
          goto done;
        }
        if (first) {
          if (d > byte_max) byte_max = d;
          set_bit(cur, i);
          first = 0;
        } else if (d > byte_max) {
          byte_max = d;
          memset(cur, 0, nw * 4);
          set_bit(cur, i);
        } else if (d == byte_max) {
          set_bit(cur, i);
        }
        pre = i;
      }
      if (n - pre > 1) or_br_skip_n_byte(&br, n - pre - 1);
      mx |= (uint64_t)byte_max << remain;
      memcpy(rb1, cur, nw * 4);
    } else {
      or_br_finish_read_byte(&br);
      size_t pre = 0;
      int first = 1;
      for (size_t i = 0; i < n; i++) {
        if (!bit_of(rb1, i)) continue;
        if (first) {
          if (i != 0) or_br_skip(&br, i * remain);
        } else if (i - pre != 1) {
          or_br_skip(&br, (i - pre - 1) * remain);
        }
        uint8_t d;
        if (or_br_read_bits(&br, remain, &d)) {
          rc = OR_PANIC;
          goto done;
        }
        if (d > byte_max) {
          byte_max = d;
          if (!first) memset(res, 0, nw * 4);
          set_bit(res, i);
        } else if (d == byte_max) {
          set_bit(res, i);
        }
        first = 0;
        pre = i;
      }
      remain = 0;
      mx |= (uint64_t)byte_max;
    }
  }
  *max_code = mx;
  *maxv = (double)(int64_t)((uint64_t)v.h.base + mx) / ldexp(1.0, (int)v.h.dlen);
  if (argmax_words) memcpy(argmax_words, res, nw * 4);
  if (argmax_count) *argmax_count = card(res, nw);
done:
  free(rb1);
  free(cur);
  free(res);
  maj_free(&v);
  return rc;
}
