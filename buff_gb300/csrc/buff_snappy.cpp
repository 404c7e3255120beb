// Snappy raw-format codec for the outlier bitmaps of the buff-major layout.
//
// The reference compresses each outlier bitmap (BitVec::to_binary) with
// parity-snappy (query/bit_vec_iter.rs:61-71).  The format is the published
// snappy raw format: a varint uncompressed length, then literal and copy
// elements.  The compressor here implements the published snappy algorithm
// (64 KiB blocks, 4-byte hashing into a 2^8..2^14 table, a skip that grows on
// misses, greedy match extension); the decompressor accepts any valid stream.
#include "buff_snappy.h"

#include <string.h>

#include <vector>

namespace buffsnappy {

namespace {

inline uint32_t load32(const uint8_t *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

inline uint32_t hash4(const uint8_t *p, int shift) { return (load32(p) * 0x1e35a7bdu) >> shift; }

void put_literal(std::vector<uint8_t> &out, const uint8_t *p, size_t len) {
  const size_t n = len - 1;
  if (n < 60) {
    out.push_back((uint8_t)(n << 2));
  } else {
    uint8_t tmp[4];
    int cnt = 0;
    for (size_t v = n; v; v >>= 8) tmp[cnt++] = (uint8_t)v;
    out.push_back((uint8_t)((59 + cnt) << 2));
    out.insert(out.end(), tmp, tmp + cnt);
  }
  out.insert(out.end(), p, p + len);
}

void put_copy_short(std::vector<uint8_t> &out, size_t offset, size_t len) {
  if (len < 12 && offset < 2048) {  // 1-byte offset form: lengths 4..11
    out.push_back((uint8_t)(1 | ((len - 4) << 2) | ((offset >> 8) << 5)));
    out.push_back((uint8_t)offset);
  } else {  // 2-byte offset form: lengths 1..64
    out.push_back((uint8_t)(2 | ((len - 1) << 2)));
    out.push_back((uint8_t)offset);
    out.push_back((uint8_t)(offset >> 8));
  }
}

void put_copy(std::vector<uint8_t> &out, size_t offset, size_t len) {
  while (len >= 68) {
    put_copy_short(out, offset, 64);
    len -= 64;
  }
  if (len > 64) {
    put_copy_short(out, offset, 60);
    len -= 60;
  }
  put_copy_short(out, offset, len);
}

void compress_block(const uint8_t *in, size_t n, std::vector<uint8_t> &out,
                    std::vector<uint16_t> &table) {
  int bits = 8;
  while (bits < 14 && ((size_t)1 << bits) < n) ++bits;
  const int shift = 32 - bits;
  table.assign((size_t)1 << bits, 0);
  const uint8_t *ip = in, *end = in + n, *emit = in;
  if (n >= 15) {
    const uint8_t *limit = in + n - 15;
    uint32_t next_hash = hash4(++ip, shift);
    for (;;) {
      uint32_t skip = 32;
      const uint8_t *next = ip, *cand;
      do {
        ip = next;
        const uint32_t h = next_hash;
        const uint32_t step = skip >> 5;
        skip += step;
        next = ip + step;
        if (next > limit) goto tail;
        next_hash = hash4(next, shift);
        cand = in + table[h];
        table[h] = (uint16_t)(ip - in);
      } while (load32(ip) != load32(cand));
      put_literal(out, emit, (size_t)(ip - emit));
      do {
        const uint8_t *start = ip;
        size_t len = 4;
        while (ip + len < end && cand[len] == ip[len]) ++len;
        ip += len;
        put_copy(out, (size_t)(start - cand), len);
        emit = ip;
        if (ip >= limit) goto tail;
        table[hash4(ip - 1, shift)] = (uint16_t)(ip - 1 - in);
        const uint32_t h = hash4(ip, shift);
        cand = in + table[h];
        table[h] = (uint16_t)(ip - in);
      } while (load32(ip) == load32(cand));
      next_hash = hash4(++ip, shift);
    }
  }
tail:
  if (emit < end) put_literal(out, emit, (size_t)(end - emit));
}

}  // namespace

std::vector<uint8_t> compress(const uint8_t *in, size_t n) {
  std::vector<uint8_t> out;
  out.reserve(32 + n + n / 6);
  for (size_t v = n;; v >>= 7) {
    if (v < 0x80) {
      out.push_back((uint8_t)v);
      break;
    }
    out.push_back((uint8_t)(v | 0x80));
  }
  std::vector<uint16_t> table;
  for (size_t off = 0; off < n; off += 65536)
    compress_block(in + off, n - off < 65536 ? n - off : 65536, out, table);
  return out;
}

bool uncompressed_length(const uint8_t *in, size_t n, size_t *len) {
  size_t v = 0;
  for (size_t i = 0, sh = 0; i < n && sh <= 35; ++i, sh += 7) {
    v |= (size_t)(in[i] & 0x7F) << sh;
    if (!(in[i] & 0x80)) {
      *len = v;
      return true;
    }
  }
  return false;
}

bool decompress(const uint8_t *in, size_t n, std::vector<uint8_t> &out) {
  size_t ulen = 0, i = 0;
  if (!uncompressed_length(in, n, &ulen)) return false;
  while (i < n && (in[i] & 0x80)) ++i;
  ++i;
  out.assign(ulen, 0);
  size_t o = 0;
  while (i < n) {
    const uint8_t tag = in[i++];
    size_t len, off;
    switch (tag & 3) {
      case 0: {
        len = (size_t)(tag >> 2) + 1;
        if (len > 60) {
          const size_t nb = len - 60;
          if (i + nb > n) return false;
          size_t v = 0;
          for (size_t k = 0; k < nb; ++k) v |= (size_t)in[i + k] << (8 * k);
          i += nb;
          len = v + 1;
        }
        if (i + len > n || o + len > ulen) return false;
        memcpy(out.data() + o, in + i, len);
        i += len;
        o += len;
        continue;
      }
      case 1:
        if (i + 1 > n) return false;
        len = 4 + ((tag >> 2) & 7);
        off = ((size_t)(tag >> 5) << 8) | in[i];
        i += 1;
        break;
      case 2:
        if (i + 2 > n) return false;
        len = (size_t)(tag >> 2) + 1;
        off = (size_t)in[i] | ((size_t)in[i + 1] << 8);
        i += 2;
        break;
      default:
        if (i + 4 > n) return false;
        len = (size_t)(tag >> 2) + 1;
        off = load32(in + i);
        i += 4;
        break;
    }
    if (off == 0 || off > o || o + len > ulen) return false;
    for (size_t k = 0; k < len; ++k, ++o) out[o] = out[o - off];
  }
  return o == ulen;
}

}  // namespace buffsnappy
