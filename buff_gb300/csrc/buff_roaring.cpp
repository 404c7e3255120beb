// Roaring portable format, host side.
//
// A bitmap is a sorted list of containers, one per 65536-row block (key =
// row >> 16).  A container built by ascending adds is an array of 16-bit
// values while it holds at most 4096 of them and a 65536-bit bitset beyond;
// run optimization then turns it into a list of (start, length - 1) runs
// whenever 2 + 4 * runs bytes are fewer than its current form (2 + 2 * card
// for an array, 8192 for a bitset).
//
// Image: a u32 cookie -- 12346 followed by the u32 container count when no
// container is a run list, else 12347 | (count - 1) << 16 followed by one
// bit per container marking the run lists -- then (key, card - 1) as two
// u16 per container, then (without run lists, or with at least 4
// containers) the u32 byte offset of every container, then the containers:
// an array as its u16 values, a bitset as 1024 little-endian u64 words, a
// run list as a u16 run count and the (start, length - 1) u16 pairs.
// Everything is little-endian.
//
// Here the containers are cut straight out of BitVec<u32> words: a block is
// 2048 words, its cardinality a popcount and its run count the number of
// set bits whose predecessor is clear.
#include "buff_roaring.h"

#include <string.h>

namespace buffroaring {
namespace {

constexpr uint32_t kCookieRun = 12347;
constexpr uint32_t kCookieNoRun = 12346;
constexpr uint32_t kNoOffsetBelow = 4;
constexpr uint32_t kArrayMax = 4096;
constexpr uint32_t kWordsPerBlock = 2048;

enum Kind : uint32_t { kArray, kBitset, kRuns };

struct Block {
  uint32_t key, card, runs;
  Kind kind;
};

void put16(std::vector<uint8_t> &v, uint32_t x) {
  v.push_back((uint8_t)x);
  v.push_back((uint8_t)(x >> 8));
}
void put32(std::vector<uint8_t> &v, uint32_t x) {
  for (int i = 0; i < 4; ++i) v.push_back((uint8_t)(x >> (8 * i)));
}
uint32_t get16(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
uint32_t get32(const uint8_t *p) {
  return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

uint32_t block_bytes(const Block &b) {
  if (b.kind == kRuns) return 2 + 4 * b.runs;
  if (b.kind == kBitset) return 8192;
  return 2 * b.card;
}

}  // namespace

std::vector<uint8_t> serialize(const uint32_t *words, uint32_t n) {
  const size_t nw = ((size_t)n + 31) / 32;
  std::vector<Block> blocks;
  for (size_t w0 = 0; w0 < nw; w0 += kWordsPerBlock) {
    const size_t w1 = w0 + kWordsPerBlock < nw ? w0 + kWordsPerBlock : nw;
    uint32_t card = 0, runs = 0, prev_msb = 0;
    for (size_t w = w0; w < w1; ++w) {
      const uint32_t x = words[w];
      card += (uint32_t)__builtin_popcount(x);
      runs += (uint32_t)__builtin_popcount(x & ~((x << 1) | prev_msb));
      prev_msb = x >> 31;
    }
    if (!card) continue;
    Block b{(uint32_t)(w0 / kWordsPerBlock), card, runs, card > kArrayMax ? kBitset : kArray};
    const uint32_t as_runs = 2 + 4 * runs;
    if (b.kind == kArray ? as_runs < 2 + 2 * card : as_runs < 8192) b.kind = kRuns;
    blocks.push_back(b);
  }
  const uint32_t nb = (uint32_t)blocks.size();
  bool any_runs = false;
  for (const Block &b : blocks) any_runs |= b.kind == kRuns;
  std::vector<uint8_t> out;
  uint32_t start;
  if (any_runs) {
    put32(out, kCookieRun | ((nb - 1) << 16));
    std::vector<uint8_t> flags((nb + 7) / 8, 0);
    for (uint32_t i = 0; i < nb; ++i)
      if (blocks[i].kind == kRuns) flags[i / 8] |= (uint8_t)(1u << (i % 8));
    out.insert(out.end(), flags.begin(), flags.end());
    start = 4 + (uint32_t)flags.size() + (nb < kNoOffsetBelow ? 4 * nb : 8 * nb);
  } else {
    put32(out, kCookieNoRun);
    put32(out, nb);
    start = 8 + 8 * nb;
  }
  for (const Block &b : blocks) {
    put16(out, b.key);
    put16(out, b.card - 1);
  }
  if (!any_runs || nb >= kNoOffsetBelow) {
    uint32_t off = start;
    for (const Block &b : blocks) {
      put32(out, off);
      off += block_bytes(b);
    }
  }
  for (const Block &b : blocks) {
    const uint32_t *bw = words + (size_t)b.key * kWordsPerBlock;
    const size_t have = nw - (size_t)b.key * kWordsPerBlock;
    const size_t cnt = have < kWordsPerBlock ? have : kWordsPerBlock;
    if (b.kind == kBitset) {
      const size_t at = out.size();
      out.resize(at + 8192, 0);
      memcpy(out.data() + at, bw, cnt * 4);  // u32 words, little-endian: the u64 layout
    } else if (b.kind == kArray) {
      for (size_t w = 0; w < cnt; ++w)
        for (uint32_t x = bw[w]; x; x &= x - 1) put16(out, (uint32_t)(w * 32) + __builtin_ctz(x));
    } else {
      put16(out, b.runs);
      bool in = false;
      uint32_t s = 0;
      for (size_t w = 0; w <= cnt; ++w) {
        const uint32_t x = w < cnt ? bw[w] : 0u;
        for (uint32_t j = 0; j < 32; ++j) {
          const bool set = (x >> j) & 1u;
          const uint32_t v = (uint32_t)(w * 32) + j;
          if (set && !in) {
            s = v;
            in = true;
          } else if (!set && in) {
            put16(out, s);
            put16(out, v - 1 - s);
            in = false;
          }
          if (w == cnt) break;
        }
      }
    }
  }
  return out;
}

bool parse(const uint8_t *b, size_t len, std::vector<uint32_t> &rows) {
  rows.clear();
  if (len < 4) return false;
  const uint32_t cookie = get32(b);
  bool any_runs;
  size_t p, nb;
  if ((cookie & 0xFFFFu) == kCookieRun) {
    any_runs = true;
    nb = (cookie >> 16) + 1;
    p = 4 + (nb + 7) / 8;
  } else if (cookie == kCookieNoRun) {
    if (len < 8) return false;
    any_runs = false;
    nb = get32(b + 4);
    p = 8;
  } else {
    return false;
  }
  if (nb > 65536 || p + 4 * nb > len) return false;
  const uint8_t *flags = b + 4, *hdr = b + p;
  p += 4 * nb;
  if (!any_runs || nb >= kNoOffsetBelow) p += 4 * nb;
  if (p > len) return false;
  int64_t prev = -1;
  for (size_t i = 0; i < nb; ++i) {
    const uint32_t key = get16(hdr + 4 * i), card = get16(hdr + 4 * i + 2) + 1;
    const bool is_runs = any_runs && ((flags[i / 8] >> (i % 8)) & 1u);
    const size_t before = rows.size();
    if (is_runs) {
      if (p + 2 > len) return false;
      const uint32_t nr = get16(b + p);
      if (p + 2 + 4 * (size_t)nr > len) return false;
      for (uint32_t r = 0; r < nr; ++r) {
        const uint32_t v0 = get16(b + p + 2 + 4 * r), l = get16(b + p + 4 + 4 * r);
        if (v0 + l > 0xFFFFu || rows.size() - before + l + 1 > card) return false;
        for (uint32_t v = v0; v <= v0 + l; ++v) rows.push_back((key << 16) | v);
      }
      p += 2 + 4 * (size_t)nr;
    } else if (card > kArrayMax) {
      if (p + 8192 > len) return false;
      for (uint32_t w = 0; w < 2048; ++w) {
        uint32_t x = get32(b + p + 4 * w);
        for (; x; x &= x - 1) rows.push_back((key << 16) | (w * 32 + __builtin_ctz(x)));
      }
      p += 8192;
    } else {
      if (p + 2 * (size_t)card > len) return false;
      for (uint32_t j = 0; j < card; ++j) rows.push_back((key << 16) | get16(b + p + 2 * j));
      p += 2 * (size_t)card;
    }
    if (rows.size() - before != card) return false;
    for (size_t j = before; j < rows.size(); ++j) {
      if ((int64_t)rows[j] <= prev) return false;
      prev = rows[j];
    }
  }
  return true;
}

}  // namespace buffroaring
