// Device helpers shared by the kernel files of the BUFF library: byte-slice
// SWAR compares, bitmap gathers, streaming loads, the quantizer on raw f64
// bits and the integer int64 -> f64 conversion.  Header-only; every function
// is inlined into its kernel.
#pragma once

#include <cuda_runtime.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

namespace buffk {
namespace dev {

constexpr uint32_t H = 0x80808080u;
constexpr int kThreads = 256;
constexpr int kU = 4;  // independent 16-byte loads a lane keeps in flight in streaming loops

__device__ __forceinline__ uint4 ld_stream(const uint8_t *p) {
  uint4 v;
  asm volatile("ld.global.nc.L1::no_allocate.v4.u32 {%0,%1,%2,%3}, [%4];"
               : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
               : "l"(p));
  return v;
}

// Per-slice compare constants for an unflipped target byte t.
struct ByteTarget {
  uint32_t lo1;  // (t & 0x7f) + 1 in every byte
  uint32_t lo0;  // (t & 0x7f) in every byte
  uint32_t th;   // all ones when t >= 0x80
};

__host__ __device__ __forceinline__ ByteTarget make_target(uint32_t t) {
  ByteTarget b;
  b.lo0 = (t & 0x7Fu) * 0x01010101u;
  b.lo1 = ((t & 0x7Fu) + 1u) * 0x01010101u;
  b.th = (t & 0x80u) ? 0xFFFFFFFFu : 0u;
  return b;
}

// SWAR compare of 4 flipped bytes w (a = w ^ 0x80 unflipped) against t.
// MSB of each byte of *gt is a > t, of *eq is a == t.  No borrow crosses a
// byte: (w|H) - lo1 and (w|H) - lo0 stay within [0, 255] per byte.
__device__ __forceinline__ void cmp4(uint32_t w, const ByteTarget &t, uint32_t &gt,
                                     uint32_t &eq) {
  uint32_t wh = w | H;
  uint32_t d1 = wh - t.lo1;  // MSB: a_lo > t_lo
  uint32_t d0 = wh - t.lo0;  // MSB: a_lo >= t_lo
  // a_hi = ~w_hi.  t_hi = 1: a > t iff a_hi & (a_lo > t_lo); t_hi = 0: a_hi | (a_lo > t_lo).
  gt = ((t.th & ~w & d1) | (~t.th & (~w | d1))) & H;
  eq = d0 & ~d1 & (w ^ t.th) & H;  // a_hi == t_hi  <=>  w_hi != t_hi
}


// The 16 r-bit tail fields of rows [16v, 16v+16): 2r bytes at byte 2r*v.
__device__ __forceinline__ void load_tail16(const uint8_t *tail, uint32_t v, uint32_t r,
                                            unsigned long long &lo, unsigned long long &hi) {
  const uint16_t *p = reinterpret_cast<const uint16_t *>(tail + (size_t)2 * r * v);
  lo = 0;
  hi = 0;
#pragma unroll
  for (uint32_t i = 0; i < 7; ++i) {
    if (i < r) {
      unsigned long long h = __ldg(p + i);
      if (i < 4)
        lo |= h << (16 * i);
      else
        hi |= h << (16 * (i - 4));
    }
  }
}

__device__ __forceinline__ uint32_t field16(unsigned long long lo, unsigned long long hi,
                                            uint32_t i, uint32_t r) {
  uint32_t p = i * r;
  unsigned long long v;
  if (p >= 64)
    v = hi >> (p - 64);
  else if (p + r > 64)
    v = (lo >> p) | (hi << (64 - p));
  else
    v = lo >> p;
  return (uint32_t)v & ((1u << r) - 1u);
}

template <typename T>
__device__ __forceinline__ long long warp_min(long long v) {
  for (int o = 16; o; o >>= 1) {
    long long x = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = x < v ? x : v;
  }
  return v;
}
__device__ __forceinline__ long long warp_max_ll(long long v) {
  for (int o = 16; o; o >>= 1) {
    long long x = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = x > v ? x : v;
  }
  return v;
}
__device__ __forceinline__ unsigned long long warp_max_ull(unsigned long long v) {
  for (int o = 16; o; o >>= 1) {
    unsigned long long x = __shfl_xor_sync(0xFFFFFFFFu, v, o);
    v = x > v ? x : v;
  }
  return v;
}
__device__ __forceinline__ unsigned long long warp_sum_ull(unsigned long long v) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
  return v;
}

// Exact f32 -> f64 widening on the integer pipes (the FP64 pipe of this part
// is narrow): returns the IEEE-754 binary64 bits of the binary32 value `fb`.
__device__ __forceinline__ unsigned long long f32_to_f64_bits(uint32_t fb) {
  const unsigned long long sgn = (unsigned long long)(fb >> 31) << 63;
  const uint32_t e = (fb >> 23) & 0xFFu;
  const uint32_t m = fb & 0x7FFFFFu;
  if (e == 0xFFu)  // inf / NaN (NaN quieted, as the host conversion does)
    return sgn | (0x7FFull << 52) | ((unsigned long long)m << 29) | (m ? (1ull << 51) : 0ull);
  if (e == 0) {
    if (m == 0) return sgn;
    const int p = 31 - __clz(m);  // subnormal: m * 2^-149, leading bit p
    return sgn | ((unsigned long long)(p - 149 + 1023) << 52) |
           (((unsigned long long)m << (52 - p)) & ((1ull << 52) - 1ull));
  }
  return sgn | ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
}

// Raw binary64 bits of the input elements, E per 16-byte vector.
template <typename T>
struct Elem;
template <>
struct Elem<double> {
  using V = ulonglong2;
  static constexpr int E = 2;
  __device__ static unsigned long long bits(const V &v, int j) { return j ? v.y : v.x; }
  __device__ static unsigned long long one(const double *x, uint32_t i) {
    return (unsigned long long)__double_as_longlong(__ldg(x + i));
  }
};
template <>
struct Elem<float> {
  using V = uint4;
  static constexpr int E = 4;
  __device__ static unsigned long long bits(const V &v, int j) {
    return f32_to_f64_bits(j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w);
  }
  __device__ static unsigned long long one(const float *x, uint32_t i) {
    return f32_to_f64_bits((uint32_t)__float_as_uint(__ldg(x + i)));
  }
};

// fetch_fixed_aligned on raw binary64 bits.
__device__ __forceinline__ long long fetch_bits(unsigned long long bdu, int pexp, uint32_t dlen) {
  const int exp = (int)((bdu >> 52) & 0x7FFu) - 1023;
  if (exp < pexp) return 0;
  const int sh = 63 - exp - (int)dlen;
  unsigned long long f = ((bdu << 11) | 0x8000000000000000ull) >> (sh & 63);
  if (bdu >> 63) f = ~(f - 1ull);
  return (long long)f;
}

// Signed-integer key with the order of the binary64 values (-0 < +0; NaNs
// are extremal).  fetch_fixed_aligned is non-decreasing on finite values
// whose shift does not wrap, so min/max can be taken on keys and quantized
// once.
__device__ __forceinline__ long long order_key(unsigned long long b) {
  return (long long)(b ^ ((unsigned long long)((long long)b >> 63) >> 1));
}
__device__ __forceinline__ unsigned long long key_bits(long long k) {
  const unsigned long long u = (unsigned long long)k;
  return u ^ ((unsigned long long)(k >> 63) >> 1);
}

// 32 flipped slice bytes (rows row0..row0+31) in eight 32-bit words.
struct Bytes32 {
  uint32_t w[8];
};

// 16 bytes global -> shared without registers (both 16-byte aligned); a
// thread's copies complete group by group (cp_commit / cp_wait<N>: at most N
// of its groups still in flight), and a warp barrier after the wait makes
// every lane's finished copies visible to the others.
__device__ __forceinline__ void cp16(uint8_t *dst, const void *src) {
  const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// 256-bit non-allocating load (sm_100+; the address is 32-byte aligned).
__device__ __forceinline__ Bytes32 ld_stream32(const uint8_t *p) {
  Bytes32 b;
  asm volatile("ld.global.nc.L1::no_allocate.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(b.w[0]), "=r"(b.w[1]), "=r"(b.w[2]), "=r"(b.w[3]), "=r"(b.w[4]),
                 "=r"(b.w[5]), "=r"(b.w[6]), "=r"(b.w[7])
               : "l"(p));
  return b;
}
// The same with an L2 prefetch of the 256-byte block around the address.
__device__ __forceinline__ Bytes32 ld_stream32_pf(const uint8_t *p) {
  Bytes32 b;
  asm volatile("ld.global.nc.L1::no_allocate.L2::256B.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(b.w[0]), "=r"(b.w[1]), "=r"(b.w[2]), "=r"(b.w[3]), "=r"(b.w[4]),
                 "=r"(b.w[5]), "=r"(b.w[6]), "=r"(b.w[7])
               : "l"(p));
  return b;
}
__device__ __forceinline__ Bytes32 ld_cand32(const uint8_t *p) {
  const uint4 lo = __ldg(reinterpret_cast<const uint4 *>(p));
  const uint4 hi = __ldg(reinterpret_cast<const uint4 *>(p + 16));
  Bytes32 b;
  b.w[0] = lo.x;
  b.w[1] = lo.y;
  b.w[2] = lo.z;
  b.w[3] = lo.w;
  b.w[4] = hi.x;
  b.w[5] = hi.y;
  b.w[6] = hi.z;
  b.w[7] = hi.w;
  return b;
}

// Byte MSBs of two words (4 rows each) -> 8 row-ordered bits in the low byte:
// with c = (m0 >> 4) | m1 the MSBs sit at bits 8b+3 (row b) and 8b+7 (row
// 4+b); multiplying by 2^29 + 2^22 + 2^15 + 2^8 moves exactly those eight bits,
// without collisions, to bits 32..39 of the 64-bit product.
__device__ __forceinline__ uint32_t msb8(uint32_t m0, uint32_t m1) {
  return __umulhi((m0 >> 4) | m1, 0x20408100u);
}
// MSBs of eight words -> the 32-bit bitmap word (bit i = byte i).
__device__ __forceinline__ uint32_t gather32(const uint32_t *m) {
  const uint32_t a = __byte_perm(msb8(m[0], m[1]), msb8(m[2], m[3]), 0x0040);
  const uint32_t b = __byte_perm(msb8(m[4], m[5]), msb8(m[6], m[7]), 0x0040);
  return __byte_perm(a, b, 0x5410);
}

// Per-byte compares of flipped bytes w against an unflipped target whose top
// bit is TH: MSB of each byte of the result.  (a = w ^ 0x80; a_lo = w_lo.)
template <bool TH>
__device__ __forceinline__ uint32_t gt4t(uint32_t w, uint32_t lo1) {
  const uint32_t d1 = (w | H) - lo1;  // MSB: a_lo > t_lo
  return TH ? (~w & d1 & H) : ((~w | d1) & H);
}
template <bool TH>
__device__ __forceinline__ uint32_t eq4t(uint32_t w, uint32_t lo0, uint32_t lo1) {
  const uint32_t wh = w | H;
  return (wh - lo0) & ~(wh - lo1) & (TH ? ~w : w) & H;
}

// Weighted popcount of one 32-bit word of a packed stream of `ts`-bit fields
// whose first bit sits at a stream bit of residue `phase` (= its position
// mod ts, < ts): sum over set bits b of 2^((phase + b) mod ts).  (The sum of
// all fields of a stream only depends on each bit's position mod ts, not on
// row boundaries.)
__device__ __forceinline__ uint32_t wpopc(uint32_t w, uint32_t phase, uint32_t ts) {
  if (ts == 1) return __popc(w);
  // bits 0, ts, 2ts, ... of a word (ts = 2..7)
  const uint32_t pat = ts == 2 ? 0x55555555u : ts == 3 ? 0x49249249u : ts == 4 ? 0x11111111u
                     : ts == 5 ? 0x42108421u : ts == 6 ? 0x41041041u : 0x10204081u;
  // bits of class c (index = c mod ts) weigh 2^((phase + c) mod ts); phase < ts
  uint32_t acc = 0;
#pragma unroll
  for (uint32_t c = 0; c < 7; ++c) {
    if (c < ts) {
      uint32_t sh = phase + c;
      if (sh >= ts) sh -= ts;
      acc += (uint32_t)__popc(w & (pat << c)) << sh;
    }
  }
  return acc;
}

constexpr uint32_t every_bit(int R) {
  uint32_t p = 0;
  for (int b = 0; b < 32; b += R) p |= 1u << b;
  return p;
}

// Tail sum of a lane's 32 rows whose R-bit fields fill the R words at tp
// (the rows all below n): bit b of word i sits at stream position 32i + b,
// which weighs 2^((32i + b) mod R) -- wpopc with the phase of every word and
// the class masks resolved at compile time (3 R^2 operations instead of
// about 7 R^2 with a run-time width).
template <int R>
__device__ __forceinline__ uint32_t tail_sum32(const uint32_t *tp) {
  uint32_t acc = 0;
#pragma unroll
  for (int i = 0; i < R; ++i) {
    const uint32_t w = tp[i];
#pragma unroll
    for (int c = 0; c < R; ++c) {
      const int sh = ((c - 32 * i) % R + R) % R;  // bits of class c in word i
      acc += (uint32_t)__popc(w & (every_bit(R) << sh)) << c;
    }
  }
  return acc;
}

// The tail sum of the whole 32-row blocks from block vt on, every nth: a
// block's 32 R-bit fields fill R words (4R bytes at 4R * block); the words
// are loaded together and summed with compile-time class masks; bits past
// tail_bits (the padding rows of the last block) are cleared.
template <int R>
__device__ __forceinline__ unsigned long long tail_blocks_sum(const uint8_t *__restrict__ tail,
                                                              unsigned long long tail_bits,
                                                              uint32_t vt, uint32_t nth) {
  const uint32_t nblk = (uint32_t)((tail_bits / R + 31) / 32);
  unsigned long long acc = 0;
  for (uint32_t b = vt; b < nblk; b += nth) {
    const uint32_t *tp = reinterpret_cast<const uint32_t *>(tail) + (size_t)b * R;
    uint32_t w[R];
#pragma unroll
    for (int i = 0; i < R; ++i) w[i] = __ldg(tp + i);
    const unsigned long long bit0 = (unsigned long long)b * 32 * R;
    if (bit0 + 32 * R > tail_bits) {
#pragma unroll
      for (int i = 0; i < R; ++i) {
        const unsigned long long wb = bit0 + 32 * i;
        if (wb >= tail_bits)
          w[i] = 0;
        else if (wb + 32 > tail_bits)
          w[i] &= (1u << (uint32_t)(tail_bits - wb)) - 1u;
      }
    }
    acc += tail_sum32<R>(w);
  }
  return acc;
}

// The slice sums (first ks slices, each a flat array of `stride` bytes whose
// padding rows hold the flipped zero 0x80) and the packed tail sum (n * ts
// bits, fields weighed by wpopc) of thread tid of nth, added into the
// block's s_acc[0..ks) and s_acc[8] (byte_fixed_sum, split_double.rs:2127-2208).
__device__ __forceinline__ void sum_slices_tail(const uint8_t *__restrict__ slices, size_t stride,
                                                uint32_t ks, const uint8_t *__restrict__ tail,
                                                uint32_t ts, unsigned long long tail_bits,
                                                uint32_t tid, uint32_t nth,
                                                unsigned long long *s_acc) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t nv = (uint32_t)(stride / 16);
  // A slice rarely divides evenly into grid-stride steps, so some threads
  // take one step more than the others.  Each slice (and the tail) starts the
  // threads at a different offset (whole warps), so no thread takes the
  // extra step in every slice: the kernel ends when the average thread does.
  const uint32_t rot = (nth / (ks + 1)) & ~31u;
  for (uint32_t s = 0; s < ks; ++s) {
    const uint8_t *sl = slices + (size_t)s * stride;
    uint32_t acc = 0;
    uint32_t vt = tid + s * rot;
    if (vt >= nth) vt -= nth;
    for (uint32_t v0 = vt; v0 < nv; v0 += kU * nth) {
      uint4 d[kU];
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        const uint32_t v = v0 + u * nth;
        d[u] = v < nv ? ld_stream(sl + (size_t)v * 16) : make_uint4(H, H, H, H);
      }
#pragma unroll
      for (int u = 0; u < kU; ++u) {
        acc = __dp4a(d[u].x ^ H, 0x01010101u, acc);
        acc = __dp4a(d[u].y ^ H, 0x01010101u, acc);
        acc = __dp4a(d[u].z ^ H, 0x01010101u, acc);
        acc = __dp4a(d[u].w ^ H, 0x01010101u, acc);
      }
    }
    const unsigned long long w = warp_sum_ull(acc);
    if (lane == 0 && w) atomicAdd(&s_acc[s], w);
  }
  if (ts) {
    uint32_t vt = tid + ks * rot;
    if (vt >= nth) vt -= nth;
    unsigned long long acc = 0;
    switch (ts) {
      case 1: acc = tail_blocks_sum<1>(tail, tail_bits, vt, nth); break;
      case 2: acc = tail_blocks_sum<2>(tail, tail_bits, vt, nth); break;
      case 3: acc = tail_blocks_sum<3>(tail, tail_bits, vt, nth); break;
      case 4: acc = tail_blocks_sum<4>(tail, tail_bits, vt, nth); break;
      case 5: acc = tail_blocks_sum<5>(tail, tail_bits, vt, nth); break;
      case 6: acc = tail_blocks_sum<6>(tail, tail_bits, vt, nth); break;
      default: acc = tail_blocks_sum<7>(tail, tail_bits, vt, nth); break;
    }
    acc = warp_sum_ull(acc);
    if (lane == 0 && acc) atomicAdd(&s_acc[8], acc);
  }
}

// `(v as f64) / 2^dlen` with integer operations only: round-to-nearest-even
// of the 64-bit integer to a 53-bit significand, then the exponent lowered by
// dlen (exact: the result stays a normal double for |v| >= 1 and dlen <= 64).
// The FP64 pipe of this part is narrow, so the conversion is done on the
// integer pipes.
__device__ __forceinline__ double i64_to_f64_scaled(long long v, int dlen) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = v < 0 ? 0x8000000000000000ull : 0ull;
  const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  int e = 63 - __clzll(a);  // a in [2^e, 2^(e+1))
  unsigned long long m;
  if (e <= 52) {
    m = a << (52 - e);
  } else {
    const int sh = e - 52;
    const unsigned long long rem = a & ((1ull << sh) - 1ull);
    const unsigned long long half = 1ull << (sh - 1);
    m = a >> sh;
    if (rem > half || (rem == half && (m & 1ull))) {
      m += 1ull;
      if (m >> 53) {
        m >>= 1;
        e += 1;
      }
    }
  }
  const unsigned long long bits =
      sgn | ((unsigned long long)(e - dlen + 1023) << 52) | (m & ((1ull << 52) - 1ull));
  return __longlong_as_double((long long)bits);
}


// The same for a = hi:lo in [1, 2^53) in 32-bit steps: the word holding the
// leading one (hi, or lo when hi is 0) shifted so that the one lands on bit
// 63 of the pair, the pair moved right 11 bits into the significand field,
// and the exponent added on top of the leading one.  Returns the high and
// low words of the double.
__device__ __forceinline__ void u53w_bits(uint32_t hi, uint32_t lo, int dlen, uint32_t &oh,
                                          uint32_t &ol) {
  const bool z = hi == 0u;
  const uint32_t H = z ? lo : hi, L = z ? 0u : lo;
  const uint32_t lz = __clz(H);
  const uint32_t NH = __funnelshift_l(L, H, lz), NL = __funnelshift_l(0u, L, lz);
  const int e1 = (z ? 31 : 63) - (int)lz - dlen + 1022;  // biased exponent - 1
  oh = (NH >> 11) + ((uint32_t)e1 << 20);
  ol = __funnelshift_r(NL, NH, 11);
}
__device__ __forceinline__ double u53w_to_f64_scaled(uint32_t hi, uint32_t lo, int dlen) {
  uint32_t oh, ol;
  u53w_bits(hi, lo, dlen, oh, ol);
  return __hiloint2double((int)oh, (int)ol);
}

// The same for a signed v with |v| < 2^53 (two's complement in 64 bits; 0
// gives +0).
__device__ __forceinline__ double s53_to_f64_scaled(unsigned long long v, int dlen) {
  const unsigned long long sg = (unsigned long long)((long long)v >> 63);
  const unsigned long long m = (v ^ sg) - sg;
  const uint32_t hi = (uint32_t)(m >> 32), lo = (uint32_t)m;
  uint32_t oh, ol;
  u53w_bits(hi, lo, dlen, oh, ol);
  // m = 0 leaves the significand words 0 (the leading-one word is 0): only
  // the exponent put into oh is cleared
  oh = (hi | lo) ? (oh | ((uint32_t)sg & 0x80000000u)) : 0u;
  return __hiloint2double((int)oh, (int)ol);
}

// The same for a value that fits in 32 bits: exact (|v| < 2^32 <= 2^53), so
// only the leading one is found and the significand placed -- a third of the
// 64-bit path's integer instructions.
__device__ __forceinline__ double i32_to_f64_scaled(int v, int dlen) {
  if (v == 0) return 0.0;
  const uint32_t sgn = v < 0 ? 0x80000000u : 0u;
  const uint32_t a = v < 0 ? 0u - (uint32_t)v : (uint32_t)v;
  const uint32_t lz = __clz(a);
  const uint32_t A = a << lz;  // leading one at bit 31
  const uint32_t hi = sgn | ((uint32_t)(31 - (int)lz - dlen + 1023) << 20) | ((A >> 11) & 0xFFFFFu);
  return __hiloint2double((int)hi, (int)(A << 21));
}

// Bit i of a 4-bit value -> byte i all ones: x * (1 + 2^7 + 2^14 + 2^21)
// places bit i at 8i without overlapping carries.
__device__ __forceinline__ uint32_t expand4(uint32_t x) {
  return ((x * 0x00204081u) & 0x01010101u) * 0xFFu;
}

// MSB of every byte of w equal to the byte in every lane of bb.
__device__ __forceinline__ uint32_t eqbytes(uint32_t w, uint32_t bb) {
  const uint32_t x = w ^ bb;
  return ~(((x & 0x7F7F7F7Fu) + 0x7F7F7F7Fu) | x) & 0x80808080u;
}

// Largest full code among rows row0..row0+31 whose leading byte is `top`
// (bit i of `cand`): every surviving candidate shares the prefix built so
// far, so one prefix and a candidate mask describe the MSB-first progressive
// max.  Each later slice is one 32-byte load; the candidates' largest byte
// and the rows holding it come from per-byte SWAR on the unflipped words.
// Out of line: it runs for few blocks.
// `next` is the slice after the leading byte and `nmore` the slices from it
// (a buff-major column's leading byte is a sparse one, its slices all dense).
static __device__ __noinline__ unsigned long long max_after_top(const uint8_t *__restrict__ next,
                                                                size_t stride, uint32_t nmore,
                                                                const uint8_t *__restrict__ tail,
                                                                uint32_t r, uint32_t row0,
                                                                uint32_t cand, uint32_t top) {
  unsigned long long prefix = top;
  for (uint32_t s = 0; s < nmore; ++s) {
    const Bytes32 b = ld_cand32(next + s * stride + row0);
    uint32_t u[8], mx = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      u[q] = (b.w[q] ^ H) & expand4((cand >> (4 * q)) & 0xFu);
      mx = __vmaxu4(mx, u[q]);
    }
    mx = __vmaxu4(mx, mx >> 16);
    mx = __vmaxu4(mx, mx >> 8);
    const uint32_t best = mx & 0xFFu;
    uint32_t e[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) e[q] = eqbytes(u[q], best * 0x01010101u);
    cand &= gather32(e);
    prefix = (prefix << 8) | best;
  }
  if (!r) return prefix;
  // 32 rows of r bits = r words at byte (row0 / 32) * 4r
  const uint32_t *tp = reinterpret_cast<const uint32_t *>(tail + (size_t)(row0 >> 5) * 4 * r);
  uint32_t tw[8];
#pragma unroll
  for (int i = 0; i < 7; ++i) tw[i] = (uint32_t)i < r ? __ldg(tp + i) : 0u;
  tw[7] = 0;
  uint32_t bt = 0;
  for (uint32_t c = cand; c; c &= c - 1) {
    const uint32_t i = __ffs(c) - 1;
    const uint32_t bit = i * r, wi = bit >> 5;
    uint32_t w0 = tw[0], w1 = tw[1];
#pragma unroll
    for (uint32_t j = 1; j < 7; ++j)
      if (wi == j) {
        w0 = tw[j];
        w1 = tw[j + 1];
      }
    bt = max(bt, __funnelshift_r(w0, w1, bit & 31) & ((1u << r) - 1u));
  }
  return (prefix << r) | bt;
}

// The same with slice 0 holding the leading byte (k slices).
__device__ __forceinline__ unsigned long long max_in_block(const uint8_t *__restrict__ slices,
                                                           size_t stride, uint32_t k,
                                                           const uint8_t *__restrict__ tail,
                                                           uint32_t r, uint32_t row0,
                                                           uint32_t cand, uint32_t top) {
  return max_after_top(slices + stride, stride, k ? k - 1 : 0u, tail, r, row0, cand, top);
}

// buff_sum_majority's combine (compress/buff_simd.rs:2294-2442), shared by
// the host call and the device-only form so both give the same bits: the
// per-byte partials (a sparse column's outlier byte sum plus its major byte
// times its other rows, then the dense slices, then the tail) scaled slice
// by slice in the reference's order; the base term is left out when a dense
// slice ends the code (Q5).
struct MajorSumArgs {
  uint64_t n;
  int64_t base;
  uint32_t m, k, r, fixed_len;
  int32_t ilen, dlen;
  uint8_t majors[8];
  uint32_t nout[8];
};

// raw: sparse byte sums at raw[0..m), dense and tail sums at raw[8..8+k-m+1).
// parts receives k (+1 with a tail) partials; returns their count.
__host__ __device__ inline uint32_t major_sum_parts(const MajorSumArgs &a,
                                                    const unsigned long long *raw,
                                                    unsigned long long *parts) {
  uint32_t np = 0;
  for (uint32_t c = 0; c < a.m; ++c)
    parts[np++] = raw[c] + (unsigned long long)a.majors[c] * (a.n - a.nout[c]);
  const uint32_t kd = a.k - a.m;
  for (uint32_t j = 0; j < kd; ++j) parts[np++] = raw[8 + j];
  if (a.r) parts[np++] = raw[8 + kd];
  return np;
}

// 2^e as a double, built from its exponent field (-1022 <= e <= 1023).
__host__ __device__ inline double pow2_exact(int e) {
  const unsigned long long bits = (unsigned long long)(e + 1023) << 52;
  double d;
  memcpy(&d, &bits, sizeof(d));
  return d;
}

// x / 2^e of the reference, as x * 2^-e: scaling by a power of two is exact,
// so both round the same real number and give the same bits.
__host__ __device__ inline double div_pow2(double x, int e) { return x * pow2_exact(-e); }

__host__ __device__ inline double major_sum_f64(const MajorSumArgs &a,
                                                const unsigned long long *parts) {
  double sum_base = (double)a.n * (double)a.base;
  sum_base = div_pow2(sum_base, a.dlen);
  double sum = 0.0;
  int32_t processed = 0;
  uint32_t remain = a.fixed_len;
  bool no_base = false;
  for (uint32_t i = 0; i < a.k; ++i) {
    remain -= 8;
    processed += 8;
    sum = sum + div_pow2((double)parts[i], processed - a.ilen);
    if (i >= a.m && remain == 0) no_base = true;  // a dense slice ends the code
  }
  if (!no_base) {
    if (remain > 0) {
      processed += (int32_t)remain;
      sum = sum + div_pow2((double)parts[a.k], processed - a.ilen);
    }
    sum += sum_base;
  }
  return sum;
}

}  // namespace dev
}  // namespace buffk
