// The headline query pair on a serialized image that has not been uploaded:
// buff_range_filter_sum_image.
//
// The reference answers every query from the encoded Vec<u8> it is handed
// (compress/buff_simd.rs:3361 takes `bytes: Vec<u8>`, split_double.rs:2127
// likewise).  When that image sits in host memory, uploading it first
// (buff_deserialize) costs one pass over the host link and a second over
// HBM; here the kernel itself reads the image where it lies -- pinned host
// memory through its device mapping, pageable memory directly where the
// device shares the host's page tables, or device memory -- and answers the
// range filter and the sum in that single pass.  The link, not HBM, bounds
// the call, and every byte crosses it once.
//
// The image's slices start at byte 20 + j*n, so they are aligned to nothing.
// Each CTA stages one 4,096-row chunk of every slice (and of the packed tail)
// into shared memory with aligned 16-byte loads covering the misaligned span,
// then thread t realigns the 32 bytes of its 32-row block with funnel shifts
// and runs the same integer steps as the resident kernels: byte sums of every
// slice (dp4a on the unflipped bytes), the tail field sum, the slice-0
// compare, refinement of candidate rows through the later slices and the
// tail, the Q3 row limit.  The partial sums are exactly those of buff_sum.
//
// buff_filter_image does the same for the four filters alone.  They need only
// slice 0 in full: it is staged as above, and the few candidate blocks (rows
// still equal to the target prefix) read their later slices and tail bytes
// straight from the image, so a filter moves about a third of the image
// across the link.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include "buff_device.cuh"
#include "buff_internal.h"

namespace {

using namespace buffk::dev;

constexpr uint32_t kImgRows = 4096;                // rows per chunk
constexpr uint32_t kImgThreads = kImgRows / 32;    // one 32-row block per thread
constexpr uint32_t kRegion = kImgRows + 32;        // staged bytes per slice (16-byte slack)

struct ImgArgs {
  const uint8_t *slices;  // image + 20: slice j at j * n
  const uint8_t *tail;    // image + 20 + k * n
  uint32_t n, k, r;
  uint32_t flipx;         // XOR that yields flipped bytes: 0 (buff-simd) or 0x80808080 (buff layout)
  uint32_t full_rows;     // rows that may be set (32 * floor(n / 32))
  uint32_t ttail;         // target tail bits
  uint64_t tail_bytes;    // ceil(n * r / 8)
  unsigned long long tb;  // target byte per slice (unflipped), slice j in bits 8j..8j+7
  uint32_t *words;        // bitmap (device-accessible)
  unsigned long long *count;
  unsigned long long *parts;  // k slice sums, then the tail field sum
};

// Copies [src, src + len) (len > 0) into dst with aligned 16-byte loads of the
// smallest aligned span covering it; returns the offset of src within dst.
// The span never leaves the 16-byte granules holding the first and the last
// byte, so it stays within the pages of the source.
__device__ __forceinline__ uint32_t stage(uint8_t *dst, const uint8_t *src, uint64_t len) {
  const uintptr_t s = reinterpret_cast<uintptr_t>(src);
  const uintptr_t a0 = s & ~(uintptr_t)15;
  const uint32_t nvec = (uint32_t)((((s + len + 15) & ~(uintptr_t)15) - a0) / 16);
  const uint4 *from = reinterpret_cast<const uint4 *>(a0);
  for (uint32_t i = threadIdx.x; i < nvec; i += kImgThreads)
    reinterpret_cast<uint4 *>(dst)[i] = from[i];
  return (uint32_t)(s - a0);
}

// The 32-byte row block starting at byte `off` of a staged region (any alignment).
__device__ __forceinline__ void unaligned32(const uint8_t *region, uint32_t off, uint32_t *w) {
  const uint32_t *x = reinterpret_cast<const uint32_t *>(region) + (off >> 2);
  const uint32_t sh = (off & 3u) * 8u;
  uint32_t lo = x[0];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const uint32_t hi = x[i + 1];
    w[i] = __funnelshift_r(lo, hi, sh);
    lo = hi;
  }
}

// The 32 R-bit tail fields of one block (words tw[0..R)): compares with the
// target, and sums the fields of the rows in `live` (rows below n).
template <int R>
__device__ __forceinline__ void tail_block(const uint32_t *tw, uint32_t ttail, uint32_t live,
                                           uint32_t &gtt, uint32_t &eqt, uint32_t &fsum) {
#pragma unroll
  for (int i = 0; i < 32; ++i) {
    const int bit = i * R, wi = bit >> 5, sh = bit & 31;
    const uint32_t hi = (wi + 1 < R) ? tw[wi + 1] : 0u;
    const uint32_t f = __funnelshift_r(tw[wi], hi, sh) & ((1u << R) - 1u);
    gtt |= (uint32_t)(f > ttail) << i;
    eqt |= (uint32_t)(f == ttail) << i;
    fsum += (live >> i & 1u) ? f : 0u;
  }
}

__global__ void __launch_bounds__(kImgThreads) k_filter_sum_image(ImgArgs a) {
  extern __shared__ __align__(16) uint8_t sm[];
  uint8_t *tail_sm = sm + (size_t)a.k * kRegion;
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  const uint32_t nchunks = (a.n + kImgRows - 1) / kImgRows;
  const uint32_t t0 = (uint32_t)(a.tb & 0xFFu);
  const uint32_t lo0 = (t0 & 0x7Fu) * 0x01010101u, lo1 = ((t0 & 0x7Fu) + 1u) * 0x01010101u;
  const bool th = t0 & 0x80u;
  unsigned long long ssum[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  unsigned long long tsum = 0, cnt = 0;
  for (uint32_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const uint32_t r0 = c * kImgRows;
    const uint32_t rows = a.n - r0 < kImgRows ? a.n - r0 : kImgRows;
    __syncthreads();  // the previous chunk's reads of the staging area are done
    uint32_t m[8];
#pragma unroll
    for (uint32_t j = 0; j < 8; ++j)
      if (j < a.k) m[j] = stage(sm + j * kRegion, a.slices + (size_t)j * a.n + r0, rows);
    uint32_t mt = 0;
    const uint64_t toff = (uint64_t)r0 * a.r / 8;  // r0 is a multiple of 8
    uint64_t tlen = 0;
    if (a.r) {
      const uint64_t tend = ((uint64_t)(r0 + rows) * a.r + 7) / 8;
      tlen = (tend < a.tail_bytes ? tend : a.tail_bytes) - toff;
      mt = stage(tail_sm, a.tail + toff, tlen);
    }
    __syncthreads();
    if (rows < kImgRows) {
      // rows past n: the zero code (flipped 0x80 in the slices, zero tail bits)
      const uint8_t pad = (uint8_t)(0x80u ^ (a.flipx & 0xFFu));
      for (uint32_t j = 0; j < a.k; ++j)
        for (uint32_t i = rows + tid; i < kImgRows + 4; i += kImgThreads)
          sm[j * kRegion + m[j] + i] = pad;
      if (a.r)
        for (uint32_t i = (uint32_t)tlen + tid; i < kImgRows / 8 * a.r + 4; i += kImgThreads)
          tail_sm[mt + i] = 0;
      __syncthreads();
    }
    if (tid * 32 >= rows) continue;
    const uint32_t row0 = r0 + tid * 32;
    uint32_t eq = 0, gt = 0;
#pragma unroll
    for (uint32_t j = 0; j < 8; ++j) {
      if (j >= a.k) break;
      uint32_t w[8];
      unaligned32(sm + j * kRegion, m[j] + tid * 32, w);
      uint32_t bs = 0;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        w[q] ^= a.flipx;
        bs = __dp4a(w[q] ^ H, 0x01010101u, bs);
      }
      ssum[j] += bs;
      uint32_t g[8], e[8];
      if (j == 0) {
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          e[q] = th ? eq4t<true>(w[q], lo0, lo1) : eq4t<false>(w[q], lo0, lo1);
          g[q] = th ? gt4t<true>(w[q], lo1) : gt4t<false>(w[q], lo1);
        }
        gt = gather32(g);
        eq = gather32(e);
      } else if (eq) {
        const ByteTarget t = make_target((uint32_t)(a.tb >> (8 * j)) & 0xFFu);
#pragma unroll
        for (int q = 0; q < 8; ++q) cmp4(w[q], t, g[q], e[q]);
        gt |= eq & gather32(g);
        eq &= gather32(e);
      }
    }
    if (a.r) {
      // 32 rows of r bits = 4r bytes at tail offset 4r * tid (4-aligned)
      const uint32_t off = mt + 4u * a.r * tid;
      const uint32_t *x = reinterpret_cast<const uint32_t *>(tail_sm) + (off >> 2);
      const uint32_t sh = (off & 3u) * 8u;
      uint32_t tw[7];
#pragma unroll
      for (uint32_t i = 0; i < 7; ++i) tw[i] = i < a.r ? __funnelshift_r(x[i], x[i + 1], sh) : 0u;
      const uint32_t nlive = a.n - row0;
      const uint32_t live = nlive >= 32 ? 0xFFFFFFFFu : ((1u << nlive) - 1u);
      uint32_t gtt = 0, eqt = 0, fsum = 0;
      switch (a.r) {
        case 1: tail_block<1>(tw, a.ttail, live, gtt, eqt, fsum); break;
        case 2: tail_block<2>(tw, a.ttail, live, gtt, eqt, fsum); break;
        case 3: tail_block<3>(tw, a.ttail, live, gtt, eqt, fsum); break;
        case 4: tail_block<4>(tw, a.ttail, live, gtt, eqt, fsum); break;
        case 5: tail_block<5>(tw, a.ttail, live, gtt, eqt, fsum); break;
        case 6: tail_block<6>(tw, a.ttail, live, gtt, eqt, fsum); break;
        default: tail_block<7>(tw, a.ttail, live, gtt, eqt, fsum); break;
      }
      tsum += fsum;
      gt |= eq & gtt;
    }
    if (row0 + 32 > a.full_rows) {
      const uint32_t lim = a.full_rows > row0 ? a.full_rows - row0 : 0u;
      gt &= lim >= 32 ? 0xFFFFFFFFu : ((1u << lim) - 1u);
    }
    a.words[row0 / 32] = gt;
    cnt += __popc(gt);
  }
  // partials: one atomic per warp and value
#pragma unroll
  for (uint32_t j = 0; j < 8; ++j) {
    if (j >= a.k) break;
    const unsigned long long v = warp_sum_ull(ssum[j]);
    if (lane == 0 && v) atomicAdd(a.parts + j, v);
  }
  if (a.r) {
    const unsigned long long v = warp_sum_ull(tsum);
    if (lane == 0 && v) atomicAdd(a.parts + a.k, v);
  }
  const unsigned long long cv = warp_sum_ull(cnt);
  if (lane == 0 && cv && a.count) atomicAdd(a.count, cv);
}

struct ImgFilterArgs {
  const uint8_t *slices;  // image + 20: slice j at j * n
  const uint8_t *tail;    // image + 20 + k * n
  uint32_t n, k_used, r;
  uint32_t flipx;         // as ImgArgs
  uint32_t full_rows;
  uint32_t ttail;
  uint32_t tail_only_eq;  // equality rows are set only by the tail step
  uint64_t tail_bytes;
  unsigned long long tb;
  uint32_t *words;
  unsigned long long *count;
};

// The `vb` valid bytes (1..32) at p, read from the image through 16-byte
// granules that hold valid bytes (so never past the pages of the image), as
// 8 words; bytes past vb read as `pad`.  scr: 16 words of this thread's
// shared scratch.
__device__ __forceinline__ void block_from_image(const uint8_t *p, uint32_t vb, uint32_t pad,
                                                 uint32_t *scr, uint32_t *w) {
  const uintptr_t s = reinterpret_cast<uintptr_t>(p);
  const uintptr_t a0 = s & ~(uintptr_t)15;
  const uint32_t m = (uint32_t)(s - a0);
  const uint32_t nv = (uint32_t)((((s + vb + 15) & ~(uintptr_t)15) - a0) / 16);
  const uint4 *from = reinterpret_cast<const uint4 *>(a0);
  uint4 *sc = reinterpret_cast<uint4 *>(scr);
#pragma unroll
  for (uint32_t v = 0; v < 3; ++v) sc[v] = v < nv ? from[v] : make_uint4(0u, 0u, 0u, 0u);
  if (vb < 32) {
    uint8_t *b = reinterpret_cast<uint8_t *>(scr);
    for (uint32_t i = m + vb; i < m + 32; ++i) b[i] = (uint8_t)pad;
  }
  unaligned32(reinterpret_cast<const uint8_t *>(scr), m, w);
}

template <bool IS_RANGE>
__global__ void __launch_bounds__(kImgThreads) k_filter_image(ImgFilterArgs a) {
  extern __shared__ __align__(16) uint8_t sm[];
  const uint32_t tid = threadIdx.x, lane = tid & 31;
  uint32_t *scr = reinterpret_cast<uint32_t *>(sm + kRegion) + tid * 16;
  const uint32_t nchunks = (a.n + kImgRows - 1) / kImgRows;
  const uint32_t t0 = (uint32_t)(a.tb & 0xFFu);
  const uint32_t lo0 = (t0 & 0x7Fu) * 0x01010101u, lo1 = ((t0 & 0x7Fu) + 1u) * 0x01010101u;
  const bool th = t0 & 0x80u;
  const bool deep = a.k_used > 1 || a.r;
  const uint32_t pad = 0x80u ^ (a.flipx & 0xFFu);
  unsigned long long cnt = 0;
  for (uint32_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const uint32_t r0 = c * kImgRows;
    const uint32_t rows = a.n - r0 < kImgRows ? a.n - r0 : kImgRows;
    __syncthreads();
    const uint32_t m0 = stage(sm, a.slices + r0, rows);
    __syncthreads();
    if (rows < kImgRows) {
      for (uint32_t i = rows + tid; i < kImgRows + 4; i += kImgThreads) sm[m0 + i] = (uint8_t)pad;
      __syncthreads();
    }
    if (tid * 32 >= rows) continue;
    const uint32_t row0 = r0 + tid * 32;
    const uint32_t vb = a.n - row0 < 32 ? a.n - row0 : 32u;
    uint32_t w[8], g[8], e[8];
    unaligned32(sm, m0 + tid * 32, w);
    uint32_t eor = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      w[q] ^= a.flipx;
      e[q] = th ? eq4t<true>(w[q], lo0, lo1) : eq4t<false>(w[q], lo0, lo1);
      eor |= e[q];
    }
    uint32_t eq = eor ? gather32(e) : 0u;
    uint32_t gt = 0;
    if (IS_RANGE) {
#pragma unroll
      for (int q = 0; q < 8; ++q) g[q] = th ? gt4t<true>(w[q], lo1) : gt4t<false>(w[q], lo1);
      gt = gather32(g);
    }
    if (eq) {
      if (deep) {
        for (uint32_t j = 1; j < a.k_used && eq; ++j) {
          block_from_image(a.slices + (size_t)j * a.n + row0, vb, pad, scr, w);
          const ByteTarget t = make_target((uint32_t)(a.tb >> (8 * j)) & 0xFFu);
#pragma unroll
          for (int q = 0; q < 8; ++q) cmp4(w[q] ^ a.flipx, t, g[q], e[q]);
          gt |= eq & gather32(g);
          eq &= gather32(e);
        }
        if (a.r && eq) {
          // 32 rows of r bits = 4r bytes at tail byte 4r * (row0 / 32)
          const uint64_t off = (uint64_t)4 * a.r * (row0 / 32);
          const uint64_t left = a.tail_bytes - off;
          const uint32_t tlen = (uint32_t)(left < 4 * a.r ? left : 4 * a.r);
          uint32_t tw[8];
          block_from_image(a.tail + off, tlen, 0u, scr, tw);
          const uint32_t live = vb >= 32 ? 0xFFFFFFFFu : ((1u << vb) - 1u);
          uint32_t gtt = 0, eqt = 0, fs = 0;
          switch (a.r) {
            case 1: tail_block<1>(tw, a.ttail, live, gtt, eqt, fs); break;
            case 2: tail_block<2>(tw, a.ttail, live, gtt, eqt, fs); break;
            case 3: tail_block<3>(tw, a.ttail, live, gtt, eqt, fs); break;
            case 4: tail_block<4>(tw, a.ttail, live, gtt, eqt, fs); break;
            case 5: tail_block<5>(tw, a.ttail, live, gtt, eqt, fs); break;
            case 6: tail_block<6>(tw, a.ttail, live, gtt, eqt, fs); break;
            default: tail_block<7>(tw, a.ttail, live, gtt, eqt, fs); break;
          }
          gt |= eq & gtt;
          eq &= eqt;
        }
      } else if (a.tail_only_eq) {
        eq = 0;
      }
    }
    uint32_t res = IS_RANGE ? gt : eq;
    if (row0 + 32 > a.full_rows) {
      const uint32_t lim = a.full_rows > row0 ? a.full_rows - row0 : 0u;
      res &= lim >= 32 ? 0xFFFFFFFFu : ((1u << lim) - 1u);
    }
    a.words[row0 / 32] = res;
    cnt += __popc(res);
  }
  const unsigned long long cv = warp_sum_ull(cnt);
  if (lane == 0 && cv && a.count) atomicAdd(a.count, cv);
}

// The slices of a serialized image copied into a column's aligned slices
// (buff_deserialize from host memory the device can reach): a CTA stages one
// 4,096-row chunk of one slice with aligned 16-byte loads, then writes it to
// slice j at j * stride with 16-byte stores (XOR flipx: the buff layout's
// unflipped bytes become flipped), rows from n to the end of the chunk
// holding the flipped zero byte.  Each image byte crosses the host link
// once and lands in place, where a pitched copy engine transfer runs
// slower.
__global__ void __launch_bounds__(kImgThreads) k_upload_slices(const uint8_t *slices, uint32_t n,
                                                               uint32_t k, size_t stride,
                                                               uint32_t flipx, uint8_t *dst) {
  __shared__ __align__(16) uint8_t sm[kRegion + 16];
  const uint32_t tid = threadIdx.x;
  const uint32_t nchunks = (uint32_t)((stride + kImgRows - 1) / kImgRows);
  for (uint64_t it = blockIdx.x; it < (uint64_t)nchunks * k; it += gridDim.x) {
    const uint32_t j = (uint32_t)(it / nchunks), c = (uint32_t)(it % nchunks);
    const uint32_t r0 = c * kImgRows;
    const uint32_t rows = r0 < n ? (n - r0 < kImgRows ? n - r0 : kImgRows) : 0u;
    const uint32_t span = (uint32_t)(stride - r0 < kImgRows ? stride - r0 : kImgRows);
    __syncthreads();
    const uint32_t m = rows ? stage(sm, slices + (size_t)j * n + r0, rows) : 0u;
    __syncthreads();
    uint8_t *out = dst + (size_t)j * stride + r0;
    for (uint32_t v = tid; v * 16 < span; v += kImgThreads) {
      const uint32_t o = v * 16;
      uint32_t w[4];
      const uint32_t *x = reinterpret_cast<const uint32_t *>(sm) + ((m + o) >> 2);
      const uint32_t sh = ((m + o) & 3u) * 8u;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        w[q] = __funnelshift_r(x[q], x[q + 1], sh) ^ flipx;
        // rows past n: the flipped zero byte
        const uint32_t row = o + 4 * q;
        if (row + 4 > rows) {
#pragma unroll
          for (int b = 0; b < 4; ++b)
            if (row + b >= rows) w[q] = (w[q] & ~(0xFFu << (8 * b))) | (0x80u << (8 * b));
        }
      }
      *reinterpret_cast<uint4 *>(out + o) = make_uint4(w[0], w[1], w[2], w[3]);
    }
  }
}

// The body of a serialized image (the k slices, then the packed tail)
// written by the device straight into its destination -- host memory the
// device can reach (buff_serialize): blockIdx.y names the segment (slice j,
// or the tail at y = k), whose bytes go to dst + y * n.  A thread writes one
// 16-byte aligned block of the destination with one store, gathered from
// the two aligned 16-byte source vectors that hold it (the source offset of
// every block of a segment has the same remainder mod 16); the partial
// blocks at a segment's two ends are written byte by byte, so neighbouring
// segments and the header are never overwritten.  flipx is XORed into the
// slice bytes (0x80808080 for the buff layout's unflipped image).
__global__ void __launch_bounds__(256) k_download_image(const uint8_t *__restrict__ slices,
                                                        size_t stride, uint32_t n, uint32_t k,
                                                        const uint8_t *__restrict__ tail,
                                                        uint64_t tail_bytes, uint64_t tail_alloc,
                                                        uint32_t flipx, uint8_t *dst) {
  const uint32_t y = blockIdx.y;
  const uint8_t *src = y < k ? slices + (size_t)y * stride : tail;
  const uint64_t len = y < k ? n : tail_bytes;
  const uint64_t cap = y < k ? stride : tail_alloc;  // source bytes that may be read
  const uint32_t fx = y < k ? flipx : 0u;
  uint8_t *out = dst + (uint64_t)y * n;  // the segment's first destination byte
  if (!len) return;
  const uintptr_t a0 = reinterpret_cast<uintptr_t>(out);
  const uint64_t head = (16 - (a0 & 15)) & 15;        // bytes before the first aligned block
  uint64_t nfull = len > head ? (len - head) / 16 : 0;
  // a block with an unaligned source also reads the next 16 source bytes:
  // keep those inside the source allocation (the rest go byte by byte)
  if (head && nfull && 16 * (nfull + 1) > cap) nfull = cap / 16 - 1;
  const uint64_t tstart = head + nfull * 16;           // bytes after the last aligned block
  const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
  const uint64_t nth = (uint64_t)gridDim.x * blockDim.x;
  // source offset head + 16b of block b: remainder s = head mod 16, words at
  // src + 16 * floor((head + 16 b) / 16)
  const uint32_t srem = (uint32_t)(head & 15), sw = srem >> 2, sb = (srem & 3) * 8;
  const uint8_t *sbase = src + (head & ~15ull);
  for (uint64_t b = tid; b < nfull; b += nth) {
    const uint4 lo = __ldg(reinterpret_cast<const uint4 *>(sbase + 16 * b));
    uint4 hi = make_uint4(0, 0, 0, 0);
    if (srem) hi = __ldg(reinterpret_cast<const uint4 *>(sbase + 16 * b + 16));
    const uint32_t w[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
    uint32_t o[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t a = w[q], c = w[q + 1];
#pragma unroll
      for (uint32_t t = 1; t < 4; ++t)
        if (sw == t) {
          a = w[q + t];
          c = w[q + t + 1];
        }
      o[q] = __funnelshift_r(a, c, sb) ^ fx;
    }
    *reinterpret_cast<uint4 *>(out + head + 16 * b) = make_uint4(o[0], o[1], o[2], o[3]);
  }
  // the partial blocks at both ends, byte by byte
  const uint64_t nhead = head < len ? head : len;
  const uint64_t ntail = len > tstart ? len - tstart : 0;
  for (uint64_t e = tid; e < nhead + ntail; e += nth) {
    const uint64_t i = e < nhead ? e : tstart + (e - nhead);
    out[i] = src[i] ^ (uint8_t)fx;
  }
}

inline cudaStream_t S(void *s) { return reinterpret_cast<cudaStream_t>(s); }

// A device-accessible address for `p`: device memory as is, pinned host
// memory through its mapping, pageable host memory when the device reads the
// host's page tables; nullptr when the device cannot reach it.
const void *device_view(const void *p, int device) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  if (at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged) return p;
  if (at.type == cudaMemoryTypeHost) return at.devicePointer;
  int pageable = 0;
  cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
  return pageable ? p : nullptr;
}

int parse_header(const uint8_t *image, uint64_t len, uint64_t scale, uint32_t flags,
                 cudaStream_t s, buff_col **out) {
  uint8_t hdr[20];
  if (buffh::is_device_ptr(image)) {
    cudaError_t e = cudaMemcpyAsync(hdr, image, 20, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return buffh::cuda_status(e);
  } else {
    memcpy(hdr, image, 20);
  }
  uint32_t w[5];
  for (int i = 0; i < 5; ++i)
    w[i] = (uint32_t)hdr[4 * i] | ((uint32_t)hdr[4 * i + 1] << 8) |
           ((uint32_t)hdr[4 * i + 2] << 16) | ((uint32_t)hdr[4 * i + 3] << 24);
  buff_col *c = buffh::new_col(scale, flags);
  if (!c) return BUFF_ENOMEM;
  c->base = (int64_t)((uint64_t)w[0] | ((uint64_t)w[1] << 32));
  c->n = w[2];
  c->ilen = w[3];
  c->dlen = w[4];
  const uint32_t fl = c->ilen + c->dlen;  // the decoders' `dlen + ilen` (u32)
  if (c->n > BUFF_MAX_ROWS) {
    buffh::free_col(c);
    return BUFF_ENOTSUP;
  }
  if (fl > 64 || c->dlen > 1000) {
    buffh::free_col(c);
    return BUFF_ECORRUPT;
  }
  buffh::set_layout(c, fl);
  if (20ull + (uint64_t)c->k * c->n + ((uint64_t)c->n * c->r + 7) / 8 > len) {
    buffh::free_col(c);
    return BUFF_ECORRUPT;
  }
  c->tail_bytes = ((uint64_t)c->n * c->r + 7) / 8;
  *out = c;
  return BUFF_OK;
}

// The two-step path: upload into a resident column, then the resident call.
int via_column(const uint8_t *image, uint64_t len, uint64_t scale, uint32_t flags, double pred,
               uint32_t *words, uint64_t *count, buff_sum_result *sum, void *stream) {
  buff_col *col = nullptr;
  int rc = buff_deserialize(image, len, scale, flags, stream, &col);
  if (rc) return rc;
  uint64_t parts[9] = {0};
  rc = buff_range_filter_sum(col, pred, words, count, parts, stream);
  if (!rc) rc = buff_sum_finish(col, parts, sum);
  const int rf = buff_col_free_async(col, stream);
  return rc ? rc : rf;
}

using FilterFn = int (*)(const buff_col *, double, uint32_t *, uint64_t *, void *);

int via_column_filter(const uint8_t *image, uint64_t len, uint64_t scale, uint32_t flags,
                      int kind, double pred, uint32_t *words, uint64_t *count, void *stream) {
  static const FilterFn fns[4] = {buff_range_filter, buff_equal_filter,
                                  buff_range_filter_with_slice, buff_equal_filter_with_slice};
  buff_col *col = nullptr;
  int rc = buff_deserialize(image, len, scale, flags, stream, &col);
  if (rc) return rc;
  rc = fns[kind](col, pred, words, count, stream);
  const int rf = buff_col_free_async(col, stream);
  return rc ? rc : rf;
}

}  // namespace

extern "C" int buff_filter_image(const uint8_t *image, uint64_t len, uint64_t scale,
                                 uint32_t flags, int kind, double pred, uint32_t *words,
                                 uint64_t *count, void *stream) {
  if (!image || kind < 0 || kind > 3) return BUFF_EINVAL;
  if (len < 20) return BUFF_ECORRUPT;
  cudaStream_t s = S(stream);
  buff_col *c = nullptr;
  int rc = parse_header(image, len, scale, flags, s, &c);
  if (rc) return rc;
  const uint32_t n = c->n, nw = (n + 31) / 32;
  if (n && !words) {
    buffh::free_col(c);
    return BUFF_EINVAL;
  }
  buffk::FilterArgs fa;
  int action = 2;
  if ((rc = buffh::plan_filter(c, pred, kind, &fa, &action))) {
    buffh::free_col(c);
    return rc;
  }
  if (n == 0 || action != 2) {
    // no kernel: every word is 0, or every word is ones up to row n
    buffh::free_col(c);
    const uint32_t fill = action == 1 ? 0xFFFFFFFFu : 0u;
    const uint64_t cnt = action == 1 ? n : 0u;
    if (nw && buffh::is_device_ptr(words)) {
      rc = buffh::cuda_status(buffk::launch_fill_words(words, n, fill, nullptr, s));
    } else {
      for (uint32_t i = 0; i < nw; ++i)
        words[i] = (i == nw - 1 && (n & 31)) ? (fill & ((1u << (n & 31)) - 1u)) : fill;
    }
    if (!rc && count) {
      if (buffh::is_device_ptr(count))
        rc = buffh::cuda_status(cudaMemcpyAsync(count, &cnt, 8, cudaMemcpyHostToDevice, s));
      else
        *count = cnt;
    }
    if (!rc) rc = buffh::cuda_status(cudaStreamSynchronize(s));
    return rc;
  }
  const uint8_t *img = static_cast<const uint8_t *>(device_view(image, c->device));
  uint32_t *dwords = static_cast<uint32_t *>(const_cast<void *>(device_view(words, c->device)));
  if (c->k == 0 || !img || !dwords) {  // packed codes, or buffers the device cannot reach
    buffh::free_col(c);
    return via_column_filter(image, len, scale, flags, kind, pred, words, count, stream);
  }
  ImgFilterArgs a;
  memset(&a, 0, sizeof(a));
  a.slices = img + 20;
  a.tail = img + 20 + (uint64_t)c->k * n;
  a.n = n;
  a.k_used = fa.k_used;
  a.r = fa.r;
  a.flipx = (flags & BUFF_FLAG_BUFF_LAYOUT) ? 0x80808080u : 0u;
  a.full_rows = fa.full_rows;
  a.ttail = fa.ttail;
  a.tail_only_eq = fa.tail_only_eq;
  a.tail_bytes = c->tail_bytes;
  for (uint32_t j = 0; j < fa.k_used; ++j) a.tb |= (unsigned long long)fa.tbyte[j] << (8 * j);
  a.words = dwords;
  unsigned long long *d = nullptr;
  unsigned long long host = 0;
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&d), sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = buffk::zero_u64(d, 1, s);
  if (e == cudaSuccess) {
    a.count = d;
    void (*fn)(ImgFilterArgs) = fa.is_range ? k_filter_image<true> : k_filter_image<false>;
    const size_t smem = kRegion + (size_t)kImgThreads * 64;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kImgThreads, smem);
    if (per_sm < 1) per_sm = 1;
    const uint32_t nchunks = (n + kImgRows - 1) / kImgRows;
    uint32_t grid = (uint32_t)(per_sm * buffk::num_sms(c->device));
    if (grid > nchunks) grid = nchunks;
    fn<<<grid, kImgThreads, smem, s>>>(a);
    buffk::count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(&host, d, 8, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (d) cudaFreeAsync(d, s);
  rc = buffh::cuda_status(e);
  if (!rc && count) {
    if (buffh::is_device_ptr(count))
      rc = buffh::cuda_status(cudaMemcpyAsync(count, &host, 8, cudaMemcpyHostToDevice, s));
    else
      *count = host;
    if (!rc && buffh::is_device_ptr(count)) rc = buffh::cuda_status(cudaStreamSynchronize(s));
  }
  buffh::free_col(c);
  return rc;
}

extern "C" int buff_range_filter_sum_image(const uint8_t *image, uint64_t len, uint64_t scale,
                                           uint32_t flags, double pred, uint32_t *words,
                                           uint64_t *count, buff_sum_result *sum,
                                           void *stream) {
  if (!image || !sum) return BUFF_EINVAL;
  if (len < 20) return BUFF_ECORRUPT;
  cudaStream_t s = S(stream);
  buff_col *c = nullptr;
  int rc = parse_header(image, len, scale, flags, s, &c);
  if (rc) return rc;
  if (c->n && !words) {
    buffh::free_col(c);
    return BUFF_EINVAL;
  }
  const int64_t fp = buffh::fetch_fixed(pred, c->precision_exp, c->dlen);
  const uint8_t *img = static_cast<const uint8_t *>(device_view(image, c->device));
  uint32_t *dwords = c->n ? static_cast<uint32_t *>(const_cast<void *>(device_view(words, c->device)))
                          : nullptr;
  // Plans that are not one pass over full slices (the intended semantics,
  // codes narrower than a byte, the early return, no rows), and buffers the
  // device cannot reach, take the two-step path.
  if ((flags & BUFF_FLAG_INTENDED) || c->k == 0 || fp < c->base || c->n == 0 || !img ||
      !dwords) {
    buffh::free_col(c);
    return via_column(image, len, scale, flags, pred, words, count, sum, stream);
  }
  ImgArgs a;
  memset(&a, 0, sizeof(a));
  const uint64_t t = (uint64_t)(fp - c->base);
  const uint32_t fl = c->fixed_len;
  a.slices = img + 20;
  a.tail = img + 20 + (uint64_t)c->k * c->n;
  a.n = c->n;
  a.k = c->k;
  a.r = c->r;
  a.flipx = (flags & BUFF_FLAG_BUFF_LAYOUT) ? 0x80808080u : 0u;
  a.full_rows = c->n / 32 * 32;
  for (uint32_t j = 0; j < c->k; ++j)
    a.tb |= (unsigned long long)(uint8_t)(t >> (fl - 8 * (j + 1))) << (8 * j);
  a.ttail = c->r ? (uint32_t)(t & ((1ull << c->r) - 1)) : 0u;
  a.tail_bytes = c->tail_bytes;
  a.words = dwords;
  unsigned long long *d = nullptr;  // 9 partials, then the count
  uint64_t host[10] = {0};
  cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&d), 10 * sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = buffk::zero_u64(d, 10, s);
  if (e == cudaSuccess) {
    a.parts = d;
    a.count = d + 9;
    // k slice regions, then the tail: 512r bytes of a chunk plus 64 of slack
    // (16 of misalignment, the word past a block's last tail word, the pad)
    const size_t smem = (size_t)c->k * kRegion + kImgRows / 8 * c->r + 64;
    int per_sm = 0, sms = buffk::num_sms(c->device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_filter_sum_image, kImgThreads, smem);
    if (per_sm < 1) per_sm = 1;
    const uint32_t nchunks = (c->n + kImgRows - 1) / kImgRows;
    uint32_t grid = (uint32_t)(per_sm * sms);
    if (grid > nchunks) grid = nchunks;
    k_filter_sum_image<<<grid, kImgThreads, smem, s>>>(a);
    buffk::count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(host, d, 10 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (d) cudaFreeAsync(d, s);
  rc = buffh::cuda_status(e);
  if (!rc) {
    if (count) {
      if (buffh::is_device_ptr(count))
        rc = buffh::cuda_status(cudaMemcpyAsync(count, host + 9, 8, cudaMemcpyHostToDevice, s));
      else
        *count = host[9];
    }
    if (!rc) rc = buff_sum_finish(c, host, sum);
  }
  buffh::free_col(c);
  return rc;
}

namespace buffk {
// Writes the `nslices` slices of c (XOR flipx) and then its packed tail into
// `dst` through k_download_image when the device can write there in place;
// returns false (nothing done) when it cannot.
bool download_body(const buff_col *c, uint8_t *dst, uint32_t nslices, uint32_t flipx,
                   cudaStream_t s, cudaError_t *err) {
  uint8_t *d = static_cast<uint8_t *>(const_cast<void *>(device_view(dst, c->device)));
  if (!d || !c->n) return false;
  const uint64_t big = c->n > c->tail_bytes ? c->n : c->tail_bytes;
  uint64_t gx = (big / 16 + 255) / 256;
  const uint64_t cap = (uint64_t)8 * num_sms(c->device) / (nslices + 1) + 1;
  if (gx > cap) gx = cap;
  if (gx < 1) gx = 1;
  dim3 grid((unsigned)gx, nslices + 1);
  k_download_image<<<grid, 256, 0, s>>>(c->slices, c->stride, c->n, nslices, c->tail,
                                        c->tail_bytes, c->tail_alloc, flipx, d);
  count_launch();
  *err = cudaGetLastError();
  return true;
}

// The body of c's image (`nslices` slices XOR flipx, then the packed tail;
// body_bytes long) written to host memory dst.  Pinned memory is written by
// the device in place; pageable memory through a device staging copy and one
// copy-engine transfer: the device faulting a fresh pageable buffer's pages
// in ran ~6x slower than the copy engine (185 MB: 48.6 against 7.9 ms), and
// the buffer a caller hands over is usually fresh.  Returns false (nothing
// done) when neither can be set up; the caller then uses pitched copies.
bool body_to_host(const buff_col *c, uint8_t *dst, uint64_t body_bytes, uint32_t nslices,
                  uint32_t flipx, cudaStream_t s, cudaError_t *err) {
  if (!c->n) return false;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, dst) == cudaSuccess && at.type == cudaMemoryTypeHost)
    return download_body(c, dst, nslices, flipx, s, err);
  cudaGetLastError();
  uint8_t *stage = nullptr;
  if (cudaMallocAsync(reinterpret_cast<void **>(&stage), body_bytes, s) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  cudaError_t e = cudaSuccess;
  download_body(c, stage, nslices, flipx, s, &e);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dst, stage, body_bytes, cudaMemcpyDeviceToHost, s);
  const cudaError_t f = cudaFreeAsync(stage, s);
  *err = e != cudaSuccess ? e : f;
  return true;
}

// Copies the k slices of a serialized image (image + 20, slice j at j * n;
// host or device memory) into c->slices through k_upload_slices when the
// device can read the image in place; returns false (nothing done) when it
// cannot, so the caller uses a pitched copy.
bool upload_slices(const uint8_t *image, buff_col *c, uint32_t flipx, cudaStream_t s,
                   cudaError_t *err) {
  const uint8_t *img = static_cast<const uint8_t *>(device_view(image, c->device));
  if (!img || !c->k || !c->n) return false;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_upload_slices, kImgThreads, 0);
  if (per_sm < 1) per_sm = 1;
  const uint64_t items = (uint64_t)c->k * ((c->stride + kImgRows - 1) / kImgRows);
  uint64_t grid = (uint64_t)per_sm * num_sms(c->device);
  if (grid > items) grid = items;
  k_upload_slices<<<(unsigned)grid, kImgThreads, 0, s>>>(img + 20, c->n, c->k, c->stride, flipx,
                                                        c->slices);
  count_launch();
  *err = cudaGetLastError();
  return true;
}
}  // namespace buffk
