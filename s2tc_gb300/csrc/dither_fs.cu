// dither_fs.cu -- DITHER_FLOYDSTEINBERG (s2tc_algorithm.cpp:1218-1261,
// 1350-1411) as a wavefront.
//
// Texel (x, y) needs the error of (x-1, y) and of (x-1..x+1, y-1), so row y can
// run two texels behind row y-1.  Each CTA owns a band of kRows rows, one
// thread per row; at step t the thread of band row r handles x = t - 2r, and
// the rows exchange their down-going errors through shared memory once per
// step.  Bands are chained through a carry row in global memory: the band's
// last row accumulates the errors it sends down, publishes how many entries
// are final, and the next band's first row waits (bounded) for them.  Bands
// take tickets in launch order, so every band waits only on a band that is
// already running.
//
// The alpha channel runs as a second one-channel pass.  Like the reference,
// it starts from what the red pass left in its first error row (the last
// row's red errors, s2tc_algorithm.cpp:1354, 1380-1382).
#include <cuda/atomic>
#include <cuda_runtime.h>

#include <cstdint>

#include "dither.h"

namespace s2tc {
namespace {

constexpr int kRows = 128;        // rows per band = threads per CTA
constexpr int kChunk = 16;        // texels loaded / stored per thread at a time
constexpr int kSpinLimit = 1 << 22;

using Progress = cuda::atomic_ref<int, cuda::thread_scope_device>;

struct FsStep {
  int q, e7, e3, e5, e1;
};

// One Floyd-Steinberg step on 12-bit values; MAXV == 1 is the 1-bit variant.
template <int SHIFT, int MAXV>
__device__ __forceinline__ FsStep fs_step(int err_in, int src) {
  FsStep o;
  const int v = ((src << 4) | (src >> 4)) + err_in;
  int loop;
  if (MAXV == 1) {
    o.q = v >= 2048;
    loop = o.q ? 4095 : 0;
  } else {
    o.q = min(max(v >> (SHIFT + 4), 0), MAXV);
    loop = o.q * 4095 / MAXV;
  }
  int e = v - loop;
  o.e7 = (e * 7 + 8) / 16;
  e -= o.e7;
  o.e3 = (e * 3 + 4) / 9;
  e -= o.e3;
  o.e5 = (e * 5 + 3) / 6;
  e -= o.e5;
  o.e1 = e;
  return o;
}

struct FsArgs {
  const uint8_t* src;
  int width, height, srccomps;
  uint8_t* dst;           // texel words viewed as bytes
  int nbands;
  int* carry;             // (nbands + 1) rows of NCH * width ints; row b feeds band b
  int* progress;          // final carry entries per row, nbands + 1
  int* leftover;          // red pass: last row's red errors, width ints
  const int* seed_row;    // alpha pass: initial errors of row 0 (the red leftover), or null
  unsigned int* ticket;
  int* error;
  int alpha_mode;         // 1 or 4 bits, alpha pass only
};

// NCH == 3: red/green/blue pass, where AP is the constant alpha written for
// 3-component input (ignored for 4 components: the alpha byte is filled by a
// later pass).  NCH == 1: alpha pass, where AP is the alpha bit count (1 or 4).
template <int NCH, int SC, int AP>
__global__ void __launch_bounds__(kRows) k_fs(FsArgs a) {
  __shared__ int xch[2][kRows][NCH][3];  // (e3, e5, e1) sent down by each row
  __shared__ int s_band;
  const int r = threadIdx.x;
  if (r == 0) s_band = int(atomicAdd(a.ticket, 1u));
  __syncthreads();
  const int band = s_band;
  const int y = band * kRows + r;
  const bool row_ok = y < a.height;
  const int w = a.width;
  const int last_row_of_band = min(kRows, a.height - band * kRows) - 1;
  int* carry_in = a.carry + (size_t)band * NCH * w;
  int* carry_out = a.carry + (size_t)(band + 1) * NCH * w;
  int known = 0;  // carry_in entries known final (thread 0)

  int pend[NCH][3];
#pragma unroll
  for (int c = 0; c < NCH; ++c) pend[c][0] = pend[c][1] = pend[c][2] = 0;
  uint32_t in_buf[kChunk];
  uint8_t out_buf[NCH][kChunk];

  const int nsteps = w + 2 * (kRows - 1);
  int buf = 0;
  for (int t = 0; t < nsteps; ++t) {
    const int x = t - 2 * r;
    const bool act = row_ok && x >= 0 && x < w;
    int sent[NCH][3];
#pragma unroll
    for (int c = 0; c < NCH; ++c) sent[c][0] = sent[c][1] = sent[c][2] = 0;
    if (act) {
      const int slot = x % kChunk;
      if (slot == 0) {
        // load texels [x, x + kChunk) of this row
        const uint8_t* s = a.src + ((size_t)y * w + x) * SC;
#pragma unroll
        for (int k = 0; k < kChunk; ++k) {
          uint32_t v = 0;
          if (x + k < w) {
            if (NCH == 3) v = uint32_t(s[k * SC]) | (uint32_t(s[k * SC + 1]) << 8) | (uint32_t(s[k * SC + 2]) << 16);
            else v = uint32_t(s[k * SC + 3]);
          }
          in_buf[k] = v;
        }
      }
      if (r == 0 && (band > 0 || a.seed_row)) {
        // errors coming from the row above this band
        if (band > 0) {
          if (known <= x) {
            Progress p(a.progress[band]);
            int v = p.load(cuda::memory_order_acquire);
            int spins = 0;
            while (v <= x && spins < kSpinLimit) {
              __nanosleep(32);
              v = p.load(cuda::memory_order_acquire);
              ++spins;
            }
            if (v <= x) atomicExch(a.error, 1);
            known = v;
          }
#pragma unroll
          for (int c = 0; c < NCH; ++c) pend[c][0] += __ldcg(carry_in + (size_t)c * w + x);
        } else {
          pend[0][0] += a.seed_row[x];
        }
      }
#pragma unroll
      for (int c = 0; c < NCH; ++c) {
        const int srcv = int((in_buf[slot] >> (8 * c)) & 0xFF);
        FsStep f;
        if (NCH == 1) {
          f = AP == 1 ? fs_step<7, 1>(pend[c][0], srcv) : fs_step<4, 15>(pend[c][0], srcv);
        } else {
          f = c == 1 ? fs_step<2, 63>(pend[c][0], srcv) : fs_step<3, 31>(pend[c][0], srcv);
        }
        if (NCH == 3 && c == 0 && y == a.height - 1 && ((a.height - 1) & 1) == 0) a.leftover[x] = pend[c][0];
        pend[c][1] += f.e7;
        sent[c][0] = f.e3;
        sent[c][1] = f.e5;
        sent[c][2] = f.e1;
        out_buf[c][slot] = uint8_t(f.q);
      }
      if (NCH == 3 && y == a.height - 1 && ((a.height - 1) & 1) == 1) {
        // the red pass leaves the errors it sent below the last row
        if (x > 0) a.leftover[x - 1] += sent[0][0];
        a.leftover[x] += sent[0][1];
        if (x + 1 < w) a.leftover[x + 1] += sent[0][2];
      }
      if (r == last_row_of_band && band + 1 < a.nbands) {
#pragma unroll
        for (int c = 0; c < NCH; ++c) {
          int* co = carry_out + (size_t)c * w;
          if (x > 0) co[x - 1] += sent[c][0];
          co[x] += sent[c][1];
          if (x + 1 < w) co[x + 1] += sent[c][2];
        }
        // entries 0..x-1 are final now
        if ((x & 31) == 31 || x == w - 1) {
          __threadfence();
          Progress p(a.progress[band + 1]);
          p.store(x == w - 1 ? w : x, cuda::memory_order_release);
        }
      }
      if (slot == kChunk - 1 || x == w - 1) {
        // flush texels [x - slot, x] of this row
        const int x0 = x - slot;
        for (int k = 0; k <= slot; ++k) {
          uint8_t* o = a.dst + ((size_t)y * w + x0 + k) * 4;
          if (NCH == 3) {
            const uint32_t al = SC == 3 ? uint32_t(AP) : 0u;
            *reinterpret_cast<uint32_t*>(o) =
                uint32_t(out_buf[0][k]) | (uint32_t(out_buf[1 % NCH][k]) << 8) | (uint32_t(out_buf[2 % NCH][k]) << 16) |
                (al << 24);
          } else {
            o[3] = out_buf[0][k];
          }
        }
      }
    }
    // exchange with the row below
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
      xch[buf][r][c][0] = sent[c][0];
      xch[buf][r][c][1] = sent[c][1];
      xch[buf][r][c][2] = sent[c][2];
    }
    __syncthreads();
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
      pend[c][0] = pend[c][1];
      pend[c][1] = pend[c][2];
      pend[c][2] = 0;
      if (r > 0) {
        pend[c][0] += xch[buf][r - 1][c][0];
        pend[c][1] += xch[buf][r - 1][c][1];
        pend[c][2] += xch[buf][r - 1][c][2];
      }
    }
    buf ^= 1;
  }
}

// 8-bit alpha passes through unchanged (s2tc_algorithm.cpp:1387-1392).
__global__ void __launch_bounds__(256) k_alpha_copy(const uint8_t* __restrict__ src, uint8_t* dst, long long npx) {
  const long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < npx) dst[p * 4 + 3] = src[p * 4 + 3];
}

}  // namespace

size_t dither_fs_scratch_bytes(int width, int height) {
  const long long nbands = (height + kRows - 1) / kRows;
  // carry rows (3 channels), progress words, leftover row, ticket + flags
  return size_t(nbands + 1) * 3 * width * sizeof(int) + size_t(nbands + 1) * sizeof(int) + size_t(width) * sizeof(int) +
         512;
}

cudaError_t launch_dither_fs(DitherArgs d, uint8_t* scratch, cudaStream_t s) {
  const int w = d.width, h = d.height;
  const int nbands = (h + kRows - 1) / kRows;
  FsArgs a;
  a.src = d.src;
  a.width = w;
  a.height = h;
  a.srccomps = d.srccomps;
  a.dst = reinterpret_cast<uint8_t*>(d.dst);
  a.nbands = nbands;
  size_t off = 0;
  a.carry = reinterpret_cast<int*>(scratch + off);
  off += size_t(nbands + 1) * 3 * w * sizeof(int);
  a.progress = reinterpret_cast<int*>(scratch + off);
  off += size_t(nbands + 1) * sizeof(int);
  a.leftover = reinterpret_cast<int*>(scratch + off);
  off += size_t(w) * sizeof(int);
  off = (off + 15) & ~size_t(15);
  a.ticket = reinterpret_cast<unsigned int*>(scratch + off);
  a.error = d.error;
  a.seed_row = nullptr;
  cudaError_t e = cudaMemsetAsync(scratch, 0, off + 16, s);
  if (e != cudaSuccess) return e;
  const int abits = d.alphabits;
  // red/green/blue pass; for 3-component input the alpha byte is the constant
  count_launches(1);
  if (d.srccomps == 3) {
    if (abits == 1) k_fs<3, 3, 1><<<nbands, kRows, 0, s>>>(a);
    else if (abits == 4) k_fs<3, 3, 15><<<nbands, kRows, 0, s>>>(a);
    else k_fs<3, 3, 255><<<nbands, kRows, 0, s>>>(a);
    return cudaGetLastError();
  }
  k_fs<3, 4, 0><<<nbands, kRows, 0, s>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (abits == 8) {
    const long long npx = (long long)w * h;
    count_launches(1);
    k_alpha_copy<<<unsigned((npx + 255) / 256), 256, 0, s>>>(d.src, a.dst, npx);
    return cudaGetLastError();
  }
  // alpha pass, seeded with the red leftover row
  FsArgs b = a;
  b.seed_row = a.leftover;
  b.leftover = nullptr;
  // fresh carry rows, progress and ticket for the second pass
  e = cudaMemsetAsync(a.carry, 0, size_t(nbands + 1) * 3 * w * sizeof(int) + size_t(nbands + 1) * sizeof(int), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(a.ticket, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  count_launches(1);
  if (abits == 1) k_fs<1, 4, 1><<<nbands, kRows, 0, s>>>(b);
  else k_fs<1, 4, 4><<<nbands, kRows, 0, s>>>(b);
  return cudaGetLastError();
}

}  // namespace s2tc
