// tools.cu -- GPU kernels for the reference's command-line tools:
//   - s2tc_compress (s2tc_compress.c:594-719): mip reduction
//     (Image_MipReduce32, :426-493) and the header's "alpha pixels" test; the
//     pipeline itself is s2tc_compress_dds in capi.cpp;
//   - s2tc_decompress (s2tc_decompress.c:156-207): a whole-image decoder with
//     the fetch_2d_texel_* semantics (s2tc_libtxc_dxtn.cpp:35-140), including
//     the checkerboard decode of indices 2 and 3;
//   - s2tc_from_s3tc (s2tc_from_s3tc.cpp:77-269): the per-block rewrite of an
//     S3TC file into S2TC.
// All three are elementwise over texels or blocks and bound by HBM.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>

#include "dither.h"
#include "s2tc_gb300.h"
#include "tools.h"

namespace s2tc {
namespace {

constexpr int kThreads = 256;

unsigned grid_for(long long n) {
  const long long g = (n + kThreads - 1) / kThreads;
  return unsigned(g < 1 ? 1 : g > (1ll << 30) ? (1ll << 30) : g);
}

// Per-channel mean of byte lanes: (a + b) >> 1 and (a + b + c + d) >> 2 on
// four channels at once, in 16-bit lanes.
__device__ __forceinline__ uint32_t avg2(uint32_t a, uint32_t b) {
  const uint32_t lo = ((a & 0x00FF00FFu) + (b & 0x00FF00FFu)) >> 1;
  const uint32_t hi = (((a >> 8) & 0x00FF00FFu) + ((b >> 8) & 0x00FF00FFu)) >> 1;
  return (lo & 0x00FF00FFu) | ((hi & 0x00FF00FFu) << 8);
}
__device__ __forceinline__ uint32_t avg4(uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
  const uint32_t lo = ((a & 0x00FF00FFu) + (b & 0x00FF00FFu) + (c & 0x00FF00FFu) + (d & 0x00FF00FFu)) >> 2;
  const uint32_t hi =
      (((a >> 8) & 0x00FF00FFu) + ((b >> 8) & 0x00FF00FFu) + ((c >> 8) & 0x00FF00FFu) + ((d >> 8) & 0x00FF00FFu)) >> 2;
  return (lo & 0x00FF00FFu) | ((hi & 0x00FF00FFu) << 8);
}

// Image_MipReduce32 (s2tc_compress.c:426-493) out of place; the in-place
// original never reads a texel it has already written, so the results agree.
__global__ void k_mip_reduce(const uint32_t* __restrict__ in, int w, int h, uint32_t* __restrict__ out, int w2,
                             int h2) {
  const long long n = (long long)w2 * h2;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const int y = int(k / w2), x = int(k % w2);
    uint32_t v;
    if (w > 1 && h > 1) {
      const uint32_t* p = in + (long long)(2 * y) * w + 2 * x;
      v = avg4(__ldg(p), __ldg(p + 1), __ldg(p + w), __ldg(p + w + 1));
    } else if (w > 1) {
      const uint32_t* p = in + (long long)y * w + 2 * x;
      v = avg2(__ldg(p), __ldg(p + 1));
    } else {
      const uint32_t* p = in + (long long)(2 * y) * w + x;
      v = avg2(__ldg(p), __ldg(p + w));
    }
    out[k] = v;
  }
}

__global__ void k_any_alpha(const uint32_t* __restrict__ px, long long n, int* flag) {
  bool any = false;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    any |= (__ldg(px + k) >> 24) != 255u;
  if (__any_sync(0xFFFFFFFFu, any) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

// ------------------------------------------------------------------ decode

__device__ __forceinline__ uint32_t expand565(uint32_t c) {
  const uint32_t r = (c >> 11) & 31, g = (c >> 5) & 63, b = c & 31;
  return ((r << 3) | (r >> 2)) | (((g << 2) | (g >> 4)) << 8) | (((b << 3) | (b >> 2)) << 16);
}

__device__ __forceinline__ uint64_t load8(const uint8_t* p) {
  if ((reinterpret_cast<uintptr_t>(p) & 7) == 0) return *reinterpret_cast<const uint64_t*>(p);
  uint64_t v = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) v |= uint64_t(p[i]) << (8 * i);
  return v;
}

__device__ __forceinline__ void store8(uint8_t* p, uint64_t v) {
  if ((reinterpret_cast<uintptr_t>(p) & 7) == 0) {
    *reinterpret_cast<uint64_t*>(p) = v;
    return;
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) p[i] = uint8_t(v >> (8 * i));
}

// One thread per block: the 16 texels of fetch_2d_texel_{rgb,rgba}_dxt1 /
// _rgba_dxt3 / _rgba_dxt5, written as RGBA8 (BGRA8 with `bgra`, the byte
// order s2tc_decompress writes) rows `pitch` bytes apart.
template <int DXT>
__global__ void k_decode(const uint8_t* __restrict__ blocks, int rgba_dxt1, int width, int height,
                         uint8_t* __restrict__ out, long long pitch, int bgra) {
  const int bw = (width + 3) / 4, bh = (height + 3) / 4;
  const long long nb = (long long)bw * bh;
  const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nb) return;
  const int bx = int(k % bw), by = int(k / bw);
  constexpr int bs = DXT == DXT1 ? 8 : 16;
  const uint8_t* blk = blocks + k * bs;
  const uint64_t colour = load8(blk + bs - 8);
  const uint64_t alpha = DXT == DXT1 ? 0 : load8(blk);
  const uint32_t c = uint32_t(colour) & 0xFFFFu, c1 = uint32_t(colour >> 16) & 0xFFFFu;
  const uint32_t idx = uint32_t(colour >> 32);
  uint32_t col0 = expand565(c), col1 = expand565(c1);
  if (bgra) {
    col0 = __byte_perm(col0, 0, 0x3012);
    col1 = __byte_perm(col1, 0, 0x3012);
  }
  const uint32_t a0 = uint32_t(alpha) & 0xFFu, a1 = uint32_t(alpha >> 8) & 0xFFu;
  const bool trans_ok = DXT == DXT1 && c1 >= c;  // index 3 is transparent black
  const uint32_t trans_a = rgba_dxt1 ? 0u : 255u;
  // all 16 texels without branches (slot s = 4y + x; index bits 2s)
  uint32_t t[16];
#pragma unroll
  for (int s = 0; s < 16; ++s) {
    const int x = s & 3, y = s >> 2;
    const bool odd = ((x ^ y) & 1) != 0;
    const uint32_t sel = (idx >> (2 * s)) & 3u;
    const bool one = sel == 1 || (sel >= 2 && odd);
    const bool trans = trans_ok && sel == 3;
    uint32_t rgb = one ? col1 : col0;
    rgb = trans ? 0u : rgb;
    uint32_t a = trans ? trans_a : 255u;
    if (DXT == DXT3) {
      const uint32_t a4 = uint32_t(alpha >> (4 * s)) & 15u;
      a = a4 | (a4 << 4);
    } else if (DXT == DXT5) {
      const uint32_t ab = uint32_t(alpha >> (16 + 3 * s)) & 7u;
      const bool hi = a1 >= a0;
      a = (ab >= 2 && odd) ? a1 : a0;
      a = (ab == 7 && hi) ? 255u : a;
      a = (ab == 6 && hi) ? 0u : a;
      a = ab == 1 ? a1 : a;
    }
    t[s] = rgb | (a << 24);
  }
  const int cw = min(4, width - 4 * bx), ch = min(4, height - 4 * by);
  uint8_t* o = out + (long long)(4 * by) * pitch + (long long)(4 * bx) * 4;
  if (cw == 4 && ch == 4 && ((reinterpret_cast<uintptr_t>(o) | uintptr_t(pitch)) & 15) == 0) {
#pragma unroll
    for (int y = 0; y < 4; ++y)
      *reinterpret_cast<uint4*>(o + y * pitch) = make_uint4(t[4 * y], t[4 * y + 1], t[4 * y + 2], t[4 * y + 3]);
    return;
  }
  for (int y = 0; y < ch; ++y)
    for (int x = 0; x < cw; ++x) {
      uint8_t* q = o + y * pitch + 4 * x;
      if ((reinterpret_cast<uintptr_t>(q) & 3) == 0) {
        *reinterpret_cast<uint32_t*>(q) = t[4 * y + x];
      } else {
        for (int b = 0; b < 4; ++b) q[b] = uint8_t(t[4 * y + x] >> (8 * b));
      }
    }
}

// --------------------------------------------------------------- from_s3tc

// Colour half (s2tc_from_s3tc.cpp:77-143): indices become 0/1, then the
// endpoints take S2TC order (inverting the indices on a swap).  `alpha`: the
// DXT1 variant that keeps index 3 transparent when c1 >= c0.
__device__ __forceinline__ uint64_t s3tc_colour(uint64_t v, bool alpha) {
  uint32_t c = uint32_t(v) & 0xFFFFu, c1 = uint32_t(v >> 16) & 0xFFFFu, px = uint32_t(v >> 32);
  const uint32_t two = (px & 0x22882288u) >> 1;
  bool swap;
  if (c1 >= c) {
    px = alpha ? (px & ~((~px & 0x55555555u) << 1)) | two : (px & ((~px & 0xAAAAAAAAu) >> 1)) | two;
    swap = !alpha;
  } else {
    px = (px & ((~px & 0xAAAAAAAAu) >> 1)) | two;
    swap = alpha;
  }
  if (swap) {
    const uint32_t t = c;
    c = c1;
    c1 = t;
    px ^= 0x55555555u;
  }
  return uint64_t(c) | (uint64_t(c1) << 16) | (uint64_t(px) << 32);
}

// DXT5 alpha half (s2tc_from_s3tc.cpp:145-190).
__device__ __forceinline__ uint64_t s3tc_alpha(uint64_t v) {
  uint32_t a = uint32_t(v) & 0xFFu, a1 = uint32_t(v >> 8) & 0xFFu;
  uint64_t px = v >> 16;
  constexpr uint64_t ones = 01111111111111111ull, pick = 00101101001011010ull;
  if (a1 >= a) {
    const uint64_t sel = (px >> 1) ^ (px >> 2);
    px = (px & ~((sel & ones) * 7)) | (sel & pick);
  } else {
    const uint64_t sel = (px >> 1) | (px >> 2);
    px = (px & ~((sel & ones) * 7)) | (sel & pick);
    const uint32_t t = a;
    a = a1;
    a1 = t;
    px ^= ones;
  }
  return uint64_t(a) | (uint64_t(a1) << 8) | ((px & 0xFFFFFFFFFFFFull) << 16);
}

template <int DXT>
__global__ void k_from_s3tc(const uint8_t* src, uint8_t* dst, long long nblocks) {
  constexpr int bs = DXT == DXT1 ? 8 : 16;
  for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < nblocks;
       k += (long long)gridDim.x * blockDim.x) {
    const uint8_t* s = src + k * bs;
    uint8_t* d = dst + k * bs;
    if (DXT == DXT1) {
      store8(d, s3tc_colour(load8(s), true));
    } else if (((reinterpret_cast<uintptr_t>(s) | reinterpret_cast<uintptr_t>(d)) & 15) == 0) {
      const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(s);  // src may be dst
      *reinterpret_cast<ulonglong2*>(d) =
          make_ulonglong2(DXT == DXT5 ? s3tc_alpha(v.x) : v.x, s3tc_colour(v.y, false));
    } else {
      const uint64_t lo = load8(s), hi = load8(s + 8);
      store8(d + 8, s3tc_colour(hi, false));
      store8(d, DXT == DXT5 ? s3tc_alpha(lo) : lo);
    }
  }
}

int fail(int status, const char* fn, const char* msg) {
  std::fprintf(stderr, "s2tc_gb300: %s: %s\n", fn, msg);
  return status;
}

int cuda_fail(const char* fn, cudaError_t e) {
  std::fprintf(stderr, "s2tc_gb300: %s: %s\n", fn, cudaGetErrorString(e));
  return S2TC_ERR_CUDA;
}

int fourcc_dxt(const unsigned char* hdr) {
  const uint32_t f = uint32_t(hdr[84]) | (uint32_t(hdr[85]) << 8) | (uint32_t(hdr[86]) << 16) |
                     (uint32_t(hdr[87]) << 24);
  switch (f) {
    case 0x31545844u: return DXT1;
    case 0x33545844u: return DXT3;
    case 0x35545844u: return DXT5;
    default: return -1;
  }
}

uint32_t le32(const unsigned char* p) {
  return uint32_t(p[0]) | (uint32_t(p[1]) << 8) | (uint32_t(p[2]) << 16) | (uint32_t(p[3]) << 24);
}

int gl_dxt(unsigned int format, int* rgba_dxt1) {
  *rgba_dxt1 = format != S2TC_GL_COMPRESSED_RGB_S3TC_DXT1_EXT;
  switch (format) {
    case S2TC_GL_COMPRESSED_RGB_S3TC_DXT1_EXT:
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT1_EXT: return DXT1;
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT3_EXT: return DXT3;
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT5_EXT: return DXT5;
    default: return -1;
  }
}

cudaError_t launch_decode(const uint8_t* blocks, int dxt, int rgba_dxt1, int width, int height, uint8_t* out,
                          long long pitch, int bgra, cudaStream_t s) {
  const long long nb = (long long)((width + 3) / 4) * ((height + 3) / 4);
  const unsigned g = unsigned((nb + kThreads - 1) / kThreads);
  count_launches(1);
  switch (dxt) {
    case DXT1: k_decode<DXT1><<<g, kThreads, 0, s>>>(blocks, rgba_dxt1, width, height, out, pitch, bgra); break;
    case DXT3: k_decode<DXT3><<<g, kThreads, 0, s>>>(blocks, rgba_dxt1, width, height, out, pitch, bgra); break;
    default: k_decode<DXT5><<<g, kThreads, 0, s>>>(blocks, rgba_dxt1, width, height, out, pitch, bgra); break;
  }
  return cudaGetLastError();
}

cudaError_t launch_from_s3tc(const uint8_t* src, uint8_t* dst, long long nblocks, int dxt, cudaStream_t s) {
  if (nblocks <= 0) return cudaSuccess;
  const unsigned g = grid_for(nblocks);
  count_launches(1);
  switch (dxt) {
    case DXT1: k_from_s3tc<DXT1><<<g, kThreads, 0, s>>>(src, dst, nblocks); break;
    case DXT3: k_from_s3tc<DXT3><<<g, kThreads, 0, s>>>(src, dst, nblocks); break;
    default: k_from_s3tc<DXT5><<<g, kThreads, 0, s>>>(src, dst, nblocks); break;
  }
  return cudaGetLastError();
}

// Device scratch of one host-buffer tool call, freed on every return path.
struct Scratch {
  void* p = nullptr;
  ~Scratch() {
    if (p) cudaFree(p);
  }
};

}  // namespace

cudaError_t launch_mip_reduce(const uint8_t* in, int w, int h, uint8_t* out, cudaStream_t s) {
  int w2 = w, h2 = h;
  mip_next(w2, h2);
  count_launches(1);
  k_mip_reduce<<<grid_for((long long)w2 * h2), kThreads, 0, s>>>(reinterpret_cast<const uint32_t*>(in), w, h,
                                                                   reinterpret_cast<uint32_t*>(out), w2, h2);
  return cudaGetLastError();
}

cudaError_t launch_any_alpha(const uint8_t* rgba, long long npx, int* flag, cudaStream_t s) {
  count_launches(1);
  const long long g = std::min<long long>(grid_for(npx), 152 * 8);
  k_any_alpha<<<unsigned(g), kThreads, 0, s>>>(reinterpret_cast<const uint32_t*>(rgba), npx, flag);
  return cudaGetLastError();
}

}  // namespace s2tc

extern "C" {

int s2tc_gpu_decode(const void* d_blocks, unsigned int format, int width, int height, void* d_out,
                    long long dst_pitch, int bgra, void* stream) {
  using namespace s2tc;
  int rgba_dxt1 = 1;
  const int dxt = gl_dxt(format, &rgba_dxt1);
  if (dxt < 0) return fail(S2TC_ERR_FORMAT, "s2tc_gpu_decode", "bad format");
  if (width < 0 || height < 0) return fail(S2TC_ERR_ARGUMENT, "s2tc_gpu_decode", "bad size");
  if (width == 0 || height == 0) return S2TC_OK;
  if (!d_blocks || !d_out) return fail(S2TC_ERR_ARGUMENT, "s2tc_gpu_decode", "null buffer");
  if (dst_pitch == 0) dst_pitch = (long long)width * 4;
  if (dst_pitch < (long long)width * 4) return fail(S2TC_ERR_ARGUMENT, "s2tc_gpu_decode", "dst_pitch below width*4");
  const cudaError_t e = launch_decode(static_cast<const uint8_t*>(d_blocks), dxt, rgba_dxt1, width, height,
                                      static_cast<uint8_t*>(d_out), dst_pitch, bgra ? 1 : 0,
                                      static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? S2TC_OK : cuda_fail("s2tc_gpu_decode", e);
}

int s2tc_gpu_from_s3tc(const void* d_src, void* d_dst, long long nblocks, unsigned int format, void* stream) {
  using namespace s2tc;
  int rgba_dxt1 = 1;
  const int dxt = gl_dxt(format, &rgba_dxt1);
  if (dxt < 0) return fail(S2TC_ERR_FORMAT, "s2tc_gpu_from_s3tc", "bad format");
  if (nblocks < 0 || (nblocks > 0 && (!d_src || !d_dst))) return fail(S2TC_ERR_ARGUMENT, "s2tc_gpu_from_s3tc", "bad argument");
  const cudaError_t e = launch_from_s3tc(static_cast<const uint8_t*>(d_src), static_cast<uint8_t*>(d_dst), nblocks,
                                         dxt, static_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? S2TC_OK : cuda_fail("s2tc_gpu_from_s3tc", e);
}

int s2tc_decompress_dds(const void* dds, long long size, void* tga, long long tga_size, long long* written) {
  using namespace s2tc;
  const unsigned char* in = static_cast<const unsigned char*>(dds);
  if (written) *written = 0;
  if (!in || !tga || size < 128) return fail(S2TC_ERR_ARGUMENT, "s2tc_decompress_dds", "bad argument");
  const int height = int(le32(in + 12)), width = int(le32(in + 16));
  const int dxt = fourcc_dxt(in);
  if (dxt < 0) {
    std::fprintf(stderr, "Only DXT1, DXT3, DXT5 are supported!\n");
    return S2TC_ERR_FORMAT;
  }
  if (width <= 0 || height <= 0 || width > 65535 || height > 65535)
    return fail(S2TC_ERR_ARGUMENT, "s2tc_decompress_dds", "bad image size");
  const long long bs = dxt == s2tc::DXT1 ? 8 : 16;
  const long long blocks = (long long)((width + 3) / 4) * ((height + 3) / 4) * bs;
  const long long pixels = (long long)width * height * 4;
  if (size < 128 + blocks) return fail(S2TC_ERR_ARGUMENT, "s2tc_decompress_dds", "file shorter than its base level");
  if (tga_size < 18 + pixels) return fail(S2TC_ERR_ARGUMENT, "s2tc_decompress_dds", "output buffer too small");
  Scratch sc;
  cudaError_t e = cudaMalloc(&sc.p, size_t(blocks + pixels) + 16);
  if (e != cudaSuccess) return cuda_fail("s2tc_decompress_dds", e);
  uint8_t* d_blk = static_cast<uint8_t*>(sc.p);
  uint8_t* d_px = d_blk + ((blocks + 15) & ~15ll);
  unsigned char* out = static_cast<unsigned char*>(tga);
  e = cudaMemcpy(d_blk, in + 128, size_t(blocks), cudaMemcpyHostToDevice);
  // the decoder uses the RGBA variant for DXT1 (s2tc_decompress.c:163-166)
  if (e == cudaSuccess) e = launch_decode(d_blk, dxt, 1, width, height, d_px, (long long)width * 4, 1, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(out + 18, d_px, size_t(pixels), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail("s2tc_decompress_dds", e);
  std::memset(out, 0, 18);
  out[2] = 2;
  out[12] = uint8_t(width % 256);
  out[13] = uint8_t(width / 256);
  out[14] = uint8_t(height % 256);
  out[15] = uint8_t(height / 256);
  out[16] = 32;
  out[17] = 0x28;
  if (written) *written = 18 + pixels;
  return S2TC_OK;
}

int s2tc_from_s3tc_dds(const void* dds, long long size, void* out, long long out_size, long long* written) {
  using namespace s2tc;
  const unsigned char* in = static_cast<const unsigned char*>(dds);
  if (written) *written = 0;
  if (!in || !out || size < 128) return fail(S2TC_ERR_ARGUMENT, "s2tc_from_s3tc_dds", "bad argument");
  const int dxt = fourcc_dxt(in);
  if (dxt < 0) {
    std::fprintf(stderr, "Only DXT1, DXT3, DXT5 are supported!\n");
    return S2TC_ERR_FORMAT;
  }
  const long long bs = dxt == s2tc::DXT1 ? 8 : 16;
  const long long n = (size - 128) / bs;  // a trailing partial block is dropped
  if (out_size < 128 + n * bs) return fail(S2TC_ERR_ARGUMENT, "s2tc_from_s3tc_dds", "output buffer too small");
  unsigned char* o = static_cast<unsigned char*>(out);
  std::memmove(o, in, 128);
  if (n == 0) {
    if (written) *written = 128;
    return S2TC_OK;
  }
  Scratch sc;
  cudaError_t e = cudaMalloc(&sc.p, size_t(n * bs));
  if (e == cudaSuccess) e = cudaMemcpy(sc.p, in + 128, size_t(n * bs), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = launch_from_s3tc(static_cast<uint8_t*>(sc.p), static_cast<uint8_t*>(sc.p), n, dxt, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(o + 128, sc.p, size_t(n * bs), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail("s2tc_from_s3tc_dds", e);
  if (written) *written = 128 + n * bs;
  return S2TC_OK;
}

}  // extern "C"
