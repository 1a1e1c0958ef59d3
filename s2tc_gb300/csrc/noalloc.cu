// noalloc.cu -- s2tc_gpu_compress_noalloc: image compression that allocates no
// memory, for callers that cannot call cudaMalloc.
//
// Some hosts of this library own every device allocation themselves: a
// renderer or game engine whose frame budget forbids allocator calls (they
// can block on the driver and stall the frame), a program that sub-allocates a
// fixed pool handed out at start-up, a process running under a strict memory
// cap.  s2tc_gpu_compress serves its scratch (the dither scan's state and the
// 5:6:5 texel words between the dither and encoder kernels) from a grow-only
// arena created with cudaMalloc, which such callers cannot accept.  This entry
// point instead keeps that scratch in one fixed array in the module's device
// memory, `g_noalloc_scratch` below, which the CUDA runtime places on every
// GPU that loads the library and which stays there until the process exits.
// The caller passes device pointers for the input pixels and the output
// blocks, exactly as for s2tc_gpu_compress.
//
// Limits and rules:
//   - images of at most kNoallocMaxTexels texels (4 Mi, e.g. 2048x2048); larger
//     ones are rejected with S2TC_ERR_TOO_LARGE;
//   - with Floyd-Steinberg dither the wavefront's carry rows (16 bytes per
//     texel column, rounded up to 8 columns, per 256 texel rows) must also fit
//     the kScanBytes region: width rounded up to 8 times ceil(height / 256) at
//     most 65520, so a 65536x64 image is rejected although it is under 4 Mi
//     texels;
//   - RANDOM_COLORS > 0 needs the caller's replayed rand() words (d_rand); the
//     host replay path would need a device buffer;
//   - the first call on a device resolves the array's device address
//     (cudaGetSymbolAddress) with that device current; make that first call
//     before any stream capture;
//   - every call shares the one array and finds the previous call's contents
//     in it; the call clears what the kernels need zeroed and waits for its
//     stream before returning, and calls in one process are serialised, but
//     calls whose work overlaps on the GPU (another instance of this library on
//     the same device, or work enqueued around the call that touches the array)
//     race on it.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "dither.h"
#include "encode.h"
#include "s2tc_gb300.h"
#include "s2tc_types.h"

namespace {

constexpr long long kNoallocMaxTexels = 1ll << 22;
constexpr size_t kTexelBytes = size_t(kNoallocMaxTexels) * 4;  // 5:6:5 texel words
constexpr size_t kScanBytes = size_t(1) << 20;                // dither scan state
constexpr size_t kFlagBytes = 256;                             // timeout flag
constexpr size_t kNoallocBytes = kTexelBytes + kScanBytes + kFlagBytes;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_addr[kMaxDevices] = {nullptr};

// The array's device address on the current device (set up once per device).
int scratch_address(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    std::fprintf(stderr, "s2tc_gb300: cudaGetDevice: %s\n", cudaGetErrorString(e));
    return S2TC_ERR_CUDA;
  }
  if (!g_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      std::fprintf(stderr, "s2tc_gb300: cudaGetSymbolAddress: %s\n", cudaGetErrorString(e));
      return S2TC_ERR_CUDA;
    }
    g_addr[dev] = static_cast<unsigned char*>(p);
  }
  *out = g_addr[dev];
  return S2TC_OK;
}

int fmt_dxt(unsigned int fmt) {
  switch (fmt) {
    case S2TC_GL_COMPRESSED_RGB_S3TC_DXT1_EXT:
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT1_EXT: return s2tc::DXT1;
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT3_EXT: return s2tc::DXT3;
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT5_EXT: return s2tc::DXT5;
    default: return -1;
  }
}

int fail(int status, const char* msg) {
  std::fprintf(stderr, "s2tc_gb300: s2tc_gpu_compress_noalloc: %s\n", msg);
  return status;
}

}  // namespace

extern "C" int s2tc_gpu_compress_noalloc(int srccomps, int width, int height, const void* d_src,
                                         unsigned int destformat, void* d_dst, long long dst_pitch,
                                         const s2tc_options* opt, const unsigned int* d_rand, void* stream) {
  using namespace s2tc;
  const int dxt = fmt_dxt(destformat);
  if (dxt < 0) return fail(S2TC_ERR_FORMAT, "bad destination format");
  if (!opt || width < 0 || height < 0) return fail(S2TC_ERR_ARGUMENT, "bad argument");
  if (width == 0 || height == 0) return S2TC_OK;
  if (!d_src || !d_dst) return fail(S2TC_ERR_ARGUMENT, "null buffer");
  const long long npx = (long long)width * height;
  if (npx > kNoallocMaxTexels) return fail(S2TC_ERR_TOO_LARGE, "image larger than 4 Mi texels");
  const int bw = (width + 3) / 4, bh = (height + 3) / 4, bs = dxt == s2tc::DXT1 ? 8 : 16;
  if (dst_pitch < (long long)bw * bs) return fail(S2TC_ERR_ARGUMENT, "dst_pitch smaller than a block row");
  s2tc_options o = *opt;
  if (o.dither != DI_NONE && o.dither != DI_FLOYDSTEINBERG) o.dither = DI_SIMPLE;
  if (o.metric < 0 || o.metric > 7) o.metric = CD_WAVG;
  if (o.refine != RF_NEVER && o.refine != RF_LOOP) o.refine = RF_ALWAYS;
  const bool normal = o.nrandom >= 0 || o.metric == CD_NORMALMAP;
  if (normal && o.nrandom > 0 && !d_rand) return fail(S2TC_ERR_ARGUMENT, "RANDOM_COLORS > 0 needs d_rand");
  const size_t scan = o.dither == DI_FLOYDSTEINBERG ? dither_fs_scratch_bytes(width, height) : dither_scratch_bytes(npx);
  if (scan > kScanBytes) return fail(S2TC_ERR_TOO_LARGE, "dither state larger than the fixed scratch");

  std::lock_guard<std::mutex> lock(g_mu);
  unsigned char* base = nullptr;
  int st = scratch_address(&base);
  if (st != S2TC_OK) return st;
  uint32_t* texels = reinterpret_cast<uint32_t*>(base);
  uint8_t* scan_state = base + kTexelBytes;
  int* flag = reinterpret_cast<int*>(base + kTexelBytes + kScanBytes);
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  cudaError_t e = cudaMemsetAsync(flag, 0, sizeof(int), s);
  DitherArgs da{};
  da.src = static_cast<const uint8_t*>(d_src);
  da.width = width;
  da.height = height;
  da.srccomps = srccomps == 3 ? 3 : 4;
  da.alphabits = dxt == s2tc::DXT1 ? 1 : dxt == s2tc::DXT3 ? 4 : 8;
  da.dst = texels;
  da.error = flag;
  if (e == cudaSuccess) e = launch_dither(da, o.dither, scan_state, s);
  EncodeArgs ea{};
  ea.t565 = texels;
  ea.width = width;
  ea.height = height;
  ea.bw = bw;
  ea.bh = bh;
  ea.by0 = 0;
  ea.nby = bh;
  ea.dst = static_cast<uint8_t*>(d_dst);
  ea.pitch = dst_pitch;
  ea.aligned = ((reinterpret_cast<uintptr_t>(d_dst) % bs) == 0 && (dst_pitch % bs) == 0) ? 1 : 0;
  ea.nrandom = o.nrandom;
  ea.rnd = (normal && o.nrandom > 0) ? d_rand : nullptr;
  ea.prev_a1_first = -1;
  ea.leftover_out = nullptr;
  if (e == cudaSuccess) e = launch_encode(ea, dxt, o.metric, normal, o.refine, s);
  int timed_out = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&timed_out, flag, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    std::fprintf(stderr, "s2tc_gb300: s2tc_gpu_compress_noalloc: %s\n", cudaGetErrorString(e));
    return S2TC_ERR_CUDA;
  }
  if (timed_out) return fail(S2TC_ERR_TIMEOUT, "a bounded wait in the dither scan gave up");
  return S2TC_OK;
}
