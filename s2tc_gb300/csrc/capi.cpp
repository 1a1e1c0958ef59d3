// capi.cpp -- the C ABI of libs2tc_gb300.so: the reference's libtxc_dxtn entry
// points (tx_compress_dxtn, fetch_2d_texel_*), its encoder API
// (s2tc_encode_block_func, rgb565_image) and the GPU extension API.
//
// The host layer owns one CUDA stream and a grow-only device arena per
// process; every compression is dither kernel -> block encoder kernel on that
// stream.  There is no CPU encoding path: when CUDA is unavailable the entry
// points report the error and write nothing.
#include "s2tc_gb300.h"

#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>
#include <strings.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "dither.h"
#include "encode.h"
#include "rand_glibc.h"
#include "tools.h"
#include "s2tc_types.h"

namespace s2tc {
namespace {

thread_local std::string g_last_error;

void set_error(const std::string& msg) {
  g_last_error = msg;
  std::fprintf(stderr, "s2tc_gb300: %s\n", msg.c_str());
}

bool cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Grow-only device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  bool reserve(size_t n, const char* what) {
    if (n <= cap) return true;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = n + n / 4 + 4096;
    if (!cuda_ok(cudaMalloc(&p, want), what)) return false;
    cap = want;
    return true;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct PinnedBuf {
  void* p = nullptr;
  size_t cap = 0;
  bool reserve(size_t n, const char* what) {
    if (n <= cap) return true;
    if (p) cudaFreeHost(p);
    p = nullptr;
    cap = 0;
    size_t want = n + n / 4 + 4096;
    if (!cuda_ok(cudaMallocHost(&p, want), what)) return false;
    cap = want;
    return true;
  }
};

// Process-wide GPU context: stream + arena.  Calls are serialised by `mu`.
struct Context {
  std::mutex mu;
  bool ready = false;
  cudaStream_t stream = nullptr;
  cudaEvent_t arena_free = nullptr;  // recorded after the last work that used the arena
  // s2tc_gpu_set_timing: per-stage CUDA events of the last kTimingSlots calls
  static constexpr int kTimingSlots = 4096;
  bool timing = false;
  std::vector<cudaEvent_t> ev;   // 3 per slot: before dither, between, after encode
  long long timed_calls = 0;
  DevBuf src, t565, dst, scratch, rnd, err;
  DevBuf mips, blocks;  // s2tc_compress_dds: every level's pixels and blocks
  DevBuf rnd_win;       // the rand() stream position for the device generator
  // pipelined tx_compress_dxtn: upload and download streams, per-range events
  // chunks of block rows take the encode streams in turn, so that one
  // chunk's encode fills the last, partial wave of the ones before it
  static constexpr int kEncodeStreams = 4;
  cudaStream_t copy_in = nullptr, copy_out = nullptr, encode_stream[kEncodeStreams] = {};
  cudaEvent_t pipe_first = nullptr;  // the first range's encode (it reads the carried endpoint)
  static constexpr int kPipeRanges = 128;
  cudaEvent_t pipe_in[kPipeRanges] = {}, pipe_mid[kPipeRanges] = {}, pipe_out[kPipeRanges] = {};
  bool pipe_ready = false;
  bool init_pipe() {
    if (pipe_ready) return true;
    if (!cuda_ok(cudaStreamCreateWithFlags(&copy_in, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaStreamCreateWithFlags(&copy_out, cudaStreamNonBlocking), "cudaStreamCreate") ||
        !cuda_ok(cudaEventCreateWithFlags(&pipe_first, cudaEventDisableTiming), "cudaEventCreate"))
      return false;
    for (cudaStream_t& e : encode_stream)
      if (!cuda_ok(cudaStreamCreateWithFlags(&e, cudaStreamNonBlocking), "cudaStreamCreate")) return false;
    for (int i = 0; i < kPipeRanges; ++i)
      if (!cuda_ok(cudaEventCreateWithFlags(&pipe_in[i], cudaEventDisableTiming), "cudaEventCreate") ||
          !cuda_ok(cudaEventCreateWithFlags(&pipe_mid[i], cudaEventDisableTiming), "cudaEventCreate") ||
          !cuda_ok(cudaEventCreateWithFlags(&pipe_out[i], cudaEventDisableTiming), "cudaEventCreate"))
        return false;
    pipe_ready = true;
    return true;
  }
  PinnedBuf host_rnd, host_out;
  DevBuf small_dev;      // small quick-mode calls: pixels, scan state, flag, blocks
  PinnedBuf small_host;  // ... and their pinned mirror
  PinnedBuf host_flag;  // where the timeout flag is read back to
  int pageable_access = 0;  // the device reads and writes pageable host memory coherently

  bool init() {
    if (ready) return true;
    int n = 0;
    if (!cuda_ok(cudaGetDeviceCount(&n), "cudaGetDeviceCount")) return false;
    if (n == 0) {
      set_error("no CUDA device");
      return false;
    }
    if (!cuda_ok(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking), "cudaStreamCreate")) return false;
    if (!cuda_ok(cudaEventCreateWithFlags(&arena_free, cudaEventDisableTiming), "cudaEventCreate")) return false;
    if (!err.reserve(sizeof(int) * 4, "cudaMalloc(error flag)")) return false;
    if (!host_flag.reserve(sizeof(int), "cudaMallocHost(error flag)")) return false;
    if (!cuda_ok(cudaMemset(err.p, 0, sizeof(int) * 4), "cudaMemset")) return false;
    // err[2]: the carried alpha endpoint of tx_compress_dxtn calls (-1: none yet)
    if (!cuda_ok(cudaMemset(err.as<int>() + 2, 0xFF, sizeof(int)), "cudaMemset")) return false;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&pageable_access, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
      cudaGetLastError();
      pageable_access = 0;
    }
    if (!cuda_ok(nm_table_init(stream), "NORMALMAP table")) return false;
    ready = true;
    return true;
  }
};

Context& ctx() {
  static Context* c = new Context();  // never destroyed: CUDA may be torn down first at exit
  return *c;
}

int format_dxt(unsigned int fmt) {
  switch (fmt) {
    case S2TC_GL_COMPRESSED_RGB_S3TC_DXT1_EXT:
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT1_EXT: return DXT1;
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT3_EXT: return DXT3;
    case S2TC_GL_COMPRESSED_RGBA_S3TC_DXT5_EXT: return DXT5;
    default: return -1;
  }
}

// Environment knobs, parsed exactly as s2tc_libtxc_dxtn.cpp:156-216.
s2tc_options read_env() {
  s2tc_options o;
  o.metric = CD_WAVG;
  o.nrandom = -1;
  o.refine = RF_ALWAYS;
  o.dither = DI_SIMPLE;
  if (const char* v = std::getenv("S2TC_DITHER_MODE")) {
    if (!strcasecmp(v, "NONE")) o.dither = DI_NONE;
    else if (!strcasecmp(v, "SIMPLE")) o.dither = DI_SIMPLE;
    else if (!strcasecmp(v, "FLOYDSTEINBERG")) o.dither = DI_FLOYDSTEINBERG;
    else std::fprintf(stderr, "Invalid dither mode: %s\n", v);
  }
  if (const char* v = std::getenv("S2TC_COLORDIST_MODE")) {
    if (!strcasecmp(v, "RGB")) o.metric = CD_RGB;
    else if (!strcasecmp(v, "YUV")) o.metric = CD_YUV;
    else if (!strcasecmp(v, "SRGB")) o.metric = CD_SRGB;
    else if (!strcasecmp(v, "SRGB_MIXED")) o.metric = CD_SRGB_MIXED;
    else if (!strcasecmp(v, "AVG")) o.metric = CD_AVG;
    else if (!strcasecmp(v, "WAVG")) o.metric = CD_WAVG;
    else if (!strcasecmp(v, "W0AVG")) o.metric = CD_W0AVG;
    else if (!strcasecmp(v, "NORMALMAP")) o.metric = CD_NORMALMAP;
    else std::fprintf(stderr, "Invalid color dist mode: %s\n", v);
  }
  if (const char* v = std::getenv("S2TC_RANDOM_COLORS")) o.nrandom = std::atoi(v);
  if (const char* v = std::getenv("S2TC_REFINE_COLORS")) {
    if (!strcasecmp(v, "NEVER")) o.refine = RF_NEVER;
    else if (!strcasecmp(v, "ALWAYS")) o.refine = RF_ALWAYS;
    else if (!strcasecmp(v, "LOOP")) o.refine = RF_LOOP;
    else std::fprintf(stderr, "Invalid refinement mode: %s\n", v);
  }
  return o;
}

// Out-of-range enum values select the reference's `default:` branches.
s2tc_options normalise(const s2tc_options& in) {
  s2tc_options o = in;
  if (o.dither != DI_NONE && o.dither != DI_FLOYDSTEINBERG) o.dither = DI_SIMPLE;
  if (o.metric < 0 || o.metric > 7) o.metric = CD_WAVG;
  if (o.refine != RF_NEVER && o.refine != RF_LOOP) o.refine = RF_ALWAYS;
  return o;
}

// The random-candidate search runs when the all-texels mode is selected
// (nrandom >= 0, or NORMALMAP which never uses the quick mode) and nrandom > 0.
bool normal_mode(const s2tc_options& o) { return o.nrandom >= 0 || o.metric == CD_NORMALMAP; }
int rand_per_block(const s2tc_options& o, int dxt) {
  return (normal_mode(o) && o.nrandom > 0) ? o.nrandom * (dxt == DXT5 ? 4 : 3) : 0;
}

// Rand words for one chunk of blocks: libc rand(), in the reference's call
// order, into pinned memory, then to the device.
constexpr long long kRandChunkWords = 1ll << 24;


// Encodes every block of a texel-word image (the encoder half of a call):
// one launch, or chunks of block rows when rand() words are replayed on the
// host.  See compress_device_locked for `carry`.
int encode_locked(Context& c, const uint32_t* t565, int width, int height, int dxt, uint8_t* d_dst, long long pitch,
                  const s2tc_options& opt, const unsigned int* d_rand, cudaStream_t s, int* carry) {
  const int bw = (width + 3) / 4, bh = (height + 3) / 4;
  EncodeArgs ea{};
  ea.t565 = t565;
  ea.width = width;
  ea.height = height;
  ea.bw = bw;
  ea.bh = bh;
  ea.dst = d_dst;
  ea.pitch = pitch;
  const int bs = block_bytes(dxt);
  ea.aligned = ((reinterpret_cast<uintptr_t>(d_dst) % bs) == 0 && (pitch % bs) == 0) ? 1 : 0;
  ea.nrandom = opt.nrandom;
  ea.prev_a1_first = -1;
  ea.prev_a1_dev = nullptr;
  ea.leftover_out = nullptr;
  const bool normal = normal_mode(opt);
  const int per_block = rand_per_block(opt, dxt);
  if (carry && dxt == DXT5 && normal && per_block == 0) {
    ea.prev_a1_dev = carry;
    ea.leftover_out = carry;
  }
  if (per_block == 0) {
    ea.by0 = 0;
    ea.nby = bh;
    ea.rnd = nullptr;
    if (!cuda_ok(launch_encode(ea, dxt, opt.metric, normal, opt.refine, s), "encode launch")) return ST_CUDA_ERROR;
  } else if (!d_rand && (long long)bw * bh * per_block >= kRandDeviceMin && rand_usable()) {
    // libc's rand() stream generated on the GPU from its current position
    // (libc's state jumps ahead by the words taken)
    const long long words = (long long)bw * bh * per_block;
    RandWindow win;
    if (!c.rnd.reserve(size_t(words) * 4, "cudaMalloc(rand)")) return ST_OUT_OF_MEMORY;
    if (!c.rnd_win.reserve(sizeof(RandWindow), "cudaMalloc(rand window)")) return ST_OUT_OF_MEMORY;
    if (!rand_take(words, &win)) {
      set_error("libc rand() state could not be read");
      return ST_CUDA_ERROR;
    }
    if (!cuda_ok(cudaMemcpyAsync(c.rnd_win.p, &win, sizeof(win), cudaMemcpyHostToDevice, s), "rand window upload"))
      return ST_CUDA_ERROR;
    if (!cuda_ok(rand_fill(c.rnd_win.as<RandWindow>(), c.rnd.as<uint32_t>(), words, s), "rand fill"))
      return ST_CUDA_ERROR;
    ea.by0 = 0;
    ea.nby = bh;
    ea.rnd = c.rnd.as<uint32_t>();
    if (!cuda_ok(launch_encode(ea, dxt, opt.metric, normal, opt.refine, s), "encode launch")) return ST_CUDA_ERROR;
  } else {
    // block rows in chunks so the replayed rand words stay bounded (one
    // chunk when the caller supplies the words)
    const long long row_words = (long long)bw * per_block;
    int rows_per_chunk = d_rand ? bh : int(std::max(1ll, kRandChunkWords / std::max(1ll, row_words)));
    if (!d_rand) {
      const size_t chunk_bytes = size_t(std::min<long long>(bh, rows_per_chunk)) * row_words * 4;
      if (!c.rnd.reserve(chunk_bytes, "cudaMalloc(rand)")) return ST_OUT_OF_MEMORY;
      if (!c.host_rnd.reserve(chunk_bytes, "cudaMallocHost(rand)")) return ST_OUT_OF_MEMORY;
    }
    for (int by0 = 0; by0 < bh; by0 += rows_per_chunk) {
      const int nby = std::min(rows_per_chunk, bh - by0);
      const long long words = (long long)nby * row_words;
      ea.by0 = by0;
      ea.nby = nby;
      if (d_rand) {
        ea.rnd = d_rand + (long long)by0 * row_words;
      } else {
        // the previous chunk's upload must finish before the staging buffer is refilled
        if (!cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize")) return ST_CUDA_ERROR;
        unsigned int* h = static_cast<unsigned int*>(c.host_rnd.p);
        for (long long i = 0; i < words; ++i) h[i] = unsigned(std::rand());
        if (!cuda_ok(cudaMemcpyAsync(c.rnd.p, h, size_t(words) * 4, cudaMemcpyHostToDevice, s), "rand upload"))
          return ST_CUDA_ERROR;
        ea.rnd = c.rnd.as<uint32_t>();
      }
      if (!cuda_ok(launch_encode(ea, dxt, opt.metric, normal, opt.refine, s), "encode launch")) return ST_CUDA_ERROR;
    }
  }
  return ST_OK;
}

// The strip kernel's view of an RGBA8 source for its TMA copies: the image
// as a 2-D tensor of rows of 256 texels (32-bit words), texels / 256 rows of
// 1024 bytes, one row per copy.  False (vector loads instead) for a source
// that is not 16-byte aligned, an image under 256 texels, or a driver without
// the tensor-map entry point.
bool rgba_rows_map(const void* src, long long npx, CUtensorMap* map, long long* rows) {
  if ((reinterpret_cast<uintptr_t>(src) & 15) != 0 || npx < 256) return false;
  static const PFN_cuTensorMapEncodeTiled_v12000 encode = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
            cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return PFN_cuTensorMapEncodeTiled_v12000(nullptr);
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }();
  if (!encode) return false;
  const cuuint64_t dims[2] = {256, cuuint64_t(npx / 256)};
  const cuuint64_t strides[1] = {1024};
  const cuuint32_t box[2] = {256, 1};
  const cuuint32_t elem[2] = {1, 1};
  if (encode(map, CU_TENSOR_MAP_DATA_TYPE_UINT32, 2, const_cast<void*>(src), dims, strides, box, elem,
             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  *rows = npx / 256;
  return true;
}

// The quick mode (darkest/brightest selection) with NONE or SIMPLE dither on
// images up to kStripMaxWidth texels wide runs as one fused strip kernel.
bool strip_mode(const s2tc_options& opt, int width, int height, StripPlan* plan) {
#ifdef S2TC_STRIP_OFF
  return false;  // build-time switch: the two-kernel path only (for comparisons)
#endif
  return !normal_mode(opt) && opt.dither != DI_FLOYDSTEINBERG && strip_plan(width, height, *plan);
}

// Arguments of a strip launch over the whole image.
StripArgs strip_args(const StripPlan& plan, int sc, int width, int height, const uint8_t* d_src, int dxt, int dither,
                     uint8_t* d_dst, long long pitch, int* error) {
  StripArgs a{};
  a.src = d_src;
  a.width = width;
  a.height = height;
  a.srccomps = sc;
  a.alphabits = alpha_bits(dxt);
  a.dither = dither == DI_NONE ? DI_NONE : DI_SIMPLE;
  a.dst = d_dst;
  a.pitch = pitch;
  const int bs = block_bytes(dxt);
  a.aligned = ((reinterpret_cast<uintptr_t>(d_dst) % bs) == 0 && (pitch % bs) == 0) ? 1 : 0;
  a.seg = plan.seg;
  a.rows_per_band = plan.rows_per_band;
  a.band_base = 0;
  a.nbands = plan.bands;
  a.image_bands = plan.bands;
  a.scan.error = error;
  return a;
}

// `carry` (device int, may be null): the second alpha endpoint that the
// previous call's last block left behind.  The reference encodes every block
// of every call in the same stack frame, and a DXT5 image whose first block
// has a single texel (a 1x1 image, e.g. the last level of a mip chain) reads
// its second alpha candidate from that frame without writing it first
// (s2tc_algorithm.cpp:996-1001), i.e. it sees the previous call's leftover.
// All-texel DXT5 calls read and update it; other calls leave it alone.
int compress_device_locked(Context& c, int srccomps, int width, int height, const uint8_t* d_src, int dxt,
                           uint8_t* d_dst, long long pitch, const s2tc_options& opt, const unsigned int* d_rand,
                           cudaStream_t s, int* carry = nullptr) {
  const int sc = srccomps == 3 ? 3 : 4;
  const long long npx = (long long)width * height;
  StripPlan plan;
  if (strip_mode(opt, width, height, &plan)) {
    // one fused launch: the texel words stay in shared memory
    if (!c.scratch.reserve(dither_batch_scratch_bytes(plan.bands), "cudaMalloc(scratch)")) return ST_OUT_OF_MEMORY;
    if (!cuda_ok(cudaStreamWaitEvent(s, c.arena_free, 0), "cudaStreamWaitEvent")) return ST_CUDA_ERROR;
    StripArgs sa = strip_args(plan, sc, width, height, d_src, dxt, opt.dither, d_dst, pitch, c.err.as<int>());
    CUtensorMap map;
    sa.use_tma = sc == 4 && rgba_rows_map(d_src, npx, &map, &sa.tma_rows);
    cudaEvent_t* tev = c.timing ? &c.ev[3 * (c.timed_calls % Context::kTimingSlots)] : nullptr;
    // the stage timing puts the fused kernel under "encode"
    if (tev && (!cuda_ok(cudaEventRecord(tev[0], s), "cudaEventRecord") ||
                !cuda_ok(cudaEventRecord(tev[1], s), "cudaEventRecord")))
      return ST_CUDA_ERROR;
    if (!cuda_ok(launch_strip(sa, &map, dxt, opt.metric, opt.refine, c.scratch.as<uint8_t>(), s), "strip launch"))
      return ST_CUDA_ERROR;
    if (tev) {
      if (!cuda_ok(cudaEventRecord(tev[2], s), "cudaEventRecord")) return ST_CUDA_ERROR;
      c.timed_calls++;
    }
    return cuda_ok(cudaEventRecord(c.arena_free, s), "cudaEventRecord") ? ST_OK : ST_CUDA_ERROR;
  }
  if (!c.t565.reserve(size_t(npx) * 4 + 16, "cudaMalloc(texels)")) return ST_OUT_OF_MEMORY;
  size_t scratch = dither_scratch_bytes(npx);
  if (opt.dither == DI_FLOYDSTEINBERG) scratch = dither_fs_scratch_bytes(width, height);
  if (!c.scratch.reserve(scratch, "cudaMalloc(scratch)")) return ST_OUT_OF_MEMORY;
  // the arena may still be in use by work on another stream
  if (!cuda_ok(cudaStreamWaitEvent(s, c.arena_free, 0), "cudaStreamWaitEvent")) return ST_CUDA_ERROR;

  DitherArgs da{};
  da.src = d_src;
  da.width = width;
  da.height = height;
  da.srccomps = sc;
  da.alphabits = alpha_bits(dxt);
  da.dst = c.t565.as<uint32_t>();
  da.error = c.err.as<int>();
  cudaEvent_t* tev = c.timing ? &c.ev[3 * (c.timed_calls % Context::kTimingSlots)] : nullptr;
  if (tev && !cuda_ok(cudaEventRecord(tev[0], s), "cudaEventRecord")) return ST_CUDA_ERROR;
  if (!cuda_ok(launch_dither(da, opt.dither, c.scratch.as<uint8_t>(), s), "dither launch")) return ST_CUDA_ERROR;
  if (tev && !cuda_ok(cudaEventRecord(tev[1], s), "cudaEventRecord")) return ST_CUDA_ERROR;

  const int st = encode_locked(c, c.t565.as<uint32_t>(), width, height, dxt, d_dst, pitch, opt, d_rand, s, carry);
  if (st != ST_OK) return st;
  if (tev) {
    if (!cuda_ok(cudaEventRecord(tev[2], s), "cudaEventRecord")) return ST_CUDA_ERROR;
    c.timed_calls++;
  }
  if (!cuda_ok(cudaEventRecord(c.arena_free, s), "cudaEventRecord")) return ST_CUDA_ERROR;
  return ST_OK;
}

// Enqueues on `s` the read-back (into pinned memory) and the reset of the
// kernels' sticky timeout flag.
bool enqueue_flag(Context& c, cudaStream_t s) {
  return cuda_ok(cudaMemcpyAsync(c.host_flag.p, c.err.p, sizeof(int), cudaMemcpyDeviceToHost, s), "error flag read") &&
         cuda_ok(cudaMemsetAsync(c.err.p, 0, sizeof(int), s), "cudaMemsetAsync");
}

// The flag's verdict, once the stream that read it back has been waited for.
int take_flag(Context& c) {
  int& flag = *static_cast<int*>(c.host_flag.p);
  if (flag) {
    flag = 0;
    set_error("a bounded wait in the dither scan gave up");
    return ST_TIMEOUT;
  }
  return ST_OK;
}

// Waits for `s`, then reads and clears the kernels' sticky timeout flag.
int check_error_flag(Context& c, cudaStream_t s) {
  if (!enqueue_flag(c, s)) return ST_CUDA_ERROR;
  if (!cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize")) return ST_CUDA_ERROR;
  return take_flag(c);
}

// The same when the flag's read-back is the last thing the call's work needs
// (every copy and kernel of the call is ordered before it on `s`): the host
// polls the pinned word that the read-back overwrites, which returns sooner
// than the stream wait; past kFlagPollLimit the stream wait takes over.
constexpr auto kFlagPollLimit = std::chrono::milliseconds(20);
int finish_polled(Context& c, cudaStream_t s) {
  volatile int* hf = static_cast<volatile int*>(c.host_flag.p);
  *hf = -1;  // the read-back writes 0 or 1
  if (!enqueue_flag(c, s)) return ST_CUDA_ERROR;
  bool seen = false;
  const auto t0 = std::chrono::steady_clock::now();
  for (unsigned int i = 1;; ++i) {
    if (*hf != -1) {
      seen = true;
      break;
    }
    if ((i & 1023u) == 0 && std::chrono::steady_clock::now() - t0 > kFlagPollLimit) break;
  }
  std::atomic_thread_fence(std::memory_order_acquire);
  if (!seen && !cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize")) return ST_CUDA_ERROR;
  return take_flag(c);
}

bool host_pinned(const void* p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

// tx_compress_dxtn on a large image, pipelined: the image goes up in ranges of
// whole dither tiles on one copy stream; the compute stream scans each range
// as it lands (the scan's look-back reaches into the ranges before it); the
// encode streams, in turn, encode the block rows whose four texel rows are
// complete while the next range is dithered; a second copy stream brings those rows
// back (per chunk when `dest` is pinned, else at the end).  Same kernels and
// bytes as the unpipelined path.  Returns false when the image does not
// qualify (the caller then takes that path).
// Dither ranges: a dither launch ends 45 to 75 us after the last byte of its
// range lands, whatever its size (a tile's latency plus the wait for SM slots
// behind the queued encoder CTAs), and the launches run one after another on
// one stream.  The host's stream operations are cheap by comparison (about
// 10 us a range).  So the ranges double in size from kPipeFirstTiles: the
// first is dithered a few microseconds into the call and the chain of
// launches stays ahead of the upload.  The encoder takes the finished block
// rows in chunks of at most 1/kPipeEncodeChunks of the image, each with its own
// download, so that little is left to do after the last dither range.  At
// 4096^2 DXT5 all-16 LOOP (0.67 ms of kernels) a call took 0.84 ms in 12
// equal ranges on two encode streams, 0.81 ms in the doubling ranges with 16
// chunks on four (one stream: 1.02 ms, two: 0.85 ms).
constexpr long long kPipeMinTexels = 1ll << 22;
constexpr long long kPipeFirstTiles = 16;
constexpr long long kPipeMaxRangeTiles = 512;
constexpr int kPipeEncodeChunks = 16;

// Tile ends of the dither ranges of a `tiles`-tile image: 16, 32, 64, ...
// tiles, each at most max(kPipeMaxRangeTiles, tiles / 48) (so at most about
// 60 ranges); a remainder below kPipeFirstTiles joins the range before it.
// Returns their number, or 0 past `max_ranges`.
int dither_ranges(long long tiles, long long* ends, int max_ranges) {
  const long long cap = std::max(kPipeMaxRangeTiles, (tiles + 47) / 48);
  long long t = 0, step = kPipeFirstTiles;
  int n = 0;
  while (t < tiles) {
    if (n == max_ranges) return 0;
    t = std::min(tiles, t + std::min(step, cap));
    if (tiles - t < kPipeFirstTiles) t = tiles;
    ends[n++] = t;
    step *= 2;
  }
  return n;
}

// The strip pipeline's ranges hold at least kPipeRangeTiles dither tiles'
// worth of texels and are at most kPipeTargetRanges.
constexpr long long kPipeRangeTiles = 64;
constexpr long long kPipeTargetRanges = 12;
static_assert(kPipeTargetRanges <= Context::kPipeRanges, "one event set per range");

// The same for the fused strip kernel (quick mode): the image goes up in
// ranges of bands on the copy stream, one strip launch per range on the
// compute stream (its look-back reaches into the ranges before it), and each
// range's block rows come back on the second copy stream when `dest` is
// pinned.  The launches run one after another, and each takes at least the
// latency of one band (50 to 80 us for 4096-texel rows), so a range carries
// about kStripRangeBytes of pixels: its upload (about 85 us at the measured
// 190 GB/s of the host link) then hides the launch before it.  4096^2 DXT1
// quick: 0.62 ms per call in 12 ranges, 0.59 in 11 ranges of 6 MB, 0.465 in 7
// of 10 MB, 0.447 in 4 of 16 MB; the bare upload is 0.35 ms.
constexpr long long kStripRangeBytes = 16ll << 20;
bool compress_host_pipelined_strip(Context& c, int sc, int width, int height, const unsigned char* src, int dxt,
                                   unsigned char* dest, long long diff, const s2tc_options& opt,
                                   const StripPlan& plan) {
  cudaStream_t s = c.stream;
  const long long npx = (long long)width * height;
  const int bw = (width + 3) / 4, bh = (height + 3) / 4;
  const long long row_bytes = (long long)bw * block_bytes(dxt);
  const long long band_texels = 4ll * plan.rows_per_band * width;
  const long long min_bands = std::max(1ll, (kPipeRangeTiles * dither_tile_texels() + band_texels - 1) / band_texels);
  const long long target = std::min(kPipeTargetRanges, std::max(1ll, (npx * sc + kStripRangeBytes - 1) / kStripRangeBytes));
  const long long per_range = std::max(min_bands, (plan.bands + target - 1) / target);
  const int ranges = int((plan.bands + per_range - 1) / per_range);
  if (!c.src.reserve(size_t(npx) * sc + 16, "cudaMalloc(src)")) return true;
  if (!c.dst.reserve(size_t(row_bytes) * bh + 16, "cudaMalloc(dst)")) return true;
  if (!c.scratch.reserve(dither_batch_scratch_bytes(plan.bands), "cudaMalloc(scratch)")) return true;
  if (!cuda_ok(cudaStreamWaitEvent(s, c.arena_free, 0), "cudaStreamWaitEvent")) return true;
  if (!cuda_ok(cudaStreamWaitEvent(c.copy_in, c.arena_free, 0), "cudaStreamWaitEvent")) return true;
  const bool pinned_out = host_pinned(dest);
  uint8_t* d_src = c.src.as<uint8_t>();
  uint8_t* d_dst = c.dst.as<uint8_t>();
  StripArgs sa = strip_args(plan, sc, width, height, d_src, dxt, opt.dither, d_dst, row_bytes, c.err.as<int>());
  CUtensorMap map;
  sa.use_tma = sc == 4 && rgba_rows_map(d_src, npx, &map, &sa.tma_rows);
  for (int r = 0; r < ranges; ++r) {
    const long long b0 = r * per_range, b1 = std::min(plan.bands, b0 + per_range);
    const long long p0 = b0 * band_texels, p1 = std::min(npx, b1 * band_texels);
    const int y0 = int(b0 * plan.rows_per_band), y1 = int(std::min<long long>(bh, b1 * plan.rows_per_band));
    sa.band_base = b0;
    sa.nbands = b1 - b0;
    if (!cuda_ok(cudaMemcpyAsync(d_src + p0 * sc, src + p0 * sc, size_t(p1 - p0) * sc, cudaMemcpyHostToDevice,
                                 c.copy_in),
                 "input upload") ||
        !cuda_ok(cudaEventRecord(c.pipe_in[r], c.copy_in), "cudaEventRecord") ||
        !cuda_ok(cudaStreamWaitEvent(s, c.pipe_in[r], 0), "cudaStreamWaitEvent") ||
        !cuda_ok(launch_strip(sa, &map, dxt, opt.metric, opt.refine, c.scratch.as<uint8_t>(), s), "strip launch"))
      return true;
    if (pinned_out) {
      if (!cuda_ok(cudaEventRecord(c.pipe_out[r], s), "cudaEventRecord") ||
          !cuda_ok(cudaStreamWaitEvent(c.copy_out, c.pipe_out[r], 0), "cudaStreamWaitEvent") ||
          !cuda_ok(cudaMemcpy2DAsync(dest + (long long)y0 * (row_bytes + diff), size_t(row_bytes + diff),
                                     d_dst + (long long)y0 * row_bytes, size_t(row_bytes), size_t(row_bytes),
                                     size_t(y1 - y0), cudaMemcpyDeviceToHost, c.copy_out),
                   "output download"))
        return true;
    }
  }
  if (!pinned_out &&
      !cuda_ok(cudaMemcpy2DAsync(dest, size_t(row_bytes + diff), d_dst, size_t(row_bytes), size_t(row_bytes),
                                 size_t(bh), cudaMemcpyDeviceToHost, s),
               "output download"))
    return true;
  if (!cuda_ok(cudaEventRecord(c.pipe_out[0], c.copy_out), "cudaEventRecord") ||
      !cuda_ok(cudaStreamWaitEvent(s, c.pipe_out[0], 0), "cudaStreamWaitEvent") ||
      !cuda_ok(cudaEventRecord(c.arena_free, s), "cudaEventRecord"))
    return true;
  finish_polled(c, s);
  return true;
}

bool compress_host_pipelined(Context& c, int sc, int width, int height, const unsigned char* src, int dxt,
                             unsigned char* dest, long long diff, const s2tc_options& opt, bool* done) {
  *done = false;
  const long long npx = (long long)width * height;
  if (npx < kPipeMinTexels || opt.dither == DI_FLOYDSTEINBERG || diff < 0) return false;
  StripPlan plan;
  if (strip_mode(opt, width, height, &plan)) {
    if (!c.init_pipe()) return false;
    *done = true;
    return compress_host_pipelined_strip(c, sc, width, height, src, dxt, dest, diff, opt, plan);
  }
  const bool normal = normal_mode(opt);
  const int per_block = rand_per_block(opt, dxt);
  if (per_block > 0 && !rand_usable()) return false;
  const long long tile = dither_tile_texels();
  const long long tiles = (npx + tile - 1) / tile;
  long long ends[Context::kPipeRanges];
  // at most half the events for the dither ranges: encode chunks end at
  // range ends or at multiples of chunk_rows, so there are fewer than
  // ranges + kPipeEncodeChunks of them
  const int ranges = dither_ranges(tiles, ends, Context::kPipeRanges / 2);
  static_assert(Context::kPipeRanges / 2 + kPipeEncodeChunks < Context::kPipeRanges, "one event per chunk");
  if (ranges == 0 || !c.init_pipe()) return false;
  *done = true;
  cudaStream_t s = c.stream;
  const int bw = (width + 3) / 4, bh = (height + 3) / 4, bs = block_bytes(dxt);
  const long long row_bytes = (long long)bw * bs;
  const int chunk_rows = std::max(1, (bh + kPipeEncodeChunks - 1) / kPipeEncodeChunks);
  if (!c.src.reserve(size_t(npx) * sc + 16, "cudaMalloc(src)")) return true;
  if (!c.dst.reserve(size_t(row_bytes) * bh + 16, "cudaMalloc(dst)")) return true;
  if (!c.t565.reserve(size_t(npx) * 4 + 16, "cudaMalloc(texels)")) return true;
  if (!c.scratch.reserve(dither_scratch_bytes(npx), "cudaMalloc(scratch)")) return true;
  if (!cuda_ok(cudaStreamWaitEvent(s, c.arena_free, 0), "cudaStreamWaitEvent")) return true;
  if (!cuda_ok(cudaStreamWaitEvent(c.copy_in, c.arena_free, 0), "cudaStreamWaitEvent")) return true;
  const bool pinned_out = host_pinned(dest);
  uint8_t* d_src = c.src.as<uint8_t>();
  uint8_t* d_dst = c.dst.as<uint8_t>();
  // random-candidate words: the whole call's share of libc's stream, on the device
  const uint32_t* rnd = nullptr;
  if (per_block > 0) {
    const long long words = (long long)bw * bh * per_block;
    RandWindow win;
    if (!c.rnd.reserve(size_t(words) * 4, "cudaMalloc(rand)") ||
        !c.rnd_win.reserve(sizeof(RandWindow), "cudaMalloc(rand window)"))
      return true;
    if (!rand_take(words, &win)) {
      set_error("libc rand() state could not be read");
      return true;
    }
    if (!cuda_ok(cudaMemcpyAsync(c.rnd_win.p, &win, sizeof(win), cudaMemcpyHostToDevice, s), "rand window upload") ||
        !cuda_ok(rand_fill(c.rnd_win.as<RandWindow>(), c.rnd.as<uint32_t>(), words, s), "rand fill"))
      return true;
    rnd = c.rnd.as<uint32_t>();
  }
  DitherArgs da{};
  da.src = d_src;
  da.width = width;
  da.height = height;
  da.srccomps = sc;
  da.alphabits = alpha_bits(dxt);
  da.dst = c.t565.as<uint32_t>();
  da.error = c.err.as<int>();
  da.alpha_const = (1 << da.alphabits) - 1;
  EncodeArgs ea{};
  ea.t565 = c.t565.as<uint32_t>();
  ea.width = width;
  ea.height = height;
  ea.bw = bw;
  ea.bh = bh;
  ea.dst = d_dst;
  ea.pitch = row_bytes;
  ea.aligned = 1;
  ea.nrandom = opt.nrandom;
  ea.prev_a1_first = -1;
  if (dxt == DXT5 && normal && per_block == 0) {
    ea.prev_a1_dev = c.err.as<int>() + 2;
    ea.leftover_out = c.err.as<int>() + 2;
  }
  int rows_done = 0, nenc = 0;
  long long t0 = 0;
  for (int r = 0; r < ranges; ++r) {
    const long long t1 = ends[r];
    const long long p0 = t0 * tile, p1 = std::min(npx, t1 * tile);
    if (!cuda_ok(cudaMemcpyAsync(d_src + p0 * sc, src + p0 * sc, size_t(p1 - p0) * sc, cudaMemcpyHostToDevice,
                                 c.copy_in),
                 "input upload") ||
        !cuda_ok(cudaEventRecord(c.pipe_in[r], c.copy_in), "cudaEventRecord") ||
        !cuda_ok(cudaStreamWaitEvent(s, c.pipe_in[r], 0), "cudaStreamWaitEvent") ||
        !cuda_ok(launch_dither_range(da, opt.dither, c.scratch.as<uint8_t>(), t0, t1, s), "dither launch"))
      return true;
    t0 = t1;
    const int rows_ready = r == ranges - 1 ? bh : int((p1 / width) / 4);
    if (rows_ready <= rows_done) continue;
    if (!cuda_ok(cudaEventRecord(c.pipe_mid[r], s), "cudaEventRecord")) return true;
    while (rows_done < rows_ready) {
      const int rows_end = std::min(rows_ready, (rows_done / chunk_rows + 1) * chunk_rows);
      ea.by0 = rows_done;
      ea.nby = rows_end - rows_done;
      ea.rnd = rnd ? rnd + (long long)rows_done * bw * per_block : nullptr;
      const int k = nenc % Context::kEncodeStreams;
      cudaStream_t se = c.encode_stream[k];
      if (!cuda_ok(cudaStreamWaitEvent(se, c.pipe_mid[r], 0), "cudaStreamWaitEvent")) return true;
      // the last rows write the carried endpoint that the first rows read
      if (rows_end == bh && k != 0 &&
          !cuda_ok(cudaStreamWaitEvent(se, c.pipe_first, 0), "cudaStreamWaitEvent"))
        return true;
      if (!cuda_ok(launch_encode(ea, dxt, opt.metric, normal, opt.refine, se), "encode launch")) return true;
      if (nenc == 0 && !cuda_ok(cudaEventRecord(c.pipe_first, se), "cudaEventRecord")) return true;
      if (pinned_out &&
          (!cuda_ok(cudaEventRecord(c.pipe_out[nenc], se), "cudaEventRecord") ||
           !cuda_ok(cudaStreamWaitEvent(c.copy_out, c.pipe_out[nenc], 0), "cudaStreamWaitEvent") ||
           !cuda_ok(cudaMemcpy2DAsync(dest + (long long)rows_done * (row_bytes + diff), size_t(row_bytes + diff),
                                      d_dst + (long long)rows_done * row_bytes, size_t(row_bytes), size_t(row_bytes),
                                      size_t(rows_end - rows_done), cudaMemcpyDeviceToHost, c.copy_out),
                    "output download")))
        return true;
      ++nenc;
      rows_done = rows_end;
    }
  }
  // the compute stream joins the encode streams, then (unpinned output) downloads
  for (int k = 0; k < Context::kEncodeStreams; ++k)
    if (!cuda_ok(cudaEventRecord(c.pipe_mid[k], c.encode_stream[k]), "cudaEventRecord") ||
        !cuda_ok(cudaStreamWaitEvent(s, c.pipe_mid[k], 0), "cudaStreamWaitEvent"))
      return true;
  if (!pinned_out &&
      !cuda_ok(cudaMemcpy2DAsync(dest, size_t(row_bytes + diff), d_dst, size_t(row_bytes), size_t(row_bytes),
                                 size_t(bh), cudaMemcpyDeviceToHost, s),
               "output download"))
    return true;
  if (!cuda_ok(cudaEventRecord(c.pipe_out[0], c.copy_out), "cudaEventRecord") ||
      !cuda_ok(cudaStreamWaitEvent(s, c.pipe_out[0], 0), "cudaStreamWaitEvent") ||
      !cuda_ok(cudaEventRecord(c.arena_free, s), "cudaEventRecord"))
    return true;
  finish_polled(c, s);
  return true;
}

// Quick-mode images where the device reads host memory coherently, of any
// size: compress_host_direct (below).  Elsewhere, small images in the quick
// mode: one fused launch between one upload and one download.  A device
// arena holds [pixels | ticket | status words | flag | blocks | aggregate
// records] and a pinned buffer mirrors its first part:
// the upload carries the pixels and the zeroed ticket, status words and
// timeout flag, the download brings back the flag and the blocks.  Four CUDA
// calls per image (upload, launch, download, wait) instead of about ten: a
// 64x64 call measured 29.5 us instead of 50 us, 256x256 43 us instead of
// 72 us.  Larger images take the ordinary path: past about 64 Ki texels the
// host copies through the staging buffer cost more than the calls they save
// (1024x1024: 348 us against 96 us).
constexpr long long kSmallCallTexels = 1ll << 16;

// Where the device reads and writes pageable host memory coherently (a Grace
// host's page tables, cudaDevAttrPageableMemoryAccess), the kernel takes the
// caller's pixels and writes the caller's blocks itself: the call is one
// launch and one wait (plus one memset of the scan state when the image has
// more than one band), with no staging copies.  Overlapping output rows (a
// dstRowStride below the padded row) keep the copying paths, whose host copy
// writes the rows in order.  The wait is a poll of a flag in pinned memory
// that the last band to finish raises after its blocks (bounded: past
// kSmallPollLimit the stream wait takes over), which returns sooner than the
// stream wait.  The bands read the pixels over the host link as they need
// them, so the link's time overlaps the scan and the encoding without ranges:
// a 1024^2 call took 60.7 µs against 96.6 µs through an upload and a
// download, a 4096^2 call 0.425 ms against 0.450 ms for the pipelined ranges.
constexpr auto kSmallPollLimit = std::chrono::milliseconds(5);

// S2TC_HOST_DIRECT=0 keeps such calls on the staged and pipelined paths.
bool host_direct_enabled() {
  const char* v = std::getenv("S2TC_HOST_DIRECT");
  return !(v && v[0] == '0');
}

bool compress_host_direct(Context& c, int sc, int width, int height, const unsigned char* src, int dxt,
                          unsigned char* dest, long long diff, const s2tc_options& opt, const StripPlan& plan) {
  const int bw = (width + 3) / 4, bs = block_bytes(dxt);
  const size_t row_bytes = size_t(bw) * bs;
  const size_t o_status = 16, o_aggs = align_up(o_status + size_t(plan.bands) * 8, 16);
  if (!c.small_dev.reserve(o_aggs + size_t(plan.bands) * 72, "cudaMalloc(small call)") ||
      !c.small_host.reserve(16, "cudaMallocHost(small call)"))
    return true;
  volatile int* flag = static_cast<volatile int*>(c.small_host.p);
  volatile int* done = flag + 1;
  *flag = 0;
  *done = 0;
  uint8_t* d = c.small_dev.as<uint8_t>();
  StripArgs sa = strip_args(plan, sc, width, height, src, dxt, opt.dither, dest, (long long)row_bytes + diff,
                            const_cast<int*>(flag));
  sa.use_tma = 0;
  sa.scan.ticket = reinterpret_cast<unsigned int*>(d);
  sa.scan.status = reinterpret_cast<unsigned long long*>(d + o_status);
  sa.scan.aggs = d + o_aggs;
  sa.single_band = plan.bands == 1;
  sa.done_count = reinterpret_cast<unsigned int*>(d + 8);  // zeroed with the ticket
  sa.done_flag = const_cast<int*>(done);
  cudaStream_t s = c.stream;
  if (!sa.single_band && !cuda_ok(cudaMemsetAsync(d, 0, o_aggs, s), "cudaMemsetAsync")) return true;
  cudaEvent_t* tev = c.timing ? &c.ev[3 * (c.timed_calls % Context::kTimingSlots)] : nullptr;
  if (tev && (!cuda_ok(cudaEventRecord(tev[0], s), "cudaEventRecord") ||
              !cuda_ok(cudaEventRecord(tev[1], s), "cudaEventRecord")))
    return true;
  if (!cuda_ok(launch_strip(sa, nullptr, dxt, opt.metric, opt.refine, nullptr, s), "strip launch")) return true;
  if (tev) {
    if (!cuda_ok(cudaEventRecord(tev[2], s), "cudaEventRecord")) return true;
    c.timed_calls++;
  }
  bool seen = false;
  const auto t0 = std::chrono::steady_clock::now();
  for (unsigned int i = 1;; ++i) {
    if (*done) {
      seen = true;
      break;
    }
    if ((i & 1023u) == 0 && std::chrono::steady_clock::now() - t0 > kSmallPollLimit) break;
  }
  // the blocks and the timeout flag are read only after the flag was seen
  std::atomic_thread_fence(std::memory_order_acquire);
  if (!seen && !cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize")) return true;
  if (*flag) set_error("a bounded wait in the dither scan gave up");
  return true;
}

bool compress_host_small(Context& c, int sc, int width, int height, const unsigned char* src, int dxt,
                         unsigned char* dest, int dstRowStride, const s2tc_options& opt, bool* done) {
  *done = false;
  const long long npx = (long long)width * height;
  StripPlan plan;
  if (!strip_mode(opt, width, height, &plan)) return false;
  const int bw = (width + 3) / 4, bh = (height + 3) / 4, bs = block_bytes(dxt);
  const size_t row_bytes = size_t(bw) * bs, out_bytes = row_bytes * bh;
  {
    const long long diff =
        dstRowStride >= width * (bs / 4) ? (long long)dstRowStride - (long long)((width + 3) & ~3) * (bs / 4) : 0;
    if (c.pageable_access == 1 && diff >= 0 && host_direct_enabled()) {
      *done = true;
      return compress_host_direct(c, sc, width, height, src, dxt, dest, diff, opt, plan);
    }
  }
  if (npx > kSmallCallTexels) return false;
  *done = true;
  const size_t o_ticket = align_up(size_t(npx) * sc, 256), o_status = o_ticket + 16;
  const size_t o_flag = align_up(o_status + size_t(plan.bands) * 8, 16), o_blocks = o_flag + 16;
  const size_t o_aggs = align_up(o_blocks + out_bytes, 16), total = o_aggs + size_t(plan.bands) * 72;
  if (!c.small_dev.reserve(total, "cudaMalloc(small call)") ||
      !c.small_host.reserve(o_blocks + out_bytes, "cudaMallocHost(small call)"))
    return true;
  uint8_t* h = static_cast<uint8_t*>(c.small_host.p);
  uint8_t* d = c.small_dev.as<uint8_t>();
  std::memcpy(h, src, size_t(npx) * sc);
  std::memset(h + o_ticket, 0, o_blocks - o_ticket);
  StripArgs sa = strip_args(plan, sc, width, height, d, dxt, opt.dither, d + o_blocks, (long long)row_bytes,
                            reinterpret_cast<int*>(d + o_flag));
  sa.scan.ticket = reinterpret_cast<unsigned int*>(d + o_ticket);
  sa.scan.status = reinterpret_cast<unsigned long long*>(d + o_status);
  sa.scan.aggs = d + o_aggs;
  CUtensorMap map;
  sa.use_tma = sc == 4 && rgba_rows_map(d, npx, &map, &sa.tma_rows);
  cudaStream_t s = c.stream;
  cudaEvent_t* tev = c.timing ? &c.ev[3 * (c.timed_calls % Context::kTimingSlots)] : nullptr;
  if (!cuda_ok(cudaMemcpyAsync(d, h, o_blocks, cudaMemcpyHostToDevice, s), "input upload")) return true;
  if (tev && (!cuda_ok(cudaEventRecord(tev[0], s), "cudaEventRecord") ||
              !cuda_ok(cudaEventRecord(tev[1], s), "cudaEventRecord")))
    return true;
  if (!cuda_ok(launch_strip(sa, &map, dxt, opt.metric, opt.refine, nullptr, s), "strip launch")) return true;
  if (tev) {
    if (!cuda_ok(cudaEventRecord(tev[2], s), "cudaEventRecord")) return true;
    c.timed_calls++;
  }
  if (!cuda_ok(cudaMemcpyAsync(h + o_flag, d + o_flag, 16 + out_bytes, cudaMemcpyDeviceToHost, s), "output download") ||
      !cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize"))
    return true;
  if (*reinterpret_cast<const int*>(h + o_flag)) {
    set_error("a bounded wait in the dither scan gave up");
    return true;
  }
  // output rows: packed, or dstRowStride apart (s2tc_libtxc_dxtn.cpp:243, 261, 279); a stride below
  // the padded row overlaps rows, later rows overwriting the end of earlier ones
  const long long diff =
      dstRowStride >= width * (bs / 4) ? (long long)dstRowStride - (long long)((width + 3) & ~3) * (bs / 4) : 0;
  const uint8_t* blocks = h + o_blocks;
  if (diff == 0) {
    std::memcpy(dest, blocks, out_bytes);
  } else {
    for (int r = 0; r < bh; ++r)
      std::memmove(dest + r * (long long)(row_bytes + diff), blocks + r * row_bytes, row_bytes);
  }
  return true;
}

// Host-memory compression used by tx_compress_dxtn.
void compress_host(int srccomps, int width, int height, const unsigned char* src, int dxt, unsigned char* dest,
                   int dstRowStride, const s2tc_options& opt) {
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return;
  cudaStream_t s = c.stream;
  {
    bool done = false;
    compress_host_small(c, srccomps == 3 ? 3 : 4, width, height, src, dxt, dest, dstRowStride, opt, &done);
    if (done) return;
  }
  {
    const int bs0 = block_bytes(dxt);
    const long long diff0 = dstRowStride >= width * (bs0 / 4)
                                ? (long long)dstRowStride - (long long)((width + 3) & ~3) * (bs0 / 4)
                                : 0;
    bool done = false;
    compress_host_pipelined(c, srccomps == 3 ? 3 : 4, width, height, src, dxt, dest, diff0, opt, &done);
    if (done) return;
  }
  const int sc = srccomps == 3 ? 3 : 4;
  const size_t in_bytes = size_t(width) * height * sc;
  const int bw = (width + 3) / 4, bh = (height + 3) / 4, bs = block_bytes(dxt);
  const size_t row_bytes = size_t(bw) * bs;
  if (!c.src.reserve(in_bytes + 16, "cudaMalloc(src)")) return;
  if (!c.dst.reserve(row_bytes * bh + 16, "cudaMalloc(dst)")) return;
  if (!cuda_ok(cudaMemcpyAsync(c.src.p, src, in_bytes, cudaMemcpyHostToDevice, s), "input upload")) return;
  if (compress_device_locked(c, sc, width, height, c.src.as<uint8_t>(), dxt, c.dst.as<uint8_t>(), (long long)row_bytes,
                             opt, nullptr, s, c.err.as<int>() + 2) != ST_OK)
    return;
  // the flag read goes ahead of the output download: one wait for both (a
  // call whose bounded wait gave up reports it, its output is undefined)
  if (!enqueue_flag(c, s)) return;
  // Output rows: packed, or dstRowStride apart (s2tc_libtxc_dxtn.cpp:243, 261, 279).
  const long long diff =
      dstRowStride >= width * (bs / 4) ? (long long)dstRowStride - (long long)((width + 3) & ~3) * (bs / 4) : 0;
  if (diff == 0) {
    cuda_ok(cudaMemcpyAsync(dest, c.dst.p, row_bytes * bh, cudaMemcpyDeviceToHost, s), "output download");
  } else if (diff > 0) {
    cuda_ok(cudaMemcpy2DAsync(dest, row_bytes + diff, c.dst.p, row_bytes, row_bytes, bh, cudaMemcpyDeviceToHost, s),
            "output download");
  } else {
    // overlapping rows: later rows overwrite the end of earlier ones, in order
    if (!c.host_out.reserve(row_bytes * bh, "cudaMallocHost(output)")) return;
    if (!cuda_ok(cudaMemcpyAsync(c.host_out.p, c.dst.p, row_bytes * bh, cudaMemcpyDeviceToHost, s), "output download"))
      return;
    if (!cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize") || take_flag(c) != ST_OK) return;
    for (int r = 0; r < bh; ++r)
      std::memmove(dest + r * (long long)(row_bytes + diff), static_cast<unsigned char*>(c.host_out.p) + r * row_bytes,
                   row_bytes);
    return;
  }
  if (cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize")) take_flag(c);
}


// ------------------------------------------------------------ launch layouts

struct LayoutTable {
  std::mutex mu;
  EncodeLayout t[8][3][3][3];  // metric, format, refinement, kind
  LayoutTable() {
    for (auto& a : t)
      for (auto& b : a)
        for (auto& c : b)
          for (auto& d : c) d = EncodeLayout{128, 4, 64};
  }
};

LayoutTable& layouts() {
  static LayoutTable* l = new LayoutTable();
  return *l;
}

bool layout_key_ok(int metric, int dxt, int refine, int kind) {
  return metric >= 0 && metric < 8 && dxt >= 0 && dxt < 3 && refine >= 0 && refine < 3 && kind >= 0 && kind < 3;
}

// ------------------------------------------------------------------ batches

// A planned batch: device tables, scratch and a CUDA graph of the whole
// launch sequence (dither for every image, then the encoder kernels of each
// format), replayed by s2tc_batch_run.
struct Batch {
  std::vector<s2tc_image> items;  // images with at least one texel
  s2tc_options opt;
  bool normal = false;
  DevBuf t565, scratch, tables, rnd;
  PinnedBuf host_rnd;
  long long host_rand_words = 0;        // rand words replayed per run (host path)
  bool device_rand = false;             // ... generated on the device from a pinned window
  DevBuf rnd_win;
  std::vector<long long> rand_words;    // per image
  cudaStream_t capture = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaEvent_t done = nullptr;
  int kernels = 0;                      // kernels per run
  // prepared launch descriptors (device tables already uploaded), per group
  // of consecutive images (see kBatchGroupTexels)
  struct Group {
    DitherWork dwork{};
    int fs_first = 0, fs_count = 0;  // Floyd-Steinberg: one launch per image
    EncodeWork ework[3]{};
    bool has_fmt[3] = {false, false, false};
  };
  std::vector<Group> groups;
  std::vector<DitherArgs> fs_items;
  std::vector<size_t> fs_off;

  ~Batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (done) cudaEventDestroy(done);
    if (capture) cudaStreamDestroy(capture);
    for (DevBuf* b : {&t565, &scratch, &tables, &rnd, &rnd_win})
      if (b->p) cudaFree(b->p);
    if (host_rnd.p) cudaFreeHost(host_rnd.p);
  }
};


// A batch runs as groups of consecutive images of at most this many texels
// (the last may exceed it by one image): a group's dither writes its texel
// words (4 bytes each, 16 MB here) and its encoder launches read them back
// while they are still in the 129 MB L2.  One dither launch over a whole
// batch of 64 normal maps of 2048^2 (1.07 GB of texel words) left the
// encoder 3% slower than one launch pair per image.  A group of one image
// passes its records by value, as a single-image launch does, instead of
// through the device tables.
constexpr long long kBatchGroupTexels = 4ll << 20;

// Lay out, allocate and upload everything a batch's launches need.
int batch_prepare(Batch& b, Context& c) {
  const int n = int(b.items.size());
  const long long tile_tex = dither_tile_texels();
  // groups of consecutive images
  std::vector<int> group_of(n);
  std::vector<int> first_of_group;
  {
    long long tex = 0;
    for (int i = 0; i < n; ++i) {
      const long long npx = (long long)b.items[i].width * b.items[i].height;
      if (i == 0 || tex >= kBatchGroupTexels) {
        first_of_group.push_back(i);
        tex = 0;
      }
      group_of[i] = int(first_of_group.size()) - 1;
      tex += npx;
    }
  }
  const int ng = int(first_of_group.size());
  // tables laid out in b.tables: DitherItem[n], tile offsets[n] (from each
  // group's first tile), then per format EncodeArgs[n_f] and block offsets
  // (from each group's first block of that format)
  std::vector<DitherItem> ditems(n);
  std::vector<long long> toff(n);
  std::vector<long long> tex_off(n);
  std::vector<long long> group_tiles(ng, 0);
  long long texels = 0;
  for (int i = 0; i < n; ++i) {
    const s2tc_image& im = b.items[i];
    const long long npx = (long long)im.width * im.height;
    tex_off[i] = texels;
    texels += (npx + 3) & ~3ll;  // 16-byte aligned texel rows of each image
    toff[i] = group_tiles[group_of[i]];
    group_tiles[group_of[i]] += (npx + tile_tex - 1) / tile_tex;
  }
  if (!b.t565.reserve(size_t(texels) * 4 + 64, "cudaMalloc(batch texels)")) return ST_OUT_OF_MEMORY;
  for (int i = 0; i < n; ++i) {
    const s2tc_image& im = b.items[i];
    const int dxt = format_dxt(im.format);
    ditems[i] = DitherItem{static_cast<const uint8_t*>(im.src), im.width, im.height, im.srccomps == 3 ? 3 : 4,
                           alpha_bits(dxt), b.t565.as<uint32_t>() + tex_off[i]};
  }
  // per-format encode tables, in image order; per group and format the first
  // entry and the count
  std::vector<EncodeArgs> eargs[3];
  std::vector<long long> eoff[3];
  std::vector<int> gfirst[3], gcount[3];
  std::vector<long long> gblocks[3];
  for (int d = 0; d < 3; ++d) {
    gfirst[d].assign(ng, 0);
    gcount[d].assign(ng, 0);
    gblocks[d].assign(ng, 0);
  }
  const int per_block_words[3] = {b.opt.nrandom > 0 ? b.opt.nrandom * 3 : 0, b.opt.nrandom > 0 ? b.opt.nrandom * 3 : 0,
                                  b.opt.nrandom > 0 ? b.opt.nrandom * 4 : 0};
  long long rand_pos = 0;
  for (int i = 0; i < n; ++i) {
    const s2tc_image& im = b.items[i];
    const int dxt = format_dxt(im.format), g = group_of[i];
    EncodeArgs ea{};
    ea.t565 = b.t565.as<uint32_t>() + tex_off[i];
    ea.width = im.width;
    ea.height = im.height;
    ea.bw = (im.width + 3) / 4;
    ea.bh = (im.height + 3) / 4;
    ea.by0 = 0;
    ea.nby = ea.bh;
    ea.dst = static_cast<uint8_t*>(im.dst);
    ea.pitch = im.dst_pitch;
    const int bs = block_bytes(dxt);
    ea.aligned = ((reinterpret_cast<uintptr_t>(im.dst) % bs) == 0 && (im.dst_pitch % bs) == 0) ? 1 : 0;
    ea.nrandom = b.opt.nrandom;
    ea.prev_a1_first = -1;
    ea.leftover_out = nullptr;
    ea.rnd = nullptr;
    if (b.normal && b.opt.nrandom > 0) {
      if (im.rand) {
        ea.rnd = im.rand;
      } else {
        ea.rnd = b.rnd.as<uint32_t>() + rand_pos;
        rand_pos += (long long)ea.bw * ea.bh * per_block_words[dxt];
      }
    }
    if (gcount[dxt][g] == 0) gfirst[dxt][g] = int(eargs[dxt].size());
    gcount[dxt][g]++;
    eoff[dxt].push_back(gblocks[dxt][g]);
    gblocks[dxt][g] += (long long)ea.bw * ea.bh;
    eargs[dxt].push_back(ea);
  }
  // upload the tables (pinned staging, copied inside the graph)
  size_t off = 0;
  const size_t o_ditems = off;
  off = align_up(off + sizeof(DitherItem) * n, 16);
  const size_t o_toff = off;
  off = align_up(off + sizeof(long long) * n, 16);
  size_t o_eargs[3], o_eoff[3];
  for (int d = 0; d < 3; ++d) {
    o_eargs[d] = off;
    off = align_up(off + sizeof(EncodeArgs) * eargs[d].size(), 16);
    o_eoff[d] = off;
    off = align_up(off + sizeof(long long) * eoff[d].size(), 16);
  }
  if (!b.tables.reserve(off + 16, "cudaMalloc(batch tables)")) return ST_OUT_OF_MEMORY;
  std::vector<unsigned char> host(off + 16, 0);
  std::memcpy(host.data() + o_ditems, ditems.data(), sizeof(DitherItem) * n);
  std::memcpy(host.data() + o_toff, toff.data(), sizeof(long long) * n);
  for (int d = 0; d < 3; ++d) {
    if (!eargs[d].empty()) std::memcpy(host.data() + o_eargs[d], eargs[d].data(), sizeof(EncodeArgs) * eargs[d].size());
    if (!eoff[d].empty()) std::memcpy(host.data() + o_eoff[d], eoff[d].data(), sizeof(long long) * eoff[d].size());
  }
  // the tables are constant for the plan: upload them now, outside the graph
  if (!cuda_ok(cudaMemcpy(b.tables.p, host.data(), off, cudaMemcpyHostToDevice), "batch table upload"))
    return ST_CUDA_ERROR;
  unsigned char* tb = b.tables.as<unsigned char>();

  // scratch: SIMPLE/NONE tiles of the largest group (groups run in stream
  // order and share it), or one Floyd-Steinberg area per image
  std::vector<size_t> fs_off(n, 0);
  long long max_tiles = 0;
  for (long long t : group_tiles) max_tiles = std::max(max_tiles, t);
  size_t scratch = dither_batch_scratch_bytes(max_tiles);
  if (b.opt.dither == DI_FLOYDSTEINBERG) {
    scratch = 0;
    for (int i = 0; i < n; ++i) {
      fs_off[i] = scratch;
      scratch = align_up(scratch + dither_fs_scratch_bytes(b.items[i].width, b.items[i].height), 256);
    }
  }
  if (!b.scratch.reserve(scratch + 256, "cudaMalloc(batch scratch)")) return ST_OUT_OF_MEMORY;

  // --- launch descriptors
  b.fs_items.clear();
  b.fs_off = fs_off;
  if (b.opt.dither == DI_FLOYDSTEINBERG) {
    for (int i = 0; i < n; ++i) {
      DitherArgs da{};
      da.src = ditems[i].src;
      da.width = ditems[i].width;
      da.height = ditems[i].height;
      da.srccomps = ditems[i].srccomps;
      da.alphabits = ditems[i].alphabits;
      da.dst = ditems[i].dst;
      da.error = c.err.as<int>();
      b.fs_items.push_back(da);
    }
  }
  b.groups.assign(ng, Batch::Group{});
  for (int g = 0; g < ng; ++g) {
    Batch::Group& G = b.groups[g];
    const int i0 = first_of_group[g], i1 = g + 1 < ng ? first_of_group[g + 1] : n;
    G.fs_first = i0;
    G.fs_count = i1 - i0;
    if (b.opt.dither != DI_FLOYDSTEINBERG) {
      G.dwork = DitherWork{};
      if (i1 - i0 == 1) {
        G.dwork.single = ditems[i0];
      } else {
        G.dwork.items = reinterpret_cast<const DitherItem*>(tb + o_ditems) + i0;
        G.dwork.tile_offsets = reinterpret_cast<const long long*>(tb + o_toff) + i0;
      }
      G.dwork.nitems = i1 - i0;
      G.dwork.total_tiles = group_tiles[g];
      G.dwork.error = c.err.as<int>();
    }
    for (int d = 0; d < 3; ++d) {
      G.has_fmt[d] = gcount[d][g] > 0;
      if (!G.has_fmt[d]) continue;
      EncodeWork& w = G.ework[d];
      w = EncodeWork{};
      if (gcount[d][g] == 1) {
        w.single = eargs[d][gfirst[d][g]];
      } else {
        w.items = reinterpret_cast<const EncodeArgs*>(tb + o_eargs[d]) + gfirst[d][g];
        w.offsets = reinterpret_cast<const long long*>(tb + o_eoff[d]) + gfirst[d][g];
      }
      w.nitems = gcount[d][g];
      w.total = gblocks[d][g];
      w.nrandom = b.opt.nrandom;
    }
  }
  return ST_OK;
}

// The launch sequence of a batch on stream `s` (captured once into the graph).
int batch_launch(Batch& b, cudaStream_t s) {
  const long long l0 = launches_so_far();
  if (b.host_rand_words > 0 && b.device_rand) {
    if (!cuda_ok(cudaMemcpyAsync(b.rnd_win.p, b.host_rnd.p, sizeof(RandWindow), cudaMemcpyHostToDevice, s),
                 "batch rand window upload"))
      return ST_CUDA_ERROR;
    if (!cuda_ok(rand_fill(b.rnd_win.as<RandWindow>(), b.rnd.as<uint32_t>(), b.host_rand_words, s), "rand fill"))
      return ST_CUDA_ERROR;
  } else if (b.host_rand_words > 0) {
    if (!cuda_ok(cudaMemcpyAsync(b.rnd.p, b.host_rnd.p, size_t(b.host_rand_words) * 4, cudaMemcpyHostToDevice, s),
                 "batch rand upload"))
      return ST_CUDA_ERROR;
  }
  for (const Batch::Group& G : b.groups) {
    if (b.opt.dither == DI_FLOYDSTEINBERG) {
      for (int i = G.fs_first; i < G.fs_first + G.fs_count; ++i)
        if (!cuda_ok(launch_dither(b.fs_items[i], DI_FLOYDSTEINBERG, b.scratch.as<uint8_t>() + b.fs_off[i], s),
                     "batch dither"))
          return ST_CUDA_ERROR;
    } else {
      if (!cuda_ok(launch_dither_batch(G.dwork, b.opt.dither, b.scratch.as<uint8_t>(), s), "batch dither"))
        return ST_CUDA_ERROR;
    }
    for (int d = 0; d < 3; ++d) {
      if (!G.has_fmt[d]) continue;
      if (!cuda_ok(launch_encode(G.ework[d], d, b.opt.metric, b.normal, b.opt.refine, s), "batch encode"))
        return ST_CUDA_ERROR;
    }
  }
  b.kernels = int(launches_so_far() - l0);
  return ST_OK;
}

}  // namespace
}  // namespace s2tc

struct s2tc_batch {
  s2tc::Batch impl;
};

namespace s2tc {
namespace {

// ----------------------------------------------------------- block shims

// Leftover second alpha endpoint of the previous shim call on this thread,
// read by a following single-texel DXT5 block (see encode.cu).
thread_local int g_prev_a1 = -1;

void encode_one_block(int dxt, int metric, bool normal, int refine, unsigned char* out, const unsigned char* rgba,
                      int iw, int w, int h, int nrandom) {
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return;
  cudaStream_t s = c.stream;
  if (w < 1 || h < 1) return;
  w = w > 4 ? 4 : w;
  h = h > 4 ? 4 : h;
  // gather the block's rows into a packed w x h texel image
  uint32_t blk[16] = {0};
  for (int y = 0; y < h; ++y) std::memcpy(&blk[y * w], rgba + (size_t)y * iw * 4, size_t(w) * 4);
  s2tc_options opt{DI_NONE, metric, nrandom, refine};
  const int per_block = (normal && nrandom > 0) ? nrandom * (dxt == DXT5 ? 4 : 3) : 0;
  if (!c.t565.reserve(64 + 16, "cudaMalloc(texels)")) return;
  if (!c.dst.reserve(16, "cudaMalloc(dst)")) return;
  if (!cuda_ok(cudaStreamWaitEvent(s, c.arena_free, 0), "cudaStreamWaitEvent")) return;
  if (per_block > 0) {
    if (!c.rnd.reserve(size_t(per_block) * 4, "cudaMalloc(rand)")) return;
    if (!c.host_rnd.reserve(size_t(per_block) * 4, "cudaMallocHost(rand)")) return;
    unsigned int* hr = static_cast<unsigned int*>(c.host_rnd.p);
    for (int i = 0; i < per_block; ++i) hr[i] = unsigned(std::rand());
    if (!cuda_ok(cudaMemcpyAsync(c.rnd.p, hr, size_t(per_block) * 4, cudaMemcpyHostToDevice, s), "rand upload")) return;
  }
  if (!cuda_ok(cudaMemcpyAsync(c.t565.p, blk, sizeof(blk), cudaMemcpyHostToDevice, s), "block upload")) return;
  EncodeArgs ea{};
  ea.t565 = c.t565.as<uint32_t>();
  ea.width = w;
  ea.height = h;
  ea.bw = 1;
  ea.bh = 1;
  ea.by0 = 0;
  ea.nby = 1;
  ea.dst = c.dst.as<uint8_t>();
  ea.pitch = 16;
  ea.aligned = 1;
  ea.nrandom = opt.nrandom;
  ea.rnd = per_block > 0 ? c.rnd.as<uint32_t>() : nullptr;
  ea.prev_a1_first = g_prev_a1;
  ea.leftover_out = c.err.as<int>() + 1;
  if (!cuda_ok(launch_encode(ea, dxt, metric, normal, refine, s), "encode launch")) return;
  unsigned char tmp[16];
  int leftover = -1;
  if (!cuda_ok(cudaMemcpyAsync(tmp, c.dst.p, 16, cudaMemcpyDeviceToHost, s), "block download")) return;
  if (!cuda_ok(cudaMemcpyAsync(&leftover, c.err.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, s),
               "block download"))
    return;
  if (!cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize")) return;
  std::memcpy(out, tmp, size_t(block_bytes(dxt)));
  g_prev_a1 = leftover;
}

template <int DXT, int METRIC, bool NORMAL, int REFINE>
void block_shim(unsigned char* out, const unsigned char* rgba, int iw, int w, int h, int nrandom) {
  encode_one_block(DXT, METRIC, NORMAL, REFINE, out, rgba, iw, w, h, nrandom);
}

template <int DXT, int METRIC, bool NORMAL>
s2tc_encode_block_func_t pick_refine(int refine) {
  switch (refine) {
    case RF_NEVER: return &block_shim<DXT, METRIC, NORMAL, RF_NEVER>;
    case RF_LOOP: return &block_shim<DXT, METRIC, NORMAL, RF_LOOP>;
    default: return &block_shim<DXT, METRIC, NORMAL, RF_ALWAYS>;
  }
}
template <int DXT, int METRIC>
s2tc_encode_block_func_t pick_mode(int nrandom, int refine) {
  if (METRIC == CD_NORMALMAP || nrandom >= 0) return pick_refine<DXT, METRIC, true>(refine);
  return pick_refine<DXT, METRIC, false>(refine);
}
template <int METRIC>
s2tc_encode_block_func_t pick_dxt(int dxt, int nrandom, int refine) {
  switch (dxt) {
    case DXT1: return pick_mode<DXT1, METRIC>(nrandom, refine);
    case DXT3: return pick_mode<DXT3, METRIC>(nrandom, refine);
    default: return pick_mode<DXT5, METRIC>(nrandom, refine);
  }
}

// ---------------------------------------------------------- texel decode

void expand565(unsigned c, unsigned char* t) {
  const int r = (c >> 11) & 31, g = (c >> 5) & 63, b = c & 31;
  t[0] = (unsigned char)((r << 3) | (r >> 2));
  t[1] = (unsigned char)((g << 2) | (g >> 4));
  t[2] = (unsigned char)((b << 3) | (b >> 2));
}

// s2tc_libtxc_dxtn.cpp:35-140: decode texel (i, j).
void fetch_texel(int dxt, bool rgba_dxt1, int stride, const unsigned char* data, int i, int j, unsigned char* t) {
  const int bs = dxt == DXT1 ? 8 : 16;
  const unsigned char* blk = data + ((long long)((stride + 3) >> 2) * (j >> 2) + (i >> 2)) * bs;
  const unsigned char* cb = blk + (bs - 8);
  unsigned c = cb[0] | (cb[1] << 8), c1 = cb[2] | (cb[3] << 8);
  const int sel = (cb[4 + (j & 3)] >> (2 * (i & 3))) & 3;
  const bool odd = ((i ^ j) & 1) != 0;
  unsigned char a = 255;
  if (sel == 1) {
    c = c1;
  } else if (sel >= 2) {
    if (dxt == DXT1 && sel == 3 && c1 >= c) {
      c = 0;
      if (rgba_dxt1) a = 0;
    } else if (odd) {
      c = c1;
    }
  }
  expand565(c, t);
  if (dxt == DXT1) {
    if (rgba_dxt1) t[3] = a;
    return;
  }
  if (dxt == DXT3) {
    const int av = (blk[(j & 3) * 2 + ((i & 3) >> 1)] >> (4 * (i & 1))) & 15;
    t[3] = (unsigned char)(av | (av << 4));
    return;
  }
  unsigned a0 = blk[0], a1 = blk[1];
  const int bit = ((j & 3) * 4 + (i & 3)) * 3;
  int ab = 0;
  for (int k = 0; k < 3; ++k)
    if (blk[2 + ((bit + k) >> 3)] & (1 << ((bit + k) & 7))) ab |= 1 << k;
  unsigned av = a0;
  if (ab == 1) av = a1;
  else if (ab == 6 && a1 >= a0) av = 0;
  else if ((ab == 6 || ab == 7) && a1 >= a0) av = 255;
  else if (ab >= 2 && odd) av = a1;
  t[3] = (unsigned char)av;
}

}  // namespace
}  // namespace s2tc

using s2tc::Context;
using s2tc::count_launches;
using s2tc::DitherArgs;
using s2tc::check_error_flag;
using s2tc::compress_device_locked;
using s2tc::compress_host;
using s2tc::ctx;
using s2tc::cuda_ok;
using s2tc::fetch_texel;
using s2tc::format_dxt;
using s2tc::normalise;
using s2tc::pick_dxt;
using s2tc::rand_per_block;
using s2tc::read_env;
using s2tc::set_error;

extern "C" {

void tx_compress_dxtn(int srccomps, int width, int height, const unsigned char* srcPixData, unsigned int destformat,
                      unsigned char* dest, int dstRowStride) {
  const s2tc_options opt = read_env();
  const int dxt = format_dxt(destformat);
  if (dxt < 0) {
    std::fprintf(stderr, "libdxtn: Bad dstFormat %d in tx_compress_dxtn\n", (int)destformat);
    return;
  }
  if (width <= 0 || height <= 0) return;
  compress_host(srccomps, width, height, srcPixData, dxt, dest, dstRowStride, normalise(opt));
}

void fetch_2d_texel_rgb_dxt1(int srcRowStride, const unsigned char* pixdata, int i, int j, void* texel) {
  unsigned char* t = static_cast<unsigned char*>(texel);
  fetch_texel(s2tc::DXT1, false, srcRowStride, pixdata, i, j, t);
  t[3] = 255;
}
void fetch_2d_texel_rgba_dxt1(int srcRowStride, const unsigned char* pixdata, int i, int j, void* texel) {
  fetch_texel(s2tc::DXT1, true, srcRowStride, pixdata, i, j, static_cast<unsigned char*>(texel));
}
void fetch_2d_texel_rgba_dxt3(int srcRowStride, const unsigned char* pixdata, int i, int j, void* texel) {
  fetch_texel(s2tc::DXT3, true, srcRowStride, pixdata, i, j, static_cast<unsigned char*>(texel));
}
void fetch_2d_texel_rgba_dxt5(int srcRowStride, const unsigned char* pixdata, int i, int j, void* texel) {
  fetch_texel(s2tc::DXT5, true, srcRowStride, pixdata, i, j, static_cast<unsigned char*>(texel));
}

void rgb565_image(unsigned char* out, const unsigned char* rgba, int w, int h, int srccomps, int alphabits,
                  DitherMode dither) {
  if (w <= 0 || h <= 0) return;
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return;
  cudaStream_t s = c.stream;
  const int sc = srccomps == 3 ? 3 : 4;
  const int ab = alphabits == 1 ? 1 : alphabits == 4 ? 4 : 8;
  int d = int(dither);
  if (d != s2tc::DI_NONE && d != s2tc::DI_FLOYDSTEINBERG) d = s2tc::DI_SIMPLE;
  const long long npx = (long long)w * h;
  if (!c.src.reserve(size_t(npx) * sc + 16, "cudaMalloc(src)")) return;
  if (!c.t565.reserve(size_t(npx) * 4 + 16, "cudaMalloc(texels)")) return;
  size_t scratch = d == s2tc::DI_FLOYDSTEINBERG ? s2tc::dither_fs_scratch_bytes(w, h) : s2tc::dither_scratch_bytes(npx);
  if (!c.scratch.reserve(scratch, "cudaMalloc(scratch)")) return;
  if (!cuda_ok(cudaStreamWaitEvent(s, c.arena_free, 0), "cudaStreamWaitEvent")) return;
  if (!cuda_ok(cudaMemcpyAsync(c.src.p, rgba, size_t(npx) * sc, cudaMemcpyHostToDevice, s), "input upload")) return;
  DitherArgs da{};
  da.src = c.src.as<uint8_t>();
  da.width = w;
  da.height = h;
  da.srccomps = sc;
  da.alphabits = ab;
  da.dst = c.t565.as<uint32_t>();
  da.error = c.err.as<int>();
  if (!cuda_ok(s2tc::launch_dither(da, d, c.scratch.as<uint8_t>(), s), "dither launch")) return;
  if (check_error_flag(c, s) != s2tc::ST_OK) return;
  if (!cuda_ok(cudaMemcpyAsync(out, c.t565.p, size_t(npx) * 4, cudaMemcpyDeviceToHost, s), "output download")) return;
  cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}

s2tc_encode_block_func_t s2tc_encode_block_func(DxtMode dxt, ColorDistMode cd, int nrandom, RefinementMode refine) {
  const int d = int(dxt), r = int(refine);
  switch (int(cd)) {
    case s2tc::CD_RGB: return pick_dxt<s2tc::CD_RGB>(d, nrandom, r);
    case s2tc::CD_YUV: return pick_dxt<s2tc::CD_YUV>(d, nrandom, r);
    case s2tc::CD_SRGB: return pick_dxt<s2tc::CD_SRGB>(d, nrandom, r);
    case s2tc::CD_SRGB_MIXED: return pick_dxt<s2tc::CD_SRGB_MIXED>(d, nrandom, r);
    case s2tc::CD_AVG: return pick_dxt<s2tc::CD_AVG>(d, nrandom, r);
    case s2tc::CD_W0AVG: return pick_dxt<s2tc::CD_W0AVG>(d, nrandom, r);
    case s2tc::CD_NORMALMAP: return pick_dxt<s2tc::CD_NORMALMAP>(d, nrandom, r);
    default: return pick_dxt<s2tc::CD_WAVG>(d, nrandom, r);
  }
}

void s2tc_options_from_env(s2tc_options* opt) {
  if (opt) *opt = read_env();
}

long long s2tc_rand_words(int width, int height, unsigned int destformat, const s2tc_options* opt) {
  const int dxt = format_dxt(destformat);
  if (dxt < 0 || !opt || width <= 0 || height <= 0) return 0;
  const s2tc_options o = normalise(*opt);
  return (long long)((width + 3) / 4) * ((height + 3) / 4) * rand_per_block(o, dxt);
}

int s2tc_gpu_compress(int srccomps, int width, int height, const void* d_src, unsigned int destformat, void* d_dst,
                      long long dst_pitch, const s2tc_options* opt, const unsigned int* d_rand, void* stream) {
  const int dxt = format_dxt(destformat);
  if (dxt < 0) {
    set_error("bad destination format");
    return S2TC_ERR_FORMAT;
  }
  if (width < 0 || height < 0 || !opt || (width > 0 && height > 0 && (!d_src || !d_dst))) {
    set_error("bad argument");
    return S2TC_ERR_ARGUMENT;
  }
  if (width == 0 || height == 0) return S2TC_OK;
  const int bw = (width + 3) / 4;
  if (dst_pitch < (long long)bw * s2tc::block_bytes(dxt)) {
    set_error("dst_pitch smaller than a block row");
    return S2TC_ERR_ARGUMENT;
  }
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return S2TC_ERR_CUDA;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
  return compress_device_locked(c, srccomps, width, height, static_cast<const uint8_t*>(d_src), dxt,
                                static_cast<uint8_t*>(d_dst), dst_pitch, normalise(*opt), d_rand, s);
}

int s2tc_gpu_encode_blocks(const void* d_t565, int width, int height, int dxt, int colordist, int nrandom, int refine,
                           void* d_dst, long long dst_pitch, const unsigned int* d_rand, void* stream) {
  if (dxt < s2tc::DXT1 || dxt > s2tc::DXT5) {
    set_error("bad DxtMode");
    return S2TC_ERR_FORMAT;
  }
  if (width < 0 || height < 0 || (width > 0 && height > 0 && (!d_t565 || !d_dst))) {
    set_error("bad argument");
    return S2TC_ERR_ARGUMENT;
  }
  if (width == 0 || height == 0) return S2TC_OK;
  if (dst_pitch < (long long)((width + 3) / 4) * s2tc::block_bytes(dxt)) {
    set_error("dst_pitch smaller than a block row");
    return S2TC_ERR_ARGUMENT;
  }
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return S2TC_ERR_CUDA;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
  const s2tc_options o = normalise(s2tc_options{s2tc::DI_NONE, colordist, nrandom, refine});
  // host-replayed rand() words go through the arena's staging buffers
  if (!cuda_ok(cudaStreamWaitEvent(s, c.arena_free, 0), "cudaStreamWaitEvent")) return S2TC_ERR_CUDA;
  const int st = encode_locked(c, static_cast<const uint32_t*>(d_t565), width, height, dxt,
                               static_cast<uint8_t*>(d_dst), dst_pitch, o, d_rand, s, nullptr);
  if (st != S2TC_OK) return st;
  return cuda_ok(cudaEventRecord(c.arena_free, s), "cudaEventRecord") ? S2TC_OK : S2TC_ERR_CUDA;
}

int s2tc_gpu_synchronize(void* stream) {
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return S2TC_ERR_CUDA;
  return check_error_flag(c, stream ? static_cast<cudaStream_t>(stream) : c.stream);
}

int s2tc_gpu_set_timing(int enable) {
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return S2TC_ERR_CUDA;
  if (enable && c.ev.empty()) {
    c.ev.resize(3 * Context::kTimingSlots);
    for (auto& e : c.ev)
      if (!cuda_ok(cudaEventCreate(&e), "cudaEventCreate")) return S2TC_ERR_CUDA;
  }
  c.timing = enable != 0;
  c.timed_calls = 0;
  return S2TC_OK;
}

int s2tc_gpu_stage_ms(float* dither_ms, float* encode_ms, long long* calls) {
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  const long long n = std::min<long long>(c.timed_calls, Context::kTimingSlots);
  double a = 0, b = 0;
  for (long long i = 0; i < n; ++i) {
    cudaEvent_t* e = &c.ev[3 * i];
    float x = 0, y = 0;
    if (!cuda_ok(cudaEventSynchronize(e[2]), "cudaEventSynchronize")) return S2TC_ERR_CUDA;
    if (!cuda_ok(cudaEventElapsedTime(&x, e[0], e[1]), "cudaEventElapsedTime")) return S2TC_ERR_CUDA;
    if (!cuda_ok(cudaEventElapsedTime(&y, e[1], e[2]), "cudaEventElapsedTime")) return S2TC_ERR_CUDA;
    a += x;
    b += y;
  }
  if (dither_ms) *dither_ms = float(a);
  if (encode_ms) *encode_ms = float(b);
  if (calls) *calls = n;
  return S2TC_OK;
}

long long s2tc_gpu_kernel_launches(void) { return s2tc::launches_so_far(); }

int s2tc_test_dither_hold(long long hold_tile, int spin_limit) {
  s2tc::set_dither_test_hold(hold_tile, spin_limit);
  return S2TC_OK;
}

int s2tc_gpu_compress_each(const s2tc_image* items, int count, const s2tc_options* opt, void* stream) {
  if (!opt || count < 0 || (count > 0 && !items)) {
    set_error("bad argument");
    return S2TC_ERR_ARGUMENT;
  }
  const s2tc_options o = normalise(*opt);
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return S2TC_ERR_CUDA;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
  for (int i = 0; i < count; ++i) {
    const s2tc_image& im = items[i];
    const int dxt = format_dxt(im.format);
    if (dxt < 0) {
      set_error("bad destination format in item " + std::to_string(i));
      return S2TC_ERR_FORMAT;
    }
    if (im.width <= 0 || im.height <= 0) continue;
    const int st = s2tc::compress_device_locked(c, im.srccomps, im.width, im.height, static_cast<const uint8_t*>(im.src),
                                                dxt, static_cast<uint8_t*>(im.dst), im.dst_pitch, o, im.rand, s);
    if (st != S2TC_OK) return st;
  }
  return S2TC_OK;
}

int s2tc_batch_create(s2tc_batch** out, const s2tc_image* items, int count, const s2tc_options* opt) {
  if (!out || !opt || count < 0 || (count > 0 && !items)) {
    set_error("bad argument");
    return S2TC_ERR_ARGUMENT;
  }
  *out = nullptr;
  s2tc_options o = normalise(*opt);
  for (int i = 0; i < count; ++i) {
    const s2tc_image& im = items[i];
    if (format_dxt(im.format) < 0) {
      set_error("bad destination format in batch item " + std::to_string(i));
      return S2TC_ERR_FORMAT;
    }
    if (im.width < 0 || im.height < 0 ||
        (im.width > 0 && im.height > 0 &&
         (!im.src || !im.dst || im.dst_pitch < (long long)((im.width + 3) / 4) * s2tc::block_bytes(format_dxt(im.format))))) {
      set_error("bad batch item " + std::to_string(i));
      return S2TC_ERR_ARGUMENT;
    }
  }
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return S2TC_ERR_CUDA;
  s2tc_batch* h = new s2tc_batch();
  s2tc::Batch& b = h->impl;
  b.opt = o;
  b.normal = o.nrandom >= 0 || o.metric == s2tc::CD_NORMALMAP;
  for (int i = 0; i < count; ++i)
    if (items[i].width > 0 && items[i].height > 0) b.items.push_back(items[i]);
  // rand words replayed on the host for images without their own stream
  if (b.normal && o.nrandom > 0) {
    for (const s2tc_image& im : b.items) {
      const long long words =
          (long long)((im.width + 3) / 4) * ((im.height + 3) / 4) * o.nrandom * (format_dxt(im.format) == s2tc::DXT5 ? 4 : 3);
      b.rand_words.push_back(im.rand ? 0 : words);
      b.host_rand_words += im.rand ? 0 : words;
    }
    if (b.host_rand_words > 0) {
      // the words come from the device generator (a pinned window per run)
      // unless libc's state cannot be read
      b.device_rand = s2tc::rand_usable() && cuda_ok(s2tc::rand_prepare(), "rand table upload");
      const size_t staging = b.device_rand ? sizeof(s2tc::RandWindow) : size_t(b.host_rand_words) * 4;
      if (!b.rnd.reserve(size_t(b.host_rand_words) * 4, "cudaMalloc(batch rand)") ||
          !b.host_rnd.reserve(staging, "cudaMallocHost(batch rand)") ||
          (b.device_rand && !b.rnd_win.reserve(sizeof(s2tc::RandWindow), "cudaMalloc(rand window)"))) {
        delete h;
        return S2TC_ERR_NOMEM;
      }
    }
  }
  int st = S2TC_OK;
  if (!cuda_ok(cudaStreamCreateWithFlags(&b.capture, cudaStreamNonBlocking), "cudaStreamCreate") ||
      !cuda_ok(cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming), "cudaEventCreate")) {
    delete h;
    return S2TC_ERR_CUDA;
  }
  if (!b.items.empty()) {
    st = s2tc::batch_prepare(b, c);
    if (st != S2TC_OK) {
      delete h;
      return st;
    }
    if (!cuda_ok(cudaStreamBeginCapture(b.capture, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture")) {
      delete h;
      return S2TC_ERR_CUDA;
    }
    st = s2tc::batch_launch(b, b.capture);
    cudaGraph_t g = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b.capture, &g);
    b.graph = g;
    if (st == S2TC_OK && !cuda_ok(e, "cudaStreamEndCapture")) st = S2TC_ERR_CUDA;
    if (st == S2TC_OK && !cuda_ok(cudaGraphInstantiate(&b.exec, b.graph, 0), "cudaGraphInstantiate"))
      st = S2TC_ERR_CUDA;
  }
  if (st != S2TC_OK) {
    delete h;
    return st;
  }
  *out = h;
  return S2TC_OK;
}

int s2tc_batch_run(s2tc_batch* h, void* stream) {
  if (!h) {
    set_error("null batch");
    return S2TC_ERR_ARGUMENT;
  }
  s2tc::Batch& b = h->impl;
  if (b.items.empty()) return S2TC_OK;
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c.stream;
  // a previous run of this plan must be done with the staging and scratch
  if (!cuda_ok(cudaEventSynchronize(b.done), "cudaEventSynchronize")) return S2TC_ERR_CUDA;
  if (b.host_rand_words > 0 && b.device_rand) {
    // libc rand() in image order, exactly as one tx_compress_dxtn call per
    // image would draw it: the stream's position now, generated on the device
    if (!s2tc::rand_take(b.host_rand_words, static_cast<s2tc::RandWindow*>(b.host_rnd.p))) {
      set_error("libc rand() state could not be read");
      return S2TC_ERR_CUDA;
    }
  } else if (b.host_rand_words > 0) {
    unsigned int* hr = static_cast<unsigned int*>(b.host_rnd.p);
    for (long long i = 0; i < b.host_rand_words; ++i) hr[i] = unsigned(std::rand());
  }
  if (!cuda_ok(cudaGraphLaunch(b.exec, s), "cudaGraphLaunch")) return S2TC_ERR_CUDA;
  s2tc::count_launches(b.kernels);
  if (!cuda_ok(cudaEventRecord(b.done, s), "cudaEventRecord")) return S2TC_ERR_CUDA;
  return S2TC_OK;
}

void s2tc_batch_destroy(s2tc_batch* h) {
  if (!h) return;
  cudaEventSynchronize(h->impl.done);
  delete h;
}

int s2tc_batch_kernels(const s2tc_batch* h) { return h ? h->impl.kernels : 0; }

long long s2tc_dds_size(int width, int height, unsigned int format) {
  const int dxt = format_dxt(format);
  if (dxt < 0 || width <= 0 || height <= 0) return -1;
  const long long bs = s2tc::block_bytes(dxt);
  long long n = 128;
  int w = width, h = height;
  for (;;) {
    n += (long long)((w + 3) / 4) * ((h + 3) / 4) * bs;
    if (w == 1 && h == 1) break;
    s2tc::mip_next(w, h);
  }
  return n;
}

// s2tc_compress (s2tc_compress.c:594-719) from its RGBA buffer on: the DDS
// header, then every mip level from the base to 1x1.  The levels are built on
// the device (one mip kernel per level), then each is compressed exactly as a
// tx_compress_dxtn call would (same kernels, libc rand() replayed per level in
// order, the leftover alpha endpoint carried from level to level), on one
// stream with a single synchronisation at the end.
int s2tc_compress_dds(const void* rgba, int width, int height, unsigned int format, const s2tc_options* opt, void* out,
                      long long out_size, long long* written) {
  using namespace s2tc;
  if (written) *written = 0;
  const int dxt = format_dxt(format);
  if (dxt < 0) {
    set_error("bad destination format");
    return S2TC_ERR_FORMAT;
  }
  if (!rgba || !out || width <= 0 || height <= 0 || width > 32768 || height > 32768) {
    set_error("bad argument");
    return S2TC_ERR_ARGUMENT;
  }
  const long long total = s2tc_dds_size(width, height, format);
  if (out_size < total) {
    set_error("output buffer smaller than s2tc_dds_size");
    return S2TC_ERR_ARGUMENT;
  }
  const s2tc_options o = normalise(opt ? *opt : read_env());
  const long long bs = block_bytes(dxt);
  // level sizes and offsets
  struct Level {
    int w, h;
    long long px_off, blk_off;
  };
  std::vector<Level> levels;
  long long px_total = 0, blk_total = 0;
  for (int w = width, h = height;;) {
    levels.push_back(Level{w, h, px_total, blk_total});
    px_total += ((long long)w * h * 4 + 15) & ~15ll;
    blk_total += (long long)((w + 3) / 4) * ((h + 3) / 4) * bs;
    if (w == 1 && h == 1) break;
    mip_next(w, h);
  }
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return S2TC_ERR_CUDA;
  cudaStream_t s = c.stream;
  if (!c.mips.reserve(size_t(px_total) + 16, "cudaMalloc(mip levels)")) return S2TC_ERR_NOMEM;
  if (!c.blocks.reserve(size_t(blk_total) + 16, "cudaMalloc(blocks)")) return S2TC_ERR_NOMEM;
  uint8_t* px = c.mips.as<uint8_t>();
  uint8_t* blk = c.blocks.as<uint8_t>();
  int* alpha_flag = c.err.as<int>() + 3;
  if (!cuda_ok(cudaStreamWaitEvent(s, c.arena_free, 0), "cudaStreamWaitEvent")) return S2TC_ERR_CUDA;
  if (!cuda_ok(cudaMemcpyAsync(px, rgba, size_t(width) * height * 4, cudaMemcpyHostToDevice, s), "input upload"))
    return S2TC_ERR_CUDA;
  if (!cuda_ok(cudaMemsetAsync(alpha_flag, 0, sizeof(int), s), "cudaMemsetAsync")) return S2TC_ERR_CUDA;
  if (!cuda_ok(launch_any_alpha(px, (long long)width * height, alpha_flag, s), "alpha test")) return S2TC_ERR_CUDA;
  for (size_t l = 1; l < levels.size(); ++l)
    if (!cuda_ok(launch_mip_reduce(px + levels[l - 1].px_off, levels[l - 1].w, levels[l - 1].h, px + levels[l].px_off,
                                   s),
                 "mip reduce"))
      return S2TC_ERR_CUDA;
  for (const Level& L : levels) {
    const int st = compress_device_locked(c, 4, L.w, L.h, px + L.px_off, dxt, blk + L.blk_off,
                                          (long long)((L.w + 3) / 4) * bs, o, nullptr, s, c.err.as<int>() + 2);
    if (st != ST_OK) return st;
  }
  unsigned char* o8 = static_cast<unsigned char*>(out);
  int alpha = 0;
  if (!cuda_ok(cudaMemcpyAsync(o8 + 128, blk, size_t(blk_total), cudaMemcpyDeviceToHost, s), "output download"))
    return S2TC_ERR_CUDA;
  if (!cuda_ok(cudaMemcpyAsync(&alpha, alpha_flag, sizeof(int), cudaMemcpyDeviceToHost, s), "flag download"))
    return S2TC_ERR_CUDA;
  const int st = check_error_flag(c, s);
  if (st != ST_OK) return st;
  // the header (s2tc_compress.c:662-707)
  auto put = [&](int off, uint32_t v) {
    for (int i = 0; i < 4; ++i) o8[off + i] = uint8_t(v >> (8 * i));
  };
  int mipcount = 0;
  while (width >= (1 << mipcount) || height >= (1 << mipcount)) ++mipcount;
  std::memset(o8, 0, 128);
  std::memcpy(o8, "DDS ", 4);
  put(4, 0x7c);
  put(8, 0x000a1007);
  put(12, uint32_t(height));
  put(16, uint32_t(width));
  put(20, uint32_t(((width + 3) / 4) * ((height + 3) / 4) * bs));
  put(28, uint32_t(mipcount));
  put(76, 0x20);
  put(80, alpha ? 5 : 4);
  std::memcpy(o8 + 84, dxt == s2tc::DXT1 ? "DXT1" : dxt == s2tc::DXT3 ? "DXT3" : "DXT5", 4);
  put(108, 0x00401008);
  if (written) *written = total;
  return S2TC_OK;
}

int s2tc_encode_layout_set(const s2tc_options* opt, unsigned int format, int threads, int rand_warps,
                           int rand_ctas_per_sm) {
  using namespace s2tc;
  const int dxt = format_dxt(format);
  if (dxt < 0 || !opt) return S2TC_ERR_ARGUMENT;
  if (threads < 32 || threads > 128 || rand_warps < 1 || rand_warps > 4 || rand_ctas_per_sm < 1) {
    set_error("layout out of range (threads 32..128, warps 1..4, CTAs per SM >= 1)");
    return S2TC_ERR_ARGUMENT;
  }
  const s2tc_options o = normalise(*opt);
  const bool normal = normal_mode(o);
  const int kind = normal ? (o.nrandom > 0 ? kLayoutRand : kLayoutFull) : kLayoutQuick;
  set_encode_layout(o.metric, dxt, o.refine, kind, EncodeLayout{threads & ~31, rand_warps, rand_ctas_per_sm});
  return S2TC_OK;
}

int s2tc_encode_layout_get(const s2tc_options* opt, unsigned int format, int* threads, int* rand_warps,
                           int* rand_ctas_per_sm) {
  using namespace s2tc;
  const int dxt = format_dxt(format);
  if (dxt < 0 || !opt) return S2TC_ERR_ARGUMENT;
  const s2tc_options o = normalise(*opt);
  const bool normal = normal_mode(o);
  const int kind = normal ? (o.nrandom > 0 ? kLayoutRand : kLayoutFull) : kLayoutQuick;
  const EncodeLayout L = encode_layout(o.metric, dxt, o.refine, kind);
  if (threads) *threads = L.threads;
  if (rand_warps) *rand_warps = L.rand_warps;
  if (rand_ctas_per_sm) *rand_ctas_per_sm = L.rand_ctas_per_sm;
  return S2TC_OK;
}

// Autotuner: times the candidate layouts of one mode's encoder launch on a
// synthetic image (texel words from a fixed xorshift stream, random-candidate
// words from the device generator started at a synthetic position, so that
// libc's rand() is not consumed) and keeps the fastest.
int s2tc_autotune(const s2tc_options* opt, unsigned int format, int width, int height, float* best_ms) {
  using namespace s2tc;
  const int dxt = format_dxt(format);
  if (dxt < 0 || !opt || width < 4 || height < 4) {
    set_error("bad argument");
    return S2TC_ERR_ARGUMENT;
  }
  const s2tc_options o = normalise(*opt);
  const bool normal = normal_mode(o);
  const int kind = normal ? (o.nrandom > 0 ? kLayoutRand : kLayoutFull) : kLayoutQuick;
  std::vector<EncodeLayout> cands;
  if (kind == kLayoutRand) {
    for (int wps : {1, 2, 4})
      for (int cps : {8, 16, 32, 64}) cands.push_back(EncodeLayout{128, wps, cps});
  } else {
    for (int th : {32, 64, 96, 128}) cands.push_back(EncodeLayout{th, 4, 64});
  }
  Context& c = ctx();
  std::lock_guard<std::mutex> lock(c.mu);
  if (!c.init()) return S2TC_ERR_CUDA;
  cudaStream_t s = c.stream;
  const long long npx = (long long)width * height;
  const int bw = (width + 3) / 4, bh = (height + 3) / 4;
  const long long pitch = (long long)bw * block_bytes(dxt);
  const long long words = (long long)bw * bh * rand_per_block(o, dxt);
  std::vector<uint32_t> host(static_cast<size_t>(npx));
  uint32_t x = 0x9E3779B9u;
  const uint32_t amask = dxt == s2tc::DXT1 ? 1u : dxt == s2tc::DXT3 ? 15u : 255u;
  for (long long i = 0; i < npx; ++i) {
    x ^= x << 13;
    x ^= x >> 17;
    x ^= x << 5;
    const long long px = i % width, py = i / width;
    const bool smooth = ((px / 64) + (py / 64)) & 1;  // half the image in smooth tiles
    const uint32_t r = smooth ? uint32_t((px / 8) & 31) : (x & 31), g = smooth ? uint32_t((py / 4) & 63) : ((x >> 5) & 63);
    const uint32_t b = smooth ? uint32_t(((px + py) / 16) & 31) : ((x >> 11) & 31);
    const uint32_t a = dxt == s2tc::DXT1 ? 1u : ((x >> 16) & amask);
    host[size_t(i)] = r | (g << 8) | (b << 16) | (a << 24);
  }
  DevBuf tex, dst, rnd, win;
  struct Free {
    DevBuf* b[4];
    ~Free() {
      for (DevBuf* d : b)
        if (d->p) cudaFree(d->p);
    }
  } cleanup{{&tex, &dst, &rnd, &win}};
  if (!tex.reserve(size_t(npx) * 4, "cudaMalloc(autotune texels)") ||
      !dst.reserve(size_t(pitch) * bh, "cudaMalloc(autotune blocks)"))
    return S2TC_ERR_NOMEM;
  if (!cuda_ok(cudaMemcpy(tex.p, host.data(), size_t(npx) * 4, cudaMemcpyHostToDevice), "autotune upload"))
    return S2TC_ERR_CUDA;
  if (words > 0) {
    RandWindow w;
    for (int i = 0; i < 61; ++i) {
      x ^= x << 13;
      x ^= x >> 17;
      x ^= x << 5;
      w.ext[i] = x;
    }
    if (!rnd.reserve(size_t(words) * 4, "cudaMalloc(autotune rand)") ||
        !win.reserve(sizeof(RandWindow), "cudaMalloc(autotune window)"))
      return S2TC_ERR_NOMEM;
    if (!cuda_ok(cudaMemcpy(win.p, &w, sizeof(w), cudaMemcpyHostToDevice), "autotune window") ||
        !cuda_ok(rand_fill(win.as<RandWindow>(), rnd.as<uint32_t>(), words, s), "autotune rand"))
      return S2TC_ERR_CUDA;
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (!cuda_ok(cudaEventCreate(&e0), "cudaEventCreate") || !cuda_ok(cudaEventCreate(&e1), "cudaEventCreate"))
    return S2TC_ERR_CUDA;
  float best = 0;
  EncodeLayout best_l = cands[0];
  int st = S2TC_OK;
  for (const EncodeLayout& L : cands) {
    set_encode_layout(o.metric, dxt, o.refine, kind, L);
    float ms = 0;
    for (int rep = 0; rep < 4 && st == S2TC_OK; ++rep) {
      if (rep == 1 && !cuda_ok(cudaEventRecord(e0, s), "cudaEventRecord")) st = S2TC_ERR_CUDA;
      if (st == S2TC_OK)
        st = encode_locked(c, tex.as<uint32_t>(), width, height, dxt, dst.as<uint8_t>(), pitch, o,
                           words > 0 ? rnd.as<uint32_t>() : nullptr, s, nullptr);
    }
    if (st == S2TC_OK && (!cuda_ok(cudaEventRecord(e1, s), "cudaEventRecord") ||
                          !cuda_ok(cudaEventSynchronize(e1), "cudaEventSynchronize") ||
                          !cuda_ok(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime")))
      st = S2TC_ERR_CUDA;
    if (st != S2TC_OK) break;
    ms /= 3;
    if (best == 0 || ms < best) {
      best = ms;
      best_l = L;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  set_encode_layout(o.metric, dxt, o.refine, kind, best_l);
  if (st == S2TC_OK) st = check_error_flag(c, s);
  if (best_ms) *best_ms = best;
  return st;
}

const char* s2tc_last_error(void) { return s2tc::g_last_error.c_str(); }

}  // extern "C"

namespace s2tc {

EncodeLayout encode_layout(int metric, int dxt, int refine, int kind) {
  if (!layout_key_ok(metric, dxt, refine, kind)) return EncodeLayout{128, 4, 64};
  LayoutTable& l = layouts();
  std::lock_guard<std::mutex> lock(l.mu);
  return l.t[metric][dxt][refine][kind];
}

void set_encode_layout(int metric, int dxt, int refine, int kind, EncodeLayout layout) {
  if (!layout_key_ok(metric, dxt, refine, kind)) return;
  LayoutTable& l = layouts();
  std::lock_guard<std::mutex> lock(l.mu);
  l.t[metric][dxt][refine][kind] = layout;
}

}  // namespace s2tc
