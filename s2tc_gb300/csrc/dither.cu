// dither.cu -- RGB8/RGBA8 -> 5:6:5 texel words with the reference's dither
// modes (s2tc_algorithm.cpp:1196-1465).
//
// DITHER_NONE is elementwise.  DITHER_SIMPLE is one serial error-diffusion
// chain per channel over the whole image in raster order; it is computed here
// as an exact single-pass scan over tiles of kTile texels, one CTA per tile
// (the scan itself is in dither_scan.cuh):
//   - the tile is read from HBM once, with coalesced vector loads, into shared
//     memory as one RGBA word per texel;
//   - thread t owns the kSeg consecutive texels starting at kSeg * t.  kSeg is
//     odd, so at every step the 32 lanes of a warp read 32 distinct banks;
//   - a channel's carried error takes few values (red/blue -7..7, green -3..3,
//     4-bit alpha -15..15), so the effect of a run of texels on it is a small
//     table "start state -> end state".  Each thread computes its segment's
//     table for all start states at once, four states per 32-bit word (one
//     byte each, see swar_step / swar_step4);
//   - tables compose with byte gathers (prmt): warps scan their lanes' tables
//     with shuffles, warp 0 scans the warps' aggregates, and tiles chain their
//     aggregates through a decoupled look-back in global memory;
//   - every thread then replays its segment from its exact start state and
//     overwrites its texels in shared memory with the 5:6:5 words, which the
//     CTA writes out with coalesced vector stores;
//   - the 1-bit alpha chain (diffuse1) is a rotation: its carried error after
//     k texels is ((sum of sources + 127) mod 255) - 127, so its "table" is a
//     sum mod 255.
// The look-back spins are bounded; on timeout the kernel records an error
// flag and finishes, and the host reports it.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "dither.h"
#include "dither_scan.cuh"

namespace s2tc {
namespace {

#ifndef S2TC_DITHER_THREADS
#define S2TC_DITHER_THREADS 256
#endif
constexpr int kThreads = S2TC_DITHER_THREADS;
constexpr int kSeg = 65;                // texels per thread (odd: conflict-free)
constexpr int kTile = kThreads * kSeg;  // 16640 texels per tile
using TileSmem = ScanSmem<kThreads, kSeg>;

// Image of global tile g: the last image whose first tile is <= g.
__device__ __forceinline__ int tile_item(const DitherWork& w, long long g) {
  if (!w.items) return 0;
  int lo = 0, hi = w.nitems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(w.tile_offsets + mid) <= g) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// DITHER_SIMPLE over every tile of every image of the work list.  Tiles take
// tickets in launch order, so a tile only ever waits on tiles that started
// before it.
#ifndef S2TC_DITHER_MINBLOCKS
#define S2TC_DITHER_MINBLOCKS 3
#endif
__global__ void __launch_bounds__(kThreads, S2TC_DITHER_MINBLOCKS) k_dither_simple(DitherWork w) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  TileSmem& sm = *reinterpret_cast<TileSmem*>(smem_raw);
  __shared__ unsigned int s_ticket;
  const int t = threadIdx.x;
  init_tables(sm);
  if (t == 0) s_ticket = atomicAdd(w.ticket, 1u);
  bulk_init(sm);
  __syncthreads();
  if ((long long)s_ticket >= w.total_tiles) return;
  const long long g = w.tile_base + s_ticket;
  const int item = tile_item(w, g);
  DitherItem it = w.single;
  if (w.items) it = w.items[item];
  const long long lt = w.items ? g - __ldg(w.tile_offsets + item) : g;
  const long long npx = (long long)it.width * it.height;
  const long long p0 = lt * kTile;
  const int n = int(min((long long)kTile, npx - p0));
  const uint8_t* tsrc = it.src + p0 * 4;
  if (it.srccomps == 4 && n == kTile && (reinterpret_cast<uintptr_t>(tsrc) & 15) == 0) {
    if (!bulk_load(sm, tsrc, uint32_t(kTile) * 4u)) {
      // The copy did not complete within the bounded wait.  The error flag
      // makes the whole call report S2TC_ERR_TIMEOUT, and its output is then
      // undefined; the tile still runs to the end (with the texels loaded
      // again by plain loads after a second bounded wait for the copy) so
      // that it publishes its scan state and the tiles behind it do not all
      // wait out their own limits.
      atomicExch(w.error, 1);
      bulk_load_wait(sm);
      load_tile<kThreads>(it, p0, n, sm.px);
    }
  } else {
    load_tile<kThreads>(it, p0, n, sm.px);
  }
  __syncthreads();
  if (it.srccomps == 3) simple_tile<0>(it.alphabits, lt, g, n, w, sm, sm.px);
  else if (it.alphabits == 1) simple_tile<1>(it.alphabits, lt, g, n, w, sm, sm.px);
  else if (it.alphabits == 4) simple_tile<4>(it.alphabits, lt, g, n, w, sm, sm.px);
  else simple_tile<8>(it.alphabits, lt, g, n, w, sm, sm.px);
  __syncthreads();
  store_tile<kThreads>(it.dst, p0, n, sm.px);
}

// DITHER_NONE (s2tc_algorithm.cpp:1269-1305): plain truncation, one tile per CTA.
__global__ void __launch_bounds__(kThreads) k_dither_none(DitherWork w) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  uint32_t* px = reinterpret_cast<uint32_t*>(smem_raw);
  if ((long long)blockIdx.x >= w.total_tiles) return;
  const long long g = w.tile_base + blockIdx.x;
  const int item = tile_item(w, g);
  DitherItem it = w.single;
  if (w.items) it = w.items[item];
  const long long npx = (long long)it.width * it.height;
  const long long p0 = (w.items ? g - __ldg(w.tile_offsets + item) : g) * kTile;
  const int n = int(min((long long)kTile, npx - p0));
  load_tile<kThreads>(it, p0, n, px);
  __syncthreads();
  const uint32_t ac = uint32_t((1 << it.alphabits) - 1);
  const int ash = 8 - it.alphabits;
  const bool rgb = it.srccomps == 3;
  for (int i = threadIdx.x; i < n; i += kThreads) {
    const uint32_t p = px[i];
    const uint32_t al = rgb ? ac : (p >> 24) >> ash;
    px[i] = ((p & 0xFFu) >> 3) | ((((p >> 8) & 0xFFu) >> 2) << 8) | ((((p >> 16) & 0xFFu) >> 3) << 16) | (al << 24);
  }
  __syncthreads();
  store_tile<kThreads>(it.dst, p0, n, px);
}

std::atomic<long long> g_launches{0};
std::atomic<long long> g_hold_tile{-1};
std::atomic<int> g_spin_limit{0};

cudaError_t set_smem(const void* fn, size_t bytes) {
  return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
}

}  // namespace

void count_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

void set_dither_test_hold(long long hold_tile, int spin_limit) {
  g_hold_tile.store(hold_tile < 0 ? -1 : hold_tile);
  g_spin_limit.store(spin_limit > 0 ? spin_limit : 0);
}

void dither_test_hold_values(long long* hold_tile, int* spin_limit) {
  *hold_tile = g_hold_tile.load();
  *spin_limit = g_spin_limit.load();
}
long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

long long dither_tile_texels() { return kTile; }

size_t dither_batch_scratch_bytes(long long tiles) {
  // status words, aggregate records, ticket (plus alignment slack)
  return size_t(tiles) * (sizeof(unsigned long long) + kRec) + 256;
}

size_t dither_scratch_bytes(long long npx) { return dither_batch_scratch_bytes((npx + kTile - 1) / kTile); }

namespace {

// Launches tiles [w.tile_base, w.tile_base + w.total_tiles) of a work list
// whose scan state (status words, aggregate records, ticket) is laid out in
// `scratch` for `all_tiles` tiles.
cudaError_t launch_tiles(DitherWork w, int dither, uint8_t* scratch, long long all_tiles, cudaStream_t s) {
  if (w.total_tiles <= 0) return cudaSuccess;
  // the attribute is set once per process (the first call on any device)
  static const cudaError_t attr = [] {
    cudaError_t e = set_smem(reinterpret_cast<const void*>(k_dither_simple), sizeof(TileSmem));
    if (e == cudaSuccess) e = set_smem(reinterpret_cast<const void*>(k_dither_none), kTile * sizeof(uint32_t));
    return e;
  }();
  if (attr != cudaSuccess) return attr;
  if (dither == DI_NONE) {
    count_launches(1);
    k_dither_none<<<unsigned(w.total_tiles), kThreads, kTile * sizeof(uint32_t), s>>>(w);
    return cudaGetLastError();
  }
  w.hold_tile = g_hold_tile.load();
  w.spin_limit = g_spin_limit.load();
  w.status = reinterpret_cast<unsigned long long*>(scratch);
  w.aggs = scratch + all_tiles * sizeof(unsigned long long);
  uintptr_t tk = reinterpret_cast<uintptr_t>(w.aggs + all_tiles * kRec);
  w.ticket = reinterpret_cast<unsigned int*>((tk + 15) & ~uintptr_t(15));
  cudaError_t e =
      cudaMemsetAsync(w.status + w.tile_base, 0, w.total_tiles * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(w.ticket, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  count_launches(1);
  k_dither_simple<<<unsigned(w.total_tiles), kThreads, sizeof(TileSmem), s>>>(w);
  return cudaGetLastError();
}

DitherWork single_work(DitherArgs a) {
  DitherWork w{};
  w.items = nullptr;
  w.tile_offsets = nullptr;
  w.nitems = 1;
  w.single = DitherItem{a.src, a.width, a.height, a.srccomps == 3 ? 3 : 4, a.alphabits, a.dst};
  w.error = a.error;
  return w;
}

}  // namespace

cudaError_t launch_dither_batch(DitherWork w, int dither, uint8_t* scratch, cudaStream_t s) {
  w.tile_base = 0;
  return launch_tiles(w, dither, scratch, w.total_tiles, s);
}

cudaError_t launch_dither_range(DitherArgs a, int dither, uint8_t* scratch, long long t0, long long t1,
                                cudaStream_t s) {
  const long long npx = (long long)a.width * a.height;
  if (npx <= 0 || t1 <= t0) return cudaSuccess;
  DitherWork w = single_work(a);
  w.tile_base = t0;
  w.total_tiles = t1 - t0;
  return launch_tiles(w, dither, scratch, (npx + kTile - 1) / kTile, s);
}

cudaError_t launch_dither(DitherArgs a, int dither, uint8_t* scratch, cudaStream_t s) {
  const long long npx = (long long)a.width * a.height;
  if (npx <= 0) return cudaSuccess;
  a.alpha_const = (1 << a.alphabits) - 1;
  if (dither == DI_FLOYDSTEINBERG) return launch_dither_fs(a, scratch, s);
  DitherWork w = single_work(a);
  w.total_tiles = (npx + kTile - 1) / kTile;
  return launch_dither_batch(w, dither, scratch, s);
}

}  // namespace s2tc
