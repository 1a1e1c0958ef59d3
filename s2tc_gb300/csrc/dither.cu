// dither.cu -- RGB8/RGBA8 -> 5:6:5 texel words with the reference's dither
// modes (s2tc_algorithm.cpp:1196-1465).
//
// DITHER_NONE is elementwise.  DITHER_SIMPLE is one serial error-diffusion
// chain per channel over the whole image in raster order; it is computed here
// as an exact single-pass scan:
//   - a channel's carried error takes few values (red/blue: -7..7, green:
//     -3..3, 4-bit alpha: -15..15), so the effect of a run of texels on it is a
//     small table state -> state; tables compose;
//   - each thread builds the table of its 64-texel segment, the CTA composes
//     them (Hillis-Steele in shared memory), tiles chain their aggregates with
//     a decoupled look-back, and every thread then replays its segment from
//     its exact start state;
//   - the 5- and 6-bit channels run all start states at once, four per 32-bit
//     word (one byte each): one texel step is then a handful of byte-parallel
//     adds and masks driven by constants that depend only on the source byte
//     (see swar_step);
//   - the 1-bit alpha chain (diffuse1) is a rotation: its carried error after
//     k texels is ((sum of sources + 127) mod 255) - 127, so its "table" is a
//     sum mod 255.
// The look-back spins are bounded; on timeout the kernel records an error
// flag and finishes, and the host reports it.
#include <cuda/atomic>
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "dither.h"

namespace s2tc {
namespace {

constexpr int kThreads = 256;
constexpr int kSeg = 64;  // texels per thread, contiguous in raster order
constexpr int kTile = kThreads * kSeg;

// Table layout (bytes) inside one 72-byte record: red 15 states at 0, green 7
// at 16, blue 15 at 24, alpha at 40 (31 states for 4-bit, or one byte holding
// the mod-255 sum for 1-bit).
constexpr int kOffR = 0, kOffG = 16, kOffB = 24, kOffA = 40;
constexpr int kRec = 72;

// One step of the 1-D error diffusion (s2tc_algorithm.cpp:1198-1207).
template <int SHIFT>
__device__ __forceinline__ int qstep(int& d, int src) {
  constexpr int maxv = (1 << (8 - SHIFT)) - 1;
  const int v = src + d;
  const int q = min(max(v >> SHIFT, 0), maxv);
  d = v - ((q << SHIFT) | (q >> (8 - 2 * SHIFT)));
  return q;
}

template <int SHIFT>
struct QChan {
  static constexpr int kOff = (1 << SHIFT) - 1;  // largest carried error
  static constexpr int kStates = 2 * kOff + 1;
};

__device__ __forceinline__ int chan_of(uint32_t px, int c) { return int((px >> (8 * c)) & 0xFF); }

// Table of one channel over the thread's segment: entry s is the end state
// when the segment starts in state s.
template <int SHIFT>
__device__ __forceinline__ void seg_table(const uint32_t* px, int nvalid, int c, uint8_t* out) {
  using Q = QChan<SHIFT>;
#pragma unroll 1
  for (int s = 0; s < Q::kStates; ++s) {
    int d = s - Q::kOff;
#pragma unroll
    for (int k = 0; k < kSeg; ++k)
      if (k < nvalid) qstep<SHIFT>(d, chan_of(px[k], c));
    out[s] = uint8_t(d + Q::kOff);
  }
}

// dst = apply `first`, then `second`.
template <int AK>
__device__ __forceinline__ void compose(const uint8_t* first, const uint8_t* second, uint8_t* dst) {
#pragma unroll 1
  for (int s = 0; s < QChan<3>::kStates; ++s) {
    dst[kOffR + s] = second[kOffR + first[kOffR + s]];
    dst[kOffB + s] = second[kOffB + first[kOffB + s]];
  }
#pragma unroll 1
  for (int s = 0; s < QChan<2>::kStates; ++s) dst[kOffG + s] = second[kOffG + first[kOffG + s]];
  if (AK == 4) {
#pragma unroll 1
    for (int s = 0; s < QChan<4>::kStates; ++s) dst[kOffA + s] = second[kOffA + first[kOffA + s]];
  } else if (AK == 1) {
    dst[kOffA] = uint8_t((first[kOffA] + second[kOffA]) % 255);
  }
}

// Apply a table record to packed start states (r | g<<8 | b<<16 | a<<24).
template <int AK>
__device__ __forceinline__ uint32_t apply(const uint8_t* t, uint32_t st) {
  uint32_t r = t[kOffR + (st & 0xFF)];
  uint32_t g = t[kOffG + ((st >> 8) & 0xFF)];
  uint32_t b = t[kOffB + ((st >> 16) & 0xFF)];
  uint32_t a = 0;
  if (AK == 4) a = t[kOffA + (st >> 24)];
  if (AK == 1) a = ((st >> 24) + t[kOffA]) % 255;
  return r | (g << 8) | (b << 16) | (a << 24);
}

template <int AK>
__device__ __forceinline__ uint32_t initial_state() {
  // zero carried error in every chain
  return uint32_t(QChan<3>::kOff) | (uint32_t(QChan<2>::kOff) << 8) | (uint32_t(QChan<3>::kOff) << 16) |
         (uint32_t(AK == 4 ? QChan<4>::kOff : AK == 1 ? 127 : 0) << 24);
}

template <int AK>
__device__ __forceinline__ void identity(uint8_t* t) {
  for (int s = 0; s < QChan<3>::kStates; ++s) t[kOffR + s] = t[kOffB + s] = uint8_t(s);
  for (int s = 0; s < QChan<2>::kStates; ++s) t[kOffG + s] = uint8_t(s);
  if (AK == 4)
    for (int s = 0; s < QChan<4>::kStates; ++s) t[kOffA + s] = uint8_t(s);
  if (AK == 1) t[kOffA] = 0;
}

// ---------------------------------------------------------------- SWAR step
// For a channel quantised with shift k (k = 3: 5 bits, k = 2: 6 bits) let
// E = 2^k - 1 be the largest carried error, e = d + E in [0, 2E] the state and
// src = 2^k q + r.  With t = r + e and s = src + d = 2^k q + t - E, qstep gives
//   e' = ((t + 1) mod 2^k) + E - base - [t >= T]           (0 <= s <= 255)
// where base = (2^k q - E) >> (8 - k) and T = 2^(8-k) (base + 1) - (2^k q - E)
// (the window of t values is narrower than 2^(8-k), so s >> (8 - k) takes at
// most two values), e' = t when s < 0 (q = 0, t < E) and e' = t - E when
// s > 255 (q = maxv, t > 2E).  Both clamps are the middle formula plus or
// minus 2^k + 1, selected by [t >= T].  Every byte of a word holds one state
// biased by 16, so no lane ever borrows from its neighbour, and one step is
//   t = ub + rm; m = (t + 1) & E; g = ((t + 128 - T) >> 7) & 1; ub' = g*j1 + m + bc
// with per-source-byte constants rm, kk = 128 - T, bc, j1 (SwarConst).

struct SwarConst {
  uint32_t rm, kk, bc, j1;
};

template <int K>
__device__ __forceinline__ uint4 swar_const(int src) {
  constexpr int E = (1 << K) - 1, maxv = 255 >> K;
  const int r = src & E, q = src >> K;
  const int base = ((1 << K) * q - E) >> (8 - K);
  const int T = (1 << (8 - K)) * (base + 1) - ((1 << K) * q - E);
  const int L = q == 0 ? (1 << K) + 1 : 0, H = q == maxv ? (1 << K) + 1 : 0;
  return make_uint4(uint32_t(r) * 0x01010101u - 0x10101010u, uint32_t(128 - T) * 0x01010101u,
                    uint32_t(16 + E - base - L) * 0x01010101u, uint32_t(H + L - 1));
}

template <int K>
__device__ __forceinline__ uint32_t swar_step(uint32_t ub, const uint4& c) {
  constexpr uint32_t MASK = uint32_t((1 << K) - 1) * 0x01010101u;
  const uint32_t t = ub + c.x;
  const uint32_t m = (t + 0x01010101u) & MASK;
  const uint32_t g = ((t + c.y) >> 7) & 0x01010101u;
  return g * c.w + (m + c.z);
}

// Unpack SWAR words (states biased by 16) into a byte table.
__device__ __forceinline__ void swar_store(const uint32_t* w, int nstates, uint8_t* out) {
  for (int s = 0; s < nstates; ++s) out[s] = uint8_t(((w[s >> 2] >> (8 * (s & 3))) & 0xFF) - 16);
}

using Status = cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>;
constexpr unsigned long long kAggReady = 1ull << 32;
constexpr unsigned long long kIncReady = 2ull << 32;
constexpr int kSpinLimit = 1 << 22;

// Texel k (0..3) of a group of four, as an RGBA word, from raw words `w`
// (four texels = 16 bytes for RGBA, 12 bytes for RGB).
template <int SC>
__device__ __forceinline__ uint32_t texel_of(const uint32_t* w, int k) {
  if (SC == 4) return w[k];
  const int b0 = 3 * k;
  const uint64_t pair = uint64_t(w[b0 >> 2]) | (uint64_t(w[min((b0 >> 2) + 1, 2)]) << 32);
  return uint32_t(pair >> (8 * (b0 & 3))) & 0xFFFFFFu;
}

// Four texels [p, p + 4) of the image as RGBA words (alpha 0 for RGB input);
// texels at or beyond npx read as 0 and must not be used.
template <int SC>
__device__ __forceinline__ void load4(const uint8_t* __restrict__ src, long long p, long long npx, uint32_t* px) {
  const uint8_t* s = src + p * SC;
  if (p + 4 <= npx && (reinterpret_cast<uintptr_t>(s) & 3) == 0) {
    uint32_t w[4];
    const uint32_t* v = reinterpret_cast<const uint32_t*>(s);
#pragma unroll
    for (int i = 0; i < SC; ++i) w[i] = __ldg(v + i);
#pragma unroll
    for (int k = 0; k < 4; ++k) px[k] = texel_of<SC>(w, k);
  } else {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      uint32_t v = 0;
      if (p + k < npx) {
        const uint8_t* t = s + k * SC;
        v = uint32_t(t[0]) | (uint32_t(t[1]) << 8) | (uint32_t(t[2]) << 16);
        if (SC == 4) v |= uint32_t(t[3]) << 24;
      }
      px[k] = v;
    }
  }
}

// Shared memory of one SIMPLE-dither tile.
struct TileSmem {
  uint8_t tbl[2][kThreads][kRec];
  uint4 c3[256], c2[256];
  uint32_t carry;
};

// One SIMPLE-dither tile: texels [tile_in_image * kTile, +kTile) of `it`,
// chained through the status words `status[tile - tile_in_image ...]`.
// `g` is the tile's global index (status / aggregate slot).
template <int SC, int AK>
__device__ __forceinline__ void simple_tile(const DitherItem& it, long long tile_in_image, long long g,
                                            const DitherWork& w, TileSmem& sm) {
  const int t = threadIdx.x;
  const long long npx = (long long)it.width * it.height;
  const long long p0 = tile_in_image * kTile + (long long)t * kSeg;
  const int nvalid = int(max(0ll, min((long long)kSeg, npx - p0)));
  const int alpha_const = (1 << it.alphabits) - 1;

  // segment tables: all start states at once, four per word
  uint32_t wr[4] = {0x13121110u, 0x17161514u, 0x1B1A1918u, 0x171E1D1Cu};  // red states 0..14 (+pad)
  uint32_t wb[4] = {0x13121110u, 0x17161514u, 0x1B1A1918u, 0x171E1D1Cu};  // blue
  uint32_t wg[2] = {0x13121110u, 0x13161514u};                            // green states 0..6 (+pad)
  int asum = 0;
  uint8_t* mine = sm.tbl[0][t];
  if (AK == 4) {
    for (int s = 0; s < QChan<4>::kStates; ++s) mine[kOffA + s] = uint8_t(s);
  }
  for (int k0 = 0; k0 < nvalid; k0 += 4) {
    uint32_t px[4];
    load4<SC>(it.src, p0 + k0, npx, px);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (k0 + k < nvalid) {
        const uint32_t p = px[k];
        const uint4 cr = sm.c3[p & 0xFF], cg = sm.c2[(p >> 8) & 0xFF], cb = sm.c3[(p >> 16) & 0xFF];
#pragma unroll
        for (int i = 0; i < 4; ++i) wr[i] = swar_step<3>(wr[i], cr);
#pragma unroll
        for (int i = 0; i < 2; ++i) wg[i] = swar_step<2>(wg[i], cg);
#pragma unroll
        for (int i = 0; i < 4; ++i) wb[i] = swar_step<3>(wb[i], cb);
        if (AK == 1) asum += int(p >> 24);
        if (AK == 4) {
          // 4-bit alpha: 31 states, stepped one by one
          const int src = int(p >> 24);
          for (int s = 0; s < QChan<4>::kStates; ++s) {
            int d = int(mine[kOffA + s]) - QChan<4>::kOff;
            qstep<4>(d, src);
            mine[kOffA + s] = uint8_t(d + QChan<4>::kOff);
          }
        }
      }
    }
  }
  swar_store(wr, QChan<3>::kStates, mine + kOffR);
  swar_store(wg, QChan<2>::kStates, mine + kOffG);
  swar_store(wb, QChan<3>::kStates, mine + kOffB);
  if (AK == 1) mine[kOffA] = uint8_t(asum % 255);
  __syncthreads();

  // inclusive scan of the tables across the CTA
  int cur = 0;
  for (int off = 1; off < kThreads; off <<= 1) {
    if (t >= off) compose<AK>(sm.tbl[cur][t - off], sm.tbl[cur][t], sm.tbl[cur ^ 1][t]);
    else
      for (int i = 0; i < kRec; ++i) sm.tbl[cur ^ 1][t][i] = sm.tbl[cur][t][i];
    __syncthreads();
    cur ^= 1;
  }

  // chain the image's tiles: publish, look back, publish the inclusive state
  if (t == 0) {
    const uint8_t* agg = sm.tbl[cur][kThreads - 1];
    Status st(w.status[g]);
    uint32_t carry = initial_state<AK>();
    if (tile_in_image == 0) {
      st.store(kIncReady | apply<AK>(agg, carry), cuda::memory_order_release);
    } else {
      uint8_t* gagg = w.aggs + g * kRec;
      for (int i = 0; i < kRec; ++i) gagg[i] = agg[i];
      st.store(kAggReady, cuda::memory_order_release);
      // acc: state at the end of tile k -> state at the start of this tile;
      // the image's first tile always publishes its inclusive state, so the
      // walk never leaves the image
      uint8_t acc[kRec];
      identity<AK>(acc);
      long long k = g - 1;
      for (;;) {
        Status sk(w.status[k]);
        unsigned long long v = sk.load(cuda::memory_order_acquire);
        int spins = 0;
        while ((v >> 32) == 0 && spins < kSpinLimit) {
          __nanosleep(64);
          v = sk.load(cuda::memory_order_acquire);
          ++spins;
        }
        if ((v >> 32) == 0) {
          atomicExch(w.error, 1);
          break;
        }
        if ((v >> 32) == 2) {
          carry = apply<AK>(acc, uint32_t(v));
          break;
        }
        // acc := agg[k] then acc
        uint8_t tmp[kRec];
        compose<AK>(w.aggs + k * kRec, acc, tmp);
        for (int i = 0; i < kRec; ++i) acc[i] = tmp[i];
        --k;
      }
      st.store(kIncReady | apply<AK>(agg, carry), cuda::memory_order_release);
    }
    sm.carry = carry;
  }
  __syncthreads();

  // replay the segment from its exact start state
  const uint32_t start = t == 0 ? sm.carry : apply<AK>(sm.tbl[cur][t - 1], sm.carry);
  int dr = int(start & 0xFF) - QChan<3>::kOff;
  int dg = int((start >> 8) & 0xFF) - QChan<2>::kOff;
  int db = int((start >> 16) & 0xFF) - QChan<3>::kOff;
  int da = AK == 4 ? int(start >> 24) - QChan<4>::kOff : int(start >> 24) - 127;
  uint32_t* o = it.dst + p0;
  for (int k0 = 0; k0 < nvalid; k0 += 4) {
    uint32_t px[4], out[4];
    load4<SC>(it.src, p0 + k0, npx, px);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint32_t p = px[k];
      uint32_t q = uint32_t(qstep<3>(dr, chan_of(p, 0))) | (uint32_t(qstep<2>(dg, chan_of(p, 1))) << 8) |
                   (uint32_t(qstep<3>(db, chan_of(p, 2))) << 16);
      uint32_t qa;
      if (AK == 4) {
        qa = uint32_t(qstep<4>(da, chan_of(p, 3)));
      } else if (AK == 1) {
        // diffuse1 (s2tc_algorithm.cpp:1208-1216)
        const int v = chan_of(p, 3) + da;
        qa = v >= 128;
        da = v - (qa ? 255 : 0);
      } else if (AK == 8) {
        qa = uint32_t(chan_of(p, 3));
      } else {
        qa = uint32_t(alpha_const);
      }
      out[k] = q | (qa << 24);
    }
    if (k0 + 4 <= nvalid && (reinterpret_cast<uintptr_t>(o + k0) & 15) == 0) {
      *reinterpret_cast<uint4*>(o + k0) = make_uint4(out[0], out[1], out[2], out[3]);
    } else {
      for (int k = 0; k < min(4, nvalid - k0); ++k) o[k0 + k] = out[k];
    }
  }
}

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
__global__ void __launch_bounds__(kThreads) k_dither_simple(DitherWork w) {
  __shared__ TileSmem sm;
  __shared__ unsigned int s_ticket;
  const int t = threadIdx.x;
  sm.c3[t] = swar_const<3>(t);
  sm.c2[t] = swar_const<2>(t);
  if (t == 0) s_ticket = atomicAdd(w.ticket, 1u);
  __syncthreads();
  const long long g = s_ticket;
  if (g >= w.total_tiles) return;
  const int item = tile_item(w, g);
  const DitherItem it = w.items ? w.items[item] : w.single;
  const long long lt = w.items ? g - __ldg(w.tile_offsets + item) : g;
  if (it.srccomps == 3) simple_tile<3, 0>(it, lt, g, w, sm);
  else if (it.alphabits == 1) simple_tile<4, 1>(it, lt, g, w, sm);
  else if (it.alphabits == 4) simple_tile<4, 4>(it, lt, g, w, sm);
  else simple_tile<4, 8>(it, lt, g, w, sm);
}

// DITHER_NONE (s2tc_algorithm.cpp:1269-1305): plain truncation, one tile per CTA.
__global__ void __launch_bounds__(kThreads) k_dither_none(DitherWork w) {
  const long long g = blockIdx.x;
  if (g >= w.total_tiles) return;
  const int item = tile_item(w, g);
  const DitherItem it = w.items ? w.items[item] : w.single;
  const long long npx = (long long)it.width * it.height;
  const long long base = (w.items ? g - __ldg(w.tile_offsets + item) : g) * kTile;
  const int sc = it.srccomps == 3 ? 3 : 4;
  const uint32_t ac = uint32_t((1 << it.alphabits) - 1);
  for (long long p = base + threadIdx.x; p < min(npx, base + kTile); p += kThreads) {
    const uint8_t* s = it.src + p * sc;
    const uint32_t r = s[0] >> 3, gg = s[1] >> 2, b = s[2] >> 3;
    const uint32_t al = sc == 4 ? uint32_t(s[3] >> (8 - it.alphabits)) : ac;
    it.dst[p] = r | (gg << 8) | (b << 16) | (al << 24);
  }
}

std::atomic<long long> g_launches{0};

}  // namespace

void count_launches(int n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
long long launches_so_far() { return g_launches.load(std::memory_order_relaxed); }

long long dither_tile_texels() { return kTile; }

size_t dither_batch_scratch_bytes(long long tiles) {
  // status words, aggregate tables, ticket (plus alignment slack)
  return size_t(tiles) * (sizeof(unsigned long long) + kRec) + 256;
}

size_t dither_scratch_bytes(long long npx) { return dither_batch_scratch_bytes((npx + kTile - 1) / kTile); }

cudaError_t launch_dither_batch(DitherWork w, int dither, uint8_t* scratch, cudaStream_t s) {
  if (w.total_tiles <= 0) return cudaSuccess;
  if (dither == DI_NONE) {
    count_launches(1);
    k_dither_none<<<unsigned(w.total_tiles), kThreads, 0, s>>>(w);
    return cudaGetLastError();
  }
  w.status = reinterpret_cast<unsigned long long*>(scratch);
  w.aggs = scratch + w.total_tiles * sizeof(unsigned long long);
  uintptr_t tk = reinterpret_cast<uintptr_t>(w.aggs + w.total_tiles * kRec);
  w.ticket = reinterpret_cast<unsigned int*>((tk + 15) & ~uintptr_t(15));
  cudaError_t e = cudaMemsetAsync(w.status, 0, w.total_tiles * sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  e = cudaMemsetAsync(w.ticket, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  count_launches(1);
  k_dither_simple<<<unsigned(w.total_tiles), kThreads, 0, s>>>(w);
  return cudaGetLastError();
}

cudaError_t launch_dither(DitherArgs a, int dither, uint8_t* scratch, cudaStream_t s) {
  const long long npx = (long long)a.width * a.height;
  if (npx <= 0) return cudaSuccess;
  a.alpha_const = (1 << a.alphabits) - 1;
  if (dither == DI_FLOYDSTEINBERG) return launch_dither_fs(a, scratch, s);
  DitherWork w{};
  w.items = nullptr;
  w.tile_offsets = nullptr;
  w.nitems = 1;
  w.single = DitherItem{a.src, a.width, a.height, a.srccomps == 3 ? 3 : 4, a.alphabits, a.dst};
  w.total_tiles = (npx + kTile - 1) / kTile;
  w.error = a.error;
  return launch_dither_batch(w, dither, scratch, s);
}

}  // namespace s2tc
