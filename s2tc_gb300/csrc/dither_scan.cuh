// dither_scan.cuh -- device side of the exact SIMPLE-dither scan
// (s2tc_algorithm.cpp:1196-1216, 1306-1348), shared by the dither kernels
// (dither.cu) and the fused strip kernel of the quick encoder (encode.cu).
//
// DITHER_SIMPLE is one serial error-diffusion chain per channel over the whole
// image in raster order; it is computed as an exact single-pass scan over
// tiles of texels, one CTA per tile:
//   - the tile is read from HBM once into shared memory as one RGBA word per
//     texel;
//   - thread t owns the SEG consecutive texels starting at SEG * t.  SEG is
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
//     overwrites its texels in shared memory with the 5:6:5 words;
//   - the 1-bit alpha chain (diffuse1) is a rotation: its carried error after
//     k texels is ((sum of sources + 127) mod 255) - 127, so its "table" is a
//     sum mod 255.
// The look-back spins are bounded; on timeout the kernel records an error
// flag and finishes, and the host reports it.
#pragma once
#include <cuda/atomic>
#include <cuda_runtime.h>

#include <cstdint>

#include "dither.h"

namespace s2tc {
namespace {

constexpr int kRecWords = 18;           // red 4, green 2, blue 4, alpha 8 words
constexpr int kRec = 4 * kRecWords;     // bytes per aggregate record in global memory

// ------------------------------------------------------------ scalar steps

// One step of the 1-D error diffusion (s2tc_algorithm.cpp:1198-1207).
template <int SHIFT>
__device__ __forceinline__ int qstep(int& d, int src) {
  constexpr int maxv = (1 << (8 - SHIFT)) - 1;
  const int v = src + d;
  const int q = min(max(v >> SHIFT, 0), maxv);
  d = v - ((q << SHIFT) | (q >> (8 - 2 * SHIFT)));
  return q;
}

// ------------------------------------------------------------- SWAR steps
// For a channel quantised with shift k (k = 3: 5 bits, k = 2: 6 bits) let
// E = 2^k - 1 be the largest carried error, e = d + E in [0, 2E] the state and
// src = 2^k q + r.  With t = r + e and s = src + d = 2^k q + t - E, qstep gives
//   e' = ((t + 1) mod 2^k) + E - base - [t >= T]           (0 <= s <= 255)
// where base = (2^k q - E) >> (8 - k) and T = 2^(8-k) (base + 1) - (2^k q - E)
// (the window of t values is narrower than 2^(8-k), so s >> (8 - k) takes at
// most two values), e' = t when s < 0 (q = 0, t < E) and e' = t - E when
// s > 255 (q = maxv, t > 2E).  Both clamps are the middle formula plus or
// minus 2^k + 1, selected by [t >= T].  Every byte of a word holds one state
// biased by 16, so no lane ever borrows from its neighbour.  With
// t1 = ub + r - 15 (per byte) one step is
//   m = t1 & E;  g = ((t1 + 127 - T) >> 7) & 1;  ub' = g*j1 + m + (16 + E - base - L)
// where L = 2^k + 1 for q = 0 (else 0), H likewise for q = maxv and
// j1 = H + L - 1.  The q-dependent constants live in a shared table of one
// word per q: byte 0 = 127 - T, byte 1 = 16 + E - base - L, byte 3 = j1.
template <int K>
__host__ __device__ __forceinline__ uint32_t swar_table_word(int q) {
  constexpr int E = (1 << K) - 1, maxv = 255 >> K;
  const int base = ((1 << K) * q - E) >> (8 - K);
  const int T = (1 << (8 - K)) * (base + 1) - ((1 << K) * q - E);
  const int L = q == 0 ? (1 << K) + 1 : 0, H = q == maxv ? (1 << K) + 1 : 0;
  return uint32_t(127 - T) | (uint32_t(16 + E - base - L) << 8) | (uint32_t(H + L - 1) << 24);
}

struct SwarC {
  uint32_t rm1, kk1, bc;
  int j1;
};

template <int K>
__device__ __forceinline__ SwarC swar_c(int src, const uint32_t* tab) {
  constexpr uint32_t E = (1u << K) - 1;
  const uint32_t tw = tab[src >> K];
  SwarC c;
  c.rm1 = (uint32_t(src) & E) * 0x01010101u - 0x0F0F0F0Fu;
  c.kk1 = __byte_perm(tw, 0, 0x0000);
  c.bc = __byte_perm(tw, 0, 0x1111);
  c.j1 = int(tw) >> 24;
  return c;
}

template <int K>
__device__ __forceinline__ uint32_t swar_step(uint32_t ub, const SwarC& c) {
  constexpr uint32_t MASK = ((1u << K) - 1) * 0x01010101u;
  const uint32_t t1 = ub + c.rm1;
  const uint32_t m = t1 & MASK;
  const uint32_t g = ((t1 + c.kk1) >> 7) & 0x01010101u;
  return g * uint32_t(c.j1) + (m + c.bc);
}

// 4-bit alpha (k = 4, 31 states): t = e + r takes up to 46 values, so
// s >> 4 takes up to three.  With src = 16 Q + r and states biased by 16,
//   e' = t + A - 17 ([t >= 15] m15 + [t >= 31] m31)
// where A = 17 - Q (0 for Q = 0, 2 for Q = 15), m15 = [Q > 0], m31 = [Q < 15]
// (the clamps at Q = 0 and Q = 15 drop one of the two corrections).  Shared
// table word per Q: byte 0 = A, byte 1 = m15, byte 2 = m31.
__host__ __device__ __forceinline__ uint32_t swar4_table_word(int Q) {
  const int A = Q == 15 ? 2 : Q == 0 ? 0 : 17 - Q;
  return uint32_t(A) | (uint32_t(Q > 0) << 8) | (uint32_t(Q < 15) << 16);
}

struct Swar4C {
  uint32_t r, a, m15, m31;
};

__device__ __forceinline__ Swar4C swar4_c(int src, const uint32_t* tab) {
  const uint32_t tw = tab[src >> 4];
  Swar4C c;
  c.r = (uint32_t(src) & 15u) * 0x01010101u;
  c.a = __byte_perm(tw, 0, 0x0000);
  c.m15 = __byte_perm(tw, 0, 0x1111);
  c.m31 = __byte_perm(tw, 0, 0x2222);
  return c;
}

__device__ __forceinline__ uint32_t swar_step4(uint32_t u, const Swar4C& c) {
  const uint32_t t = u + c.r;
  const uint32_t g15 = ((t + 0x61616161u) >> 7) & c.m15;  // 128 - 15 - 16 = 97
  const uint32_t g31 = ((t + 0x51515151u) >> 7) & c.m31;  // 128 - 31 - 16 = 81
  return (t + c.a) - 17u * (g15 + g31);
}

// ------------------------------------------------------------------ records
// The end state of each chain for every start state, one byte per state
// (states unbiased: red/blue 0..14, green 0..6, 4-bit alpha 0..30; the last
// byte of each channel is a padding state that always holds a valid state).
// For the 1-bit alpha chain a[0] is the sum of sources mod 255.
struct Rec {
  uint32_t r[4], g[2], b[4], a[8];
};

template <int AK>
__device__ __forceinline__ void rec_identity(Rec& x) {
  x.r[0] = x.b[0] = 0x03020100u;
  x.r[1] = x.b[1] = 0x07060504u;
  x.r[2] = x.b[2] = 0x0B0A0908u;
  x.r[3] = x.b[3] = 0x070E0D0Cu;
  x.g[0] = 0x03020100u;
  x.g[1] = 0x03060504u;
  if (AK == 4) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x.a[i] = 0x03020100u + 0x04040404u * uint32_t(i);
    x.a[7] = 0x0F1E1D1Cu;
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) x.a[i] = 0;
  }
}

// prmt selector from the low three bits of four byte indices.
__device__ __forceinline__ uint32_t sel3(uint32_t idx) {
  const uint32_t x = idx & 0x07070707u;
  return __byte_perm(x | (x >> 4), 0, 0x0020);
}

__device__ __forceinline__ uint32_t bytemask(uint32_t idx, int bit) {
  return ((idx >> bit) & 0x01010101u) * 0xFFu;
}

// g[idx[i]] for four byte indices below 8, 16 or 32.
__device__ __forceinline__ uint32_t gather8(const uint32_t* g, uint32_t idx) {
  return __byte_perm(g[0], g[1], sel3(idx));
}
__device__ __forceinline__ uint32_t gather16(const uint32_t* g, uint32_t idx) {
  const uint32_t s = sel3(idx);
  const uint32_t lo = __byte_perm(g[0], g[1], s), hi = __byte_perm(g[2], g[3], s);
  const uint32_t m = bytemask(idx, 3);
  return (hi & m) | (lo & ~m);
}
__device__ __forceinline__ uint32_t gather32(const uint32_t* g, uint32_t idx) {
  const uint32_t s = sel3(idx);
  const uint32_t p0 = __byte_perm(g[0], g[1], s), p1 = __byte_perm(g[2], g[3], s);
  const uint32_t p2 = __byte_perm(g[4], g[5], s), p3 = __byte_perm(g[6], g[7], s);
  const uint32_t m3 = bytemask(idx, 3), m4 = bytemask(idx, 4);
  const uint32_t lo = (p1 & m3) | (p0 & ~m3), hi = (p3 & m3) | (p2 & ~m3);
  return (hi & m4) | (lo & ~m4);
}

// out = `first`, then `second`.
template <int AK>
__device__ __forceinline__ Rec compose(const Rec& first, const Rec& second) {
  Rec o;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    o.r[i] = gather16(second.r, first.r[i]);
    o.b[i] = gather16(second.b, first.b[i]);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) o.g[i] = gather8(second.g, first.g[i]);
  if (AK == 4) {
#pragma unroll
    for (int i = 0; i < 8; ++i) o.a[i] = gather32(second.a, first.a[i]);
  } else if (AK == 1) {
    o.a[0] = (first.a[0] + second.a[0]) % 255u;
#pragma unroll
    for (int i = 1; i < 8; ++i) o.a[i] = 0;
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) o.a[i] = 0;
  }
  return o;
}

// Packed chain states: r | g << 8 | b << 16 | a << 24 (alpha: 4-bit state, or
// (carried error + 127) for the 1-bit chain).
template <int AK>
__device__ __forceinline__ uint32_t apply(const Rec& t, uint32_t st) {
  const uint32_t r = gather16(t.r, st & 0xFFu) & 0xFFu;
  const uint32_t g = gather8(t.g, (st >> 8) & 0xFFu) & 0xFFu;
  const uint32_t b = gather16(t.b, (st >> 16) & 0xFFu) & 0xFFu;
  uint32_t a = 0;
  if (AK == 4) a = gather32(t.a, st >> 24) & 0xFFu;
  if (AK == 1) a = ((st >> 24) + t.a[0]) % 255u;
  return r | (g << 8) | (b << 16) | (a << 24);
}

template <int AK>
__device__ __forceinline__ uint32_t initial_state() {
  // zero carried error in every chain
  return 7u | (3u << 8) | (7u << 16) | (uint32_t(AK == 4 ? 15 : AK == 1 ? 127 : 0) << 24);
}

template <int AK>
__device__ __forceinline__ Rec shfl_up_rec(const Rec& x, int d) {
  Rec o;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    o.r[i] = __shfl_up_sync(0xFFFFFFFFu, x.r[i], d);
    o.b[i] = __shfl_up_sync(0xFFFFFFFFu, x.b[i], d);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) o.g[i] = __shfl_up_sync(0xFFFFFFFFu, x.g[i], d);
  if (AK == 4) {
#pragma unroll
    for (int i = 0; i < 8; ++i) o.a[i] = __shfl_up_sync(0xFFFFFFFFu, x.a[i], d);
  } else if (AK == 1) {
    o.a[0] = __shfl_up_sync(0xFFFFFFFFu, x.a[0], d);
  }
  return o;
}

__device__ __forceinline__ void rec_store(uint32_t* p, const Rec& x) {
#pragma unroll
  for (int i = 0; i < 4; ++i) p[i] = x.r[i];
#pragma unroll
  for (int i = 0; i < 2; ++i) p[4 + i] = x.g[i];
#pragma unroll
  for (int i = 0; i < 4; ++i) p[6 + i] = x.b[i];
#pragma unroll
  for (int i = 0; i < 8; ++i) p[10 + i] = x.a[i];
}

__device__ __forceinline__ Rec rec_load(const uint32_t* p) {
  Rec x;
#pragma unroll
  for (int i = 0; i < 4; ++i) x.r[i] = p[i];
#pragma unroll
  for (int i = 0; i < 2; ++i) x.g[i] = p[4 + i];
#pragma unroll
  for (int i = 0; i < 4; ++i) x.b[i] = p[6 + i];
#pragma unroll
  for (int i = 0; i < 8; ++i) x.a[i] = p[10 + i];
  return x;
}

// Global aggregate records are read after an acquire of their status word;
// L2 loads (no L1) keep them coherent.
__device__ __forceinline__ Rec rec_load_global(const uint32_t* p) {
  Rec x;
#pragma unroll
  for (int i = 0; i < 4; ++i) x.r[i] = __ldcg(p + i);
#pragma unroll
  for (int i = 0; i < 2; ++i) x.g[i] = __ldcg(p + 4 + i);
#pragma unroll
  for (int i = 0; i < 4; ++i) x.b[i] = __ldcg(p + 6 + i);
#pragma unroll
  for (int i = 0; i < 8; ++i) x.a[i] = __ldcg(p + 10 + i);
  return x;
}

// --------------------------------------------------------------- tile I/O

// Shared memory of a tile of THREADS threads with SEG texels each (SEG odd:
// at every step the 32 lanes of a warp read 32 distinct banks).  `pad` words
// in front of the texels let a tile start anywhere within a 256-texel row of
// a two-dimensional tensor copy (see the fused strip kernel).
template <int THREADS, int SEG, int PAD = 0>
struct ScanSmem {
  static constexpr int kThreads = THREADS, kWarps = THREADS / 32, kSeg = SEG, kTile = THREADS * SEG;
  alignas(128) uint32_t px[PAD + kTile];  // RGBA words in, 5:6:5 words out
  uint32_t tab3[32], tab2[64], tab4[16];
  uint32_t wagg[kWarps][kRecWords];  // warps' inclusive records
  uint32_t wstart[kWarps];           // warps' start states
  uint32_t lb[32][kRecWords + 1];     // look-back window: aggregates of 32 earlier tiles
  alignas(8) unsigned long long mbar;  // completion of the tile's bulk copy
};

// The SWAR constant tables, by the CTA's first threads (before a barrier).
template <class SM>
__device__ __forceinline__ void init_tables(SM& sm) {
  const int t = threadIdx.x;
  if (t < 32) sm.tab3[t] = swar_table_word<3>(t);
  if (t < 64) sm.tab2[t] = swar_table_word<2>(t);
  if (t < 16) sm.tab4[t] = swar4_table_word(t);
}

// ------------------------------------------------ bulk copy (TMA) of a tile
// A whole RGBA8 tile is contiguous in global memory (kTile * 4 bytes): one
// thread starts bulk copies of it into shared memory (cp.async.bulk, the TMA
// unit's non-tensor form) that signal an mbarrier with their byte count, and
// every thread waits on that barrier.  Both addresses must be 16-byte aligned
// and each size a multiple of 16; callers check.  The waits are bounded: on
// timeout the error flag is set and the tile is loaded with ordinary loads.
constexpr int kBulkChunk = 16384;  // bytes per bulk copy
constexpr int kBulkSpins = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(mbar), "r"(parity)
      : "memory");
  return done != 0;
}

// Thread 0 initialises the barrier; call before a __syncthreads.
template <class SM>
__device__ __forceinline__ void bulk_init(SM& sm) {
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&sm.mbar)) : "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
}

// A second bounded wait for the barrier's phase (after a timeout).
template <class SM>
__device__ __forceinline__ void bulk_load_wait(SM& sm) {
  const uint32_t mbar = smem_u32(&sm.mbar);
  int spins = 0;
  while (!mbar_try_wait(mbar, 0) && ++spins < kBulkSpins) {
  }
}

// Copies `bytes` (a multiple of 16) from `src` into sm.px; every thread
// returns once the data is in shared memory.  Returns false on timeout.
template <class SM>
__device__ bool bulk_load(SM& sm, const uint8_t* src, uint32_t bytes) {
  const uint32_t mbar = smem_u32(&sm.mbar);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
    const uint32_t dst = smem_u32(sm.px);
    for (uint32_t off = 0; off < bytes; off += kBulkChunk) {
      const uint32_t n = bytes - off < uint32_t(kBulkChunk) ? bytes - off : uint32_t(kBulkChunk);
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst + off),
          "l"(src + off), "r"(n), "r"(mbar)
          : "memory");
    }
  }
  int spins = 0;
  while (!mbar_try_wait(mbar, 0) && ++spins < kBulkSpins) {
  }
  return spins < kBulkSpins;
}

// Texels [p0, p0 + n) of `it` into px[0, n) as RGBA words (alpha 0 for RGB),
// by the CTA's THREADS threads.
template <int THREADS>
__device__ __forceinline__ void load_tile(const DitherItem& it, long long p0, int n, uint32_t* px) {
  constexpr int kThreads = THREADS;
  const int t = threadIdx.x;
  if (it.srccomps == 4) {
    const uint8_t* s = it.src + p0 * 4;
    int done = 0;
    if ((reinterpret_cast<uintptr_t>(s) & 15) == 0) {
      const uint4* v = reinterpret_cast<const uint4*>(s);
      for (int i = t; i < (n >> 2); i += kThreads) reinterpret_cast<uint4*>(px)[i] = __ldg(v + i);
      done = n & ~3;
    } else if ((reinterpret_cast<uintptr_t>(s) & 3) == 0) {
      const uint32_t* v = reinterpret_cast<const uint32_t*>(s);
      for (int i = t; i < n; i += kThreads) px[i] = __ldg(v + i);
      done = n;
    }
    for (int i = done + t; i < n; i += kThreads) {
      const uint8_t* b = s + 4 * i;
      px[i] = uint32_t(b[0]) | (uint32_t(b[1]) << 8) | (uint32_t(b[2]) << 16) | (uint32_t(b[3]) << 24);
    }
  } else {
    const uint8_t* s = it.src + p0 * 3;
    int done = 0;
    if ((reinterpret_cast<uintptr_t>(s) & 3) == 0) {
      // four texels = three words
      const uint32_t* v = reinterpret_cast<const uint32_t*>(s);
      for (int i = t; i < (n >> 2); i += kThreads) {
        const uint32_t w0 = __ldg(v + 3 * i), w1 = __ldg(v + 3 * i + 1), w2 = __ldg(v + 3 * i + 2);
        reinterpret_cast<uint4*>(px)[i] =
            make_uint4(w0 & 0xFFFFFFu, __funnelshift_r(w0, w1, 24) & 0xFFFFFFu,
                       __funnelshift_r(w1, w2, 16) & 0xFFFFFFu, w2 >> 8);
      }
      done = n & ~3;
    }
    for (int i = done + t; i < n; i += kThreads) {
      const uint8_t* b = s + 3 * i;
      px[i] = uint32_t(b[0]) | (uint32_t(b[1]) << 8) | (uint32_t(b[2]) << 16);
    }
  }
}

// px[0, n) out to dst[p0, p0 + n).
template <int THREADS>
__device__ __forceinline__ void store_tile(uint32_t* dst, long long p0, int n, const uint32_t* px) {
  constexpr int kThreads = THREADS;
  const int t = threadIdx.x;
  uint32_t* d = dst + p0;
  int done = 0;
  if ((reinterpret_cast<uintptr_t>(d) & 15) == 0) {
    for (int i = t; i < (n >> 2); i += kThreads)
      reinterpret_cast<uint4*>(d)[i] = reinterpret_cast<const uint4*>(px)[i];
    done = n & ~3;
  }
  for (int i = done + t; i < n; i += kThreads) d[i] = px[i];
}

using Status = cuda::atomic_ref<unsigned long long, cuda::thread_scope_device>;
constexpr unsigned long long kAggReady = 1ull << 32;
constexpr unsigned long long kIncReady = 2ull << 32;
constexpr int kSpinLimit = 1 << 22;

// The state at the start of tile g of an image whose tile within the image
// is `lt`, given the tile's aggregate; publishes the tile's own records.
// The tile's start state, by one warp.  The tile publishes its aggregate,
// then its lanes read the status words of the 32 tiles before it at once: the
// nearest one that has published its end state ("inclusive") ends the walk,
// and the aggregates of the tiles between it and this one are applied to that
// state in order.  A window without any end state (only aggregates) is
// composed into one record and the walk moves 32 tiles further back.  The
// image's first tile publishes its end state without looking back, so the
// walk never leaves the image.  Finally the tile publishes its own end state.
template <int AK, class SM>
__device__ uint32_t look_back(const DitherWork& w, long long g, long long lt, const Rec& agg, SM& sm) {
  const int lane = threadIdx.x & 31;
  Status st(w.status[g]);
  const bool publish = g != w.hold_tile;  // false only under the test hook
  const int spin_limit = w.spin_limit > 0 ? w.spin_limit : kSpinLimit;
  if (lt == 0) {
    const uint32_t carry = initial_state<AK>();
    if (lane == 0 && publish) st.store(kIncReady | apply<AK>(agg, carry), cuda::memory_order_release);
    return carry;
  }
  if (lane == 0 && publish) {
    rec_store(reinterpret_cast<uint32_t*>(w.aggs + g * kRec), agg);
    st.store(kAggReady, cuda::memory_order_release);
  }
  const long long first = g - lt;  // the image's first tile
  Rec acc;                          // the tiles after the current window, up to g - 1 (lane 0)
  rec_identity<AK>(acc);
  uint32_t carry = initial_state<AK>();
  for (long long top = g - 1;; top -= 32) {
    const long long k = top - lane;
    const bool valid = k >= first;
    unsigned long long v = 0;
    if (valid) {
      Status sk(w.status[k]);
      v = sk.load(cuda::memory_order_acquire);
      int spins = 0;
      while ((v >> 32) == 0 && spins < spin_limit) {
        __nanosleep(64);
        v = sk.load(cuda::memory_order_acquire);
        ++spins;
      }
    }
    if (__any_sync(0xFFFFFFFFu, valid && (v >> 32) == 0)) {
      if (lane == 0) atomicExch(w.error, 1);
      break;
    }
    const unsigned inc = __ballot_sync(0xFFFFFFFFu, valid && (v >> 32) == 2);
    const int nagg = inc ? __ffs(int(inc)) - 1 : 32;  // lanes 0 .. nagg-1 hold aggregates
    if (lane < nagg) rec_store(sm.lb[lane], rec_load_global(reinterpret_cast<const uint32_t*>(w.aggs + k * kRec)));
    __syncwarp();
    if (inc) {
      uint32_t s = __shfl_sync(0xFFFFFFFFu, uint32_t(v), nagg);  // end state of tile top - nagg
      if (lane == 0) {
        for (int j = nagg - 1; j >= 0; --j) s = apply<AK>(rec_load(sm.lb[j]), s);
        s = apply<AK>(acc, s);
      }
      carry = __shfl_sync(0xFFFFFFFFu, s, 0);
      break;
    }
    if (lane == 0) {
      // the window's tiles in order (top - 31 .. top), then the later ones
      Rec win = rec_load(sm.lb[31]);
      for (int j = 30; j >= 0; --j) win = compose<AK>(win, rec_load(sm.lb[j]));
      acc = compose<AK>(win, acc);
    }
    __syncwarp();
  }
  if (lane == 0 && publish) st.store(kIncReady | apply<AK>(agg, carry), cuda::memory_order_release);
  return carry;
}

// One SIMPLE-dither tile: the n texels at `base` (RGBA words in shared
// memory, the tile's texels in raster order), the tile's local index `lt`
// within its image (0: the image's first tile), chained through the status
// words; `g` is the tile's global index.  On return `base` holds the tile's
// 5:6:5 words.
template <int AK, class SM>
__device__ __forceinline__ void simple_tile(int alphabits, long long lt, long long g, int n, const DitherWork& w,
                                            SM& sm, uint32_t* base) {
  constexpr int kSeg = SM::kSeg, kWarps = SM::kWarps;
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const int k0 = t * kSeg;
  const int cnt = max(0, min(kSeg, n - k0));
  const uint32_t* px = base + k0;

  // the segment's records, all start states at once (states biased by 16)
  Rec x;
  x.r[0] = x.b[0] = 0x13121110u;
  x.r[1] = x.b[1] = 0x17161514u;
  x.r[2] = x.b[2] = 0x1B1A1918u;
  x.r[3] = x.b[3] = 0x171E1D1Cu;
  x.g[0] = 0x13121110u;
  x.g[1] = 0x13161514u;
#pragma unroll
  for (int i = 0; i < 8; ++i) x.a[i] = AK == 4 ? 0x13121110u + 0x04040404u * uint32_t(i) : 0u;
  if (AK == 4) x.a[7] = 0x1F2E2D2Cu;
  uint32_t asum = 0;
#pragma unroll 1
  for (int k = 0; k < cnt; ++k) {
    const uint32_t p = px[k];
    const SwarC cr = swar_c<3>(int(p & 0xFFu), sm.tab3);
    const SwarC cg = swar_c<2>(int((p >> 8) & 0xFFu), sm.tab2);
    const SwarC cb = swar_c<3>(int((p >> 16) & 0xFFu), sm.tab3);
#pragma unroll
    for (int i = 0; i < 4; ++i) x.r[i] = swar_step<3>(x.r[i], cr);
#pragma unroll
    for (int i = 0; i < 2; ++i) x.g[i] = swar_step<2>(x.g[i], cg);
#pragma unroll
    for (int i = 0; i < 4; ++i) x.b[i] = swar_step<3>(x.b[i], cb);
    if (AK == 1) asum += p >> 24;
    if (AK == 4) {
      const Swar4C ca = swar4_c(int(p >> 24), sm.tab4);
#pragma unroll
      for (int i = 0; i < 8; ++i) x.a[i] = swar_step4(x.a[i], ca);
    }
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    x.r[i] -= 0x10101010u;
    x.b[i] -= 0x10101010u;
  }
#pragma unroll
  for (int i = 0; i < 2; ++i) x.g[i] -= 0x10101010u;
  if (AK == 4) {
#pragma unroll
    for (int i = 0; i < 8; ++i) x.a[i] -= 0x10101010u;
  }
  if (AK == 1) x.a[0] = asum % 255u;

  // inclusive scan over the warp's lanes
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const Rec o = shfl_up_rec<AK>(x, d);
    if (lane >= d) x = compose<AK>(o, x);
  }
  if (lane == 31) rec_store(sm.wagg[warp], x);
  __syncthreads();

  // warp 0: scan the warps' records, chain the tile, start state of each warp
  if (warp == 0) {
    Rec y;
    if (lane < kWarps) y = rec_load(sm.wagg[lane]);
    else rec_identity<AK>(y);
#pragma unroll
    for (int d = 1; d < kWarps; d <<= 1) {
      const Rec o = shfl_up_rec<AK>(y, d);
      if (lane >= d) y = compose<AK>(o, y);
    }
    // tile aggregate = lane kWarps-1's inclusive record
    Rec agg;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      agg.r[i] = __shfl_sync(0xFFFFFFFFu, y.r[i], kWarps - 1);
      agg.b[i] = __shfl_sync(0xFFFFFFFFu, y.b[i], kWarps - 1);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) agg.g[i] = __shfl_sync(0xFFFFFFFFu, y.g[i], kWarps - 1);
#pragma unroll
    for (int i = 0; i < 8; ++i) agg.a[i] = __shfl_sync(0xFFFFFFFFu, y.a[i], kWarps - 1);
    const uint32_t carry = look_back<AK>(w, g, lt, agg, sm);
    // start of warp l = end of warp l-1
    const uint32_t end = apply<AK>(y, carry);
    const uint32_t start = __shfl_up_sync(0xFFFFFFFFu, end, 1);
    if (lane < kWarps) sm.wstart[lane] = lane == 0 ? carry : start;
  }
  __syncthreads();

  // the lane's start state: end of the previous lane
  const uint32_t ws = sm.wstart[warp];
  const uint32_t end = apply<AK>(x, ws);
  uint32_t st = __shfl_up_sync(0xFFFFFFFFu, end, 1);
  if (lane == 0) st = ws;

  // replay the segment from its exact start state, in place
  int dr = int(st & 0xFFu) - 7;
  int dg = int((st >> 8) & 0xFFu) - 3;
  int db = int((st >> 16) & 0xFFu) - 7;
  int da = AK == 4 ? int(st >> 24) - 15 : int(st >> 24) - 127;
  const uint32_t alpha_const = uint32_t((1 << alphabits) - 1);
  uint32_t* o = base + k0;
#pragma unroll 1
  for (int k = 0; k < cnt; ++k) {
    const uint32_t p = o[k];
    uint32_t q = uint32_t(qstep<3>(dr, int(p & 0xFFu))) | (uint32_t(qstep<2>(dg, int((p >> 8) & 0xFFu))) << 8) |
                 (uint32_t(qstep<3>(db, int((p >> 16) & 0xFFu))) << 16);
    uint32_t qa;
    if (AK == 4) {
      qa = uint32_t(qstep<4>(da, int(p >> 24)));
    } else if (AK == 1) {
      // diffuse1 (s2tc_algorithm.cpp:1208-1216)
      const int v = int(p >> 24) + da;
      qa = v >= 128;
      da = v - (qa ? 255 : 0);
    } else if (AK == 8) {
      qa = p >> 24;
    } else {
      qa = alpha_const;
    }
    o[k] = q | (qa << 24);
  }
}

}  // namespace
}  // namespace s2tc
