// dither_fs.cu -- DITHER_FLOYDSTEINBERG (s2tc_algorithm.cpp:1218-1261,
// 1350-1411) as a wavefront of warps.
//
// Texel (x, y) needs the error of (x-1, y) and of (x-1..x+1, y-1), so row y can
// run two texels behind row y-1.  Rows are cut into strips of 32, and one warp
// runs one channel of one strip, one lane per row: at step t lane r handles
// x = t - 2r.  Each lane keeps the errors it sends to the row below in a
// two-entry window; the entry for x-1 is complete once texel x has sent its
// 3/16 share, and one warp shuffle per step hands it to the lane below, which
// needs it one step later.  The three colour channels are independent chains,
// so a strip's red, green and blue run as three warps of one CTA; they drop
// their 5/6/5-bit values into a shared ring of texel words that the CTA writes
// out every 32 steps.  Source texels arrive by asynchronous copies into
// shared memory two groups of eight steps ahead.
//
// A strip's last lane hands the errors it sends below to lane 0 of the next
// strip.  Strips run as clusters of eight CTAs: inside a cluster the entries
// go straight into the next CTA's shared memory (a ring of 64-bit words, value
// and position, so that a stale or unwritten slot is recognised; the reader
// tells the writer how far it has read, which keeps the writer from lapping
// it).  Between clusters they go through carry rows in global memory (tagged
// words: value plus a bias, zero meaning "not written yet", read two groups
// ahead).  No fences are needed: every entry is checked on its own; every
// wait is bounded.  Clusters take tickets in launch order, so a strip only
// waits on a strip that is already running.  No lane ever branches on its
// own: loads are clamped into the image, stores are predicated, and every
// wait is taken by the whole warp.
//
// 1- and 4-bit alpha runs as a second launch, one single-warp CTA per strip.
// Like the reference, it starts from what the red pass left in its first
// error row (s2tc_algorithm.cpp:1354, 1380-1382): the red errors of the last
// row when its index is even, else the red errors it sent below.  The red
// warp of the last strip writes that row, tagged, as the alpha pass's first
// carry row.
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "dither.h"

namespace s2tc {
namespace {

constexpr int kLanes = 32;           // rows per strip
constexpr int kLag = 2;              // steps each row runs behind the row above
constexpr int kGroup = 8;            // steps per group
constexpr int kStages = 3;           // register stages: loads run kStages-1 groups ahead
constexpr int kWindow = 32;          // steps between writes of the texel ring
constexpr int kRing = 2 * kWindow;   // texels per row in the ring
// words per ring row: lane r touches word r * stride + ((t - kLag * r) & 63) at
// step t, so stride - kLag must be odd for the 32 lanes to hit 32 banks
constexpr int kRingStride = kRing + 1;
static_assert((kRingStride - kLag) % 2 == 1 && kLag % 2 == 0, "ring banks, texel pairs");
constexpr int kCluster = 8;          // strips per cluster (their hand-overs stay on chip)
constexpr int kCarryLen = 256;       // carry ring entries per channel (a power of two)
constexpr int kSpinLimit = 1 << 22;  // polls of one carry entry
constexpr int kTagBias = 0x40000000; // global carry word = value + bias; 0 = not written

// How a warp fetches its source texels: RGBA8 rows read with asynchronous
// copies into shared memory (8-byte pairs when every row start is 8-byte
// aligned, else 4-byte words), or (RGB8, unaligned RGBA8) byte loads into
// registers.  Shared memory per warp: kStages slots of kSlotWords words per
// lane (12, so that four-word reads of eight lanes hit distinct banks).
enum LoadMode { kLoadPairs, kLoadWords, kLoadBytes };
constexpr int kSlotWords = 12;
constexpr int kStageWords = kLanes * kSlotWords;
constexpr int kWarpStageWords = kStages * kStageWords;
static_assert(kGroup == 8, "a slot holds one group");
static_assert(kCarryLen >= 8 * kGroup && (kCarryLen & (kCarryLen - 1)) == 0, "carry ring");

// q * 4095 / maxv for q in [0, maxv] as one multiply and shift by 16.
__host__ __device__ constexpr int loop_mul(int maxv) { return maxv == 31 ? 8657095 : (4095 / maxv) << 16; }
constexpr bool loop_exact(int maxv) {
  for (int q = 0; q <= maxv; ++q)
    if (((q * loop_mul(maxv)) >> 16) != q * 4095 / maxv) return false;
  return true;
}
static_assert(loop_exact(31) && loop_exact(63) && loop_exact(15), "loop multipliers");
static_assert(kWindow % kGroup == 0, "window of whole groups");

// A channel's quantiser: q = clamp(v >> (shift + 4), 0, maxv) on 12-bit values,
// or the 1-bit variant (maxv 1).
struct Quant {
  int shift, maxv, mul;
};

__device__ __forceinline__ int widen12(uint32_t b) { return int((b << 4) | (b >> 4)); }

struct FsOut {
  int q, e7, e3, e5, e1;
};

// One Floyd-Steinberg step on 12-bit values (s2tc_algorithm.cpp:1218-1261);
// BIT1 is the 1-bit variant (:1241).  `v` is the source byte widened to 12
// bits, (s << 4) | (s >> 4), plus the error that reached the texel.  The error
// shares are zero when `act` is false.
template <bool BIT1>
__device__ __forceinline__ FsOut fs_step(int v, bool act, const Quant& qt) {
  FsOut o;
  int loop;
  if (BIT1) {
    o.q = v >= 2048;
    loop = o.q ? 4095 : 0;
  } else {
    o.q = min(max(v >> (qt.shift + 4), 0), qt.maxv);
    loop = (o.q * qt.mul) >> 16;
  }
  int e = act ? v - loop : 0;
  o.e7 = (e * 7 + 8) / 16;
  e -= o.e7;
  o.e3 = (e * 3 + 4) / 9;
  e -= o.e3;
  o.e5 = (e * 5 + 3) / 6;
  o.e1 = e - o.e5;
  return o;
}

// ---------------------------------------------------------------- memory ops

// Stores v (tagged) at p when `on`; one predicated store, no branch.
__device__ __forceinline__ void st_tagged_if(bool on, int* p, int v) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %2, 0;\n\t@p st.relaxed.gpu.global.b32 [%0], %1;\n\t}" ::"l"(p),
      "r"(v + kTagBias), "r"(int(on)));
}

__device__ __forceinline__ int ld_poll(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void cp_async(uint32_t* sdst, const uint8_t* gsrc, int bytes8) {
  const uint32_t s = smem_addr(sdst);
  const size_t g = __cvta_generic_to_global(gsrc);
  if (bytes8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(s), "l"(g) : "memory");
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(s), "l"(g) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

// Every thread of every CTA of the cluster.
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// The shared::cluster address of `p` (a shared variable) in CTA `rank`.
__device__ __forceinline__ uint32_t map_rank(const void* p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_addr(p)), "r"(rank));
  return r;
}

__device__ __forceinline__ void st_cluster_u64_if(bool on, uint32_t addr, uint64_t v) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %2, 0;\n\t@p st.relaxed.cluster.shared::cluster.b64 [%0], %1;\n\t}" ::"r"(
          addr),
      "l"(v), "r"(int(on))
      : "memory");
}

__device__ __forceinline__ void st_cluster_u32_if(bool on, uint32_t addr, uint32_t v) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %2, 0;\n\t@p st.relaxed.cluster.shared::cluster.b32 [%0], %1;\n\t}" ::"r"(
          addr),
      "r"(v), "r"(int(on))
      : "memory");
}

__device__ __forceinline__ uint64_t ld_local_u64(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.volatile.shared.b64 %0, [%1];" : "=l"(v) : "r"(smem_addr(p)) : "memory");
  return v;
}

__device__ __forceinline__ uint32_t ld_local_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.volatile.shared.b32 %0, [%1];" : "=r"(v) : "r"(smem_addr(p)) : "memory");
  return v;
}

// ------------------------------------------------------------------- strips

struct FsArgs {
  const uint8_t* src;
  uint32_t* dst;
  int width, height;
  int nstrips;
  int wpad;             // carry row length, width rounded up to a whole group
  int* carry;           // carry rows between clusters: the first strip of cluster k, channel c,
                        // reads row k * channels + c (row 0: the alpha pass's seed, else unused)
  int* leftover;        // colour pass followed by an alpha pass: the alpha pass's first carry row
  int seeded;           // alpha pass: strip 0 reads its carry row (the red leftover)
  int dst8;             // 8-byte aligned destination
  unsigned int* ticket;
  int* error;
};

// A CTA's carry rings, one per channel, written by the CTA before it in the
// cluster; prog[c] is how far this CTA's successor has read what this CTA
// writes to it (written by the successor).
template <int NCH>
struct CarrySmem {
  uint64_t ring[NCH][kCarryLen];
  uint32_t prog[NCH];
  uint32_t ticket;
};

enum CarryIn { kInNone, kInRow, kInRing };
enum CarryOut { kOutNone, kOutRow, kOutRing };

// One channel of one strip, one lane per row, reading source byte `srcb`
// (3 for alpha) of SC-byte texels, fetched as LM says.
template <bool BIT1, int SC, int LM>
struct Chan {
  Quant qt;
  int srcb;
  int lane, w;
  bool row_ok;
  int wpad_end;            // last aligned group start inside a carry row
  const uint8_t* srow;
  int* error;
  // carry input
  int in_mode;
  const int* cin;          // global row (kInRow)
  const uint64_t* rin;     // this CTA's ring for the channel (kInRing)
  uint32_t prog_up;        // the predecessor's progress word for the channel (kInRing)
  // carry output
  int out_mode;
  int* emit;               // global row (kOutRow)
  uint32_t rout;           // the successor's ring for the channel (kOutRing)
  const uint32_t* prog;    // how far the successor has read (kOutRing)
  int emit_lane;
  bool emit_err;           // write the texel's own error at x (red leftover of an even last row)

  uint32_t* slot;                 // this lane's stage-0 slot (asynchronous copies)
  uint32_t inb[LM == kLoadBytes ? kStages : 1][kGroup];  // source texels of kStages groups (byte loads)
  uint32_t cur[kGroup];           // source texels of the group at hand (SC 4: whole words)
  int cinb[kStages][kGroup];      // carry entries (lane 0; 0 elsewhere)
  int e7p;                  // 7/16 share of the previous texel
  int dq;                   // complete down-going error from the row above for x
  int wa, wb;               // down-going errors of this row for x-1, x
  int q[kGroup];            // quantised values of the group

  template <int NCH>
  __device__ __forceinline__ void setup(const FsArgs& a, int strip, int rank, int ch, bool red_leftover, Quant qv,
                                        int sb, uint32_t* stage_buf, CarrySmem<NCH>& cs) {
    qt = qv;
    srcb = sb;
    w = a.width;
    error = a.error;
    wpad_end = a.wpad - kGroup;
    lane = threadIdx.x & 31;
    const int y = strip * kLanes + lane;
    row_ok = y < a.height;
    srow = a.src + size_t(row_ok ? y : 0) * w * SC;
    slot = stage_buf + lane * kSlotWords;
    in_mode = strip == 0 && !a.seeded ? kInNone : rank > 0 ? kInRing : kInRow;
    cin = a.carry + (size_t(strip / kCluster) * NCH + ch) * a.wpad;
    rin = cs.ring[ch];
    prog_up = rank > 0 ? map_rank(&cs.prog[ch], rank - 1) : 0;
    out_mode = kOutNone;
    emit = nullptr;
    rout = 0;
    prog = &cs.prog[ch];
    emit_lane = -1;
    emit_err = false;
    if (strip + 1 < a.nstrips) {
      emit_lane = kLanes - 1;
      if (rank + 1 < kCluster) {
        out_mode = kOutRing;
        rout = map_rank(&cs.ring[ch][0], rank + 1);
      } else {
        out_mode = kOutRow;
        emit = a.carry + (size_t((strip + 1) / kCluster) * NCH + ch) * a.wpad;
      }
    } else if (red_leftover) {
      out_mode = kOutRow;
      emit = a.leftover;
      emit_lane = a.height - 1 - strip * kLanes;
      emit_err = ((a.height - 1) & 1) == 0;
    }
    e7p = dq = wa = wb = 0;
#pragma unroll
    for (int st = 0; st < kStages; ++st)
#pragma unroll
      for (int k = 0; k < kGroup; ++k) cinb[st][k] = 0;
#pragma unroll
    for (int st = 0; st + 1 < kStages; ++st) {
      load_src(st, st);
      load_cin(st, st);
    }
  }

  // Source texels of group g into stage st.  The fetches are unconditional
  // (x clamped into the row; rows past the image read row 0) so that no lane
  // branches around them: a texel outside the image only feeds a step that
  // does nothing.  Asynchronous copies form one commit group per group.
  __device__ __forceinline__ void load_src(int st, int g) {
    const int x0 = g * kGroup - kLag * lane;
    if (LM == kLoadPairs) {
#pragma unroll
      for (int h = 0; h < kGroup / 2; ++h)
        cp_async(slot + st * kStageWords + 2 * h, srow + size_t(min(max(x0 + 2 * h, 0), w - 2)) * 4, 1);
      cp_async_commit();
    } else if (LM == kLoadWords) {
#pragma unroll
      for (int k = 0; k < kGroup; ++k)
        cp_async(slot + st * kStageWords + k, srow + size_t(min(max(x0 + k, 0), w - 1)) * 4, 0);
      cp_async_commit();
    } else if (SC == 4) {
#pragma unroll
      for (int k = 0; k < kGroup; ++k) {
        const uint8_t* p = srow + size_t(min(max(x0 + k, 0), w - 1)) * 4;
        inb[st][k] = uint32_t(__ldg(p)) | (uint32_t(__ldg(p + 1)) << 8) | (uint32_t(__ldg(p + 2)) << 16) |
                     (uint32_t(__ldg(p + 3)) << 24);
      }
    } else {
#pragma unroll
      for (int k = 0; k < kGroup; ++k) inb[st][k] = __ldg(srow + size_t(min(max(x0 + k, 0), w - 1)) * 3 + srcb);
    }
  }

  __device__ __forceinline__ int src_byte(uint32_t v) const { return SC == 4 ? int((v >> (8 * srcb)) & 0xFF) : int(v); }

  // Global carry words of group g into stage st.  All lanes load the same
  // words (one broadcast transaction) so that the warp never splits; only
  // lane 0 keeps them once their tags are checked.  Past the row's end the
  // words are clamped into the carry row and never used.
  __device__ __forceinline__ void load_cin(int st, int g) {
    if (in_mode != kInRow) return;
    const int x0 = min(g * kGroup, wpad_end);
#pragma unroll
    for (int h = 0; h < kGroup / 4; ++h) {
      const int4 v = __ldcg(reinterpret_cast<const int4*>(cin + x0 + 4 * h));
      cinb[st][4 * h] = v.x;
      cinb[st][4 * h + 1] = v.y;
      cinb[st][4 * h + 2] = v.z;
      cinb[st][4 * h + 3] = v.w;
    }
  }

  __device__ __forceinline__ bool cin_ready(int st, int g) const {
    const int need = min(kGroup, w - g * kGroup);
    bool ok = true;
#pragma unroll
    for (int k = 0; k < kGroup; ++k) ok &= cinb[st][k] != 0 || k >= need;
    return ok;
  }

  // Group g's carry entries (lane 0; zero for every other lane and past the
  // row's end) into stage CS.  The branches are warp-uniform.
  //  * global row: the words were loaded kStages-1 groups ahead.  A group
  //    that is not there yet means the later prefetches are stale as well, so
  //    the wait runs until the writer is kStages-1 groups further on and then
  //    reloads every stage: that lag keeps later prefetches from coming back
  //    empty.
  //  * ring: read now (shared memory is close); a slot is ready once it holds
  //    this position.  The reader then publishes how far it has read.
  template <int CS>
  __device__ __forceinline__ void take_cin(int g) {
    const int x0 = g * kGroup;
    if (in_mode == kInRow) {
      if (x0 < w && !cin_ready(CS, g)) {
        const int* pw = cin + min(x0 + kStages * kGroup - 1, w - 1);  // last entry of group g+kStages-1
        int spins = 0;
        while (ld_poll(pw) == 0 && ++spins < kSpinLimit)
          if ((spins & 255) == 0 && ld_poll(error)) break;
        spins = 0;
        do {
#pragma unroll
          for (int i = 0; i < kStages; ++i) load_cin((CS + i) % kStages, g + i);
        } while (!cin_ready(CS, g) && ++spins < 64 && !ld_poll(error));
        if (!cin_ready(CS, g) && lane == 0) atomicExch(error, 1);
      }
#pragma unroll
      for (int k = 0; k < kGroup; ++k)
        cinb[CS][k] = lane == 0 && x0 + k < w && cinb[CS][k] ? cinb[CS][k] - kTagBias : 0;
    } else if (in_mode == kInRing) {
      if (x0 >= w) {
#pragma unroll
        for (int k = 0; k < kGroup; ++k) cinb[CS][k] = 0;
        return;
      }
      uint64_t e[kGroup];
      bool ok = true;
#pragma unroll
      for (int k = 0; k < kGroup; ++k) {
        e[k] = ld_local_u64(rin + ((x0 + k) & (kCarryLen - 1)));
        ok &= uint32_t(e[k] >> 32) == uint32_t(x0 + k + 1) || x0 + k >= w;
      }
      int spins = 0;
      while (!ok && ++spins < kSpinLimit) {
        if ((spins & 1023) == 0 && ld_poll(error)) break;
        ok = true;
#pragma unroll
        for (int k = 0; k < kGroup; ++k) {
          e[k] = ld_local_u64(rin + ((x0 + k) & (kCarryLen - 1)));
          ok &= uint32_t(e[k] >> 32) == uint32_t(x0 + k + 1) || x0 + k >= w;
        }
      }
      if (!ok && lane == 0) atomicExch(error, 1);
#pragma unroll
      for (int k = 0; k < kGroup; ++k) cinb[CS][k] = lane == 0 && x0 + k < w ? int(uint32_t(e[k])) : 0;
      st_cluster_u32_if(lane == 0, prog_up, uint32_t(x0 + kGroup));
    }
  }

  // The steps of group g (its source texels in stage ST); the quantised
  // values land in q[].
  template <int ST>
  __device__ __forceinline__ void steps(int g) {
    load_src((ST + kStages - 1) % kStages, g + kStages - 1);
    load_cin((ST + kStages - 1) % kStages, g + kStages - 1);
    take_cin<ST>(g);
    if (LM == kLoadBytes) {
#pragma unroll
      for (int k = 0; k < kGroup; ++k) cur[k] = inb[ST][k];
    } else {
      // this group's copies are done once at most the two later ones are pending
      cp_async_wait<kStages - 1>();
      const uint4 lo = *reinterpret_cast<const uint4*>(slot + ST * kStageWords);
      const uint4 hi = *reinterpret_cast<const uint4*>(slot + ST * kStageWords + 4);
      cur[0] = lo.x, cur[1] = lo.y, cur[2] = lo.z, cur[3] = lo.w;
      cur[4] = hi.x, cur[5] = hi.y, cur[6] = hi.z, cur[7] = hi.w;
    }
    const int x0 = g * kGroup - kLag * lane;
    int ev[kGroup];
#pragma unroll
    for (int k = 0; k < kGroup; ++k) {
      const int x = x0 + k;
      const bool act = row_ok && unsigned(x) < unsigned(w);
      const int ein = e7p + dq + cinb[ST][k];
      const FsOut f = fs_step<BIT1>(widen12(src_byte(cur[k])) + ein, act, qt);
      q[k] = f.q;
      // the entry for x-1 is complete; x and x+1 move up the window
      const int down = wa + f.e3;
      wa = wb + f.e5;
      wb = f.e1;
      // the lane above is at x + 2: its complete entry is for x + 1
      const int up = __shfl_up_sync(0xffffffffu, down, 1);
      e7p = f.e7;
      dq = lane ? up : 0;
      ev[k] = emit_err ? ein : down;
    }
    // the emitting lane writes the group's completed entries: x-1 for each
    // texel x, or (red leftover, even last row) each texel's own error
    const int i0 = g * kGroup - kLag * emit_lane - (emit_err ? 0 : 1);  // the same in every lane
    const bool me = lane == emit_lane;
    if (out_mode == kOutRow) {
#pragma unroll
      for (int k = 0; k < kGroup; ++k) st_tagged_if(me && unsigned(i0 + k) < unsigned(w), emit + i0 + k, ev[k]);
    } else if (out_mode == kOutRing && i0 + kGroup > 0 && i0 < w) {
      // the successor must have read everything this overwrites
      int spins = 0;
      while (i0 + kGroup > int(ld_local_u32(prog)) + kCarryLen && ++spins < kSpinLimit)
        if ((spins & 1023) == 0 && ld_poll(error)) break;
#pragma unroll
      for (int k = 0; k < kGroup; ++k) {
        const int i = i0 + k;
        const uint64_t v = (uint64_t(uint32_t(i + 1)) << 32) | uint32_t(ev[k]);
        st_cluster_u64_if(me && unsigned(i) < unsigned(w), rout + uint32_t((i & (kCarryLen - 1)) * 8), v);
      }
    }
  }
};

// Ticket, ring set-up and the cluster barriers around a CTA's strip.  All
// CTAs of the cluster get strips ticket * kCluster + rank; CTAs past the last
// strip only take part in the barriers.
template <int NCH>
__device__ __forceinline__ int cluster_begin(const FsArgs& a, CarrySmem<NCH>& cs, int& rank) {
  rank = int(cluster_rank());
  for (int i = threadIdx.x; i < NCH * kCarryLen; i += blockDim.x) (&cs.ring[0][0])[i] = 0;
  if (threadIdx.x < NCH) cs.prog[threadIdx.x] = 0;
  cluster_sync();  // every CTA of the cluster runs and has its rings cleared
  if (rank == 0 && threadIdx.x == 0) {
    const uint32_t t = atomicAdd(a.ticket, 1u);
    for (int r = 0; r < kCluster; ++r) st_cluster_u32_if(true, map_rank(&cs.ticket, uint32_t(r)), t);
  }
  cluster_sync();
  return int(ld_local_u32(&cs.ticket)) * kCluster + rank;
}

// Colour pass: one CTA per strip, warp c runs channel c.  AP is the alpha
// byte: for 3-component input the constant (1, 15 or 255); for 4 components
// 255 copies the source alpha (8-bit alpha) and 0 leaves 0 for the alpha pass.
template <int SC, int AP, int LM>
__device__ __forceinline__ void colour_warp(const FsArgs& a, int strip, int rank, uint32_t (*ring)[kRingStride],
                                            uint32_t* stage_buf, CarrySmem<3>& cs, int ch) {
  const Quant qt = ch == 1 ? Quant{2, 63, loop_mul(63)} : Quant{3, 31, loop_mul(31)};
  Chan<false, SC, LM> c;
  c.setup(a, strip, rank, ch, ch == 0 && a.leftover != nullptr, qt, ch, stage_buf, cs);
  const int lane = c.lane;
  const int w = a.width;
  const int y = strip * kLanes + lane;
  const bool row_ok = y < a.height;
  uint32_t* drow = a.dst + size_t(row_ok ? y : 0) * w;
  const bool al_dst = a.dst8 && (((row_ok ? y : 0) & w & 1) == 0);
  uint8_t* ring8 = reinterpret_cast<uint8_t*>(ring[lane]);
  // the last lane reaches x = w (where it completes the entry for w-1) at
  // step w + kLag * 31; whole windows so that every texel is written out
  const int nsteps = w + kLag * (kLanes - 1) + 1;
  const int ngroups = (nsteps + kWindow - 1) / kWindow * (kWindow / kGroup);

  auto group = [&](auto stc, int g) {
    constexpr int ST = decltype(stc)::value;
    c.template steps<ST>(g);
    const int x0 = g * kGroup - kLag * lane;
#pragma unroll
    for (int k = 0; k < kGroup; ++k) {
      const int pos = (x0 + k) & (kRing - 1);
      ring8[pos * 4 + ch] = uint8_t(c.q[k]);
      if (SC == 4 && AP == 255 && ch == 0) ring8[pos * 4 + 3] = uint8_t(c.cur[k] >> 24);
    }
    if ((g + 1) % (kWindow / kGroup) == 0) {
      // window m holds each lane's texels [32m - kLag r, 32m + 32 - kLag r);
      // the ring keeps two windows, so one barrier per window is enough
      asm volatile("bar.sync 1, 96;" ::: "memory");
      const int xs = (g + 1) * kGroup - kWindow - kLag * lane;
      for (int j = ch; j < kWindow / 2; j += 3) {
        const int x = xs + 2 * j;
        if (!row_ok || x < 0 || x >= w) continue;
        uint32_t v0 = ring[lane][x & (kRing - 1)];
        uint32_t v1 = ring[lane][(x + 1) & (kRing - 1)];
        if (!(SC == 4 && AP == 255)) {
          v0 = (v0 & 0x00FFFFFFu) | (uint32_t(AP) << 24);
          v1 = (v1 & 0x00FFFFFFu) | (uint32_t(AP) << 24);
        }
        if (x + 1 < w && al_dst) {
          *reinterpret_cast<uint2*>(drow + x) = make_uint2(v0, v1);
        } else {
          drow[x] = v0;
          if (x + 1 < w) drow[x + 1] = v1;
        }
      }
    }
  };
  for (int g = 0; g < ngroups; g += kStages) {
    static_assert(kStages == 3, "stage unroll");
    group(std::integral_constant<int, 0>(), g);
    if (g + 1 < ngroups) group(std::integral_constant<int, 1>(), g + 1);
    if (g + 2 < ngroups) group(std::integral_constant<int, 2>(), g + 2);
  }
  if (LM != kLoadBytes) asm volatile("cp.async.wait_all;" ::: "memory");
}

template <int SC, int AP, int LM>
__global__ void __launch_bounds__(3 * kLanes, 1) k_fs_colour(FsArgs a) {
  __shared__ uint32_t ring[kLanes][kRingStride];
  __shared__ __align__(16) uint32_t stage[LM == kLoadBytes ? 4 : 3 * kWarpStageWords];
  __shared__ __align__(16) CarrySmem<3> cs;
  int rank;
  const int strip = cluster_begin(a, cs, rank);
  if (strip < a.nstrips) {
    const int warp = threadIdx.x >> 5;
    colour_warp<SC, AP, LM>(a, strip, rank, ring, stage + (LM == kLoadBytes ? 0 : warp * kWarpStageWords), cs,
                            warp);
  }
  cluster_sync();  // no CTA leaves while another may still write to its rings
}

// Alpha pass: one single-warp CTA per strip, writing byte 3 of each texel.
template <int AB, int LM>
__global__ void __launch_bounds__(kLanes, 1) k_fs_alpha(FsArgs a) {
  __shared__ __align__(16) uint32_t stage[LM == kLoadBytes ? 4 : kWarpStageWords];
  __shared__ __align__(16) CarrySmem<1> cs;
  int rank;
  const int strip = cluster_begin(a, cs, rank);
  if (strip < a.nstrips) {
    Chan<AB == 1, 4, LM> c;
    c.setup(a, strip, rank, 0, false, Quant{4, 15, loop_mul(15)}, 3, stage, cs);
    const int lane = c.lane;
    const int w = a.width;
    const int y = strip * kLanes + lane;
    const bool row_ok = y < a.height;
    uint8_t* d = reinterpret_cast<uint8_t*>(a.dst + size_t(row_ok ? y : 0) * w) + 3;
    const int ngroups = (w + kLag * (kLanes - 1) + 1 + kGroup - 1) / kGroup;
    auto group = [&](auto stc, int g) {
      constexpr int ST = decltype(stc)::value;
      c.template steps<ST>(g);
      const int x0 = g * kGroup - kLag * lane;
#pragma unroll
      for (int k = 0; k < kGroup; ++k)
        if (row_ok && unsigned(x0 + k) < unsigned(w)) d[size_t(x0 + k) * 4] = uint8_t(c.q[k]);
    };
    for (int g = 0; g < ngroups; g += kStages) {
      group(std::integral_constant<int, 0>(), g);
      if (g + 1 < ngroups) group(std::integral_constant<int, 1>(), g + 1);
      if (g + 2 < ngroups) group(std::integral_constant<int, 2>(), g + 2);
    }
    if (LM != kLoadBytes) asm volatile("cp.async.wait_all;" ::: "memory");
  }
  cluster_sync();
}

struct FsLayout {
  int nstrips, nrows, wpad;
  size_t rgb_bytes, alpha_bytes;
};

// One carry row per channel and cluster (the strips inside a cluster hand
// their carries over in shared memory).
FsLayout fs_layout(int width, int height) {
  FsLayout l;
  l.nstrips = (height + kLanes - 1) / kLanes;
  l.nrows = (l.nstrips + kCluster - 1) / kCluster;
  l.wpad = ((width + kGroup - 1) / kGroup) * kGroup;
  l.rgb_bytes = size_t(l.nrows) * 3 * l.wpad * sizeof(int);
  l.alpha_bytes = size_t(l.nrows) * l.wpad * sizeof(int);
  return l;
}

template <typename K>
cudaError_t launch_clusters(K kernel, unsigned ctas, unsigned threads, const FsArgs& a, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(ctas);
  cfg.blockDim = dim3(threads);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = kCluster;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kernel, a);
}

}  // namespace

size_t dither_fs_scratch_bytes(int width, int height) {
  const FsLayout l = fs_layout(width, height);
  // carry rows of both passes, then two tickets
  return l.rgb_bytes + l.alpha_bytes + 256;
}

cudaError_t launch_dither_fs(DitherArgs d, uint8_t* scratch, cudaStream_t s) {
  const int w = d.width, h = d.height;
  const FsLayout l = fs_layout(w, h);
  const bool alpha_pass = d.srccomps == 4 && (d.alphabits == 1 || d.alphabits == 4);
  FsArgs a;
  a.src = d.src;
  a.dst = d.dst;
  a.width = w;
  a.height = h;
  a.nstrips = l.nstrips;
  a.wpad = l.wpad;
  a.carry = reinterpret_cast<int*>(scratch);
  int* alpha_carry = reinterpret_cast<int*>(scratch + l.rgb_bytes);
  unsigned int* tickets = reinterpret_cast<unsigned int*>(scratch + l.rgb_bytes + l.alpha_bytes);
  a.leftover = alpha_pass ? alpha_carry : nullptr;
  a.seeded = 0;
  a.dst8 = (reinterpret_cast<uintptr_t>(d.dst) & 7) == 0;
  a.ticket = tickets;
  a.error = d.error;
  // the colour pass's row 0 is never read (the first strip has no input)
  const size_t skip = size_t(l.wpad) * 3 * sizeof(int);
  cudaError_t e = l.rgb_bytes > skip ? cudaMemsetAsync(scratch + skip, 0, l.rgb_bytes - skip, s) : cudaSuccess;
  if (e == cudaSuccess && alpha_pass) e = cudaMemsetAsync(alpha_carry, 0, l.alpha_bytes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(tickets, 0, 2 * sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  const unsigned ctas = unsigned((l.nstrips + kCluster - 1) / kCluster * kCluster);
  const unsigned block = 3 * kLanes;
  const uintptr_t sp = reinterpret_cast<uintptr_t>(d.src);
  const int lm = d.srccomps == 4 && (sp & 7) == 0 && (w & 1) == 0 ? kLoadPairs
                 : d.srccomps == 4 && (sp & 3) == 0              ? kLoadWords
                                                                  : kLoadBytes;
  count_launches(1);
  if (d.srccomps == 3) {
    if (d.alphabits == 1) return launch_clusters(k_fs_colour<3, 1, kLoadBytes>, ctas, block, a, s);
    if (d.alphabits == 4) return launch_clusters(k_fs_colour<3, 15, kLoadBytes>, ctas, block, a, s);
    return launch_clusters(k_fs_colour<3, 255, kLoadBytes>, ctas, block, a, s);
  }
  if (alpha_pass) {
    if (lm == kLoadPairs) e = launch_clusters(k_fs_colour<4, 0, kLoadPairs>, ctas, block, a, s);
    else if (lm == kLoadWords) e = launch_clusters(k_fs_colour<4, 0, kLoadWords>, ctas, block, a, s);
    else e = launch_clusters(k_fs_colour<4, 0, kLoadBytes>, ctas, block, a, s);
  } else {
    if (lm == kLoadPairs) return launch_clusters(k_fs_colour<4, 255, kLoadPairs>, ctas, block, a, s);
    if (lm == kLoadWords) return launch_clusters(k_fs_colour<4, 255, kLoadWords>, ctas, block, a, s);
    return launch_clusters(k_fs_colour<4, 255, kLoadBytes>, ctas, block, a, s);
  }
  if (e != cudaSuccess) return e;
  // alpha pass, seeded with the red leftover row
  FsArgs b = a;
  b.carry = alpha_carry;
  b.leftover = nullptr;
  b.seeded = 1;
  b.ticket = tickets + 1;
  count_launches(1);
  if (d.alphabits == 1) {
    if (lm == kLoadPairs) return launch_clusters(k_fs_alpha<1, kLoadPairs>, ctas, kLanes, b, s);
    if (lm == kLoadWords) return launch_clusters(k_fs_alpha<1, kLoadWords>, ctas, kLanes, b, s);
    return launch_clusters(k_fs_alpha<1, kLoadBytes>, ctas, kLanes, b, s);
  }
  if (lm == kLoadPairs) return launch_clusters(k_fs_alpha<4, kLoadPairs>, ctas, kLanes, b, s);
  if (lm == kLoadWords) return launch_clusters(k_fs_alpha<4, kLoadWords>, ctas, kLanes, b, s);
  return launch_clusters(k_fs_alpha<4, kLoadBytes>, ctas, kLanes, b, s);
}

}  // namespace s2tc
