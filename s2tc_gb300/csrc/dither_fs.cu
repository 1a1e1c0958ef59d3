// dither_fs.cu -- DITHER_FLOYDSTEINBERG (s2tc_algorithm.cpp:1218-1261,
// 1350-1411) as a wavefront of warps.
//
// Texel (x, y) needs the error of (x-1, y) and of (x-1..x+1, y-1), so row y can
// run two texels behind row y-1.  One warp owns a strip of 32 rows, one lane
// per row: at step t lane r handles x = t - 2r.  Each lane keeps the errors it
// sends to the row below in a two-entry window; the entry for x-1 is complete
// once texel x has sent its 3/16 share, and one warp shuffle per channel and
// step hands it to the lane below, which needs it one step later.
//
// Strips are chained through carry rows in global memory.  The strip's last
// lane writes every completed down-going entry as one tagged word (value plus a
// bias, so that zero means "not written yet"); lane 0 of the next strip reads
// the entries four at a time, two groups of four steps ahead, and spins
// (bounded) only when a word is still zero.  No fences are needed: every word
// is checked on its own.  Warps take tickets in launch order, so a strip only
// waits on a strip that is already running.
//
// The alpha channel of 1- and 4-bit alpha runs as a second launch of the same
// kernel over one channel.  Like the reference, it starts from what the red
// pass left in its first error row (s2tc_algorithm.cpp:1354, 1380-1382): the
// red errors of the last row when its index is even, else the red errors it
// sent below.  The red pass writes that row, tagged, as the alpha pass's first
// carry row.
#include <cuda_runtime.h>

#include <cstdint>

#include "dither.h"

namespace s2tc {
namespace {

constexpr int kLanes = 32;           // rows per strip
constexpr int kWarps = 4;            // strips per CTA
constexpr int kGroup = 4;            // steps per group
constexpr int kSpinLimit = 1 << 22;  // polls of one carry group
constexpr int kTagBias = 0x40000000; // carry word = value + bias; 0 = not written

// q * 4095 / 31 for q in [0, 31] as one multiply and shift.
constexpr int kLoop31Mul = 8657095;
constexpr bool loop31_exact() {
  for (int q = 0; q <= 31; ++q)
    if (((q * kLoop31Mul) >> 16) != q * 4095 / 31) return false;
  return true;
}
static_assert(loop31_exact(), "loop31 multiplier");
static_assert(4095 % 63 == 0 && 4095 % 15 == 0, "exact loops");

struct FsOut {
  int q, e7, e3, e5, e1;
};

// One Floyd-Steinberg step on 12-bit values (s2tc_algorithm.cpp:1218-1261);
// MAXV == 1 is the 1-bit variant (:1241).  `s12` is the source byte widened to
// 12 bits, (s << 4) | (s >> 4).  The error shares are zero when `act` is false.
template <int SHIFT, int MAXV>
__device__ __forceinline__ FsOut fs_step(int err_in, int s12, bool act) {
  FsOut o;
  const int v = s12 + err_in;
  int loop;
  if (MAXV == 1) {
    o.q = v >= 2048;
    loop = o.q ? 4095 : 0;
  } else {
    o.q = min(max(v >> (SHIFT + 4), 0), MAXV);
    loop = MAXV == 31 ? (o.q * kLoop31Mul) >> 16 : o.q * (4095 / MAXV);
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

__device__ __forceinline__ int widen12(uint32_t b) { return int((b << 4) | (b >> 4)); }

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

struct FsArgs {
  const uint8_t* src;
  uint32_t* dst;
  int width, height;
  int nstrips;
  int wpad;             // carry row length, width rounded up to 4
  int* carry;           // nstrips * NCH rows; strip s reads rows s*NCH.. (strip 0's only if seeded)
  int* leftover;        // red pass followed by an alpha pass: the alpha pass's first carry row
  int seeded;           // alpha pass: strip 0 reads its carry row (the red leftover)
  int src8, dst8;       // 8-byte aligned base pointers
  unsigned int* ticket;
  int* error;
};

// NCH == 3: red/green/blue pass.  For 3-component input AP is the constant
// alpha byte; for 4 components AP == 255 copies the source alpha (8-bit alpha)
// and AP == 0 leaves 0 for the alpha pass.  NCH == 1: alpha pass with AP alpha
// bits (1 or 4), writing byte 3 only.
template <int NCH, int SC, int AP>
struct Strip {
  FsArgs a;
  int lane, y, w;
  bool row_ok, al_src, al_dst, has_in;
  const int* cin;          // carry rows read by lane 0
  int* emit;               // carry rows written by the emitting lane, or null
  int emit_lane, emit_nch, emit_err;  // emit_err: write err_in (not the window) at x
  const uint8_t* srow;
  uint32_t* drow;

  uint32_t inb[3][kGroup];     // source texels of three groups
  int cinb[3][NCH][kGroup];    // lane 0: carry entries of three groups
  int pa[NCH];                 // error of the texel at hand (minus the carry, lane 0)
  int wa[NCH], wb[NCH];        // down-going errors for x-1 and x

  __device__ __forceinline__ void load_src(int st, int g) {
    const int x0 = g * kGroup - 2 * lane;
    if (SC == 4) {
      if (row_ok && x0 >= 0 && x0 + kGroup <= w && al_src) {
        const uint2 p0 = __ldg(reinterpret_cast<const uint2*>(srow + size_t(x0) * 4));
        const uint2 p1 = __ldg(reinterpret_cast<const uint2*>(srow + size_t(x0) * 4 + 8));
        inb[st][0] = p0.x;
        inb[st][1] = p0.y;
        inb[st][2] = p1.x;
        inb[st][3] = p1.y;
      } else {
#pragma unroll
        for (int k = 0; k < kGroup; ++k) {
          const int x = x0 + k;
          inb[st][k] = row_ok && unsigned(x) < unsigned(w) ? __ldg(reinterpret_cast<const uint32_t*>(srow + size_t(x) * 4)) : 0u;
        }
      }
    } else {
#pragma unroll
      for (int k = 0; k < kGroup; ++k) {
        const int x = x0 + k;
        uint32_t v = 0;
        if (row_ok && unsigned(x) < unsigned(w)) {
          const uint8_t* s = srow + size_t(x) * 3;
          v = uint32_t(__ldg(s)) | (uint32_t(__ldg(s + 1)) << 8) | (uint32_t(__ldg(s + 2)) << 16);
        }
        inb[st][k] = v;
      }
    }
  }

  // Carry words of group g into stage st.  All lanes load the same words (one
  // broadcast transaction) so that the warp never splits; only lane 0 keeps
  // them once their tags are checked.
  __device__ __forceinline__ void load_cin(int st, int g) {
    if (!has_in) return;
    const int x0 = g * kGroup;
#pragma unroll
    for (int c = 0; c < NCH; ++c) {
      int4 v = make_int4(0, 0, 0, 0);
      if (x0 < w) v = __ldcg(reinterpret_cast<const int4*>(cin + size_t(c) * a.wpad + x0));
      cinb[st][c][0] = v.x;
      cinb[st][c][1] = v.y;
      cinb[st][c][2] = v.z;
      cinb[st][c][3] = v.w;
    }
  }

  __device__ __forceinline__ bool cin_ready(int st, int g) const {
    const int need = min(kGroup, w - g * kGroup);
    bool ok = true;
#pragma unroll
    for (int c = 0; c < NCH; ++c)
#pragma unroll
      for (int k = 0; k < kGroup; ++k) ok &= cinb[st][c][k] != 0 || k >= need;
    return ok;
  }

  // Makes sure group g's carry words (stage ST) are written, then strips their
  // tags (and zeroes them for every lane but 0).  A group that is not there
  // yet means the prefetches of the next two groups are stale as well, so the
  // wait runs until the producer is three groups further on and then reloads
  // all three stages: that lag keeps later prefetches (issued two groups
  // ahead) from coming back empty.  The branch is warp-uniform.
  template <int ST>
  __device__ __forceinline__ void take_cin(int g) {
    if (!has_in) return;
    const int x0 = g * kGroup;
    if (x0 >= w) return;
    if (!cin_ready(ST, g)) {
      const int xw = min(x0 + 4 * kGroup - 1, w - 1);  // last entry of group g+3
      const int* pw = cin + size_t(NCH - 1) * a.wpad + xw;
      int spins = 0;
      while (ld_poll(pw) == 0 && ++spins < kSpinLimit)
        if ((spins & 255) == 0 && ld_poll(a.error)) break;
      spins = 0;
      do {
        load_cin(ST, g);
        load_cin((ST + 1) % 3, g + 1);
        load_cin((ST + 2) % 3, g + 2);
      } while (!cin_ready(ST, g) && ++spins < 64 && !ld_poll(a.error));
      if (!cin_ready(ST, g) && lane == 0) atomicExch(a.error, 1);
    }
#pragma unroll
    for (int c = 0; c < NCH; ++c)
#pragma unroll
      for (int k = 0; k < kGroup; ++k) cinb[ST][c][k] = lane == 0 && cinb[ST][c][k] ? cinb[ST][c][k] - kTagBias : 0;
  }

  template <int ST>
  __device__ __forceinline__ void group(int g) {
    load_src((ST + 2) % 3, g + 2);
    load_cin((ST + 2) % 3, g + 2);
    take_cin<ST>(g);
    const int x0 = g * kGroup - 2 * lane;
    uint32_t out[kGroup];
#pragma unroll
    for (int k = 0; k < kGroup; ++k) {
      const int x = x0 + k;
      const bool act = row_ok && unsigned(x) < unsigned(w);
      const uint32_t texel = inb[ST][k];
      // the emitting lane writes the entry for x-1 (complete now) or, for the
      // red leftover of an even last row, this texel's error
      const bool em = lane == emit_lane && (emit_err ? act : unsigned(x - 1) < unsigned(w));
      int* const ep = emit + (emit_err ? x : x - 1);
      uint32_t word = 0;
#pragma unroll
      for (int c = 0; c < NCH; ++c) {
        const int ein = pa[c] + cinb[ST][c][k];
        FsOut f;
        if (NCH == 1) {
          const int s12 = widen12(texel >> 24);
          f = AP == 1 ? fs_step<7, 1>(ein, s12, act) : fs_step<4, 15>(ein, s12, act);
        } else {
          const int s12 = widen12((texel >> (8 * c)) & 0xFF);
          f = c == 1 ? fs_step<2, 63>(ein, s12, act) : fs_step<3, 31>(ein, s12, act);
        }
        word |= uint32_t(f.q) << (8 * c);
        // the entry for x-1 is complete; x and x+1 move up the window
        const int down = wa[c] + f.e3;
        wa[c] = wb[c] + f.e5;
        wb[c] = f.e1;
        const int up = __shfl_up_sync(0xffffffffu, down, 1);
        pa[c] = f.e7 + (lane ? up : 0);
        st_tagged_if(em && c < emit_nch, ep + size_t(c) * a.wpad, emit_err ? ein : down);
      }
      if (NCH == 3) {
        if (SC == 3) word |= uint32_t(AP) << 24;
        else if (AP == 255) word |= texel & 0xFF000000u;
      }
      out[k] = word;
    }
    // store the group's texels
    if (NCH == 3) {
      if (row_ok && x0 >= 0 && x0 + kGroup <= w && al_dst) {
        uint2* d = reinterpret_cast<uint2*>(drow + x0);
        d[0] = make_uint2(out[0], out[1]);
        d[1] = make_uint2(out[2], out[3]);
      } else {
#pragma unroll
        for (int k = 0; k < kGroup; ++k)
          if (row_ok && unsigned(x0 + k) < unsigned(w)) drow[x0 + k] = out[k];
      }
    } else {
      uint8_t* d = reinterpret_cast<uint8_t*>(drow);
#pragma unroll
      for (int k = 0; k < kGroup; ++k)
        if (row_ok && unsigned(x0 + k) < unsigned(w)) d[size_t(x0 + k) * 4 + 3] = uint8_t(out[k]);
    }
  }

  __device__ __forceinline__ void run(int strip) {
    w = a.width;
    lane = threadIdx.x & 31;
    y = strip * kLanes + lane;
    row_ok = y < a.height;
    const int yy = row_ok ? y : 0;
    srow = a.src + size_t(yy) * w * SC;
    drow = a.dst + size_t(yy) * w;
    const bool odd_row_start = (yy & w & 1) != 0;  // y * w odd
    al_src = a.src8 && !odd_row_start;
    al_dst = a.dst8 && !odd_row_start;
    has_in = strip > 0 || a.seeded;
    cin = a.carry + size_t(strip) * NCH * a.wpad;
    const bool last = strip == a.nstrips - 1;
    emit = nullptr;
    emit_lane = -1;
    emit_nch = NCH;
    emit_err = 0;
    if (!last) {
      emit = a.carry + size_t(strip + 1) * NCH * a.wpad;
      emit_lane = kLanes - 1;
    } else if (NCH == 3 && a.leftover) {
      emit = a.leftover;
      emit_lane = a.height - 1 - strip * kLanes;
      emit_nch = 1;
      emit_err = ((a.height - 1) & 1) == 0;
    }
#pragma unroll
    for (int c = 0; c < NCH; ++c) pa[c] = wa[c] = wb[c] = 0;
#pragma unroll
    for (int st = 0; st < 3; ++st)
#pragma unroll
      for (int c = 0; c < NCH; ++c)
#pragma unroll
        for (int k = 0; k < kGroup; ++k) cinb[st][c][k] = 0;
    load_src(0, 0);
    load_src(1, 1);
    load_cin(0, 0);
    load_cin(1, 1);
    // the last lane reaches x = w (where it completes the entry for w-1) at
    // step w + 2 * 31
    const int ngroups = (w + 2 * (kLanes - 1) + 1 + kGroup - 1) / kGroup;
    for (int g = 0; g < ngroups; g += 3) {
      group<0>(g);
      if (g + 1 < ngroups) group<1>(g + 1);
      if (g + 2 < ngroups) group<2>(g + 2);
    }
  }
};

template <int NCH, int SC, int AP>
__global__ void __launch_bounds__(kLanes * kWarps) k_fs(FsArgs a) {
  int strip = 0;
  if ((threadIdx.x & 31) == 0) strip = int(atomicAdd(a.ticket, 1u));
  strip = __shfl_sync(0xffffffffu, strip, 0);
  if (strip >= a.nstrips) return;
  Strip<NCH, SC, AP> s;
  s.a = a;
  s.run(strip);
}

struct FsLayout {
  int nstrips, wpad;
  size_t rgb_bytes, alpha_bytes;
};

FsLayout fs_layout(int width, int height) {
  FsLayout l;
  l.nstrips = (height + kLanes - 1) / kLanes;
  l.wpad = (width + 3) & ~3;
  l.rgb_bytes = size_t(l.nstrips) * 3 * l.wpad * sizeof(int);
  l.alpha_bytes = size_t(l.nstrips) * l.wpad * sizeof(int);
  return l;
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
  a.src8 = (reinterpret_cast<uintptr_t>(d.src) & 7) == 0;
  a.dst8 = (reinterpret_cast<uintptr_t>(d.dst) & 7) == 0;
  a.ticket = tickets;
  a.error = d.error;
  // the carry words of strip 0 are never read in the red/green/blue pass
  const size_t skip = size_t(l.wpad) * 3 * sizeof(int);
  cudaError_t e = cudaMemsetAsync(scratch + skip, 0, l.rgb_bytes - skip, s);
  if (e == cudaSuccess && alpha_pass) e = cudaMemsetAsync(alpha_carry, 0, l.alpha_bytes, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(tickets, 0, 2 * sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  const unsigned warps = unsigned(l.nstrips);
  const unsigned grid = (warps + kWarps - 1) / kWarps;
  const unsigned block = kLanes * kWarps;
  count_launches(1);
  if (d.srccomps == 3) {
    if (d.alphabits == 1) k_fs<3, 3, 1><<<grid, block, 0, s>>>(a);
    else if (d.alphabits == 4) k_fs<3, 3, 15><<<grid, block, 0, s>>>(a);
    else k_fs<3, 3, 255><<<grid, block, 0, s>>>(a);
    return cudaGetLastError();
  }
  if (alpha_pass) k_fs<3, 4, 0><<<grid, block, 0, s>>>(a);
  else k_fs<3, 4, 255><<<grid, block, 0, s>>>(a);
  e = cudaGetLastError();
  if (e != cudaSuccess || !alpha_pass) return e;
  // alpha pass, seeded with the red leftover row
  FsArgs b = a;
  b.carry = alpha_carry;
  b.leftover = nullptr;
  b.seeded = 1;
  b.ticket = tickets + 1;
  count_launches(1);
  if (d.alphabits == 1) k_fs<1, 4, 1><<<grid, block, 0, s>>>(b);
  else k_fs<1, 4, 4><<<grid, block, 0, s>>>(b);
  return cudaGetLastError();
}

}  // namespace s2tc
