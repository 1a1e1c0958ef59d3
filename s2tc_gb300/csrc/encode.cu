// encode.cu -- the S2TC block encoder kernels (one thread per 4x4 block).
//
// This file is compiled once per colour-distance metric (-DS2TC_METRIC=<id>),
// so the 135 (format x metric x selection x refinement) instantiations of the
// reference's compile-time dispatch (s2tc_algorithm.cpp:1110-1194) spread over
// eight translation units that build in parallel.
//
// Input: the 4-byte-per-texel 5:6:5 buffer produced by the dither kernels
// (r | g<<8 | b<<16 | a<<24, row length `width` texels).  Output: 8/16-byte
// DXT1/DXT3/DXT5 blocks, block rows `pitch` bytes apart.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include <cuda.h>

#include "dither.h"
#include "dither_scan.cuh"
#include "encode.h"
#include "s2tc_device.cuh"

#ifndef S2TC_METRIC
#error "compile with -DS2TC_METRIC=<0..7>"
#endif

namespace s2tc {
namespace {

constexpr int kMetric = S2TC_METRIC;

using P = typename PrepT<kMetric>::T;

// Slot (y*4+x) of input k of a full block: inputs are gathered x-outer,
// y-inner (s2tc_algorithm.cpp:940-951).
__device__ __forceinline__ constexpr int in_slot(int k) { return (k & 3) * 4 + (k >> 2); }

// ------------------------------------------------------------------------
// Full-block search without random candidates: 16 inputs, all 120 pairs.
// The loop runs over the inputs k; the 120 pair sums stay in registers and
// every iteration adds min(d(i,k), d(j,k)) to each of them, so the loop body is
// small (a few hundred instructions) while every index into the sums is a
// compile-time constant.  Input k's prepared colour comes from a per-thread
// column in shared memory.

constexpr int kThreadsPerCta = 128;

// The metrics other than SRGB are symmetric in their arguments.
constexpr bool kSymmetric = kMetric != CD_SRGB;

// Per-thread scratch columns in shared memory (index [k][thread]).
struct Scratch16 {
  P pin[16][kThreadsPerCta];
  int ain[16][kThreadsPerCta];   // distinct alpha values of the block, ascending
  int ast[16][kThreadsPerCta];   // where each value's run starts in the sorted values
};

// Sorts 16 values ascending (bitonic network, unrolled).
__device__ __forceinline__ void sort16(int* v) {
#pragma unroll
  for (int k = 2; k <= 16; k <<= 1)
#pragma unroll
    for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const int l = i ^ j;
        if (l > i) {
          const int lo = min(v[i], v[l]), hi = max(v[i], v[l]);
          const bool up = (i & k) == 0;
          v[i] = up ? lo : hi;
          v[l] = up ? hi : lo;
        }
      }
}

// Pick the pair the reference keeps: pairs in (i, j) lexicographic order,
// taken when `bestsum < 0 || sum < bestsum` (s2tc_algorithm.cpp:404-409).
// Only pairs of inputs in `mask` (bit k: input k takes part) are candidates.
__device__ __forceinline__ void pick_pair(const int32_t* S, uint32_t mask, int& besti, int& bestj) {
  int32_t bestsum = -1;
  besti = 0;
  bestj = 1;
  int p = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i)
#pragma unroll
    for (int j = i + 1; j < 16; ++j, ++p) {
      const bool ok = ((mask >> i) & (mask >> j) & 1u) != 0;
      const bool take = ok && (bestsum < 0 || S[p] < bestsum);
      bestsum = take ? S[p] : bestsum;
      besti = take ? i : besti;
      bestj = take ? j : bestj;
    }
}

// pick_pair (above) without negative sums and with every input taking part:
// the smallest sum by a tree of minima, then the first pair that has it.  The
// sequential rule is a chain of 120 dependent compare-and-selects per block;
// this form has a dependency depth of about twenty.
__device__ __forceinline__ void pick_pair_nonneg(const int32_t* S, int& besti, int& bestj) {
  uint32_t t[60];
#pragma unroll
  for (int r = 0; r < 60; ++r) t[r] = min(uint32_t(S[2 * r]), uint32_t(S[2 * r + 1]));
#pragma unroll
  for (int st = 1; st < 60; st <<= 1)
#pragma unroll
    for (int r = 0; r + st < 60; r += 2 * st) t[r] = min(t[r], t[r + st]);
  const uint32_t m = t[0];
  // the first position with the minimum, as (i << 4) | j: eight independent
  // chains of fifteen selects, then the earliest chain that found one
  uint32_t f[8];
#pragma unroll
  for (int c = 0; c < 8; ++c) f[c] = 0xFFu;
  int p = 119;
#pragma unroll
  for (int i = 15; i >= 0; --i)
#pragma unroll
    for (int j = 15; j > i; --j, --p) f[p / 15] = uint32_t(S[p]) == m ? uint32_t((i << 4) | j) : f[p / 15];
  uint32_t r = f[7];
#pragma unroll
  for (int c = 6; c >= 0; --c) r = f[c] != 0xFFu ? f[c] : r;
  besti = int(r >> 4);
  bestj = int(r & 15);
}

// reduce_colors_inplace (s2tc_algorithm.cpp:363-414) for n = m = 16.  Between
// two inputs the reference evaluates dist(c[lo], c[hi]) once and uses it both
// ways; d(k, k) = 0.
__device__ __forceinline__ void reduce16_rgb(const P* tp, uint32_t mask, Scratch16& sc, int& besti, int& bestj) {
  const int t = threadIdx.x;
  P pin[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    pin[i] = tp[in_slot(i)];
    sc.pin[i][t] = pin[i];
  }
  int32_t S[120];
#pragma unroll
  for (int p = 0; p < 120; ++p) S[p] = 0;
  // two inputs per pass: each sum takes both minima in one three-input add
#pragma unroll 1
  for (int k = 0; k < 16; k += 2) {
    const P pk = sc.pin[k][t], pk1 = sc.pin[k + 1][t];
    // a transparent DXT1 texel is no input: its distances count as 0
    const bool in0 = (mask >> k) & 1u, in1 = (mask >> (k + 1)) & 1u;
    int32_t col[16], col1[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      col[i] = (kSymmetric || i < k) ? pdist<kMetric>(pin[i], pk) : pdist<kMetric>(pk, pin[i]);
      col1[i] = (kSymmetric || i < k + 1) ? pdist<kMetric>(pin[i], pk1) : pdist<kMetric>(pk1, pin[i]);
      col[i] = in0 ? col[i] : 0;
      col1[i] = in1 ? col1[i] : 0;
    }
    int p = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i)
#pragma unroll
      for (int j = i + 1; j < 16; ++j, ++p)
        S[p] = int32_t(uint32_t(S[p]) + uint32_t(min(col[i], col[j])) + uint32_t(min(col1[i], col1[j])));
  }
  uint32_t neg = 0;
#pragma unroll
  for (int p = 0; p < 120; ++p) neg |= uint32_t(S[p]);
  if (mask == 0xFFFFu && int32_t(neg) >= 0) {
    pick_pair_nonneg(S, besti, bestj);
    return;
  }
  pick_pair(S, mask, besti, bestj);  // negative sums (SRGB) or DXT1 transparent texels
}

// reduce_colors_inplace_2fixpoints (s2tc_algorithm.cpp:415-478) for n = m = 16
// on the alpha values.  Each input's cost is the smallest squared distance to
// the pair or to the fixed values 0 and 255; the minimum of squares of
// non-negative numbers is the square of their minimum.  Its conditional
// write-back into c[0]/c[1] reads the candidates before changing them, so the
// result is simply the winning pair.
//
// Every input k adds min(d(i,k), d(j,k)) to the sum of pair (i, j), and inputs
// with equal alpha add equal amounts, so the loop runs over the block's
// distinct alpha values (2.6 per block on a typical texture with alpha) and
// adds each one's contribution times its count: the same integer sums, in
// fewer passes over the 120 pairs.
__device__ __forceinline__ void reduce16_alpha(const int* ain, Scratch16& sc, int& besti, int& bestj) {
  const int t = threadIdx.x;
  // distinct values and their counts: a sort, then the runs
  int v[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = ain[i];
  sort16(v);
  int nd = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    if (i == 0 || v[i] != v[i - 1]) {
      sc.ain[nd][t] = v[i];
      sc.ast[nd][t] = i;
      ++nd;
    }
  }
  int32_t S[120];
#pragma unroll
  for (int p = 0; p < 120; ++p) S[p] = 0;
#pragma unroll 1
  for (int d = 0; d < nd; ++d) {
    const int ak = sc.ain[d][t];
    const int wk = (d + 1 < nd ? sc.ast[d + 1][t] : 16) - sc.ast[d][t];
    const int fk = min(ak, 255 - ak);
    int col[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      const int c = min(abs(ain[i] - ak), fk);
      col[i] = c * c;
    }
    int p = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i)
#pragma unroll
      for (int j = i + 1; j < 16; ++j, ++p) S[p] += wk * min(col[i], col[j]);
  }
  pick_pair_nonneg(S, besti, bestj);  // sums of squares: never negative
}

// ------------------------------------------------------------------------
// General search: partial blocks, DXT1 blocks with transparent texels, and
// random candidates.

// Candidate c[j] of the pair search: the first n are the block's inputs in
// x-outer, y-inner order; the rest are the random candidates of
// s2tc_algorithm.cpp:962-993 drawn from the replayed rand() words.
struct Candidates {
  C3 in[16];
  P pin[16];
  int ain[16];
  int n;
  const uint32_t* rnd;
  int stride;  // rand words per candidate: 3 (DXT1/DXT3) or 4 (DXT5)
  C3 lo;
  int lr, lg, lb;
  int alo, la;
};

__device__ __forceinline__ C3 cand_rgb(const Candidates& cs, int j) {
  if (j < cs.n) return cs.in[j];
  const uint32_t* r = cs.rnd + size_t(j - cs.n) * cs.stride;
  return C3{cs.lo.r + int(__ldg(r) % uint32_t(cs.lr)), cs.lo.g + int(__ldg(r + 1) % uint32_t(cs.lg)),
            cs.lo.b + int(__ldg(r + 2) % uint32_t(cs.lb))};
}
__device__ __forceinline__ int cand_a(const Candidates& cs, int j) {
  if (j < cs.n) return cs.ain[j];
  const uint32_t* r = cs.rnd + size_t(j - cs.n) * cs.stride;
  return cs.alo + int(__ldg(r + 3) % uint32_t(cs.la));
}

// Distance row of candidate i against the inputs, with the reference's
// argument order: between two inputs dist(c[min], c[max])
// (s2tc_algorithm.cpp:375-383), for a random candidate dist(c[i], c[k])
// (:385-392).  Entries k >= n are 0 and add nothing.
__device__ __forceinline__ void dist_row(const Candidates& cs, int i, int32_t* row) {
  if (i < cs.n) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      int32_t d = 0;
      if (k < cs.n && k != i) d = i < k ? pdist<kMetric>(cs.pin[i], cs.pin[k]) : pdist<kMetric>(cs.pin[k], cs.pin[i]);
      row[k] = d;
    }
  } else {
    const P pi = prep<kMetric>(cand_rgb(cs, i));
#pragma unroll
    for (int k = 0; k < 16; ++k) row[k] = k < cs.n ? pdist<kMetric>(pi, cs.pin[k]) : 0;
  }
}

// reduce_colors_inplace (s2tc_algorithm.cpp:363-414), sequential over pairs.
__device__ void reduce_rgb(const Candidates& cs, int m, C3& c0, C3& c1) {
  int32_t bestsum = -1;
  int besti = 0, bestj = 1;
  int32_t ri[16], rj[16];
  for (int i = 0; i < m; ++i) {
    dist_row(cs, i, ri);
    for (int j = i + 1; j < m; ++j) {
      dist_row(cs, j, rj);
      int32_t sum = 0;
#pragma unroll
      for (int k = 0; k < 16; ++k) sum = wadd(sum, min(ri[k], rj[k]));
      if (bestsum < 0 || sum < bestsum) {
        bestsum = sum;
        besti = i;
        bestj = j;
      }
    }
  }
  c0 = cand_rgb(cs, besti);
  c1 = cand_rgb(cs, bestj);
}

// reduce_colors_inplace_2fixpoints (s2tc_algorithm.cpp:415-478) on the alpha
// candidates; see reduce16_alpha for why the result is the winning pair.
__device__ void reduce_alpha(const Candidates& cs, int m, int& a0, int& a1) {
  const int n = cs.n;
  int F[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) F[k] = k < n ? min(cs.ain[k], 255 - cs.ain[k]) : 0;
  int32_t bestsum = -1;
  int besti = 0, bestj = 1;
  for (int i = 0; i < m; ++i) {
    const int ai = cand_a(cs, i);
    for (int j = i + 1; j < m; ++j) {
      const int aj = cand_a(cs, j);
      int32_t sum = 0;
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        if (k < n) {
          const int ak = cs.ain[k];
          const int v = min(min(abs(ai - ak), abs(aj - ak)), F[k]);
          sum += v * v;
        }
      }
      if (bestsum < 0 || sum < bestsum) {
        bestsum = sum;
        besti = i;
        bestj = j;
      }
    }
  }
  a0 = cand_a(cs, besti);
  a1 = cand_a(cs, bestj);
}

struct EncodedBlock {
  uint64_t lo, hi;
};

// A block takes the full-block search when it has 16 inputs: all 16 texels
// inside the image and, for DXT1, none of them transparent (the reference
// leaves alpha-0 texels out of the candidate list, :947-949).
// Inputs of a whole block in x-outer, y-inner order (bit k: input k): DXT1
// leaves transparent texels out (s2tc_algorithm.cpp:940-951).
template <int DXT>
__device__ __forceinline__ uint32_t input_mask(const BlockTexels& bt) {
  uint32_t m = 0xFFFFu;
  if (DXT == DXT1) {
#pragma unroll
    for (int k = 0; k < 16; ++k)
      if ((bt.px[in_slot(k)] >> 24) == 0) m &= ~(1u << k);
  }
  return m;
}

// Blocks of the register-resident all-texels search: 4x4 blocks with at
// least two inputs (fewer take the general search's special cases).
template <int DXT>
__device__ __forceinline__ bool is_full(const BlockTexels& bt) {
  return bt.w == 4 && bt.h == 4 && (DXT != DXT1 || __popc(input_mask<DXT>(bt)) >= 2);
}

// s2tc_encode_block<> (s2tc_algorithm.cpp:872-1108) for one block.
// FULL16 selects the register-resident search and requires a full block in
// the all-texels mode without random candidates; otherwise the general search
// runs.  `prev_a1` is the second alpha endpoint left behind by the previous
// block of the same image (used only by a single-texel DXT5 block without
// random candidates); the return value is this block's leftover for the next.
template <int DXT, bool NORMAL, int REFINE, bool FULL16>
__device__ int encode_block(const BlockTexels& bt, int nrandom, const uint32_t* rnd, int prev_a1,
                            EncodedBlock& out, Scratch16* sc) {
  constexpr bool TRANS = DXT == DXT1;
  P tp[16];
#pragma unroll
  for (int i = 0; i < 16; ++i) tp[i] = prep<kMetric>(texel_c3(bt.px[i]));
  C3 c0, c1;
  int a0 = 0, a1 = 0;
  if (!NORMAL) {
    // darkest / brightest by distance to black (:879-935), kept as texel
    // words (their colour fields; the starting values are the colours
    // 31,63,31 and 0,0,0)
    const P black = prep<kMetric>(C3{0, 0, 0});
    int32_t dmin = 0x7FFFFFFF, dmax = 0;
    uint32_t t0 = 31u | (63u << 8) | (31u << 16), t1 = 0u;
    if (DXT == DXT5) a0 = a1 = texel_a(bt.px[0]);
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
      for (int y = 0; y < 4; ++y) {
        if (x >= bt.w || y >= bt.h) continue;
        uint32_t t = bt.px[y * 4 + x];
        if (DXT == DXT1 && (t >> 24) == 0) continue;
        int32_t d = pdist<kMetric>(tp[y * 4 + x], black);
        if (d > dmax) { dmax = d; t1 = t; }
        if (d < dmin) { dmin = d; t0 = t; }
        if (DXT == DXT5) {
          int a = texel_a(t);
          if (a != 255) {
            if (a > a1) a1 = a;
            if (a < a0) a0 = a;
          }
        }
      }
    c0 = texel_c3(t0);
    c1 = texel_c3(t1);
  } else {
    if constexpr (FULL16) {
      int bi, bj;
      reduce16_rgb(tp, input_mask<DXT>(bt), *sc, bi, bj);
      // read by a run-time index, which places the block's texel words in
      // local memory while the searches hold their sums in registers; keeping
      // them in registers (selected by masks) or parking them in shared memory
      // and reading them back measured 10% and 2.5% slower
      c0 = texel_c3(bt.px[(bi & 3) * 4 + (bi >> 2)]);
      c1 = texel_c3(bt.px[(bj & 3) * 4 + (bj >> 2)]);
      if (DXT == DXT5) {
        int ain[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) ain[k] = texel_a(bt.px[in_slot(k)]);
        reduce16_alpha(ain, *sc, bi, bj);
        a0 = texel_a(bt.px[(bi & 3) * 4 + (bi >> 2)]);
        a1 = texel_a(bt.px[(bj & 3) * 4 + (bj >> 2)]);
      }
    } else {
      Candidates cs;
      cs.n = 0;
#pragma unroll
      for (int x = 0; x < 4; ++x)
#pragma unroll
        for (int y = 0; y < 4; ++y) {
          if (x >= bt.w || y >= bt.h) continue;
          uint32_t t = bt.px[y * 4 + x];
          if (DXT == DXT1 && (t >> 24) == 0) continue;
          cs.in[cs.n] = texel_c3(t);
          cs.pin[cs.n] = tp[y * 4 + x];
          cs.ain[cs.n] = texel_a(t);
          cs.n++;
        }
      if (cs.n == 0) {
        cs.n = 1;
        cs.in[0] = C3{0, 0, 0};
        cs.pin[0] = prep<kMetric>(cs.in[0]);
        cs.ain[0] = 0;
      }
      int m = cs.n;
      cs.rnd = rnd;
      cs.stride = DXT == DXT5 ? 4 : 3;
      if (nrandom > 0) {
        C3 lo = cs.in[0], hi = cs.in[0];
        int alo = DXT == DXT5 ? cs.ain[0] : 0, ahi = alo;
        for (int k = 1; k < cs.n; ++k) {
          lo.r = min(lo.r, cs.in[k].r); lo.g = min(lo.g, cs.in[k].g); lo.b = min(lo.b, cs.in[k].b);
          hi.r = max(hi.r, cs.in[k].r); hi.g = max(hi.g, cs.in[k].g); hi.b = max(hi.b, cs.in[k].b);
          if (DXT == DXT5) { alo = min(alo, cs.ain[k]); ahi = max(ahi, cs.ain[k]); }
        }
        cs.lo = lo;
        cs.lr = hi.r - lo.r + 1; cs.lg = hi.g - lo.g + 1; cs.lb = hi.b - lo.b + 1;
        cs.alo = alo; cs.la = ahi - alo + 1;
        m = cs.n + nrandom;
      } else if (cs.n == 1) {
        // single input (:996-1001): the colour is duplicated; the reference's
        // second alpha candidate is whatever the previous block left in that slot
        cs.in[1] = cs.in[0];
        cs.pin[1] = cs.pin[0];
        cs.ain[1] = prev_a1 >= 0 ? prev_a1 : cs.ain[0];
        cs.n = 2;
        m = 2;
      }
      reduce_rgb(cs, m, c0, c1);
      if (DXT == DXT5) reduce_alpha(cs, m, a0, a1);
    }
  }

  // equal endpoints are bumped apart (:1009-1027)
  if (c3_eq(c0, c1)) c1 = (c0.r == 31 && c0.g == 63 && c0.b == 31) ? c3_prev(c1) : c3_next(c1);
  if (DXT == DXT5 && a0 == a1) {
    if (a0 == 255) --a1; else ++a1;
  }

  uint32_t cbits = colour_refine<kMetric, TRANS, REFINE>(bt, tp, c0, c1);
  const uint64_t colour = uint64_t(pack565(c0)) | (uint64_t(pack565(c1)) << 16) | (uint64_t(cbits) << 32);
  int leftover = a1;
  if (DXT == DXT1) {
    out.lo = colour;
    out.hi = 0;
  } else if (DXT == DXT3) {
    uint64_t ab = 0;
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if ((i & 3) < bt.w && (i >> 2) < bt.h) ab |= uint64_t(texel_a(bt.px[i]) & 15) << (4 * i);
    out.lo = ab;
    out.hi = colour;
  } else {
    uint64_t abits = alpha_refine<REFINE>(bt, a0, a1, leftover);
    out.lo = uint64_t(a0) | (uint64_t(a1) << 8) | (abits << 16);
    out.hi = colour;
  }
  return leftover;
}

__device__ __forceinline__ void load_block(const uint32_t* __restrict__ t565, int width, int height, int bx, int by,
                                           BlockTexels& bt) {
  bt.w = min(4, width - bx * 4);
  bt.h = min(4, height - by * 4);
  const uint32_t* p = t565 + size_t(by) * 4 * width + size_t(bx) * 4;
  if (bt.w == 4 && bt.h == 4 && ((reinterpret_cast<uintptr_t>(p) | (size_t(width) * 4)) & 15) == 0) {
    // whole block, rows 16-byte aligned: one vector load per row
#pragma unroll
    for (int y = 0; y < 4; ++y) {
      const uint4 v = __ldg(reinterpret_cast<const uint4*>(p + size_t(y) * width));
      bt.px[y * 4 + 0] = v.x;
      bt.px[y * 4 + 1] = v.y;
      bt.px[y * 4 + 2] = v.z;
      bt.px[y * 4 + 3] = v.w;
    }
    return;
  }
#pragma unroll
  for (int y = 0; y < 4; ++y)
#pragma unroll
    for (int x = 0; x < 4; ++x)
      bt.px[y * 4 + x] = (x < bt.w && y < bt.h) ? __ldg(p + size_t(y) * width + x) : 0u;
}

__device__ __forceinline__ void store_block(const EncodeArgs& a, int dxt, int bx, int by, const EncodedBlock& eb) {
  uint8_t* o = a.dst + (size_t)by * a.pitch + (size_t)bx * (dxt == DXT1 ? 8 : 16);
  if (a.aligned) {
    if (dxt == DXT1) {
      *reinterpret_cast<uint64_t*>(o) = eb.lo;
    } else {
      *reinterpret_cast<ulonglong2*>(o) = make_ulonglong2(eb.lo, eb.hi);
    }
  } else {
#pragma unroll
    for (int i = 0; i < 8; ++i) o[i] = uint8_t(eb.lo >> (8 * i));
    if (dxt != DXT1) {
#pragma unroll
      for (int i = 0; i < 8; ++i) o[8 + i] = uint8_t(eb.hi >> (8 * i));
    }
  }
}

// The image and its block-within-launch index for global work item g.
__device__ __forceinline__ bool resolve(const EncodeWork& w, long long g, EncodeArgs& a, long long& bl) {
  if (g >= w.total) return false;
  if (!w.items) {
    a = w.single;
    bl = g;
    return true;
  }
  int lo = 0, hi = w.nitems - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(w.offsets + mid) <= g) lo = mid;
    else hi = mid - 1;
  }
  a = w.items[lo];
  bl = g - __ldg(w.offsets + lo);
  return true;
}

// Full blocks of the all-texels mode without random candidates.
#ifndef S2TC_FULL16_MINBLOCKS
#define S2TC_FULL16_MINBLOCKS 1
#endif
template <int DXT, int REFINE>
__global__ void __launch_bounds__(kThreadsPerCta, S2TC_FULL16_MINBLOCKS) k_encode_full16(EncodeWork w) {
  __shared__ Scratch16 sc;
  EncodeArgs a;
  long long bl;
  if (!resolve(w, (long long)blockIdx.x * blockDim.x + threadIdx.x, a, bl)) return;
  const long long b = (long long)a.by0 * a.bw + bl;
  const int by = int(b / a.bw), bx = int(b % a.bw);
  BlockTexels bt;
  load_block(a.t565, a.width, a.height, bx, by, bt);
  if (!is_full<DXT>(bt)) return;  // left to k_encode
  EncodedBlock eb;
  const int leftover = encode_block<DXT, true, REFINE, true>(bt, 0, nullptr, -1, eb, &sc);
  if (a.leftover_out && b == (long long)a.bw * a.bh - 1) *a.leftover_out = leftover;
  store_block(a, DXT, bx, by, eb);
}

// Every other block: the quick selection, random candidates, edge blocks and
// DXT1 blocks with transparent texels.  In the all-texels mode without random
// candidates the full blocks are skipped (k_encode_full16 encodes them).
template <int DXT, bool NORMAL, int REFINE>
__global__ void __launch_bounds__(kThreadsPerCta) k_encode(EncodeWork w) {
  EncodeArgs a;
  long long bl;  // block within this launch's part of the image
  if (!resolve(w, (long long)blockIdx.x * blockDim.x + threadIdx.x, a, bl)) return;
  const long long b = (long long)a.by0 * a.bw + bl;                         // block within the image
  const int by = int(b / a.bw), bx = int(b % a.bw);
  // whole DXT3/DXT5 blocks of the all-texels mode belong to k_encode_full16:
  // leave them without reading their texels
  if (NORMAL && a.nrandom <= 0 && DXT != DXT1 && a.width - bx * 4 >= 4 && a.height - by * 4 >= 4) return;
  BlockTexels bt;
  load_block(a.t565, a.width, a.height, bx, by, bt);
  if (NORMAL && a.nrandom <= 0 && is_full<DXT>(bt)) return;
  const int per_block = a.nrandom > 0 ? a.nrandom * (DXT == DXT5 ? 4 : 3) : 0;
  const uint32_t* rnd = a.rnd ? a.rnd + (size_t)bl * per_block : nullptr;
  int prev_a1 = -1;
  if (DXT == DXT5 && NORMAL && a.nrandom <= 0 && bt.w == 1 && bt.h == 1) {
    // The reference encodes blocks in raster order into the same stack
    // frame; a single-texel DXT5 block reads its second alpha candidate from
    // a slot it never writes, i.e. the value the previous block left there
    // (s2tc_algorithm.cpp:876, 996-1001).  That block is re-encoded here (the
    // general search gives the same bytes as the full-block one) to recover it.
    if (b > 0) {
      const int pby = int((b - 1) / a.bw), pbx = int((b - 1) % a.bw);
      BlockTexels pt;
      load_block(a.t565, a.width, a.height, pbx, pby, pt);
      EncodedBlock scratch;
      prev_a1 = encode_block<DXT, NORMAL, REFINE, false>(pt, a.nrandom, nullptr, -1, scratch, nullptr);
    } else {
      prev_a1 = a.prev_a1_dev ? *a.prev_a1_dev : a.prev_a1_first;
    }
  }
  EncodedBlock eb;
  const int leftover = encode_block<DXT, NORMAL, REFINE, false>(bt, a.nrandom, rnd, prev_a1, eb, nullptr);
  if (a.leftover_out && b == (long long)a.bw * a.bh - 1) *a.leftover_out = leftover;
  store_block(a, DXT, bx, by, eb);
}

// ------------------------------------------------------------------------
// Random candidates: one warp per block.
//
// The candidate list (the block's inputs, then nrandom random colours) and
// each candidate's distance row against the inputs live in shared memory.
// Lane l owns the rows i = l, l + 32, ...; all lanes walk j together, so the
// row-j loads are broadcasts.  Without negative sums (they need the SRGB
// metrics' int32 wrap-around) the reference's `bestsum < 0 || sum < bestsum`
// rule picks the first pair with the smallest sum, i.e. the smallest
// (sum, i, j); a block that sees a negative sum is replayed by one lane in
// exact sequential order.  Refinement runs with one lane per texel and warp
// reductions.

constexpr int kRandWarps = 4;
constexpr unsigned kFull = 0xFFFFFFFFu;
// Unique candidates up to which a pair search packs (sum, i, j) into 32 bits
// (positions as a * 90 + b < 8192, 13 bits).
constexpr int kKeyPositions = 90;

// Colour distance rows fit in 16 bits for the AVG family (at most
// 4*31^2 + 4*63^2 + 31^2 = 20681); they are then packed two per word.
constexpr bool kSmallDist = kMetric == CD_AVG || kMetric == CD_W0AVG || kMetric == CD_WAVG;
constexpr int kRowBytes = kSmallDist ? 32 : 64;

// Candidates are deduplicated through a per-warp table indexed by the value
// inside the block's bounding box when the box has at most kDedupSlots
// values (first occurrence and first repeat per value).
#ifndef S2TC_DEDUP_SLOTS
#define S2TC_DEDUP_SLOTS 256
#endif
constexpr int kDedupSlots = S2TC_DEDUP_SLOTS;
constexpr int kDedupWords = 2 * kDedupSlots;
static_assert(kDedupSlots >= 256, "the alpha search indexes the table by the 256 alpha values");

struct RandLayout {
  size_t p, c, a, d, e, u, t, bytes;  // section offsets and bytes per warp
};

__host__ __device__ __forceinline__ size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ __forceinline__ RandLayout rand_layout(int m) {
  RandLayout L;
  L.p = 0;
  L.c = align16(L.p + size_t(m) * sizeof(P));          // prepared candidates
  L.a = align16(L.c + size_t(m) * sizeof(uint16_t));   // candidate colours, 5:6:5
  L.d = align16(L.a + size_t(m));                       // candidate alphas
  // the alpha rows (16-bit, 32 bytes each) reuse the colour rows' space: the
  // alpha search starts after the colour search has read its last row
  L.e = L.d;
  L.u = align16(L.d + size_t(m) * kRowBytes);          // colour distance rows
  L.t = align16(L.u + size_t(m) * 2 * sizeof(uint16_t));  // unique colour / alpha indices
  L.bytes = align16(L.t + kDedupWords * sizeof(uint32_t));  // dedup table
  return L;
}

__device__ __forceinline__ C3 unpack565(uint32_t v) { return C3{int(v >> 11) & 31, int(v >> 5) & 63, int(v) & 31}; }

// One colour index pass over the block, lane s (< 16) holding slot s.
struct WarpColourPass {
  uint32_t bits, score;
  int n0, n1, s0r, s0g, s0b, s1r, s1g, s1b;
};

template <bool TRANS, bool ACC>
__device__ __forceinline__ WarpColourPass colour_pass_warp(bool inb, uint32_t px, const P& tp, C3 r0, C3 r1,
                                                          int lane) {
  WarpColourPass o;
  const P p0 = prep<kMetric>(r0), p1 = prep<kMetric>(r1);
  const bool trans = TRANS && inb && (px >> 24) == 0;
  const bool active = inb && !trans;
  int32_t d0 = 0, d1 = 0;
  if (active) {
    d0 = pdist<kMetric>(tp, p0);
    d1 = pdist<kMetric>(tp, p1);
  }
  const bool one = active && d1 < d0;
  const uint32_t idx = trans ? 3u : (one ? 1u : 0u);
  o.bits = __reduce_or_sync(kFull, lane < 16 ? idx << (2 * lane) : 0u);
  o.score = __reduce_add_sync(kFull, active ? uint32_t(one ? d1 : d0) : 0u);
  if (ACC) {
    const C3 c = texel_c3(px);
    o.n1 = __popc(__ballot_sync(kFull, one));
    o.n0 = __popc(__ballot_sync(kFull, active && !one));
    o.s1r = int(__reduce_add_sync(kFull, one ? uint32_t(c.r) : 0u));
    o.s1g = int(__reduce_add_sync(kFull, one ? uint32_t(c.g) : 0u));
    o.s1b = int(__reduce_add_sync(kFull, one ? uint32_t(c.b) : 0u));
    o.s0r = int(__reduce_add_sync(kFull, active && !one ? uint32_t(c.r) : 0u));
    o.s0g = int(__reduce_add_sync(kFull, active && !one ? uint32_t(c.g) : 0u));
    o.s0b = int(__reduce_add_sync(kFull, active && !one ? uint32_t(c.b) : 0u));
  }
  return o;
}

__device__ __forceinline__ bool warp_means(const WarpColourPass& a, C3& c0, C3& c1) {
  if (!a.n0 && !a.n1) return false;
  if (a.n0) c0 = C3{rmean(a.s0r, a.n0) & 31, rmean(a.s0g, a.n0) & 63, rmean(a.s0b, a.n0) & 31};
  if (a.n1) c1 = C3{rmean(a.s1r, a.n1) & 31, rmean(a.s1g, a.n1) & 63, rmean(a.s1b, a.n1) & 31};
  return true;
}

// colour_refine (s2tc_algorithm.cpp:767-860), warp-parallel; results uniform.
template <bool TRANS, int REFINE>
__device__ __forceinline__ uint32_t colour_refine_warp(bool inb, uint32_t px, const P& tp, C3& c0, C3& c1,
                                                       int lane) {
  uint32_t bits = 0;
  if (REFINE == RF_NEVER) {
    if (TRANS ? c3_lt(c1, c0) : c3_lt(c0, c1)) {
      C3 t = c0; c0 = c1; c1 = t;
    }
    return colour_pass_warp<TRANS, false>(inb, px, tp, c0, c1, lane).bits;
  } else if (REFINE == RF_LOOP) {
    C3 n0 = c0, n1 = c1;
    uint32_t best = 0x7FFFFFFFu;
    for (;;) {
      const WarpColourPass r = colour_pass_warp<TRANS, true>(inb, px, tp, n0, n1, lane);
      if (!(r.score < best)) break;
      bits = r.bits;
      best = r.score;
      c0 = n0;
      c1 = n1;
      if (!warp_means(r, n0, n1)) break;
    }
  } else {
    const WarpColourPass r = colour_pass_warp<TRANS, true>(inb, px, tp, c0, c1, lane);
    bits = r.bits;
    warp_means(r, c0, c1);
  }
  colour_finish<TRANS>(bits, c0, c1);
  return bits;
}

struct WarpAlphaPass {
  uint64_t bits;
  uint32_t score;
  int n0, n1, s0, s1;
};

// alpha index pass with the 0/255 fixed points (s2tc_algorithm.cpp:582-643)
template <bool ACC>
__device__ __forceinline__ WarpAlphaPass alpha_pass_warp(bool inb, uint32_t px, int r0, int r1, int lane) {
  WarpAlphaPass o;
  const int a = int(px >> 24);
  uint32_t idx = 0, d = 0;
  bool e0 = false, e1 = false;
  if (inb) {
    int32_t bd = adist(a, r0), d1 = adist(a, r1);
    int best = 0;
    if (d1 < bd) { bd = d1; best = 1; }
    const int32_t dz = a * a, df = (255 - a) * (255 - a);
    if (dz <= bd) { idx = 6; d = uint32_t(dz); }
    else if (df <= bd) { idx = 7; d = uint32_t(df); }
    else { idx = uint32_t(best); d = uint32_t(bd); e0 = best == 0; e1 = best == 1; }
  }
  const uint32_t lo = __reduce_or_sync(kFull, lane < 10 ? idx << (3 * lane) : 0u);
  const uint32_t hi = __reduce_or_sync(kFull, (lane >= 10 && lane < 16) ? idx << (3 * (lane - 10)) : 0u);
  o.bits = uint64_t(lo) | (uint64_t(hi) << 30);
  o.score = __reduce_add_sync(kFull, d);
  if (ACC) {
    o.n0 = __popc(__ballot_sync(kFull, e0));
    o.n1 = __popc(__ballot_sync(kFull, e1));
    o.s0 = int(__reduce_add_sync(kFull, e0 ? uint32_t(a) : 0u));
    o.s1 = int(__reduce_add_sync(kFull, e1 ? uint32_t(a) : 0u));
  }
  return o;
}

// alpha_refine (s2tc_algorithm.cpp:645-765), warp-parallel; results uniform.
template <int REFINE>
__device__ __forceinline__ uint64_t alpha_refine_warp(bool inb, uint32_t px, int& a0, int& a1, int lane) {
  uint64_t bits = 0;
  if (REFINE == RF_NEVER) {
    if (a1 < a0) { int t = a0; a0 = a1; a1 = t; }
    return alpha_pass_warp<false>(inb, px, a0, a1, lane).bits;
  } else if (REFINE == RF_LOOP) {
    int x0 = a0, x1 = a1;
    uint32_t best = 0x7FFFFFFFu;
    for (;;) {
      const WarpAlphaPass r = alpha_pass_warp<true>(inb, px, x0, x1, lane);
      if (!(r.score < best)) break;
      bits = r.bits;
      best = r.score;
      a0 = x0;
      a1 = x1;
      if (!r.n0 && !r.n1) break;
      if (r.n0) x0 = rmean(r.s0, r.n0) & 255;
      if (r.n1) x1 = rmean(r.s1, r.n1) & 255;
    }
  } else {
    const WarpAlphaPass r = alpha_pass_warp<true>(inb, px, a0, a1, lane);
    bits = r.bits;
    if (r.n0) a0 = rmean(r.s0, r.n0) & 255;
    if (r.n1) a1 = rmean(r.s1, r.n1) & 255;
  }
  alpha_finish(bits, a0, a1);
  return bits;
}

__device__ __forceinline__ uint64_t warp_min_u64(uint64_t v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const uint64_t w = __shfl_xor_sync(kFull, v, o);
    v = w < v ? w : v;
  }
  return v;
}

__device__ __forceinline__ uint32_t vmin_u16x2(uint32_t a, uint32_t b) {
  uint32_t d;
  asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
  return d;
}

// Sum over the 16 inputs of min(row a, row b).
__device__ __forceinline__ int32_t pair_sum(const int4* a, const int4* b) {
  int32_t s = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    s = wadd(s, min(a[q].x, b[q].x));
    s = wadd(s, min(a[q].y, b[q].y));
    s = wadd(s, min(a[q].z, b[q].z));
    s = wadd(s, min(a[q].w, b[q].w));
  }
  return s;
}
// Same for rows of sixteen 16-bit values (two per word).
__device__ __forceinline__ uint32_t pair_sum16(const uint4* a, const uint4* b) {
  uint32_t s = 0;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    s = __dp2a_lo(vmin_u16x2(a[q].x, b[q].x), 0x0101u, s);
    s = __dp2a_lo(vmin_u16x2(a[q].y, b[q].y), 0x0101u, s);
    s = __dp2a_lo(vmin_u16x2(a[q].z, b[q].z), 0x0101u, s);
    s = __dp2a_lo(vmin_u16x2(a[q].w, b[q].w), 0x0101u, s);
  }
  return s;
}
// Sum over the 16 inputs of min(row a, row b)^2 for alpha rows (values <= 255
// in 16-bit halves): four minima packed as bytes, squared and summed by dp4a.
__device__ __forceinline__ uint32_t pair_sq_sum16(const uint4* a, const uint4* b) {
  uint32_t s = 0;
#pragma unroll
  for (int q = 0; q < 2; ++q) {
    uint32_t v = __byte_perm(vmin_u16x2(a[q].x, b[q].x), vmin_u16x2(a[q].y, b[q].y), 0x6420);
    s = __dp4a(v, v, s);
    v = __byte_perm(vmin_u16x2(a[q].z, b[q].z), vmin_u16x2(a[q].w, b[q].w), 0x6420);
    s = __dp4a(v, v, s);
  }
  return s;
}

#ifndef S2TC_PAIR_UNROLL
#define S2TC_PAIR_UNROLL 4
#endif
constexpr int kPairUnroll = S2TC_PAIR_UNROLL;  // partner rows unrolled per tile row
// Walks every pair i < j < mm: 8-row tiles (I, J), I <= J, four groups of
// eight lanes per warp, each group one tile at a time; lane r of a group owns
// row I*8 + r and visits the tile's eight partner rows.  `load(k, row)` reads
// row k, `sum(a, b)` combines two rows, `visit(i, j, s, valid)` sees every
// pair once with `valid` set (and some clamped non-pairs with it clear).
template <class RowT, class Load, class Sum, class Visit>
__device__ __forceinline__ void tiled_pairs(int mm, int lane, Load load, Sum sum, Visit visit) {
  const int g = lane >> 3, r = lane & 7;
  const int nblk = (mm + 7) >> 3;
  const int T = nblk * (nblk + 1) / 2;
  for (int t0 = 0; t0 < T; t0 += 4) {
    const int t = t0 + g;
    int I = 0, rem = t;
    while (I < nblk && rem >= nblk - I) {
      rem -= nblk - I;
      ++I;
    }
    const bool ok = t < T;
    const int J = I + rem;
    const int i = I * 8 + r;
    RowT ri;
    load(min(i, mm - 1), ri);
#pragma unroll kPairUnroll
    for (int jj = 0; jj < 8; ++jj) {
      const int j = J * 8 + jj;
      RowT rj;
      load(min(j, mm - 1), rj);
      const auto v = sum(ri, rj);
      visit(i, j, v, ok && j < mm && j > i);
    }
  }
}

struct RowI32 {
  int4 q[4];
};
struct RowU16 {
  uint4 q[2];
};

// Unique candidates in index order.  Equal candidates have equal distance
// rows under a symmetric metric, hence equal pair sums, and the reference's
// first minimum is then always a pair of first occurrences (i, j) or a pair
// (x, y) of a value's first occurrence and its first repeat (its sum is the
// row sum of x).  `slot(j)` maps candidate j into [0, nslots) (equal slots
// for equal candidates); without a table (nslots == 0) every candidate is
// unique.  Writes the unique indices to `uniq`, and for each unique x its
// first repeat (or 0xFFFFFFFF) to tab[kDedupSlots + slot(x)]; returns the count.
template <class Slot>
__device__ __forceinline__ int dedup(int mm, int lane, int nslots, Slot slot, uint16_t* uniq, uint32_t* tab) {
  if (nslots == 0) {
    for (int j = lane; j < mm; j += 32) uniq[j] = uint16_t(j);
    __syncwarp();
    return mm;
  }
  uint32_t* first = tab;
  uint32_t* rep = tab + kDedupSlots;
  for (int k = lane; k < nslots; k += 32) {
    first[k] = 0xFFFFFFFFu;
    rep[k] = 0xFFFFFFFFu;
  }
  __syncwarp();
  for (int j = lane; j < mm; j += 32) atomicMin(first + slot(j), uint32_t(j));
  __syncwarp();
  int nu = 0;
  for (int base = 0; base < mm; base += 32) {
    const int j = base + lane;
    bool u = false;
    if (j < mm) {
      const int sj = slot(j);
      u = first[sj] == uint32_t(j);
      if (!u) atomicMin(rep + sj, uint32_t(j));
    }
    const unsigned bal = __ballot_sync(kFull, u);
    if (u) uniq[nu + __popc(bal & ((1u << lane) - 1u))] = uint16_t(j);
    nu += __popc(bal);
  }
  __syncwarp();
  return nu;
}

// CTAs per SM the register budget allows: at 64 random candidates a CTA of
// four warps holds about 22 KB of shared memory with 16-bit distance rows
// (seven CTAs: 72 registers, measured 5% faster than five on the mip chains)
// and 35 KB with 32-bit rows (six CTAs: 80 registers and a few spilled words,
// 1.4% faster than five on a normal map).
#ifndef S2TC_RAND_MINBLOCKS
#define S2TC_RAND_MINBLOCKS (kSmallDist ? 7 : 6)
#endif
template <int DXT, int REFINE>
__global__ void __launch_bounds__(32 * kRandWarps, S2TC_RAND_MINBLOCKS) k_encode_rand(EncodeWork w, int m) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const RandLayout L = rand_layout(m);
  unsigned char* base = smem + size_t(warp) * L.bytes;
  P* sP = reinterpret_cast<P*>(base + L.p);
  uint16_t* sC = reinterpret_cast<uint16_t*>(base + L.c);
  uint8_t* sA = base + L.a;
  unsigned char* sD = base + L.d;  // colour rows, kRowBytes each (row a: a-th unique candidate)
  unsigned char* sE = base + L.e;  // alpha rows, 32 bytes each
  uint16_t* sUc = reinterpret_cast<uint16_t*>(base + L.u);  // unique colour candidates
  uint16_t* sUa = sUc + m;                                   // unique alpha candidates
  uint32_t* sTab = reinterpret_cast<uint32_t*>(base + L.t);
  const int nrandom = w.nrandom;
  const int stride = DXT == DXT5 ? 4 : 3;
  const long long nb = w.total;

  const int warps = int(blockDim.x >> 5);
  for (long long g = (long long)blockIdx.x * warps + warp; g < nb; g += (long long)gridDim.x * warps) {
    EncodeArgs a;
    long long bl;
    resolve(w, g, a, bl);
    const long long b = (long long)a.by0 * a.bw + bl;
    const int by = int(b / a.bw), bx = int(b % a.bw);
    const int bw_ = min(4, a.width - bx * 4), bh_ = min(4, a.height - by * 4);
    // lanes 0..15 hold the block's slots (y*4 + x)
    const int sx = lane & 3, sy = (lane >> 2) & 3;
    const bool inb = lane < 16 && sx < bw_ && sy < bh_;
    uint32_t px = 0;
    if (inb) px = __ldg(a.t565 + (size_t(by) * 4 + sy) * a.width + size_t(bx) * 4 + sx);
    const bool valid = inb && !(DXT == DXT1 && (px >> 24) == 0);
    const int pos = sx * 4 + sy;  // x-outer, y-inner input order (:940-951)
    const unsigned mask = __reduce_or_sync(kFull, valid ? 1u << pos : 0u);
    int n = __popc(mask);
    const C3 c = texel_c3(px);
    const P tp = prep<kMetric>(c);
    if (valid) {
      const int rank = __popc(mask & ((1u << pos) - 1u));
      sP[rank] = tp;
      sC[rank] = uint16_t(pack565(c));
      sA[rank] = uint8_t(px >> 24);
    }
    // bounding box of the inputs (:962-983); an empty block has one black input
    C3 lo, hi;
    lo.r = int(__reduce_min_sync(kFull, valid ? unsigned(c.r) : 255u));
    lo.g = int(__reduce_min_sync(kFull, valid ? unsigned(c.g) : 255u));
    lo.b = int(__reduce_min_sync(kFull, valid ? unsigned(c.b) : 255u));
    hi.r = int(__reduce_max_sync(kFull, valid ? unsigned(c.r) : 0u));
    hi.g = int(__reduce_max_sync(kFull, valid ? unsigned(c.g) : 0u));
    hi.b = int(__reduce_max_sync(kFull, valid ? unsigned(c.b) : 0u));
    int alo = 0, ahi = 0;
    if (DXT == DXT5) {
      alo = int(__reduce_min_sync(kFull, valid ? (px >> 24) : 255u));
      ahi = int(__reduce_max_sync(kFull, valid ? (px >> 24) : 0u));
    }
    if (n == 0) {
      n = 1;
      lo = hi = C3{0, 0, 0};
      alo = ahi = 0;
      if (lane == 0) {
        sP[0] = prep<kMetric>(C3{0, 0, 0});
        sC[0] = 0;
        sA[0] = 0;
      }
    }
    const int mm = n + nrandom;
    const int lr = hi.r - lo.r + 1, lg = hi.g - lo.g + 1, lb = hi.b - lo.b + 1, la = ahi - alo + 1;
    // random candidates (:984-992), rand() words in the reference's call order
    const uint32_t* rnd = a.rnd + size_t(bl) * size_t(nrandom) * stride;
    for (int j = n + lane; j < mm; j += 32) {
      const uint32_t* r = rnd + size_t(j - n) * stride;
      const C3 cj{lo.r + int(__ldg(r) % uint32_t(lr)), lo.g + int(__ldg(r + 1) % uint32_t(lg)),
                  lo.b + int(__ldg(r + 2) % uint32_t(lb))};
      sP[j] = prep<kMetric>(cj);
      sC[j] = uint16_t(pack565(cj));
      if (DXT == DXT5) sA[j] = uint8_t(alo + int(__ldg(r + 3) % uint32_t(la)));
    }
    __syncwarp();
    // deduplicate the colour candidates (symmetric metrics, small boxes)
    const int cbox = lr * lg * lb;
    const int ncs = (kSymmetric && cbox <= kDedupSlots) ? cbox : 0;
    const int nuc = dedup(mm, lane, ncs,
                          [&](int j) {
                            const C3 q = unpack565(sC[j]);
                            return ((q.r - lo.r) * lg + (q.g - lo.g)) * lb + (q.b - lo.b);
                          },
                          sUc, sTab);
    // distance rows against the inputs (:375-392); entries k >= n are 0
    for (int ua = lane; ua < nuc; ua += 32) {
      const int i = sUc[ua];
      const P pi = sP[i];
      int32_t row[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        int32_t d = 0;
        if (k < n && k != i) {
          const P pk = sP[k];
          d = (kSymmetric || i >= n || i < k) ? pdist<kMetric>(pi, pk) : pdist<kMetric>(pk, pi);
        }
        row[k] = d;
      }
      if (kSmallDist) {
        uint4* dr = reinterpret_cast<uint4*>(sD + size_t(ua) * kRowBytes);
#pragma unroll
        for (int q = 0; q < 2; ++q)
          dr[q] = make_uint4(uint32_t(row[8 * q]) | (uint32_t(row[8 * q + 1]) << 16),
                             uint32_t(row[8 * q + 2]) | (uint32_t(row[8 * q + 3]) << 16),
                             uint32_t(row[8 * q + 4]) | (uint32_t(row[8 * q + 5]) << 16),
                             uint32_t(row[8 * q + 6]) | (uint32_t(row[8 * q + 7]) << 16));
      } else {
        int4* dr = reinterpret_cast<int4*>(sD + size_t(ua) * kRowBytes);
#pragma unroll
        for (int q = 0; q < 4; ++q) dr[q] = make_int4(row[4 * q], row[4 * q + 1], row[4 * q + 2], row[4 * q + 3]);
      }
    }
    __syncwarp();

    // colour pair search: the smallest (sum, i, j) is the pair the
    // reference keeps when no sum is negative
    int ci, cj;
    {
      uint64_t best = ~0ull;
      bool neg = false;
      if (kSmallDist && nuc <= kKeyPositions) {
        // 32-bit keys (sum << 13 | a * 90 + b): the sums of 16-bit rows stay
        // below 2^19, and the unique list is in ascending candidate order, so
        // its positions order pairs as the candidates' indices do
        uint32_t best32 = 0xFFFFFFFFu;
        tiled_pairs<RowU16>(
            nuc, lane,
            [&](int k, RowU16& rw) {
              const uint4* q = reinterpret_cast<const uint4*>(sD + size_t(k) * kRowBytes);
              rw.q[0] = q[0];
              rw.q[1] = q[1];
            },
            [](const RowU16& x, const RowU16& y) { return pair_sum16(x.q, y.q); },
            [&](int a, int b, uint32_t v, bool valid) {
              const uint32_t key = (v << 13) | uint32_t(a * kKeyPositions + b);
              best32 = min(best32, valid ? key : 0xFFFFFFFFu);
            });
        best32 = __reduce_min_sync(kFull, best32);
        if (best32 != 0xFFFFFFFFu) {  // none when every candidate has one value
          const int pa = int((best32 & 8191u) / kKeyPositions), pb = int((best32 & 8191u) % kKeyPositions);
          best = (uint64_t(best32 >> 13) << 32) | (uint32_t(ncs ? sUc[pa] : pa) << 16) | uint32_t(ncs ? sUc[pb] : pb);
        }
      } else if (kSmallDist) {
        tiled_pairs<RowU16>(
            nuc, lane,
            [&](int k, RowU16& rw) {
              const uint4* q = reinterpret_cast<const uint4*>(sD + size_t(k) * kRowBytes);
              rw.q[0] = q[0];
              rw.q[1] = q[1];
            },
            [](const RowU16& x, const RowU16& y) { return pair_sum16(x.q, y.q); },
            [&](int a, int b, uint32_t v, bool valid) {
              if (!valid || v > uint32_t(best >> 32)) return;  // cannot win; skip the index lookups
              const uint32_t ia = ncs ? sUc[a] : a, ib = ncs ? sUc[b] : b;
              const uint64_t key = (uint64_t(v) << 32) | (ia << 16) | ib;
              best = key < best ? key : best;
            });
      } else {
        tiled_pairs<RowI32>(
            nuc, lane,
            [&](int k, RowI32& rw) {
              const int4* q = reinterpret_cast<const int4*>(sD + size_t(k) * kRowBytes);
#pragma unroll
              for (int t = 0; t < 4; ++t) rw.q[t] = q[t];
            },
            [](const RowI32& x, const RowI32& y) { return pair_sum(x.q, y.q); },
            [&](int a, int b, int32_t v, bool valid) {
              if (!valid) return;
              neg |= v < 0;
              if (v < 0 || uint32_t(v) > uint32_t(best >> 32)) return;
              const uint32_t ia = ncs ? sUc[a] : a, ib = ncs ? sUc[b] : b;
              const uint64_t key = (uint64_t(uint32_t(v)) << 32) | (ia << 16) | ib;
              best = key < best ? key : best;
            });
      }
      if (ncs > 0) {
        // pairs of a value's first occurrence and its first repeat: the row sum
        for (int ua = lane; ua < nuc; ua += 32) {
          const int x = sUc[ua];
          const C3 q = unpack565(sC[x]);
          const uint32_t y = sTab[kDedupSlots + ((q.r - lo.r) * lg + (q.g - lo.g)) * lb + (q.b - lo.b)];
          if (y == 0xFFFFFFFFu) continue;
          int32_t v = 0;
          if (kSmallDist) {
            const uint4* r = reinterpret_cast<const uint4*>(sD + size_t(ua) * kRowBytes);
            uint32_t t = 0;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
              t = __dp2a_lo(r[h].x, 0x0101u, t);
              t = __dp2a_lo(r[h].y, 0x0101u, t);
              t = __dp2a_lo(r[h].z, 0x0101u, t);
              t = __dp2a_lo(r[h].w, 0x0101u, t);
            }
            v = int32_t(t);
          } else {
            const int32_t* r = reinterpret_cast<const int32_t*>(sD + size_t(ua) * kRowBytes);
            for (int k = 0; k < 16; ++k) v = wadd(v, r[k]);
          }
          neg |= v < 0;
          const uint64_t key = (uint64_t(uint32_t(v)) << 32) | (uint32_t(x) << 16) | y;
          if (v >= 0 && key < best) best = key;
        }
      }
      if (!kSmallDist && __any_sync(kFull, neg)) {
        // negative sums: replay the reference's rule in pair order on one lane
        int bi = 0, bj = 1;
        if (lane == 0) {
          // rows of the original candidates, recomputed (rare path)
          auto dist_ik = [&](int i, int k) -> int32_t {
            if (k >= n || k == i) return 0;
            return (kSymmetric || i >= n || i < k) ? pdist<kMetric>(sP[i], sP[k]) : pdist<kMetric>(sP[k], sP[i]);
          };
          int32_t bestsum = -1;
          for (int i = 0; i < mm; ++i)
            for (int j = i + 1; j < mm; ++j) {
              int32_t sum = 0;
              for (int k = 0; k < 16; ++k) sum = wadd(sum, min(dist_ik(i, k), dist_ik(j, k)));
              if (bestsum < 0 || sum < bestsum) {
                bestsum = sum;
                bi = i;
                bj = j;
              }
            }
        }
        ci = __shfl_sync(kFull, bi, 0);
        cj = __shfl_sync(kFull, bj, 0);
      } else {
        best = warp_min_u64(best);
        ci = int((best >> 16) & 0xFFFF);
        cj = int(best & 0xFFFF);
      }
    }
    C3 c0 = unpack565(sC[ci]), c1 = unpack565(sC[cj]);
    int a0 = 0, a1 = 0;
    if (DXT == DXT5) {
      // alpha pair search (:415-478) over the distinct alpha values; sums of
      // squares of bytes never overflow
      __syncwarp();
      const int nua = dedup(mm, lane, 256, [&](int j) { return int(sA[j]); }, sUa, sTab);
      for (int ua = lane; ua < nua; ua += 32) {
        const int ai = sA[sUa[ua]];
        uint32_t v[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) {
          const int ak = sA[k];
          v[k] = k < n ? uint32_t(min(abs(ai - ak), min(ak, 255 - ak))) : 0u;
        }
        uint4* er = reinterpret_cast<uint4*>(sE + size_t(ua) * 32);
        er[0] = make_uint4(v[0] | (v[1] << 16), v[2] | (v[3] << 16), v[4] | (v[5] << 16), v[6] | (v[7] << 16));
        er[1] = make_uint4(v[8] | (v[9] << 16), v[10] | (v[11] << 16), v[12] | (v[13] << 16), v[14] | (v[15] << 16));
      }
      __syncwarp();
      uint64_t best = ~0ull;
      if (nua <= kKeyPositions) {
        // 32-bit keys: a capped alpha distance is at most 127, so the sums stay
        // below 16 * 127^2 < 2^18 (see the colour search)
        uint32_t best32 = 0xFFFFFFFFu;
        tiled_pairs<RowU16>(
            nua, lane,
            [&](int k, RowU16& rw) {
              const uint4* q = reinterpret_cast<const uint4*>(sE + size_t(k) * 32);
              rw.q[0] = q[0];
              rw.q[1] = q[1];
            },
            [](const RowU16& x, const RowU16& y) { return pair_sq_sum16(x.q, y.q); },
            [&](int a, int b, uint32_t v, bool valid) {
              const uint32_t key = (v << 13) | uint32_t(a * kKeyPositions + b);
              best32 = min(best32, valid ? key : 0xFFFFFFFFu);
            });
        best32 = __reduce_min_sync(kFull, best32);
        if (best32 != 0xFFFFFFFFu) {
          const int pa = int((best32 & 8191u) / kKeyPositions), pb = int((best32 & 8191u) % kKeyPositions);
          best = (uint64_t(best32 >> 13) << 32) | (uint32_t(sUa[pa]) << 16) | uint32_t(sUa[pb]);
        }
      } else {
        tiled_pairs<RowU16>(
            nua, lane,
            [&](int k, RowU16& rw) {
              const uint4* q = reinterpret_cast<const uint4*>(sE + size_t(k) * 32);
              rw.q[0] = q[0];
              rw.q[1] = q[1];
            },
            [](const RowU16& x, const RowU16& y) { return pair_sq_sum16(x.q, y.q); },
            [&](int a, int b, uint32_t v, bool valid) {
              if (!valid || v > uint32_t(best >> 32)) return;
              const uint64_t key = (uint64_t(v) << 32) | (uint32_t(sUa[a]) << 16) | uint32_t(sUa[b]);
              best = key < best ? key : best;
            });
      }
      for (int ua = lane; ua < nua; ua += 32) {
        const int x = sUa[ua];
        const uint32_t y = sTab[kDedupSlots + sA[x]];
        if (y == 0xFFFFFFFFu) continue;
        const uint4* r = reinterpret_cast<const uint4*>(sE + size_t(ua) * 32);
        uint32_t t = 0;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint32_t p = __byte_perm(r[h].x, r[h].y, 0x6420);
          t = __dp4a(p, p, t);
          p = __byte_perm(r[h].z, r[h].w, 0x6420);
          t = __dp4a(p, p, t);
        }
        const uint64_t key = (uint64_t(t) << 32) | (uint32_t(x) << 16) | y;
        best = key < best ? key : best;
      }
      best = warp_min_u64(best);
      a0 = sA[(best >> 16) & 0xFFFF];
      a1 = sA[best & 0xFFFF];
    }
    __syncwarp();  // the next block overwrites the candidate lists

    // equal endpoints are bumped apart (:1009-1027)
    if (c3_eq(c0, c1)) c1 = (c0.r == 31 && c0.g == 63 && c0.b == 31) ? c3_prev(c1) : c3_next(c1);
    if (DXT == DXT5 && a0 == a1) {
      if (a0 == 255) --a1; else ++a1;
    }
    const uint32_t cbits = colour_refine_warp<DXT == DXT1, REFINE>(inb, px, tp, c0, c1, lane);
    EncodedBlock eb;
    const uint64_t colour = uint64_t(pack565(c0)) | (uint64_t(pack565(c1)) << 16) | (uint64_t(cbits) << 32);
    if (DXT == DXT1) {
      eb.lo = colour;
      eb.hi = 0;
    } else if (DXT == DXT3) {
      const uint32_t nib = inb ? ((px >> 24) & 15) : 0u;
      const uint32_t lo32 = __reduce_or_sync(kFull, lane < 8 ? nib << (4 * lane) : 0u);
      const uint32_t hi32 = __reduce_or_sync(kFull, (lane >= 8 && lane < 16) ? nib << (4 * (lane - 8)) : 0u);
      eb.lo = uint64_t(lo32) | (uint64_t(hi32) << 32);
      eb.hi = colour;
    } else {
      const uint64_t abits = alpha_refine_warp<REFINE>(inb, px, a0, a1, lane);
      eb.lo = uint64_t(a0) | (uint64_t(a1) << 8) | (abits << 16);
      eb.hi = colour;
    }
    if (lane == 0) store_block(a, DXT, bx, by, eb);
  }
}

// Shared memory the warp kernel needs for `m` candidates and `warps` warps per
// CTA, or 0 when it does not fit (the thread-per-block kernel then handles
// the launch).
size_t rand_smem_bytes(int m, int warps) {
  const size_t bytes = rand_layout(m).bytes * warps;
  return bytes <= 200 * 1024 ? bytes : 0;
}

// Raises the kernel's dynamic shared memory limit only when a launch needs more
// than any earlier one (the attribute persists), then launches.
template <int DXT, int REFINE>
cudaError_t launch_rand(const EncodeWork& a, int m, size_t smem, unsigned grid, int warps, cudaStream_t s) {
  static int limit = 48 * 1024;
  if (int(smem) > limit) {
    const cudaError_t e =
        cudaFuncSetAttribute(k_encode_rand<DXT, REFINE>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
    if (e != cudaSuccess) return e;
    limit = int(smem);
  }
  k_encode_rand<DXT, REFINE><<<grid, 32 * warps, smem, s>>>(a, m);
  return cudaGetLastError();
}

// The launch layout comes from the tuning table (encode_layout): threads per
// CTA of the thread-per-block kernels, and warps per CTA and CTAs per SM of
// the warp kernel's persistent grid.  Every layout encodes the same bytes.
template <int DXT, bool NORMAL>
cudaError_t launch_r(const EncodeWork& a, int refine, cudaStream_t s) {
  const long long nb = a.total;
  if (nb == 0) return cudaSuccess;
  if (NORMAL && a.nrandom > 0) {
    const EncodeLayout L = encode_layout(kMetric, DXT, refine, kLayoutRand);
    const int warps = std::max(1, std::min(kRandWarps, L.rand_warps));
    const int m = 16 + a.nrandom;
    const size_t smem = rand_smem_bytes(m, warps);
    if (smem > 0) {
      count_launches(1);
      const unsigned rgrid =
          unsigned(std::min<long long>((nb + warps - 1) / warps, 152ll * std::max(1, L.rand_ctas_per_sm)));
      switch (refine) {
        case RF_NEVER: return launch_rand<DXT, RF_NEVER>(a, m, smem, rgrid, warps, s);
        case RF_LOOP: return launch_rand<DXT, RF_LOOP>(a, m, smem, rgrid, warps, s);
        default: return launch_rand<DXT, RF_ALWAYS>(a, m, smem, rgrid, warps, s);
      }
    }
  }
  const int kind = NORMAL ? (a.nrandom > 0 ? kLayoutRand : kLayoutFull) : kLayoutQuick;
  const EncodeLayout L = encode_layout(kMetric, DXT, refine, kind);
  const int threads = std::max(32, std::min(kThreadsPerCta, L.threads & ~31));
  const unsigned grid = unsigned((nb + threads - 1) / threads);
  if (NORMAL && a.nrandom <= 0) {
    // the full-block kernel's shared columns are laid out for kThreadsPerCta
    const unsigned grid16 = unsigned((nb + kThreadsPerCta - 1) / kThreadsPerCta);
    count_launches(1);
    switch (refine) {
      case RF_NEVER: k_encode_full16<DXT, RF_NEVER><<<grid16, kThreadsPerCta, 0, s>>>(a); break;
      case RF_LOOP: k_encode_full16<DXT, RF_LOOP><<<grid16, kThreadsPerCta, 0, s>>>(a); break;
      default: k_encode_full16<DXT, RF_ALWAYS><<<grid16, kThreadsPerCta, 0, s>>>(a); break;
    }
    // every block of a DXT3/DXT5 image whose sides are multiples of 4 is
    // whole, and k_encode would leave every one of them
    if (DXT != DXT1 && !a.items && a.single.width % 4 == 0 && a.single.height % 4 == 0)
      return cudaGetLastError();
  }
  count_launches(1);
  switch (refine) {
    case RF_NEVER: k_encode<DXT, NORMAL, RF_NEVER><<<grid, threads, 0, s>>>(a); break;
    case RF_LOOP: k_encode<DXT, NORMAL, RF_LOOP><<<grid, threads, 0, s>>>(a); break;
    default: k_encode<DXT, NORMAL, RF_ALWAYS><<<grid, threads, 0, s>>>(a); break;
  }
  return cudaGetLastError();
}

template <int DXT>
cudaError_t launch_d(const EncodeWork& a, bool normal, int refine, cudaStream_t s) {
  // NORMALMAP never uses the quick selection (s2tc_algorithm.cpp:1127-1143)
  if (normal || kMetric == CD_NORMALMAP) return launch_r<DXT, true>(a, refine, s);
  return launch_r<DXT, (kMetric == CD_NORMALMAP)>(a, refine, s);
}

// ------------------------------------------------------------------------
// Fused strip kernel of the quick mode: the NONE or SIMPLE dither and the
// quick encoder (darkest/brightest selection) in one launch.
//
// A CTA takes a band of whole block rows, i.e. one contiguous raster range of
// the image: 4 * rows_per_band texel rows.  RGBA8 sources come in by the TMA
// unit: the image seen as a 2-D tensor of rows of 256 texels (one 32-bit word
// each), one cp.async.bulk.tensor copy per row, issued by the 32 lanes of warp
// 0 and completing on one mbarrier.  The inner coordinate is always 0, so
// every copy starts on a 16-byte boundary; the band begins `p0 % 256` words
// into the first row, and the texels after the last whole row of the image
// come in by plain loads.  Other sources (RGB8, unaligned) take vector loads.
// The band's SIMPLE scan is the dither kernel's (dither_scan.cuh), chained
// to the bands before it by the same decoupled look-back; its 5:6:5 words
// stay in shared memory, where the band's blocks are read and encoded, one
// thread per block, and written out in block order.  HBM then sees the
// source once and the blocks once.

constexpr int kStripPad = 512;  // words before the band: its offset in the first tensor row, and the last row's rest
template <int SEG>
using StripSmem = ScanSmem<kStripThreads, SEG, kStripPad>;

__device__ __forceinline__ void tma_row(uint32_t dst, const CUtensorMap* map, int row, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
      "[%4];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(0), "r"(row), "r"(mbar)
      : "memory");
}

// RGBA word of texel i of a packed RGBA8 image.
__device__ __forceinline__ uint32_t rgba_word(const uint8_t* src, long long i) {
  const uint8_t* b = src + 4 * i;
  if ((reinterpret_cast<uintptr_t>(b) & 3) == 0) return __ldg(reinterpret_cast<const uint32_t*>(b));
  return uint32_t(b[0]) | (uint32_t(b[1]) << 8) | (uint32_t(b[2]) << 16) | (uint32_t(b[3]) << 24);
}

// Two CTAs per SM (128 registers); three (85 registers, with spills) measured
// the same.
template <int DXT, int REFINE, int SEG>
__global__ void __launch_bounds__(kStripThreads, 2) k_strip_quick(const __grid_constant__ CUtensorMap tmap,
                                                                  StripArgs a) {
  extern __shared__ unsigned char smem_raw[];
  StripSmem<SEG>& sm =
      *reinterpret_cast<StripSmem<SEG>*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  __shared__ unsigned int s_ticket;
  const int t = threadIdx.x;
  init_tables(sm);
  if (t == 0) s_ticket = a.single_band ? blockIdx.x : atomicAdd(a.scan.ticket, 1u);
  bulk_init(sm);
  __syncthreads();
  if ((long long)s_ticket >= a.nbands) return;
  const long long band = a.band_base + s_ticket;
  const int W = a.width, H = a.height, bw = (W + 3) / 4, bh = (H + 3) / 4;
  const int by0 = int(band * a.rows_per_band);
  const int nby = min(a.rows_per_band, bh - by0);
  const int rows = min(4 * nby, H - 4 * by0);
  const long long p0 = (long long)by0 * 4 * W;
  const int n = rows * W;
  uint32_t* base = sm.px;
  if (a.use_tma) {
    base = sm.px + int(p0 & 255);
    const long long row0 = p0 >> 8;
    const long long covered = a.tma_rows << 8;  // texels inside the tensor
    const long long end = min(p0 + n, covered);
    const int nrows = end > (row0 << 8) ? int((end - (row0 << 8) + 255) >> 8) : 0;
    const uint32_t mbar = smem_u32(&sm.mbar);
    if (t < 32) {
      if (t == 0)
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(uint32_t(nrows) * 1024u)
                     : "memory");
      __syncwarp();
      for (int r = t; r < nrows; r += 32) tma_row(smem_u32(sm.px + r * 256), &tmap, int(row0 + r), mbar);
    }
    int spins = 0;
    while (!mbar_try_wait(mbar, 0) && ++spins < kBulkSpins) {
    }
    // one decision for the whole CTA (the branch below has a barrier)
    if (__syncthreads_or(spins >= kBulkSpins)) {
      // the copies did not complete within the bounded wait: the call reports
      // S2TC_ERR_TIMEOUT (output undefined); the band goes on with plain loads
      // after a second bounded wait, so that the bands behind it do not wait
      // out their own limits
      if (t == 0) atomicExch(a.scan.error, 1);
      bulk_load_wait(sm);
      __syncthreads();
      for (int i = t; i < n; i += kStripThreads) base[i] = rgba_word(a.src, p0 + i);
    }
    for (long long i = max(p0, covered) - p0 + t; i < n; i += kStripThreads) base[i] = rgba_word(a.src, p0 + i);
  } else {
    load_tile<kStripThreads>(DitherItem{a.src, W, H, a.srccomps, a.alphabits, nullptr}, p0, n, base);
  }
  __syncthreads();
  if (a.dither == DI_SIMPLE) {
    if (a.srccomps == 3) simple_tile<0>(a.alphabits, band, band, n, a.scan, sm, base);
    else if (a.alphabits == 1) simple_tile<1>(a.alphabits, band, band, n, a.scan, sm, base);
    else if (a.alphabits == 4) simple_tile<4>(a.alphabits, band, band, n, a.scan, sm, base);
    else simple_tile<8>(a.alphabits, band, band, n, a.scan, sm, base);
  } else {
    // DITHER_NONE (s2tc_algorithm.cpp:1269-1305): plain truncation
    const uint32_t ac = uint32_t((1 << a.alphabits) - 1);
    const int ash = 8 - a.alphabits;
    for (int i = t; i < n; i += kStripThreads) {
      const uint32_t q = base[i];
      const uint32_t al = a.srccomps == 3 ? ac : (q >> 24) >> ash;
      base[i] = ((q & 0xFFu) >> 3) | ((((q >> 8) & 0xFFu) >> 2) << 8) | ((((q >> 16) & 0xFFu) >> 3) << 16) | (al << 24);
    }
  }
  __syncthreads();
  // the band's blocks, one thread per block, in block order
  const bool vec = (W & 3) == 0;
  for (int k = t; k < nby * bw; k += kStripThreads) {
    const int ly = k / bw, bx = k - ly * bw;
    BlockTexels bt;
    bt.w = min(4, W - 4 * bx);
    bt.h = min(4, rows - 4 * ly);
    const uint32_t* q = base + 4 * ly * W + 4 * bx;
    if (vec && bt.w == 4 && bt.h == 4) {
#pragma unroll
      for (int y = 0; y < 4; ++y) {
        const uint4 v = *reinterpret_cast<const uint4*>(q + y * W);
        bt.px[y * 4 + 0] = v.x;
        bt.px[y * 4 + 1] = v.y;
        bt.px[y * 4 + 2] = v.z;
        bt.px[y * 4 + 3] = v.w;
      }
    } else {
#pragma unroll
      for (int y = 0; y < 4; ++y)
#pragma unroll
        for (int x = 0; x < 4; ++x) bt.px[y * 4 + x] = (x < bt.w && y < bt.h) ? q[y * W + x] : 0u;
    }
    EncodedBlock eb;
    encode_block<DXT, false, REFINE, false>(bt, -1, nullptr, -1, eb, nullptr);
    uint8_t* o = a.dst + (size_t)(by0 + ly) * a.pitch + (size_t)bx * (DXT == DXT1 ? 8 : 16);
    if (a.aligned) {
      if (DXT == DXT1) *reinterpret_cast<uint64_t*>(o) = eb.lo;
      else *reinterpret_cast<ulonglong2*>(o) = make_ulonglong2(eb.lo, eb.hi);
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) o[i] = uint8_t(eb.lo >> (8 * i));
      if (DXT != DXT1) {
#pragma unroll
        for (int i = 0; i < 8; ++i) o[8 + i] = uint8_t(eb.hi >> (8 * i));
      }
    }
  }
  if (a.done_flag) {
    // every thread's blocks are visible system-wide before the last band to
    // finish raises the flag that the host polls
    __threadfence_system();
    __syncthreads();
    if (t == 0) {
      const unsigned int prev = a.single_band ? 0u : atomicAdd(a.done_count, 1u);
      if ((long long)prev + 1 == a.nbands) {
        __threadfence_system();
        *reinterpret_cast<volatile int*>(a.done_flag) = 1;
      }
    }
  }
}

template <int DXT, int REFINE, int SEG>
cudaError_t launch_strip_k(const StripArgs& a, const CUtensorMap& map, cudaStream_t s) {
  const size_t smem = sizeof(StripSmem<SEG>) + 128;
  static const cudaError_t attr = cudaFuncSetAttribute(k_strip_quick<DXT, REFINE, SEG>,
                                                       cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  if (attr != cudaSuccess) return attr;
  count_launches(1);
  k_strip_quick<DXT, REFINE, SEG><<<unsigned(a.nbands), kStripThreads, smem, s>>>(map, a);
  return cudaGetLastError();
}

template <int DXT, int REFINE>
cudaError_t launch_strip_r(const StripArgs& a, const CUtensorMap& map, cudaStream_t s) {
  return a.seg == 65 ? launch_strip_k<DXT, REFINE, 65>(a, map, s) : launch_strip_k<DXT, REFINE, 17>(a, map, s);
}

template <int DXT>
cudaError_t launch_strip_d(const StripArgs& a, const CUtensorMap& map, int refine, cudaStream_t s) {
  switch (refine) {
    case RF_NEVER: return launch_strip_r<DXT, RF_NEVER>(a, map, s);
    case RF_LOOP: return launch_strip_r<DXT, RF_LOOP>(a, map, s);
    default: return launch_strip_r<DXT, RF_ALWAYS>(a, map, s);
  }
}

#if S2TC_METRIC == 7
__global__ void k_nm_table() {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < (1 << 16)) {
    const NUnit v = nm_unit(C3{(k >> 11) & 31, (k >> 5) & 63, k & 31});
    g_nm_table[k] = make_float4(v.x, v.y, v.z, 0.0f);
  }
}
__global__ void k_nm_ready() { g_nm_ready = 1; }
#endif

}  // namespace

#define S2TC_CAT2(a, b) a##b
#define S2TC_CAT(a, b) S2TC_CAT2(a, b)

#if S2TC_METRIC == 7
cudaError_t nm_table_init(cudaStream_t s) {
  count_launches(2);
  k_nm_table<<<256, 256, 0, s>>>();
  k_nm_ready<<<1, 1, 0, s>>>();
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  return e;
}
#endif

cudaError_t S2TC_CAT(launch_strip_m, S2TC_METRIC)(StripArgs a, const void* tmap, int dxt, int refine,
                                                  uint8_t* scratch, cudaStream_t s) {
  // NORMALMAP never uses the quick selection (s2tc_algorithm.cpp:1127-1143)
  if (kMetric == CD_NORMALMAP || a.nbands <= 0) return kMetric == CD_NORMALMAP ? cudaErrorNotSupported : cudaSuccess;
  if (a.seg != 65 && a.seg != 17) return cudaErrorInvalidValue;
  if (a.band_base < 0 || a.band_base + a.nbands > a.image_bands) return cudaErrorInvalidValue;
  dither_test_hold_values(&a.scan.hold_tile, &a.scan.spin_limit);
  if (scratch) {
    // the layout of launch_dither_batch's scratch for image_bands tiles
    a.scan.status = reinterpret_cast<unsigned long long*>(scratch);
    a.scan.aggs = scratch + a.image_bands * sizeof(unsigned long long);
    uintptr_t tk = reinterpret_cast<uintptr_t>(a.scan.aggs + a.image_bands * kRecWords * 4);
    a.scan.ticket = reinterpret_cast<unsigned int*>((tk + 15) & ~uintptr_t(15));
    cudaError_t e = cudaMemsetAsync(a.scan.status + a.band_base, 0, a.nbands * sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(a.scan.ticket, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return e;
  } else if (!a.scan.status || !a.scan.aggs || (!a.scan.ticket && !a.single_band) || a.band_base != 0 ||
             (a.single_band && a.nbands != 1)) {
    return cudaErrorInvalidValue;
  }
  if (a.done_flag && !a.done_count && !a.single_band) return cudaErrorInvalidValue;
  CUtensorMap map;
  if (a.use_tma) map = *static_cast<const CUtensorMap*>(tmap);
  else std::memset(&map, 0, sizeof(map));
  switch (dxt) {
    case DXT1: return launch_strip_d<DXT1>(a, map, refine, s);
    case DXT3: return launch_strip_d<DXT3>(a, map, refine, s);
    default: return launch_strip_d<DXT5>(a, map, refine, s);
  }
}

cudaError_t S2TC_CAT(launch_encode_m, S2TC_METRIC)(const EncodeWork& a, int dxt, bool normal, int refine,
                                                   cudaStream_t s) {
  switch (dxt) {
    case DXT1: return launch_d<DXT1>(a, normal, refine, s);
    case DXT3: return launch_d<DXT3>(a, normal, refine, s);
    default: return launch_d<DXT5>(a, normal, refine, s);
  }
}

}  // namespace s2tc
