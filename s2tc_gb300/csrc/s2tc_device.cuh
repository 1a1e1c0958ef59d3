// s2tc_device.cuh -- device-side building blocks of the S2TC block encoder:
// 5:6:5 colour helpers, the eight colour-distance metrics, index passes,
// refinement and block packing.  Everything here is integer arithmetic with
// 32-bit wrap-around except the NORMALMAP and SRGB_MIXED float steps, which use
// explicitly rounded single-precision intrinsics (no fused multiply-add) so the
// results equal the reference's x86-64 SSE code.
//
// Reference: s2tc_algorithm.cpp (divVerent/s2tc); line numbers are cited per
// function.
#pragma once
#include <cstdint>

#include "s2tc_types.h"

namespace s2tc {

// ----------------------------------------------------------------- colours

struct C3 {
  int r, g, b;
};

__device__ __forceinline__ C3 texel_c3(uint32_t t) {
  return C3{int(t & 0xFF), int((t >> 8) & 0xFF), int((t >> 16) & 0xFF)};
}
__device__ __forceinline__ int texel_a(uint32_t t) { return int(t >> 24); }

__device__ __forceinline__ bool c3_eq(C3 a, C3 b) { return a.r == b.r && a.g == b.g && a.b == b.b; }
// Lexicographic r,g,b order, which is the numeric order of the 5:6:5 word
// (s2tc_algorithm.cpp:70-81).
__device__ __forceinline__ int c3_key(C3 a) { return (a.r << 11) | (a.g << 5) | a.b; }
__device__ __forceinline__ bool c3_lt(C3 a, C3 b) { return c3_key(a) < c3_key(b); }
// Wrapping step through the 5:6:5 space (s2tc_algorithm.cpp:82-131).
__device__ __forceinline__ C3 c3_from_key(int k) { return C3{(k >> 11) & 31, (k >> 5) & 63, k & 31}; }
__device__ __forceinline__ C3 c3_next(C3 a) { return c3_from_key((c3_key(a) + 1) & 0xFFFF); }
__device__ __forceinline__ C3 c3_prev(C3 a) { return c3_from_key((c3_key(a) + 0xFFFF) & 0xFFFF); }

// ----------------------------------------------------------------- metrics
// s2tc_algorithm.cpp:215-361.  `a` is the first argument of the reference's
// call; SRGB is not symmetric in its arguments.

__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) { return int32_t(uint32_t(a) + uint32_t(b)); }
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) { return int32_t(uint32_t(a) * uint32_t(b)); }
template <int N>
__device__ __forceinline__ int32_t shrr(int32_t a) { return wadd(a, 1 << (N - 1)) >> N; }

__device__ __forceinline__ int srgb_luma(int r, int g, int b) {
  // (int)(sqrtf((float)y) + 0.5f), s2tc_algorithm.cpp:285-296
  int y = 37 * (r * r * 84 + g * g * 72 + b * b * 28);
  float f = __fadd_rn(__fsqrt_rn(__int2float_rn(y)), 0.5f);
  return __float2int_rz(f);
}

struct NUnit {
  float x, y, z;
};
// Unit vector of a normal-map texel (s2tc_algorithm.cpp:320-341).
__device__ __forceinline__ NUnit nm_unit(C3 c) {
  NUnit v;
  v.x = __fsub_rn(__fmul_rn(__fdiv_rn(__int2float_rn(c.r), 31.0f), 2.0f), 1.0f);
  v.y = __fsub_rn(__fmul_rn(__fdiv_rn(__int2float_rn(c.g), 63.0f), 2.0f), 1.0f);
  v.z = __fsub_rn(__fmul_rn(__fdiv_rn(__int2float_rn(c.b), 31.0f), 2.0f), 1.0f);
  float n = __fadd_rn(__fadd_rn(__fmul_rn(v.x, v.x), __fmul_rn(v.y, v.y)), __fmul_rn(v.z, v.z));
  if (n > 0.0f) {
    n = __fdiv_rn(1.0f, __fsqrt_rn(n));
    v.x = __fmul_rn(v.x, n);
    v.y = __fmul_rn(v.y, n);
    v.z = __fmul_rn(v.z, n);
  }
  return v;
}
// 100000 * |vb - va|^2 truncated to int (s2tc_algorithm.cpp:343-352).
__device__ __forceinline__ int32_t nm_dist(NUnit a, NUnit b) {
  float t = __fsub_rn(b.x, a.x);
  float s = __fmul_rn(t, t);
  t = __fsub_rn(b.y, a.y);
  s = __fadd_rn(s, __fmul_rn(t, t));
  t = __fsub_rn(b.z, a.z);
  s = __fadd_rn(s, __fmul_rn(t, t));
  return __float2int_rz(__fmul_rn(100000.0f, s));
}

// NORMALMAP's prepared form of every 5:6:5 colour, computed once per device by
// nm_unit itself (encode.cu, nm_table_init) into a 1 MB table in the
// translation unit of that metric; until the table is ready (flag set after
// the table kernel has completed) the form is computed on the spot.  Either
// way the bits are nm_unit's.
#if defined(S2TC_METRIC) && S2TC_METRIC == 7
static __device__ float4 g_nm_table[1 << 16];
static __device__ int g_nm_ready;
__device__ __forceinline__ NUnit nm_prepared(C3 c) {
  if (g_nm_ready) {
    const float4 v = __ldg(&g_nm_table[(c.r << 11) | (c.g << 5) | c.b]);
    return NUnit{v.x, v.y, v.z};
  }
  return nm_unit(c);
}
#else
__device__ __forceinline__ NUnit nm_prepared(C3 c) { return nm_unit(c); }
#endif

// Each metric is evaluated on a per-colour "prepared" form computed once per
// colour: the squared components for SRGB, (Y, U, V) with the square-rooted
// luma for SRGB_MIXED, the unit vector for NORMALMAP, the plain components
// for RGB and YUV.  pdist(prep(a), prep(b)) equals the reference's dist(a, b)
// exactly.
//
// The AVG family is a weighted sum of squares with weights 1 or 4 = 2^2, so
// its prepared form packs the components times their weight's square root as
// bytes (at most 2 * 63 = 126): byte-wise differences then fit signed bytes
// and one dp4a sums their squares.  The differences come from one 32-bit
// subtraction that cannot borrow across bytes: (a | 0x80 per byte) - b keeps
// every byte in [2, 254], and flipping bit 7 back gives the signed difference.
struct Pk {
  uint32_t v;  // byte 0: red, 1: green, 2: blue, each times 1 or 2; byte 3: 0
};

template <int METRIC>
struct PrepT {
  using T = C3;
};
template <>
struct PrepT<CD_NORMALMAP> {
  using T = NUnit;
};
template <>
struct PrepT<CD_AVG> {
  using T = Pk;
};
template <>
struct PrepT<CD_WAVG> {
  using T = Pk;
};
template <>
struct PrepT<CD_W0AVG> {
  using T = Pk;
};

__device__ __forceinline__ int32_t pk_dist(Pk a, Pk b) {
  const uint32_t x = ((a.v | 0x80808080u) - b.v) ^ 0x80808080u;
  return __dp4a(int(x), int(x), 0);
}

template <int METRIC>
__device__ __forceinline__ typename PrepT<METRIC>::T prep(C3 c) {
  if constexpr (METRIC == CD_SRGB) {
    return C3{c.r * c.r, c.g * c.g, c.b * c.b};
  } else if constexpr (METRIC == CD_SRGB_MIXED) {
    const int y = srgb_luma(c.r, c.g, c.b);
    return C3{y, c.r * 191 - y, c.b * 191 - y};
  } else if constexpr (METRIC == CD_NORMALMAP) {
    return nm_prepared(c);
  } else if constexpr (METRIC == CD_AVG) {  // 4 dr^2 + dg^2 + 4 db^2
    return Pk{uint32_t(2 * c.r) | (uint32_t(c.g) << 8) | (uint32_t(2 * c.b) << 16)};
  } else if constexpr (METRIC == CD_WAVG) {  // 4 dr^2 + 4 dg^2 + db^2
    return Pk{uint32_t(2 * c.r) | (uint32_t(2 * c.g) << 8) | (uint32_t(c.b) << 16)};
  } else if constexpr (METRIC == CD_W0AVG) {  // dr^2 + dg^2 + db^2
    return Pk{uint32_t(c.r) | (uint32_t(c.g) << 8) | (uint32_t(c.b) << 16)};
  } else {
    return c;
  }
}

template <int METRIC>
__device__ __forceinline__ int32_t pdist(const typename PrepT<METRIC>::T& a, const typename PrepT<METRIC>::T& b) {
  if constexpr (METRIC == CD_NORMALMAP) {
    return nm_dist(a, b);
  } else if constexpr (METRIC == CD_AVG || METRIC == CD_W0AVG || METRIC == CD_WAVG) {
    return pk_dist(a, b);
  } else if constexpr (METRIC == CD_YUV || METRIC == CD_RGB) {
    int dr = a.r - b.r, dg = a.g - b.g, db = a.b - b.b;
    int y = METRIC == CD_YUV ? dr * 60 + dg * 59 + db * 22 : dr * 42 + dg * 72 + db * 14;
    int u = dr * 202 - y, v = db * 202 - y;
    return wadd(wadd(wmul(y, y) << 1, shrr<3>(wmul(u, u))), shrr<4>(wmul(v, v)));
  } else if constexpr (METRIC == CD_SRGB) {
    // components are already squared
    int dr = a.r - b.r, dg = a.g - b.g, db = a.b - b.b;
    int y = dr * 84 + dg * 72 + db * 28;
    int u = dr * 409 - y, v = db * 409 - y;
    int32_t sy = wmul(shrr<3>(y), shrr<4>(y));
    int32_t su = wmul(shrr<3>(u), shrr<4>(u));
    int32_t sv = wmul(shrr<3>(v), shrr<4>(v));
    return wadd(wadd(shrr<4>(sy), shrr<8>(su)), shrr<9>(sv));
  } else {  // CD_SRGB_MIXED: (Y, U, V)
    int y = a.r - b.r, u = a.g - b.g, v = a.b - b.b;
    return wadd(wadd(wmul(y, y) << 3, shrr<1>(wmul(u, u))), shrr<2>(wmul(v, v)));
  }
}

template <int METRIC>
__device__ __forceinline__ int32_t cdist(C3 a, C3 b) {
  return pdist<METRIC>(prep<METRIC>(a), prep<METRIC>(b));
}

__device__ __forceinline__ int32_t adist(int a, int b) { return (a - b) * (a - b); }

// ------------------------------------------------------ block texel access

// One 4x4 (or edge w x h) block held as 16 texel words, slot y*4+x.  Each word
// is r | g<<8 | b<<16 | a<<24 with r,b in 0..31, g in 0..63 and a quantised to
// the format's alpha bits.
struct BlockTexels {
  uint32_t px[16];
  int w, h;
};

// ------------------------------------------------------ colour index pass

// Channel sums of a set of texels, two words: red and blue (texel word bits
// 0-7 and 16-23) in one, green (bits 8-15) in the other.  Sixteen texels sum
// to at most 16 * 63 per channel, so no field carries into the next.
struct ColourSums {
  uint32_t rb, g;
};
__device__ __forceinline__ uint32_t texel_rb(uint32_t t) { return t & 0x00FF00FFu; }
__device__ __forceinline__ uint32_t texel_g(uint32_t t) { return t & 0x0000FF00u; }

// The sums of the block's texels that take part in the colour passes (inside
// the image; for DXT1 not transparent) and their number.
template <bool TRANS>
__device__ __forceinline__ ColourSums colour_totals(const BlockTexels& bt, int& n) {
  ColourSums s{0u, 0u};
  n = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int x = i & 3, y = i >> 2;
    if (x >= bt.w || y >= bt.h) continue;
    const uint32_t t = bt.px[i];
    if (TRANS && (t >> 24) == 0) continue;
    s.rb += texel_rb(t);
    s.g += texel_g(t);
    ++n;
  }
  return s;
}

// s2tc_algorithm.cpp:582-643 (colour, two references): nearest endpoint per
// texel, ties to endpoint 0; DXT1 alpha-0 texels take index 3.  `tp` holds the
// block's texels in prepared form (slot y*4+x).  The reference visits texels
// x-outer, y-inner; the results (per-texel indices, sums) do not depend on
// the order.  With ACC, `acc` gets the channel sums of the texels that chose
// endpoint 1 (those of endpoint 0 are the totals minus these; the counts come
// from the index word).
template <int METRIC, bool TRANS, bool ACC>
__device__ __forceinline__ uint32_t colour_pass(const BlockTexels& bt, const typename PrepT<METRIC>::T* tp, C3 r0,
                                                C3 r1, uint32_t& bits, ColourSums& acc) {
  uint32_t score = 0;
  bits = 0;
  if (ACC) acc = ColourSums{0u, 0u};
  const auto p0 = prep<METRIC>(r0), p1 = prep<METRIC>(r1);
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int x = i & 3, y = i >> 2;
    if (x >= bt.w || y >= bt.h) continue;
    uint32_t t = bt.px[i];
    if (TRANS && (t >> 24) == 0) {
      bits |= 3u << (2 * i);
      continue;
    }
    int32_t d0 = pdist<METRIC>(tp[i], p0), d1 = pdist<METRIC>(tp[i], p1);
    const bool one = d1 < d0;
    if (ACC) {
      acc.rb += texel_rb(t) * uint32_t(one);
      acc.g += texel_g(t) * uint32_t(one);
    }
    bits |= uint32_t(one) << (2 * i);
    score += uint32_t(one ? d1 : d0);
  }
  return score;
}

// Rounded mean ((s << 1) + n) / (n << 1) (s2tc_algorithm.cpp:542-551) for the
// sums of at most 16 texels: 1 <= n <= 16 and 0 <= s <= 16 * 255.  The integer
// quotient q of x = 2s + n < 2^13 by d = 2n <= 32 is taken in float: x / d lies
// in [q, q + 1 - 1/d] with 1/d >= 2^-5; the correctly rounded reciprocal, the
// fused multiply-add and its one rounding (results below 2^12 + 1) miss x / d
// by less than 2^-10, so after adding 2^-6 the value stays in (q, q + 1) and
// its floor is q.  (Exhaustively equal to the integer division over that
// domain: tests/test_arith.py.)
__device__ __forceinline__ int rmean(int s, int n) {
  const float r = __frcp_rn(float(n << 1));
  return __float2int_rd(__fmaf_rn(float((s << 1) + n), r, 0.015625f));
}

// s2tc_algorithm.cpp:542-551, from the block's totals (`tot`, `n` texels),
// endpoint 1's sums and the index word of the same pass.
__device__ __forceinline__ bool colour_means(const ColourSums& tot, int n, const ColourSums& a1, uint32_t bits, C3& c0,
                                             C3& c1) {
  if (!n) return false;
  const uint32_t lo = bits & 0x55555555u, hi = (bits >> 1) & 0x55555555u;
  const int n1 = __popc(lo & ~hi);  // indices equal to 1
  const int n0 = n - n1;
  const uint32_t rb0 = tot.rb - a1.rb, g0 = tot.g - a1.g;  // no field goes below 0
  if (n0) c0 = C3{rmean(int(rb0 & 0xFFFFu), n0) & 31, rmean(int(g0 >> 8), n0) & 63, rmean(int(rb0 >> 16), n0) & 31};
  if (n1)
    c1 = C3{rmean(int(a1.rb & 0xFFFFu), n1) & 31, rmean(int(a1.g >> 8), n1) & 63, rmean(int(a1.rb >> 16), n1) & 31};
  return true;
}

// Equal-endpoint fix and canonical order (s2tc_algorithm.cpp:796-813).
template <bool TRANS>
__device__ __forceinline__ void colour_finish(uint32_t& bits, C3& c0, C3& c1) {
  if (c3_eq(c0, c1)) {
    c1 = (c0.r == 31 && c0.g == 63 && c0.b == 31) ? c3_prev(c1) : c3_next(c1);
    // indices other than 1 become 0
    uint32_t lo = bits & 0x55555555u, hi = (bits >> 1) & 0x55555555u;
    bits = lo & ~hi;
  }
  if (TRANS ? c3_lt(c1, c0) : c3_lt(c0, c1)) {
    C3 t = c0; c0 = c1; c1 = t;
    // xor bit 0 of every index whose bit 1 is clear
    uint32_t hi = (bits >> 1) & 0x55555555u;
    bits ^= ~hi & 0x55555555u;
  }
}

// Colour refinement NEVER / ALWAYS / LOOP (s2tc_algorithm.cpp:767-860).
template <int METRIC, bool TRANS, int REFINE>
__device__ __forceinline__ uint32_t colour_refine(const BlockTexels& bt, const typename PrepT<METRIC>::T* tp, C3& c0,
                                                  C3& c1) {
  uint32_t bits;
  ColourSums acc;
  if (REFINE == RF_NEVER) {
    if (TRANS ? c3_lt(c1, c0) : c3_lt(c0, c1)) {
      C3 t = c0; c0 = c1; c1 = t;
    }
    colour_pass<METRIC, TRANS, false>(bt, tp, c0, c1, bits, acc);
    return bits;
  }
  int n;
  const ColourSums tot = colour_totals<TRANS>(bt, n);
  if (REFINE == RF_LOOP) {
    C3 n0 = c0, n1 = c1;
    uint32_t best = 0x7FFFFFFFu;
    bits = 0;
    for (;;) {
      uint32_t b2;
      uint32_t s2 = colour_pass<METRIC, TRANS, true>(bt, tp, n0, n1, b2, acc);
      if (!(s2 < best)) break;
      bits = b2;
      best = s2;
      c0 = n0;
      c1 = n1;
      if (!colour_means(tot, n, acc, b2, n0, n1)) break;
    }
  } else {
    colour_pass<METRIC, TRANS, true>(bt, tp, c0, c1, bits, acc);
    colour_means(tot, n, acc, bits, c0, c1);
  }
  colour_finish<TRANS>(bits, c0, c1);
  return bits;
}

// --------------------------------------------------------- DXT5 alpha pass

// s2tc_algorithm.cpp:582-643 with bpp=3 and the 0/255 fixed points.
template <bool ACC>
__device__ __forceinline__ uint32_t alpha_pass(const BlockTexels& bt, int r0, int r1, uint64_t& bits,
                                               int& n0, int& n1, int& s0, int& s1) {
  uint32_t score = 0;
  bits = 0;
  if (ACC) n0 = n1 = s0 = s1 = 0;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const int x = i & 3, y = i >> 2;
    if (x >= bt.w || y >= bt.h) continue;
    int a = int(bt.px[i] >> 24);
    int32_t bd = adist(a, r0), d1 = adist(a, r1);
    int best = 0;
    if (d1 < bd) { bd = d1; best = 1; }
    int32_t dz = a * a;
    if (dz <= bd) {
      bits |= uint64_t(6) << (3 * i);
      score += uint32_t(dz);
      continue;
    }
    int32_t df = (255 - a) * (255 - a);
    if (df <= bd) {
      bits |= uint64_t(7) << (3 * i);
      score += uint32_t(df);
      continue;
    }
    if (ACC) {
      if (best) { n1++; s1 += a; } else { n0++; s0 += a; }
    }
    bits |= uint64_t(best) << (3 * i);
    score += uint32_t(bd);
  }
  return score;
}

// s2tc_algorithm.cpp:673-705
__device__ __forceinline__ void alpha_finish(uint64_t& bits, int& a0, int& a1) {
  if (a0 == a1) {
    if (a0 == 255) --a1; else ++a1;
#pragma unroll
    for (int i = 0; i < 16; ++i)
      if (((bits >> (3 * i)) & 7) == 1) bits &= ~(uint64_t(7) << (3 * i));
  }
  if (a1 < a0) {
    int t = a0; a0 = a1; a1 = t;
#pragma unroll
    for (int i = 0; i < 16; ++i) {
      uint64_t v = (bits >> (3 * i)) & 7, nv;
      if (v == 0) nv = 1;
      else if (v == 1) nv = 0;
      else if (v >= 6) nv = v;
      else nv = 7 - v;
      bits = (bits & ~(uint64_t(7) << (3 * i))) | (nv << (3 * i));
    }
  }
}

// s2tc_algorithm.cpp:645-765.  Returns the value of the second endpoint that a
// following single-texel block would read (see encode_block).
template <int REFINE>
__device__ __forceinline__ uint64_t alpha_refine(const BlockTexels& bt, int& a0, int& a1, int& leftover) {
  uint64_t bits = 0;
  int n0, n1, s0, s1;
  if (REFINE == RF_NEVER) {
    leftover = a1;
    if (a1 < a0) { int t = a0; a0 = a1; a1 = t; }
    alpha_pass<false>(bt, a0, a1, bits, n0, n1, s0, s1);
    return bits;
  } else if (REFINE == RF_LOOP) {
    int x0 = a0, x1 = a1;
    uint32_t best = 0x7FFFFFFFu;
    for (;;) {
      uint64_t b2;
      uint32_t s2 = alpha_pass<true>(bt, x0, x1, b2, n0, n1, s0, s1);
      if (!(s2 < best)) break;
      bits = b2;
      best = s2;
      a0 = x0;
      a1 = x1;
      if (!n0 && !n1) break;
      if (n0) x0 = rmean(s0, n0) & 255;
      if (n1) x1 = rmean(s1, n1) & 255;
    }
  } else {
    alpha_pass<true>(bt, a0, a1, bits, n0, n1, s0, s1);
    if (n0) a0 = rmean(s0, n0) & 255;
    if (n1) a1 = rmean(s1, n1) & 255;
  }
  alpha_finish(bits, a0, a1);
  leftover = a1;
  return bits;
}

// ------------------------------------------------------------------ packing

__device__ __forceinline__ uint32_t pack565(C3 c) { return uint32_t((c.r << 11) | (c.g << 5) | c.b); }

}  // namespace s2tc
