/*
 * s2tc_oracle.c -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C, single-threaded restatement of the S2TC encode path of
 * divVerent/s2tc (files s2tc_algorithm.cpp and s2tc_libtxc_dxtn.cpp).  It is
 * the checker that the GPU encoder is compared against, and the "port" CPU
 * baseline that bench.py times.  Nothing in the shipped library links it, and
 * only tests/, __graft_entry__.smoke() and bench.py's CPU legs load it.
 *
 * Parity pin: tests/test_oracle_pin.py compares every entry point below with
 * the reference library compiled from its own sources (oracle/Makefile, target
 * `ref`), over exhaustive small sizes and every mode, and tests/golden/ holds
 * vectors produced by that compiled reference (tests/golden/make_golden.py).
 *
 * Arithmetic rules that the reference's compiler output follows and this file
 * restates explicitly:
 *   - 32-bit signed arithmetic wraps (the SRGB metric overflows; gcc -O3 emits
 *     plain wrapping imul/add for it).  Wrapping is written out with unsigned
 *     arithmetic so no flag is needed.
 *   - `>>` on negative ints is an arithmetic shift.
 *   - float code is IEEE single precision, every operation rounded, no fused
 *     multiply-add (x86-64 SSE without -march).  Build with -ffp-contract=off
 *     so that aarch64 gcc does not fuse.
 *   - rand() is libc's, called in the same order as the reference (or, for
 *     tests, the same words from an array: s2tc_oracle_set_rand_words).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>

#include "s2tc_oracle.h"

/* ---------------------------------------------------------------- helpers */

typedef struct { int r, g, b; } o_rgb;   /* 5:6:5 colour: r,b 0..31, g 0..63 */

/* The metrics, and the functions that take one as an o_metric, are inlined
 * into each per-metric copy of the block encoder, where the metric is a
 * constant. */
#define ALWAYS_INLINE __attribute__((always_inline)) inline

static inline int32_t w_add(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t w_sub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t w_mul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }
/* SHRR: shift right, rounded (s2tc_algorithm.cpp:215), on wrapped values. */
static inline int32_t shrr(int32_t a, int n) { return w_add(a, 1 << (n - 1)) >> n; }

static inline int rgb_eq(o_rgb a, o_rgb b) { return a.r == b.r && a.g == b.g && a.b == b.b; }
/* Lexicographic r,g,b order (s2tc_algorithm.cpp:70-81). */
static inline int rgb_lt(o_rgb a, o_rgb b)
{
	if (a.r != b.r) return a.r < b.r;
	if (a.g != b.g) return a.g < b.g;
	return a.b < b.b;
}
/* Step to the previous 5:6:5 value, wrapping 0 -> max (s2tc_algorithm.cpp:82-106). */
static o_rgb rgb_prev(o_rgb c)
{
	if (c.b > 0) { c.b--; return c; }
	c.b = 31;
	if (c.g > 0) { c.g--; return c; }
	c.g = 63;
	if (c.r > 0) { c.r--; return c; }
	c.r = 31;
	return c;
}
/* Step to the next 5:6:5 value, wrapping max -> 0 (s2tc_algorithm.cpp:107-131). */
static o_rgb rgb_next(o_rgb c)
{
	if (c.b < 31) { c.b++; return c; }
	c.b = 0;
	if (c.g < 63) { c.g++; return c; }
	c.g = 0;
	if (c.r < 31) { c.r++; return c; }
	c.r = 0;
	return c;
}

/* ---------------------------------------------------------------- metrics */
/* s2tc_algorithm.cpp:217-361.  Argument order matters: SRGB is not symmetric. */

ALWAYS_INLINE
static int32_t d_avg(o_rgb a, o_rgb b)
{
	int dr = a.r - b.r, dg = a.g - b.g, db = a.b - b.b;
	return 4 * dr * dr + dg * dg + 4 * db * db;
}
ALWAYS_INLINE
static int32_t d_w0avg(o_rgb a, o_rgb b)
{
	int dr = a.r - b.r, dg = a.g - b.g, db = a.b - b.b;
	return dr * dr + dg * dg + db * db;
}
ALWAYS_INLINE
static int32_t d_wavg(o_rgb a, o_rgb b)
{
	int dr = a.r - b.r, dg = a.g - b.g, db = a.b - b.b;
	return 4 * dr * dr + 4 * dg * dg + db * db;
}
/* Shared tail of the YUV and RGB metrics: 2y^2 + SHRR(u^2,3) + SHRR(v^2,4). */
static int32_t d_luma_chroma(int dr, int db, int y)
{
	int32_t u = dr * 202 - y, v = db * 202 - y;
	return w_add(w_add(w_mul(y, y) * 2, shrr(w_mul(u, u), 3)), shrr(w_mul(v, v), 4));
}
ALWAYS_INLINE
static int32_t d_yuv(o_rgb a, o_rgb b)
{
	int dr = a.r - b.r, dg = a.g - b.g, db = a.b - b.b;
	return d_luma_chroma(dr, db, dr * 60 + dg * 59 + db * 22);
}
ALWAYS_INLINE
static int32_t d_rgb(o_rgb a, o_rgb b)
{
	int dr = a.r - b.r, dg = a.g - b.g, db = a.b - b.b;
	return d_luma_chroma(dr, db, dr * 42 + dg * 72 + db * 14);
}
ALWAYS_INLINE
static int32_t d_srgb(o_rgb a, o_rgb b)
{
	int32_t dr = a.r * a.r - b.r * b.r;
	int32_t dg = a.g * a.g - b.g * b.g;
	int32_t db = a.b * a.b - b.b * b.b;
	int32_t y = dr * 84 + dg * 72 + db * 28;
	int32_t u = dr * 409 - y, v = db * 409 - y;
	int32_t sy = w_mul(shrr(y, 3), shrr(y, 4));
	int32_t su = w_mul(shrr(u, 3), shrr(u, 4));
	int32_t sv = w_mul(shrr(v, 3), shrr(v, 4));
	return w_add(w_add(shrr(sy, 4), shrr(su, 8)), shrr(sv, 9));
}
/* Luma of the squared ("linear") components, square-rooted back
 * (s2tc_algorithm.cpp:285-296): (int)(sqrtf((float)y) + 0.5f). */
static int srgb_luma(o_rgb a)
{
	int y = 37 * (a.r * a.r * 84 + a.g * a.g * 72 + a.b * a.b * 28);
	float f = sqrtf((float)y);
	f = f + 0.5f;
	return (int)f;
}
ALWAYS_INLINE
static int32_t d_srgb_mixed(o_rgb a, o_rgb b)
{
	int ay = srgb_luma(a), by = srgb_luma(b);
	int y = ay - by;
	int u = (a.r * 191 - ay) - (b.r * 191 - by);
	int v = (a.b * 191 - ay) - (b.b * 191 - by);
	return w_add(w_add(w_mul(y, y) * 8, shrr(w_mul(u, u), 1)), shrr(w_mul(v, v), 2));
}
/* Unit-vector distance (s2tc_algorithm.cpp:317-354).  Every float operation is
 * written in the reference's evaluation order. */
static void nm_unit(o_rgb c, float v[3])
{
	float n;
	v[0] = (float)c.r / 31.0f * 2.0f - 1.0f;
	v[1] = (float)c.g / 63.0f * 2.0f - 1.0f;
	v[2] = (float)c.b / 31.0f * 2.0f - 1.0f;
	n = v[0] * v[0] + v[1] * v[1];
	n = n + v[2] * v[2];
	if (n > 0.0f) {
		n = 1.0f / sqrtf(n);
		v[0] = v[0] * n;
		v[1] = v[1] * n;
		v[2] = v[2] * n;
	}
}
ALWAYS_INLINE
static int32_t d_normalmap(o_rgb a, o_rgb b)
{
	float va[3], vb[3], s, t;
	nm_unit(a, va);
	nm_unit(b, vb);
	t = vb[0] - va[0];
	s = t * t;
	t = vb[1] - va[1];
	s = s + t * t;
	t = vb[2] - va[2];
	s = s + t * t;
	return (int32_t)(100000.0f * s);
}

typedef int32_t (*o_metric)(o_rgb, o_rgb);
/* random candidates held on the stack; more take a heap buffer */
enum { kStackRandom = 64 };
static o_metric metric_fn(int metric)
{
	switch (metric) {
	case S2TC_O_RGB: return d_rgb;
	case S2TC_O_YUV: return d_yuv;
	case S2TC_O_SRGB: return d_srgb;
	case S2TC_O_SRGB_MIXED: return d_srgb_mixed;
	case S2TC_O_AVG: return d_avg;
	case S2TC_O_W0AVG: return d_w0avg;
	case S2TC_O_NORMALMAP: return d_normalmap;
	case S2TC_O_WAVG:
	default: return d_wavg;
	}
}

static inline int32_t d_alpha(int a, int b) { return (a - b) * (a - b); }

int32_t s2tc_oracle_color_dist(int metric, int ar, int ag, int ab, int br, int bg, int bb)
{
	o_rgb a = { ar, ag, ab }, b = { br, bg, bb };
	return metric_fn(metric)(a, b);
}

/* ------------------------------------------------------ endpoint reduction */

/* Pair search over candidates (s2tc_algorithm.cpp:363-414): inputs are the
 * first n candidates, all m are endpoint candidates.  Distances between two
 * inputs are evaluated once, as dist(c[lo], c[hi]), and used both ways. */
ALWAYS_INLINE
static void reduce_rgb(o_rgb *c, int n, int m, o_metric dist, int32_t *dm)
{
	int i, j, k;
	int32_t bestsum = -1;
	int besti = 0, bestj = 1;
	for (i = 0; i < n; ++i) {
		dm[i * n + i] = 0;
		for (j = i + 1; j < n; ++j)
			dm[i * n + j] = dm[j * n + i] = dist(c[i], c[j]);
	}
	for (i = n; i < m; ++i)
		for (k = 0; k < n; ++k)
			dm[i * n + k] = dist(c[i], c[k]);
	for (i = 0; i < m; ++i)
		for (j = i + 1; j < m; ++j) {
			int32_t sum = 0;
			const int32_t *ri = dm + i * n, *rj = dm + j * n;
			for (k = 0; k < n; ++k)
				sum = w_add(sum, rj[k] < ri[k] ? rj[k] : ri[k]);
			if (bestsum < 0 || sum < bestsum) {
				bestsum = sum;
				besti = i;
				bestj = j;
			}
		}
	{
		o_rgb lo = c[besti];
		c[1] = c[bestj];
		c[0] = lo;
	}
}

/* DXT5 alpha variant (s2tc_algorithm.cpp:415-478): every input may also be
 * served by the fixed values 0 and 255; c[0]/c[1] are only written when the
 * winning pair does not already sit there. */
static void reduce_alpha(uint8_t *c, int n, int m, int32_t *dm)
{
	int i, j, k;
	int32_t bestsum = -1;
	int besti = 0, bestj = 1;
	int32_t *fix = dm + m * n;   /* min(dist to 0, dist to 255) per input */
	for (i = 0; i < n; ++i) {
		dm[i * n + i] = 0;
		for (j = i + 1; j < n; ++j)
			dm[i * n + j] = dm[j * n + i] = d_alpha(c[i], c[j]);
	}
	for (i = n; i < m; ++i)
		for (k = 0; k < n; ++k)
			dm[i * n + k] = d_alpha(c[i], c[k]);
	for (k = 0; k < n; ++k) {
		int32_t d0 = d_alpha(0, c[k]), d1 = d_alpha(255, c[k]);
		fix[k] = d1 < d0 ? d1 : d0;
	}
	for (i = 0; i < m; ++i)
		for (j = i + 1; j < m; ++j) {
			int32_t sum = 0;
			const int32_t *ri = dm + i * n, *rj = dm + j * n;
			for (k = 0; k < n; ++k) {
				int32_t v = rj[k] < ri[k] ? rj[k] : ri[k];
				if (fix[k] < v) v = fix[k];
				sum = w_add(sum, v);
			}
			if (bestsum < 0 || sum < bestsum) {
				bestsum = sum;
				besti = i;
				bestj = j;
			}
		}
	if (besti != 0) c[0] = c[besti];
	if (bestj != 1) c[1] = c[bestj];
}

/* ----------------------------------------------- index assignment + refine */

static inline o_rgb texel_rgb(const uint8_t *p) { o_rgb c = { p[0], p[1], p[2] }; return c; }

/* Rounded mean ((S<<1)+n)/(n<<1) (s2tc_algorithm.cpp:542-551). */
static inline int rmean(int s, int n) { return ((s << 1) + n) / (n << 1); }

/* Colour index pass (s2tc_algorithm.cpp:582-643 with bpp=2, two references).
 * Visits texels x-outer, y-inner.  Returns the unsigned score; when `acc` is
 * set, also returns per-endpoint sums of the texels that chose it. */
ALWAYS_INLINE
static uint32_t colour_pass(uint32_t *bits, const uint8_t *blk, int iw, int w, int h,
			    o_metric dist, int have_trans, o_rgb r0, o_rgb r1,
			    int acc, int cnt[2], int sum[2][3])
{
	uint32_t score = 0;
	int x, y;
	*bits = 0;
	if (acc) memset(cnt, 0, 2 * sizeof(int)), memset(sum, 0, 6 * sizeof(int));
	for (x = 0; x < w; ++x)
		for (y = 0; y < h; ++y) {
			const uint8_t *p = blk + (y * iw + x) * 4;
			int i = y * 4 + x, best = 0;
			int32_t bd, d1;
			o_rgb t;
			if (have_trans && p[3] == 0) {
				*bits |= 3u << (2 * i);
				continue;
			}
			t = texel_rgb(p);
			bd = dist(t, r0);
			d1 = dist(t, r1);
			if (d1 < bd) { bd = d1; best = 1; }
			if (acc) {
				cnt[best]++;
				sum[best][0] += t.r; sum[best][1] += t.g; sum[best][2] += t.b;
			}
			*bits |= (uint32_t)best << (2 * i);
			score += (uint32_t)bd;
		}
	return score;
}

/* New endpoints from the pass sums; false when no texel chose either. */
static int colour_means(const int cnt[2], int sum[2][3], o_rgb *c0, o_rgb *c1)
{
	if (!cnt[0] && !cnt[1]) return 0;
	if (cnt[0]) {
		c0->r = rmean(sum[0][0], cnt[0]) & 31;
		c0->g = rmean(sum[0][1], cnt[0]) & 63;
		c0->b = rmean(sum[0][2], cnt[0]) & 31;
	}
	if (cnt[1]) {
		c1->r = rmean(sum[1][0], cnt[1]) & 31;
		c1->g = rmean(sum[1][1], cnt[1]) & 63;
		c1->b = rmean(sum[1][2], cnt[1]) & 31;
	}
	return 1;
}

/* Equal-endpoint fix and canonical order after refinement
 * (s2tc_algorithm.cpp:796-813 / 828-845). */
static void colour_finish(uint32_t *bits, o_rgb *c0, o_rgb *c1, int have_trans)
{
	int i;
	if (rgb_eq(*c0, *c1)) {
		if (c0->r == 31 && c0->g == 63 && c0->b == 31) *c1 = rgb_prev(*c1);
		else *c1 = rgb_next(*c1);
		for (i = 0; i < 16; ++i)
			if (((*bits >> (2 * i)) & 3) != 1) *bits &= ~(3u << (2 * i));
	}
	if (have_trans ? rgb_lt(*c1, *c0) : rgb_lt(*c0, *c1)) {
		o_rgb t = *c0; *c0 = *c1; *c1 = t;
		for (i = 0; i < 16; ++i)
			if (!((*bits >> (2 * i)) & 2)) *bits ^= 1u << (2 * i);
	}
}

/* Colour refinement NEVER / ALWAYS / LOOP (s2tc_algorithm.cpp:767-860). */
ALWAYS_INLINE
static uint32_t colour_refine(const uint8_t *blk, int iw, int w, int h, o_metric dist,
			      int have_trans, int refine, o_rgb *c0, o_rgb *c1)
{
	uint32_t bits = 0;
	int cnt[2], sum[2][3];
	if (refine == S2TC_O_NEVER) {
		if (have_trans ? rgb_lt(*c1, *c0) : rgb_lt(*c0, *c1)) {
			o_rgb t = *c0; *c0 = *c1; *c1 = t;
		}
		colour_pass(&bits, blk, iw, w, h, dist, have_trans, *c0, *c1, 0, cnt, sum);
		return bits;
	}
	if (refine == S2TC_O_LOOP) {
		o_rgb n0 = *c0, n1 = *c1;
		uint32_t best = 0x7FFFFFFFu;
		for (;;) {
			uint32_t b2;
			uint32_t s2 = colour_pass(&b2, blk, iw, w, h, dist, have_trans, n0, n1, 1, cnt, sum);
			if (!(s2 < best)) break;
			bits = b2;
			best = s2;
			*c0 = n0;
			*c1 = n1;
			if (!colour_means(cnt, sum, &n0, &n1)) break;
		}
	} else {
		colour_pass(&bits, blk, iw, w, h, dist, have_trans, *c0, *c1, 1, cnt, sum);
		colour_means(cnt, sum, c0, c1);
	}
	colour_finish(&bits, c0, c1, have_trans);
	return bits;
}

/* DXT5 alpha index pass (s2tc_algorithm.cpp:582-643 with bpp=3 and the 0/255
 * fixed points): ties go to the endpoint, then to 0, then to 255. */
static uint32_t alpha_pass(uint64_t *bits, const uint8_t *blk, int iw, int w, int h,
			   int r0, int r1, int acc, int cnt[2], int sum[2])
{
	uint32_t score = 0;
	int x, y;
	*bits = 0;
	if (acc) cnt[0] = cnt[1] = sum[0] = sum[1] = 0;
	for (x = 0; x < w; ++x)
		for (y = 0; y < h; ++y) {
			int a = blk[(y * iw + x) * 4 + 3];
			int i = y * 4 + x, best = 0;
			int32_t bd = d_alpha(a, r0), d1 = d_alpha(a, r1), dz, df;
			if (d1 < bd) { bd = d1; best = 1; }
			dz = d_alpha(a, 0);
			if (dz <= bd) {
				*bits |= (uint64_t)6 << (3 * i);
				score += (uint32_t)dz;
				continue;
			}
			df = d_alpha(a, 255);
			if (df <= bd) {
				*bits |= (uint64_t)7 << (3 * i);
				score += (uint32_t)df;
				continue;
			}
			if (acc) { cnt[best]++; sum[best] += a; }
			*bits |= (uint64_t)best << (3 * i);
			score += (uint32_t)bd;
		}
	return score;
}

static int alpha_means(const int cnt[2], const int sum[2], int *a0, int *a1)
{
	if (!cnt[0] && !cnt[1]) return 0;
	if (cnt[0]) *a0 = rmean(sum[0], cnt[0]) & 255;
	if (cnt[1]) *a1 = rmean(sum[1], cnt[1]) & 255;
	return 1;
}

/* s2tc_algorithm.cpp:673-705 / 719-751. */
static void alpha_finish(uint64_t *bits, int *a0, int *a1)
{
	int i;
	if (*a0 == *a1) {
		if (*a0 == 255) --*a1; else ++*a1;
		for (i = 0; i < 16; ++i)
			if (((*bits >> (3 * i)) & 7) == 1) *bits &= ~((uint64_t)7 << (3 * i));
	}
	if (*a1 < *a0) {
		int t = *a0; *a0 = *a1; *a1 = t;
		for (i = 0; i < 16; ++i) {
			uint64_t v = (*bits >> (3 * i)) & 7, nv;
			if (v == 0) nv = 1;
			else if (v == 1) nv = 0;
			else if (v >= 6) nv = v;
			else nv = 7 - v;
			*bits = (*bits & ~((uint64_t)7 << (3 * i))) | (nv << (3 * i));
		}
	}
}

/* s2tc_algorithm.cpp:645-765. */
static uint64_t alpha_refine(const uint8_t *blk, int iw, int w, int h, int refine, int *a0, int *a1)
{
	uint64_t bits = 0;
	int cnt[2], sum[2];
	if (refine == S2TC_O_NEVER) {
		if (*a1 < *a0) { int t = *a0; *a0 = *a1; *a1 = t; }
		alpha_pass(&bits, blk, iw, w, h, *a0, *a1, 0, cnt, sum);
		return bits;
	}
	if (refine == S2TC_O_LOOP) {
		int n0 = *a0, n1 = *a1;
		uint32_t best = 0x7FFFFFFFu;
		for (;;) {
			uint64_t b2;
			uint32_t s2 = alpha_pass(&b2, blk, iw, w, h, n0, n1, 1, cnt, sum);
			if (!(s2 < best)) break;
			bits = b2;
			best = s2;
			*a0 = n0;
			*a1 = n1;
			if (!alpha_means(cnt, sum, &n0, &n1)) break;
		}
	} else {
		alpha_pass(&bits, blk, iw, w, h, *a0, *a1, 1, cnt, sum);
		alpha_means(cnt, sum, a0, a1);
	}
	alpha_finish(&bits, a0, a1);
	return bits;
}

/* ------------------------------------------------------------ block encoder */

/* Where the random candidates' words come from: libc's rand(), as in the
 * reference (s2tc_algorithm.cpp:986-990), or a caller-supplied array of the
 * same words (s2tc_oracle_set_rand_words), which lets a test hold an encoder
 * fed with stored words against this restatement without replaying libc's
 * stream.  Words are consumed in the reference's call order either way. */
static const uint32_t *o_words;
static long o_words_n, o_words_pos;

void s2tc_oracle_set_rand_words(const uint32_t *words, long n)
{
	o_words = words;
	o_words_n = words ? n : 0;
	o_words_pos = 0;
}

long s2tc_oracle_rand_words_used(void) { return o_words_pos; }

static inline int o_rand(void)
{
	if (!o_words) return rand();
	/* past the end: a value that no test expects, and the count tells */
	if (o_words_pos >= o_words_n) { ++o_words_pos; return 0; }
	return (int)o_words[o_words_pos++];
}

static void put_colour_block(uint8_t *out, o_rgb c0, o_rgb c1, uint32_t bits)
{
	out[0] = (uint8_t)(((c0.g & 7) << 5) | c0.b);
	out[1] = (uint8_t)((c0.r << 3) | (c0.g >> 3));
	out[2] = (uint8_t)(((c1.g & 7) << 5) | c1.b);
	out[3] = (uint8_t)((c1.r << 3) | (c1.g >> 3));
	out[4] = (uint8_t)bits; out[5] = (uint8_t)(bits >> 8);
	out[6] = (uint8_t)(bits >> 16); out[7] = (uint8_t)(bits >> 24);
}

/* Encode one 4x4 (or edge w x h) block of the 4-byte 5:6:5+alpha texel buffer
 * (s2tc_algorithm.cpp:872-1108).  `rgba` points at the block's first texel and
 * `iw` is the buffer's row length in texels. */
ALWAYS_INLINE
static int encode_block(uint8_t *out, const uint8_t *rgba, int iw, int w, int h,
			int dxt, int metric, o_metric dist, int nrandom, int refine, int prev_a1)
{
	int leftover;
	int nr = nrandom > 0 ? nrandom : 0;
	int normal_mode = metric == S2TC_O_NORMALMAP || nrandom >= 0;   /* :1139 */
	o_rgb c_stack[16 + kStackRandom];
	uint8_t ca_stack[16 + kStackRandom];
	int32_t dm_stack[(16 + kStackRandom + 2) * 16];
	o_rgb *c = nr <= kStackRandom ? c_stack : (o_rgb *)malloc(sizeof(o_rgb) * (16 + nr));
	uint8_t *ca = nr <= kStackRandom ? ca_stack : (uint8_t *)malloc(16 + nr);
	int x, y;
	int a0 = 0, a1 = 0;

	if (!normal_mode) {
		/* darkest and brightest by distance to black (:879-935) */
		const o_rgb black = { 0, 0, 0 };
		int32_t dmin = 0x7FFFFFFF, dmax = 0;
		c[0].r = 31; c[0].g = 63; c[0].b = 31;
		c[1] = black;
		if (dxt == S2TC_O_DXT5) ca[0] = ca[1] = rgba[3];
		for (x = 0; x < w; ++x)
			for (y = 0; y < h; ++y) {
				const uint8_t *p = rgba + (x + y * iw) * 4;
				o_rgb t = texel_rgb(p);
				int32_t d;
				if (dxt == S2TC_O_DXT1 && p[3] == 0) continue;
				d = dist(t, black);
				if (d > dmax) { dmax = d; c[1] = t; }
				if (d < dmin) { dmin = d; c[0] = t; }
				if (dxt == S2TC_O_DXT5 && p[3] != 255) {
					if (p[3] > ca[1]) ca[1] = p[3];
					if (p[3] < ca[0]) ca[0] = p[3];
				}
			}
	} else {
		int n = 0, m;
		for (x = 0; x < w; ++x)
			for (y = 0; y < h; ++y) {
				const uint8_t *p = rgba + (x + y * iw) * 4;
				if (dxt == S2TC_O_DXT1 && p[3] == 0) continue;
				c[n] = texel_rgb(p);
				ca[n] = p[3];
				++n;
			}
		if (n == 0) {
			n = 1;
			c[0].r = c[0].g = c[0].b = 0;
			ca[0] = 0;
		}
		m = n;
		if (nrandom > 0) {
			/* random candidates inside the per-channel bounding box (:962-993) */
			o_rgb lo = c[0], hi = c[0];
			int alo = dxt == S2TC_O_DXT5 ? ca[0] : 0, ahi = alo;
			int lr, lg, lb, la, r;
			for (x = 1; x < n; ++x) {
				if (c[x].r < lo.r) lo.r = c[x].r;
				if (c[x].g < lo.g) lo.g = c[x].g;
				if (c[x].b < lo.b) lo.b = c[x].b;
				if (c[x].r > hi.r) hi.r = c[x].r;
				if (c[x].g > hi.g) hi.g = c[x].g;
				if (c[x].b > hi.b) hi.b = c[x].b;
				if (dxt == S2TC_O_DXT5) {
					if (ca[x] < alo) alo = ca[x];
					if (ca[x] > ahi) ahi = ca[x];
				}
			}
			lr = hi.r - lo.r + 1; lg = hi.g - lo.g + 1; lb = hi.b - lo.b + 1;
			la = ahi - alo + 1;
			for (r = 0; r < nrandom; ++r) {
				c[m].r = lo.r + o_rand() % lr;
				c[m].g = lo.g + o_rand() % lg;
				c[m].b = lo.b + o_rand() % lb;
				if (dxt == S2TC_O_DXT5) ca[m] = (uint8_t)(alo + o_rand() % la);
				++m;
			}
		} else if (n == 1) {
			/* single input: duplicate the colour (:996-1001).  The reference
			 * leaves the second alpha candidate unset here, so it holds what
			 * the previous block encoded by the same caller left in that
			 * stack slot (`prev_a1`, see the return value).  With no previous
			 * block (prev_a1 < 0) the reference's value is indeterminate;
			 * this restatement then duplicates the alpha too. */
			c[1] = c[0];
			ca[1] = prev_a1 >= 0 ? (uint8_t)prev_a1 : ca[0];
			m = n = 2;
		}
		{
			int32_t *dm = nr <= kStackRandom ? dm_stack
				: (int32_t *)malloc(sizeof(int32_t) * (size_t)(m + 2) * (size_t)n);
			reduce_rgb(c, n, m, dist, dm);
			if (dxt == S2TC_O_DXT5) reduce_alpha(ca, n, m, dm);
			if (dm != dm_stack) free(dm);
		}
	}

	/* equal endpoints are bumped apart (:1009-1027) */
	if (rgb_eq(c[0], c[1])) {
		if (c[0].r == 31 && c[0].g == 63 && c[0].b == 31) c[1] = rgb_prev(c[1]);
		else c[1] = rgb_next(c[1]);
	}
	if (dxt == S2TC_O_DXT5) {
		a0 = ca[0];
		a1 = ca[1];
		if (a0 == a1) {
			if (a0 == 255) --a1; else ++a1;
		}
	}
	leftover = a1;

	{
		o_rgb c0 = c[0], c1 = c[1];
		uint32_t cbits = colour_refine(rgba, iw, w, h, dist, dxt == S2TC_O_DXT1, refine, &c0, &c1);
		if (dxt == S2TC_O_DXT1) {
			put_colour_block(out, c0, c1, cbits);
		} else if (dxt == S2TC_O_DXT3) {
			/* explicit 4-bit alpha (:862-870) */
			uint64_t ab = 0;
			int i;
			for (x = 0; x < w; ++x)
				for (y = 0; y < h; ++y)
					ab |= (uint64_t)rgba[(y * iw + x) * 4 + 3] << (4 * (y * 4 + x));
			for (i = 0; i < 8; ++i) out[i] = (uint8_t)(ab >> (8 * i));
			put_colour_block(out + 8, c0, c1, cbits);
		} else {
			uint64_t ab = alpha_refine(rgba, iw, w, h, refine, &a0, &a1);
			int i;
			if (refine != S2TC_O_NEVER) leftover = a1;
			out[0] = (uint8_t)a0;
			out[1] = (uint8_t)a1;
			for (i = 0; i < 6; ++i) out[2 + i] = (uint8_t)(ab >> (8 * i));
			put_colour_block(out + 8, c0, c1, cbits);
		}
	}
	if (c != c_stack) free(c);
	if (ca != ca_stack) free(ca);
	return leftover;
}

/* One copy of the block encoder per distance metric, so that each copy calls
 * its metric directly (the reference's ColorDist template parameter,
 * s2tc_algorithm.cpp:1110-1180) and the compiler inlines it. */
int s2tc_oracle_encode_block_ex(uint8_t *out, const uint8_t *rgba, int iw, int w, int h,
				int dxt, int metric, int nrandom, int refine, int prev_a1)
{
#define ENC(D) encode_block(out, rgba, iw, w, h, dxt, metric, D, nrandom, refine, prev_a1)
	switch (metric) {
	case S2TC_O_RGB: return ENC(d_rgb);
	case S2TC_O_YUV: return ENC(d_yuv);
	case S2TC_O_SRGB: return ENC(d_srgb);
	case S2TC_O_SRGB_MIXED: return ENC(d_srgb_mixed);
	case S2TC_O_AVG: return ENC(d_avg);
	case S2TC_O_W0AVG: return ENC(d_w0avg);
	case S2TC_O_NORMALMAP: return ENC(d_normalmap);
	case S2TC_O_WAVG:
	default: return ENC(d_wavg);
	}
#undef ENC
}

void s2tc_oracle_encode_block(uint8_t *out, const uint8_t *rgba, int iw, int w, int h,
			      int dxt, int metric, int nrandom, int refine)
{
	s2tc_oracle_encode_block_ex(out, rgba, iw, w, h, dxt, metric, nrandom, refine, -1);
}

/* --------------------------------------------------------------- dithering */

/* One step of the 1-D error diffusion (s2tc_algorithm.cpp:1198-1207). */
static inline int diff_step(int *err, int src, int shift)
{
	int maxv = (1 << (8 - shift)) - 1;
	int v = src + *err;
	int q = v >> shift;
	if (q > maxv) q = maxv;
	if (q < 0) q = 0;
	*err = v - ((q << shift) | (q >> (8 - 2 * shift)));
	return q;
}
/* 1-bit variant (s2tc_algorithm.cpp:1208-1216). */
static inline int diff_step1(int *err, int src)
{
	int v = src + *err;
	int q = v >= 128;
	*err = v - (q ? 255 : 0);
	return q;
}
/* Floyd-Steinberg step on 12-bit values (s2tc_algorithm.cpp:1218-1261):
 * `cur` is this texel's slot in the current error row (its own error at
 * cur[1]), `nxt` the slot in the next row.  maxv==1 with shift 7 gives the
 * 1-bit variant. */
static inline int fs_step(int *cur, int *nxt, int src, int shift, int maxv)
{
	int v = ((src << 4) | (src >> 4)) + cur[1];
	int q, e, e7, e3, e5;
	if (maxv == 1) {
		q = v >= 2048;
		e = v - (q ? 4095 : 0);
	} else {
		q = v >> (shift + 4);
		if (q > maxv) q = maxv;
		if (q < 0) q = 0;
		e = v - q * 4095 / maxv;
	}
	e7 = (e * 7 + 8) / 16; e -= e7;
	e3 = (e * 3 + 4) / 9;  e -= e3;
	e5 = (e * 5 + 3) / 6;  e -= e5;
	cur[2] += e7;
	nxt[0] += e3;
	nxt[1] += e5;
	nxt[2] += e;
	return q;
}

/* RGB8/RGBA8 -> 4-byte texels r5 g6 b5 a(alphabits) (s2tc_algorithm.cpp:1263-1465). */
void s2tc_oracle_rgb565_image(uint8_t *out, const uint8_t *src, int w, int h, int srccomps,
			      int alphabits, int dither)
{
	long npx = (long)w * h, i;
	if (srccomps != 3) srccomps = 4;
	if (alphabits != 1 && alphabits != 4) alphabits = 8;
	if (dither != S2TC_O_DITHER_NONE && dither != S2TC_O_DITHER_FS) dither = S2TC_O_DITHER_SIMPLE;

	if (dither == S2TC_O_DITHER_NONE) {
		for (i = 0; i < npx; ++i) {
			out[i * 4 + 0] = src[i * srccomps + 0] >> 3;
			out[i * 4 + 1] = src[i * srccomps + 1] >> 2;
			out[i * 4 + 2] = src[i * srccomps + 2] >> 3;
		}
		for (i = 0; i < npx; ++i)
			out[i * 4 + 3] = srccomps == 3 ? (uint8_t)((1 << alphabits) - 1)
				       : (uint8_t)(src[i * 4 + 3] >> (8 - alphabits));
	} else if (dither == S2TC_O_DITHER_SIMPLE) {
		int er = 0, eg = 0, eb = 0, ea = 0;
		for (i = 0; i < npx; ++i) {
			out[i * 4 + 0] = (uint8_t)diff_step(&er, src[i * srccomps + 0], 3);
			out[i * 4 + 1] = (uint8_t)diff_step(&eg, src[i * srccomps + 1], 2);
			out[i * 4 + 2] = (uint8_t)diff_step(&eb, src[i * srccomps + 2], 3);
		}
		for (i = 0; i < npx; ++i) {
			if (srccomps == 3) out[i * 4 + 3] = (uint8_t)((1 << alphabits) - 1);
			else if (alphabits == 8) out[i * 4 + 3] = src[i * 4 + 3];
			else if (alphabits == 1) out[i * 4 + 3] = (uint8_t)diff_step1(&ea, src[i * 4 + 3]);
			else out[i * 4 + 3] = (uint8_t)diff_step(&ea, src[i * 4 + 3], 8 - alphabits);
		}
	} else {
		/* Six error rows of w+2 ints: current/next for r,g,b.  The alpha
		 * pass below reuses the first two rows without clearing the first,
		 * so it starts from the red pass's leftovers, as the reference does
		 * (s2tc_algorithm.cpp:1354, 1380-1382). */
		int pw = w + 2, x, y;
		int *rows = (int *)calloc((size_t)6 * pw, sizeof(int));
		for (y = 0; y < h; ++y) {
			int *cur = rows + ((y & 1) ? 3 : 0) * pw;
			int *nxt = rows + ((y & 1) ? 0 : 3) * pw;
			memset(nxt, 0, sizeof(int) * 3 * pw);
			for (x = 0; x < w; ++x) {
				const uint8_t *s = src + ((long)y * w + x) * srccomps;
				uint8_t *o = out + ((long)y * w + x) * 4;
				o[0] = (uint8_t)fs_step(cur + x, nxt + x, s[0], 3, 31);
				o[1] = (uint8_t)fs_step(cur + pw + x, nxt + pw + x, s[1], 2, 63);
				o[2] = (uint8_t)fs_step(cur + 2 * pw + x, nxt + 2 * pw + x, s[2], 3, 31);
			}
		}
		if (srccomps == 3 || alphabits == 8) {
			for (i = 0; i < npx; ++i)
				out[i * 4 + 3] = srccomps == 3 ? (uint8_t)((1 << alphabits) - 1) : src[i * 4 + 3];
		} else {
			for (y = 0; y < h; ++y) {
				int *cur = rows + (y & 1) * pw;
				int *nxt = rows + !(y & 1) * pw;
				memset(nxt, 0, sizeof(int) * pw);
				for (x = 0; x < w; ++x) {
					long p = (long)y * w + x;
					out[p * 4 + 3] = (uint8_t)(alphabits == 1
						? fs_step(cur + x, nxt + x, src[p * 4 + 3], 7, 1)
						: fs_step(cur + x, nxt + x, src[p * 4 + 3], 8 - alphabits,
							  (1 << alphabits) - 1));
				}
			}
		}
		free(rows);
	}
}

/* ------------------------------------------------------- libtxc_dxtn entry */

int s2tc_oracle_format_dxt(unsigned int fmt)
{
	switch (fmt) {
	case 0x83F0: case 0x83F1: return S2TC_O_DXT1;
	case 0x83F2: return S2TC_O_DXT3;
	case 0x83F3: return S2TC_O_DXT5;
	default: return -1;
	}
}

/* tx_compress_dxtn with the knobs passed explicitly
 * (s2tc_libtxc_dxtn.cpp:142-299).  `prev_a1` carries the second alpha
 * endpoint that the last block of the previous call left in the encoder's
 * stack slot (-1: none, the first block duplicates its own alpha); on return
 * it holds this call's leftover.  Returns 0, or -1 for a bad format (nothing
 * written). */
int s2tc_oracle_compress_ex(int srccomps, int width, int height, const uint8_t *src,
			    unsigned int fmt, uint8_t *dest, int dst_row_stride,
			    int dither, int metric, int nrandom, int refine, int *prev_a1)
{
	int dxt = s2tc_oracle_format_dxt(fmt);
	int bs, i, j;
	long row_diff;
	uint8_t *t565, *o = dest;
	if (dxt < 0) return -1;
	t565 = (uint8_t *)malloc((size_t)width * height * 4 + 1);
	s2tc_oracle_rgb565_image(t565, src, width, height, srccomps,
				 dxt == S2TC_O_DXT1 ? 1 : dxt == S2TC_O_DXT3 ? 4 : 8, dither);
	bs = dxt == S2TC_O_DXT1 ? 8 : 16;
	row_diff = dst_row_stride >= width * (bs / 4)
		 ? dst_row_stride - ((width + 3) & ~3) * (bs / 4) : 0;
	for (j = 0; j < height; j += 4) {
		int bh = height > j + 3 ? 4 : height - j;
		for (i = 0; i < width; i += 4) {
			int bw = width > i + 3 ? 4 : width - i;
			*prev_a1 = s2tc_oracle_encode_block_ex(o, t565 + ((long)j * width + i) * 4, width,
							       bw, bh, dxt, metric, nrandom, refine, *prev_a1);
			o += bs;
		}
		o += row_diff;
	}
	free(t565);
	return 0;
}

int s2tc_oracle_compress(int srccomps, int width, int height, const uint8_t *src,
			 unsigned int fmt, uint8_t *dest, int dst_row_stride,
			 int dither, int metric, int nrandom, int refine)
{
	int prev_a1 = -1;
	return s2tc_oracle_compress_ex(srccomps, width, height, src, fmt, dest, dst_row_stride,
				       dither, metric, nrandom, refine, &prev_a1);
}

/* ---------------------------------------------------------- texel decoders */
/* fetch_2d_texel_* (s2tc_libtxc_dxtn.cpp:35-140): decode texel (i,j) of an
 * image whose row is `stride` texels wide. */

static void expand565(unsigned c, uint8_t *t)
{
	int r = (c >> 11) & 31, g = (c >> 5) & 63, b = c & 31;
	t[0] = (uint8_t)((r << 3) | (r >> 2));
	t[1] = (uint8_t)((g << 2) | (g >> 4));
	t[2] = (uint8_t)((b << 3) | (b >> 2));
}

void s2tc_oracle_fetch(int dxt, int rgba_dxt1, int stride, const uint8_t *data, int i, int j, uint8_t *t)
{
	int bs = dxt == S2TC_O_DXT1 ? 8 : 16;
	const uint8_t *blk = data + ((long)((stride + 3) >> 2) * (j >> 2) + (i >> 2)) * bs;
	const uint8_t *cb = blk + (bs - 8);
	unsigned c = cb[0] | (cb[1] << 8), c1 = cb[2] | (cb[3] << 8);
	int sel = (cb[4 + (j & 3)] >> (2 * (i & 3))) & 3;
	int odd = (i ^ j) & 1;
	t[3] = 255;
	if (sel == 1) c = c1;
	else if (sel >= 2) {
		if (dxt == S2TC_O_DXT1 && sel == 3 && c1 >= c) {
			c = 0;
			if (rgba_dxt1) t[3] = 0;
		} else if (odd) c = c1;
	}
	expand565(c, t);
	if (dxt == S2TC_O_DXT3) {
		int a = (blk[(j & 3) * 2 + ((i & 3) >> 1)] >> (4 * (i & 1))) & 15;
		t[3] = (uint8_t)(a | (a << 4));
	} else if (dxt == S2TC_O_DXT5) {
		unsigned a = blk[0], a1 = blk[1];
		int bit = ((j & 3) * 4 + (i & 3)) * 3, ab = 0, k;
		for (k = 0; k < 3; ++k)
			if (blk[2 + ((bit + k) >> 3)] & (1 << ((bit + k) & 7))) ab |= 1 << k;
		if (ab == 1) a = a1;
		else if (ab == 6 && a1 >= a) a = 0;
		else if ((ab == 6 || ab == 7) && a1 >= a) a = 255;
		else if (ab >= 2 && odd) a = a1;
		t[3] = (uint8_t)a;
	}
}

/* ------------------------------------------------------ command-line tools */
/* The pipelines of the reference's three tools, with their file formats kept
 * in memory: s2tc_compress (RGBA in, DDS with a full mip chain out),
 * s2tc_decompress (DDS in, TGA out) and s2tc_from_s3tc (S3TC DDS in, S2TC DDS
 * out).  Image loading (LoadTGA_BGRA) is left to the caller: the input here is
 * the RGBA buffer that s2tc_compress.c:634-639 produces. */

/* Image_MipReduce32 towards 1x1 (s2tc_compress.c:426-493), out of place: a
 * dimension above 1 halves (rounding down, the odd last row/column is
 * dropped); 2x2, 2x1 or 1x2 boxes average with a truncating shift. */
void s2tc_oracle_mip_reduce(const uint8_t *in, uint8_t *out, int *width, int *height)
{
	int w = *width, h = *height, x, y, c;
	long row = (long)w * 4;
	if (w > 1) {
		w >>= 1;
		if (h > 1) {
			h >>= 1;
			for (y = 0; y < h; ++y)
				for (x = 0; x < w; ++x)
					for (c = 0; c < 4; ++c) {
						const uint8_t *p = in + 2 * y * row + 8 * x + c;
						out[((long)y * w + x) * 4 + c] = (uint8_t)((p[0] + p[4] + p[row] + p[row + 4]) >> 2);
					}
		} else {
			for (y = 0; y < h; ++y)
				for (x = 0; x < w; ++x)
					for (c = 0; c < 4; ++c) {
						const uint8_t *p = in + y * row + 8 * x + c;
						out[((long)y * w + x) * 4 + c] = (uint8_t)((p[0] + p[4]) >> 1);
					}
		}
	} else if (h > 1) {
		h >>= 1;
		for (y = 0; y < h; ++y)
			for (x = 0; x < w; ++x)
				for (c = 0; c < 4; ++c) {
					const uint8_t *p = in + 2 * y * row + 4 * x + c;
					out[((long)y * w + x) * 4 + c] = (uint8_t)((p[0] + p[row]) >> 1);
				}
	}
	*width = w;
	*height = h;
}

static void put32(uint8_t *p, uint32_t v)
{
	p[0] = (uint8_t)v; p[1] = (uint8_t)(v >> 8); p[2] = (uint8_t)(v >> 16); p[3] = (uint8_t)(v >> 24);
}

static uint32_t get32(const uint8_t *p)
{
	return p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

/* Bytes of the DDS file s2tc_compress writes for a width x height image. */
long s2tc_oracle_dds_size(int width, int height, unsigned int fmt)
{
	int dxt = s2tc_oracle_format_dxt(fmt), w = width, h = height;
	long n = 128, bs = dxt == S2TC_O_DXT1 ? 8 : 16;
	if (dxt < 0 || width < 1 || height < 1) return -1;
	for (;;) {
		n += (long)((w + 3) / 4) * ((h + 3) / 4) * bs;
		if (w == 1 && h == 1) break;
		if (w > 1) w >>= 1;
		if (h > 1) h >>= 1;
	}
	return n;
}

/* s2tc_compress's output for an RGBA image (s2tc_compress.c:641-719): the
 * 128-byte DDS header (mip count, base level size, "alpha pixels" flag when any
 * base texel has alpha != 255, FourCC), then every level from the base down to
 * 1x1, each compressed like tx_compress_dxtn with packed block rows.  Returns
 * the bytes written, or -1 for a bad format or size. */
long s2tc_oracle_dds(const uint8_t *rgba, int width, int height, unsigned int fmt,
		     int dither, int metric, int nrandom, int refine, uint8_t *out)
{
	int dxt = s2tc_oracle_format_dxt(fmt), mipcount = 0, w = width, h = height, alpha = 0;
	int prev_a1 = -1;  /* the encoder's stack slot, carried from level to level */
	long i, npx = (long)width * height, bs = dxt == S2TC_O_DXT1 ? 8 : 16;
	uint8_t *pic, *next, *o;
	if (dxt < 0 || width < 1 || height < 1) return -1;
	while (width >= (1 << mipcount) || height >= (1 << mipcount)) ++mipcount;
	for (i = 0; i < npx; ++i)
		if (rgba[i * 4 + 3] != 255) { alpha = 1; break; }
	memset(out, 0, 128);
	memcpy(out, "DDS ", 4);
	put32(out + 4, 0x7c);
	put32(out + 8, 0x000a1007);
	put32(out + 12, (uint32_t)height);
	put32(out + 16, (uint32_t)width);
	put32(out + 20, (uint32_t)(((width + 3) / 4) * ((height + 3) / 4) * bs));
	put32(out + 28, (uint32_t)mipcount);
	put32(out + 76, 0x20);
	put32(out + 80, alpha ? 5 : 4);
	memcpy(out + 84, dxt == S2TC_O_DXT1 ? "DXT1" : dxt == S2TC_O_DXT3 ? "DXT3" : "DXT5", 4);
	put32(out + 108, 0x00401008);
	o = out + 128;
	pic = (uint8_t *)malloc((size_t)npx * 4 + 4);
	next = (uint8_t *)malloc((size_t)npx * 4 + 4);
	memcpy(pic, rgba, (size_t)npx * 4);
	for (;;) {
		long lvl = (long)((w + 3) / 4) * ((h + 3) / 4) * bs;
		uint8_t *t;
		s2tc_oracle_compress_ex(4, w, h, pic, fmt, o, ((w + 3) / 4) * (int)bs, dither, metric, nrandom, refine,
					&prev_a1);
		o += lvl;
		if (w == 1 && h == 1) break;
		s2tc_oracle_mip_reduce(pic, next, &w, &h);
		t = pic; pic = next; next = t;
	}
	free(pic);
	free(next);
	return (long)(o - out);
}

/* s2tc_decompress (s2tc_decompress.c:156-207): the base level of a DXT1/3/5
 * DDS (height and width from header words 3 and 4, FourCC from word 21; DXT1
 * decodes with the RGBA variant) as an 18-byte TGA header and top-down BGRA
 * rows.  Returns the bytes written, or -1 for another FourCC. */
long s2tc_oracle_decompress(const uint8_t *dds, uint8_t *tga)
{
	int height = (int)get32(dds + 12), width = (int)get32(dds + 16), x, y, dxt;
	uint32_t fourcc = get32(dds + 84);
	uint8_t *o = tga + 18;
	if (fourcc == 0x31545844) dxt = S2TC_O_DXT1;
	else if (fourcc == 0x33545844) dxt = S2TC_O_DXT3;
	else if (fourcc == 0x35545844) dxt = S2TC_O_DXT5;
	else return -1;
	memset(tga, 0, 18);
	tga[2] = 2;
	tga[12] = (uint8_t)(width % 256);
	tga[13] = (uint8_t)(width / 256);
	tga[14] = (uint8_t)(height % 256);
	tga[15] = (uint8_t)(height / 256);
	tga[16] = 32;
	tga[17] = 0x28;
	for (y = 0; y < height; ++y)
		for (x = 0; x < width; ++x) {
			uint8_t t[4];
			s2tc_oracle_fetch(dxt, 1, width, dds + 128, x, y, t);
			o[0] = t[2]; o[1] = t[1]; o[2] = t[0]; o[3] = t[3];
			o += 4;
		}
	return (long)(o - tga);
}

/* s2tc_from_s3tc's colour block rewrite (s2tc_from_s3tc.cpp:77-143): every
 * index becomes 0 or 1 (index 2 and 3 map to the endpoint chosen by the
 * reference's bit formula), then the endpoints are put in S2TC order (c0 < c1
 * for a DXT1 block that keeps its transparent texels, else c0 > c1), with the
 * indices inverted on a swap.  `alpha` selects the DXT1 variant that keeps
 * index 3 as transparent when c1 >= c0. */
static void from_s3tc_colour(uint8_t *b, int alpha)
{
	unsigned c = b[0] | (b[1] << 8), c1 = b[2] | (b[3] << 8), t;
	uint32_t px = get32(b + 4);
	int swap;
	if (c1 >= c) {
		if (alpha) px = (px & ~((~px & 0x55555555u) << 1)) | ((px & 0x22882288u) >> 1);
		else px = (px & ((~px & 0xAAAAAAAAu) >> 1)) | ((px & 0x22882288u) >> 1);
		swap = !alpha;
	} else {
		px = (px & ((~px & 0xAAAAAAAAu) >> 1)) | ((px & 0x22882288u) >> 1);
		swap = alpha;
	}
	if (swap) {
		t = c; c = c1; c1 = t;
		px ^= 0x55555555u;
	}
	b[0] = (uint8_t)c; b[1] = (uint8_t)(c >> 8); b[2] = (uint8_t)c1; b[3] = (uint8_t)(c1 >> 8);
	put32(b + 4, px);
}

/* DXT5 alpha block rewrite (s2tc_from_s3tc.cpp:145-190): 3-bit indices 2..5
 * (and 6, 7 when a1 < a0) become 0 or 1, then a0 <= a1 order with the 0/1
 * indices inverted on a swap. */
static void from_s3tc_alpha(uint8_t *b)
{
	unsigned a = b[0], a1 = b[1], t;
	uint64_t px = 0, sel;
	const uint64_t ones = 01111111111111111ull, pick = 00101101001011010ull;
	int k;
	for (k = 0; k < 6; ++k) px |= (uint64_t)b[2 + k] << (8 * k);
	if (a1 >= a) {
		sel = (px >> 1) ^ (px >> 2);
		px = (px & ~((sel & ones) * 7)) | (sel & pick);
	} else {
		sel = (px >> 1) | (px >> 2);
		px = (px & ~((sel & ones) * 7)) | (sel & pick);
		t = a; a = a1; a1 = t;
		px ^= ones;
	}
	b[0] = (uint8_t)a;
	b[1] = (uint8_t)a1;
	for (k = 0; k < 6; ++k) b[2 + k] = (uint8_t)(px >> (8 * k));
}

/* One block of format `dxt` (s2tc_from_s3tc.cpp:255-262). */
void s2tc_oracle_from_s3tc_block(int dxt, uint8_t *blk)
{
	if (dxt == S2TC_O_DXT1) {
		from_s3tc_colour(blk, 1);
	} else {
		from_s3tc_colour(blk + 8, 0);
		if (dxt == S2TC_O_DXT5) from_s3tc_alpha(blk);
	}
}

/* s2tc_from_s3tc on a whole file (s2tc_from_s3tc.cpp:209-269): the 128-byte
 * header is copied, then every whole block that follows is converted (a
 * trailing partial block is dropped, as the reference's fread loop does).
 * Returns the bytes written, or -1 for another FourCC or a file shorter than
 * the header. */
long s2tc_oracle_from_s3tc(const uint8_t *in, long size, uint8_t *out)
{
	uint32_t fourcc;
	int dxt;
	long bs, n, i;
	if (size < 128) return -1;
	fourcc = get32(in + 84);
	if (fourcc == 0x31545844) dxt = S2TC_O_DXT1;
	else if (fourcc == 0x33545844) dxt = S2TC_O_DXT3;
	else if (fourcc == 0x35545844) dxt = S2TC_O_DXT5;
	else return -1;
	bs = dxt == S2TC_O_DXT1 ? 8 : 16;
	n = (size - 128) / bs;
	memcpy(out, in, 128);
	memcpy(out + 128, in + 128, (size_t)(n * bs));
	for (i = 0; i < n; ++i) s2tc_oracle_from_s3tc_block(dxt, out + 128 + i * bs);
	return 128 + n * bs;
}
