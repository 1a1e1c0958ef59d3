/*
 * s2tc_oracle.h -- TEST INFRASTRUCTURE ONLY: the CPU restatement of the S2TC
 * encode path used as the checker (see s2tc_oracle.c).  The enum values are
 * those of the reference's s2tc_algorithm.h:31-63.
 */
#ifndef S2TC_ORACLE_H
#define S2TC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { S2TC_O_DXT1 = 0, S2TC_O_DXT3 = 1, S2TC_O_DXT5 = 2 };
enum { S2TC_O_RGB = 0, S2TC_O_YUV, S2TC_O_SRGB, S2TC_O_SRGB_MIXED,
       S2TC_O_AVG, S2TC_O_WAVG, S2TC_O_W0AVG, S2TC_O_NORMALMAP };
enum { S2TC_O_NEVER = 0, S2TC_O_ALWAYS = 1, S2TC_O_LOOP = 2 };
enum { S2TC_O_DITHER_NONE = 0, S2TC_O_DITHER_SIMPLE = 1, S2TC_O_DITHER_FS = 2 };

int32_t s2tc_oracle_color_dist(int metric, int ar, int ag, int ab, int br, int bg, int bb);
void s2tc_oracle_encode_block(uint8_t *out, const uint8_t *rgba, int iw, int w, int h,
			      int dxt, int metric, int nrandom, int refine);
/* Returns the second alpha endpoint as the reference leaves it in its stack
 * slot (after refinement for ALWAYS/LOOP, before the final ordering swap for
 * NEVER); a following single-texel DXT5 block of the same call reads it. */
int s2tc_oracle_encode_block_ex(uint8_t *out, const uint8_t *rgba, int iw, int w, int h,
				int dxt, int metric, int nrandom, int refine, int prev_a1);
void s2tc_oracle_rgb565_image(uint8_t *out, const uint8_t *src, int w, int h, int srccomps,
			      int alphabits, int dither);
int s2tc_oracle_format_dxt(unsigned int fmt);
/* The random candidates read their words from `words` (n of them) instead of
 * libc's rand(); NULL restores rand().  _used() counts the words taken since. */
void s2tc_oracle_set_rand_words(const uint32_t *words, long n);
long s2tc_oracle_rand_words_used(void);
int s2tc_oracle_compress(int srccomps, int width, int height, const uint8_t *src,
			 unsigned int fmt, uint8_t *dest, int dst_row_stride,
			 int dither, int metric, int nrandom, int refine);
void s2tc_oracle_fetch(int dxt, int rgba_dxt1, int stride, const uint8_t *data, int i, int j,
		       uint8_t *texel);
/* the reference's command-line tools, in memory */
void s2tc_oracle_mip_reduce(const uint8_t *in, uint8_t *out, int *width, int *height);
long s2tc_oracle_dds_size(int width, int height, unsigned int fmt);
long s2tc_oracle_dds(const uint8_t *rgba, int width, int height, unsigned int fmt,
		     int dither, int metric, int nrandom, int refine, uint8_t *out);
long s2tc_oracle_decompress(const uint8_t *dds, uint8_t *tga);
void s2tc_oracle_from_s3tc_block(int dxt, uint8_t *blk);
long s2tc_oracle_from_s3tc(const uint8_t *in, long size, uint8_t *out);

#ifdef __cplusplus
}
#endif
#endif
