/*
 * s2tc_gb300.h -- C ABI of the GB300 S2TC encoder library (libs2tc_gb300.so).
 *
 * Part 1 is a drop-in for the reference's libtxc_dxtn plugin ABI and encoder
 * API: same symbol names, argument meaning, environment knobs, output bytes
 * and error behaviour.  Part 2 is the GPU extension (device pointers, streams,
 * batches, status codes).  All types are plain C; no CUDA or GL header is
 * needed to include this file (GLint = int, GLubyte = unsigned char,
 * GLenum = unsigned int, GLvoid = void, as in <GL/gl.h>).
 */
#ifndef S2TC_GB300_H
#define S2TC_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------
 * Part 1: reference-compatible entry points
 * ------------------------------------------------------------------------ */

/* GL_EXT_texture_compression_s3tc format enums accepted as `destformat`. */
#define S2TC_GL_COMPRESSED_RGB_S3TC_DXT1_EXT  0x83F0
#define S2TC_GL_COMPRESSED_RGBA_S3TC_DXT1_EXT 0x83F1
#define S2TC_GL_COMPRESSED_RGBA_S3TC_DXT3_EXT 0x83F2
#define S2TC_GL_COMPRESSED_RGBA_S3TC_DXT5_EXT 0x83F3

/* Enums with the reference's values (s2tc_algorithm.h:31-63). */
typedef enum { DITHER_NONE, DITHER_SIMPLE, DITHER_FLOYDSTEINBERG } DitherMode;
typedef enum { DXT1, DXT3, DXT5 } DxtMode;
typedef enum { REFINE_NEVER, REFINE_ALWAYS, REFINE_LOOP } RefinementMode;
typedef enum { RGB, YUV, SRGB, SRGB_MIXED, AVG, WAVG, W0AVG, NORMALMAP } ColorDistMode;

/* Compress a packed RGB8 (srccomps 3) or RGBA8 (any other srccomps) image of
 * width x height texels from host memory into S2TC DXT1/DXT3/DXT5 blocks at
 * `dest`, block rows dstRowStride bytes apart when dstRowStride is at least
 * the packed row size (else packed).  Reads S2TC_DITHER_MODE,
 * S2TC_COLORDIST_MODE, S2TC_RANDOM_COLORS and S2TC_REFINE_COLORS on every
 * call.  A bad format prints "libdxtn: Bad dstFormat ..." and writes
 * nothing.  The work runs on the GPU; the call returns when `dest` is written.
 * Replaces: txc_dxtn.h:47-49, s2tc_libtxc_dxtn.cpp:142-299. */
void tx_compress_dxtn(int srccomps, int width, int height, const unsigned char *srcPixData,
		      unsigned int destformat, unsigned char *dest, int dstRowStride);

/* Decode one texel (i, j) of a DXTn image whose rows are srcRowStride texels
 * wide into RGB(A)8 `texel`.  Host functions (one texel per call).
 * Replaces: txc_dxtn.h:38-45, s2tc_libtxc_dxtn.cpp:35-140. */
void fetch_2d_texel_rgb_dxt1(int srcRowStride, const unsigned char *pixdata, int i, int j, void *texel);
void fetch_2d_texel_rgba_dxt1(int srcRowStride, const unsigned char *pixdata, int i, int j, void *texel);
void fetch_2d_texel_rgba_dxt3(int srcRowStride, const unsigned char *pixdata, int i, int j, void *texel);
void fetch_2d_texel_rgba_dxt5(int srcRowStride, const unsigned char *pixdata, int i, int j, void *texel);

/* Quantise a host RGB8/RGBA8 image to 4-byte texels (r 0..31, g 0..63,
 * b 0..31, alpha with `alphabits` 1/4/8 bits) with the given dither, on the GPU.
 * Replaces: s2tc_algorithm.h:38, s2tc_algorithm.cpp:1453-1465. */
void rgb565_image(unsigned char *out, const unsigned char *rgba, int w, int h, int srccomps, int alphabits,
		  DitherMode dither);

/* Per-block encoder selected by format, metric, candidate count and
 * refinement, as in the reference; the returned function encodes one block of
 * a host 4-byte texel buffer (row length iw) and runs it on the GPU, one
 * launch per call (a compatibility path: batch through tx_compress_dxtn or the
 * extension API for throughput).
 * Replaces: s2tc_algorithm.h:65-66, s2tc_algorithm.cpp:1164-1194. */
typedef void (*s2tc_encode_block_func_t)(unsigned char *out, const unsigned char *rgba, int iw, int w, int h,
					 int nrandom);
s2tc_encode_block_func_t s2tc_encode_block_func(DxtMode dxt, ColorDistMode cd, int nrandom, RefinementMode refine);

/* ------------------------------------------------------------------------
 * Part 2: GPU extension API
 * ------------------------------------------------------------------------ */

/* Status codes. */
#define S2TC_OK 0
#define S2TC_ERR_ARGUMENT 1
#define S2TC_ERR_FORMAT 2
#define S2TC_ERR_CUDA 3
#define S2TC_ERR_NOMEM 4
#define S2TC_ERR_TIMEOUT 5
#define S2TC_ERR_TOO_LARGE 6

/* Encoder knobs with the meaning of the S2TC_* environment variables. */
typedef struct s2tc_options {
	int dither;  /* DitherMode */
	int metric;  /* ColorDistMode */
	int nrandom; /* S2TC_RANDOM_COLORS: <0 quick, 0 all texels, >0 extra random candidates */
	int refine;  /* RefinementMode */
} s2tc_options;

/* Fill `opt` from the environment exactly as tx_compress_dxtn does (defaults
 * SIMPLE / WAVG / -1 / ALWAYS; invalid values print the reference's message and
 * keep the default). */
void s2tc_options_from_env(s2tc_options *opt);

/* Compress one image that already lives in device memory, on `stream` (a
 * cudaStream_t, or NULL for the library's stream).  `d_dst` receives the
 * blocks, block rows dst_pitch bytes apart.  For opt->nrandom > 0 the random
 * candidates come from `d_rand` (nrandom*(3 or 4) rand() words per block in
 * raster order) or, when d_rand is NULL, from libc rand() replayed on the
 * host.  Scratch memory comes from the library's device arena.  Returns a
 * status code; asynchronous with respect to the host unless rand() is
 * replayed. */
int s2tc_gpu_compress(int srccomps, int width, int height, const void *d_src, unsigned int destformat, void *d_dst,
		      long long dst_pitch, const s2tc_options *opt, const unsigned int *d_rand, void *stream);

/* ---- batches: many images (textures, mip levels) of uneven sizes ---- */

/* One image of a batch: device pointers, as for s2tc_gpu_compress.  `rand`
 * optionally gives the image's replayed rand() words (nrandom*(3|4) per block
 * in raster order); when NULL and the knobs select random candidates, each run
 * draws them from libc rand() on the host, in image order, as one
 * tx_compress_dxtn call per image would. */
typedef struct s2tc_image {
	const void *src;
	int width, height, srccomps;
	unsigned int format;
	void *dst;
	long long dst_pitch;
	const unsigned int *rand;
} s2tc_image;

/* Compress each image with its own launches, one after another on `stream`
 * (the per-image path that batches replace; same bytes). */
int s2tc_gpu_compress_each(const s2tc_image *items, int count, const s2tc_options *opt, void *stream);

typedef struct s2tc_batch s2tc_batch;

/* Plan a batch: allocates the device scratch and tables for all images and
 * captures the whole launch sequence (the dither of every image, then one
 * encoder launch per block format) in a CUDA graph.  The images' pointers and
 * sizes are fixed for the plan; their contents may change between runs. */
int s2tc_batch_create(s2tc_batch **out, const s2tc_image *items, int count, const s2tc_options *opt);
/* Replay the plan on `stream` (NULL: the library's stream); asynchronous.
 * Runs of one plan are serialised. */
int s2tc_batch_run(s2tc_batch *batch, void *stream);
/* Number of kernels one run launches. */
int s2tc_batch_kernels(const s2tc_batch *batch);
void s2tc_batch_destroy(s2tc_batch *batch);

/* ---- serving: a request loop with continuous batching ---- */

typedef struct s2tc_server s2tc_server;

/* Start a server whose requests share `budget_bytes` of device memory (input,
 * texel words, output and rand words of every admitted request).  A
 * scheduler thread admits waiting requests in arrival order as memory frees
 * up and launches each group of admitted requests as one round of batched
 * kernels; rounds overlap on the GPU.  Pass pinned host buffers so that the
 * uploads and downloads overlap too. */
int s2tc_server_create(s2tc_server **out, long long budget_bytes);
/* Queue one compression (host pixels in, host blocks out, block rows
 * dst_pitch bytes apart or packed when 0); returns immediately with an id.
 * Random candidates draw libc rand() here, in submission order.  A request
 * larger than the whole budget is rejected with S2TC_ERR_TOO_LARGE. */
int s2tc_server_submit(s2tc_server *server, const void *src, int srccomps, int width, int height,
		       unsigned int format, const s2tc_options *opt, void *dst, long long dst_pitch,
		       long long *id);
/* The same for device-resident requests: `d_src` and `d_dst` are device
 * pointers; nothing is copied, the pool holds only the request's texel words
 * (and random-candidate words), and the blocks are written straight into
 * `d_dst` (block rows `dst_pitch` bytes apart, 0 = packed).  The input must
 * stay valid and the output untouched until s2tc_server_wait returns. */
int s2tc_server_submit_device(s2tc_server *server, const void *d_src, int srccomps, int width, int height,
			      unsigned int format, const s2tc_options *opt, void *d_dst, long long dst_pitch,
			      long long *id);
/* Block until request `id` is done; its latency (submission to completion)
 * in milliseconds.  Each id can be waited for once. */
int s2tc_server_wait(s2tc_server *server, long long id, double *latency_ms);
/* Rounds launched, requests done, most rounds in flight at once, most
 * requests in one round, device pool high-water mark in bytes. */
int s2tc_server_stats(s2tc_server *server, long long *rounds, long long *done, int *max_inflight_rounds,
		      int *max_round_requests, long long *pool_high_water);
/* Finish the queued requests and stop. */
void s2tc_server_destroy(s2tc_server *server);

/* Wait for `stream` (NULL: the library's stream) and report whether any
 * kernel since the last check gave up a bounded wait (S2TC_ERR_TIMEOUT). */
int s2tc_gpu_synchronize(void *stream);

/* Test hook of the timeout path; no counterpart in the reference.  Launches
 * of the SIMPLE dither made (or captured into a graph) after this call keep
 * dither tile `hold_tile` of their work list (16640 texels per tile, raster
 * order; -1: none) from publishing its scan state, and give up each
 * look-back wait after `spin_limit` polls (0: the library's default limit,
 * about 4 M polls).  The tiles that wait on the held tile give up, and the
 * call reports S2TC_ERR_TIMEOUT (s2tc_gpu_synchronize, or the error text of
 * tx_compress_dxtn) with undefined output; nothing faults or hangs.  Call it
 * with (-1, 0) to restore normal operation. */
int s2tc_test_dither_hold(long long hold_tile, int spin_limit);

/* Number of rand() words an image consumes: blocks * nrandom * (4 for DXT5,
 * else 3) when the random-candidate search is active, else 0. */
long long s2tc_rand_words(int width, int height, unsigned int destformat, const s2tc_options *opt);

/* Profiling hook: while enabled, every compression records CUDA events on its
 * stream before the dither kernel, between the dither and encoder kernels and
 * after the encoder (up to 4096 calls after each enable).  s2tc_gpu_stage_ms
 * waits for them and returns the summed stage durations in milliseconds and
 * the number of calls they cover. */
int s2tc_gpu_set_timing(int enable);
int s2tc_gpu_stage_ms(float *dither_ms, float *encode_ms, long long *calls);

/* Number of CUDA kernels this library has launched since it was loaded. */
long long s2tc_gpu_kernel_launches(void);

/* The per-block encoder that s2tc_encode_block_func(dxt, colordist, nrandom,
 * refine) selects (s2tc_algorithm.h:65-66, s2tc_algorithm.cpp:1110-1194),
 * over every 4x4 block of a device-resident texel image in the layout
 * rgb565_image produces (one word r | g<<8 | b<<16 | a<<24 per texel, rows of
 * `width` words): the batched form of that per-block function.  Blocks are
 * encoded as tx_compress_dxtn's block loop encodes them (edge blocks of
 * min(4, width - x) x min(4, height - y) texels); block rows go `dst_pitch`
 * bytes apart.  RANDOM_COLORS > 0 draws libc rand() on the host unless
 * `d_rand` supplies the replayed words.  Asynchronous on `stream`. */
int s2tc_gpu_encode_blocks(const void *d_t565, int width, int height, int dxt, int colordist, int nrandom,
			   int refine, void *d_dst, long long dst_pitch, const unsigned int *d_rand, void *stream);

/* Compress one device-resident image without allocating any memory.  No
 * counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc (engines whose frame budget or memory pool forbids allocator
 * calls).  Same arguments and bytes as s2tc_gpu_compress, but the scratch
 * (dither state and 5:6:5 texel words) lives in one fixed device array of the
 * library, held on every GPU that loads it until exit; images are limited to
 * 4 Mi texels (S2TC_ERR_TOO_LARGE beyond; with Floyd-Steinberg dither also
 * ceil(width/8)*8 * ceil(height/256) <= 65520, so that its carry rows fit the
 * array's 1 MiB scan region: a 65536x64 image is rejected, every image up to
 * 2048x2048 fits), RANDOM_COLORS > 0 needs `d_rand`,
 * and the call waits for `stream` before returning.  The first call on a
 * device sets up the array's address: make it before any stream capture.
 * Calls are serialised within the process; calls whose GPU work overlaps
 * (e.g. from another library instance) race on the shared array. */
int s2tc_gpu_compress_noalloc(int srccomps, int width, int height, const void *d_src, unsigned int destformat,
			      void *d_dst, long long dst_pitch, const s2tc_options *opt, const unsigned int *d_rand,
			      void *stream);

/* Launch layout of the encoder for one mode (format, colour distance,
 * RANDOM_COLORS > 0 / = 0 / quick, refinement): threads per CTA of the
 * thread-per-block kernels (32..128), and warps per CTA (1..4) and CTAs per
 * SM of the random-candidate kernel's persistent grid.  No counterpart in the
 * reference: layouts change speed only, never bytes.  s2tc_autotune times
 * the candidate layouts of a mode on a synthetic width x height image (it
 * does not consume libc rand()) and keeps the fastest for the rest of the
 * process; `best_ms` (may be NULL) receives that layout's encoder time.
 * s2tc_encode_layout_set sets one by hand. */
int s2tc_autotune(const s2tc_options *opt, unsigned int format, int width, int height, float *best_ms);
int s2tc_encode_layout_set(const s2tc_options *opt, unsigned int format, int threads, int rand_warps,
			   int rand_ctas_per_sm);
int s2tc_encode_layout_get(const s2tc_options *opt, unsigned int format, int *threads, int *rand_warps,
			   int *rand_ctas_per_sm);

/* ---------------------------------------------------------------------
 * Part 3: the reference's command-line tools, in memory, on the GPU.
 * --------------------------------------------------------------------- */

/* Bytes of the DDS file s2tc_compress writes for a width x height image in
 * `format` (header + every mip level down to 1x1), or -1 for a bad format or
 * size. */
long long s2tc_dds_size(int width, int height, unsigned int format);

/* s2tc_compress (s2tc_compress.c:594-719) from the RGBA8 buffer it builds
 * after loading its TGA (s2tc_compress.c:634-639): writes the DDS file (128-
 * byte header, then every mip level from `width` x `height` down to 1x1,
 * Image_MipReduce32 box filter, s2tc_compress.c:426-493) into `out`, which
 * must hold s2tc_dds_size bytes.  `format` is the GL enum the tool's `-t`
 * selects (DXT1 = GL_COMPRESSED_RGBA_S3TC_DXT1_EXT).  `opt` NULL reads the
 * S2TC_* environment like tx_compress_dxtn.  Levels are built and encoded on
 * the GPU; rand() is drawn per level in order, as the tool's
 * tx_compress_dxtn calls draw it. */
int s2tc_compress_dds(const void *rgba, int width, int height, unsigned int format, const s2tc_options *opt,
		      void *out, long long out_size, long long *written);

/* Decode a whole image of S2TC/S3TC blocks (packed block rows) on the GPU
 * with the semantics of fetch_2d_texel_rgb_dxt1 (format
 * GL_COMPRESSED_RGB_S3TC_DXT1_EXT), _rgba_dxt1, _rgba_dxt3 and _rgba_dxt5
 * (s2tc_libtxc_dxtn.cpp:35-140), including their checkerboard decode of
 * indices 2 and 3.  Output: RGBA8 texels (BGRA8 when `bgra` is non-zero),
 * rows `dst_pitch` bytes apart (0: width*4).  Asynchronous on `stream`. */
int s2tc_gpu_decode(const void *d_blocks, unsigned int format, int width, int height, void *d_out,
		    long long dst_pitch, int bgra, void *stream);

/* s2tc_decompress (s2tc_decompress.c:156-207) in memory: the base level of a
 * DXT1/DXT3/DXT5 DDS file as an uncompressed 32-bit TGA (18-byte header, BGRA
 * rows top to bottom); `tga` must hold 18 + width*height*4 bytes.  Another
 * FourCC prints the tool's message and returns S2TC_ERR_FORMAT. */
int s2tc_decompress_dds(const void *dds, long long size, void *tga, long long tga_size, long long *written);

/* s2tc_from_s3tc's per-block rewrite (s2tc_from_s3tc.cpp:77-190) of `nblocks`
 * device-resident blocks of `format` (DXT1 blocks keep transparent texels;
 * DXT3/DXT5 colour halves and DXT5 alpha halves are rewritten).  `d_src` may
 * equal `d_dst`.  Asynchronous on `stream`. */
int s2tc_gpu_from_s3tc(const void *d_src, void *d_dst, long long nblocks, unsigned int format, void *stream);

/* s2tc_from_s3tc (s2tc_from_s3tc.cpp:209-269) in memory: copies the 128-byte
 * header and converts every whole block after it (a trailing partial block is
 * dropped, as the tool's read loop does).  `out` must hold `size` bytes. */
int s2tc_from_s3tc_dds(const void *dds, long long size, void *out, long long out_size, long long *written);

/* Text of the last error this thread saw (empty when none). */
const char *s2tc_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
