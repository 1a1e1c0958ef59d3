// dither.h -- launch interface of the dither kernels (dither.cu, dither_fs.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "s2tc_types.h"

namespace s2tc {

// Kernels launched by this library since load (all translation units).
void count_launches(int n);
long long launches_so_far();

struct DitherArgs {
  const uint8_t* src;  // packed RGB8/RGBA8, `width * srccomps` bytes per row
  int width, height, srccomps;
  int alphabits;       // 1 (DXT1), 4 (DXT3) or 8 (DXT5)
  uint32_t* dst;       // width*height texel words r | g<<8 | b<<16 | a<<24
  int* error;          // set to 1 when a bounded wait gives up
  // filled in by launch_dither
  int alpha_const;
  unsigned long long* status;
  uint8_t* aggs;
  unsigned int* ticket;
};

// One image of a batched dither launch.
struct DitherItem {
  const uint8_t* src;
  int width, height, srccomps, alphabits;
  uint32_t* dst;
};

// Batched DITHER_NONE / DITHER_SIMPLE over many images: the images' 16384-texel
// tiles are numbered consecutively (`tile_offsets[i]` = first tile of image i,
// images with no texels left out) and every CTA takes one tile.
struct DitherWork {
  const DitherItem* items;      // device array, or null for the single image below
  const long long* tile_offsets;  // device array, nitems entries
  int nitems;
  DitherItem single;
  long long total_tiles;         // tiles of this launch
  long long tile_base;           // global index of its first tile (0 unless a launch covers a range)
  int* error;
  unsigned long long* status;   // total_tiles status words (zeroed before launch)
  uint8_t* aggs;                // total_tiles aggregate tables
  unsigned int* ticket;         // zeroed before launch
  // test hook (set_dither_test_hold): the look-back's spin limit (0: the
  // default) and a tile that publishes nothing (-1: none)
  int spin_limit;
  long long hold_tile;
};

// Test hook of the timeout path: launches of the SIMPLE dither made after this
// call keep tile `hold_tile` (global index within a launch's work list; -1:
// none) from publishing its scan state, and give up each look-back wait after
// `spin_limit` polls (0: the default limit).  The tiles behind a held tile
// time out, set the error flag and finish; the call reports S2TC_ERR_TIMEOUT.
void set_dither_test_hold(long long hold_tile, int spin_limit);
// The values set_dither_test_hold set last (for other kernels that run the scan).
void dither_test_hold_values(long long* hold_tile, int* spin_limit);

// Texels per tile of the batched/SIMPLE dither kernels.
long long dither_tile_texels();

// Scratch bytes that launch_dither needs for an image of `npx` texels, and
// that launch_dither_batch needs for `tiles` tiles in total.
size_t dither_scratch_bytes(long long npx);
size_t dither_batch_scratch_bytes(long long tiles);
size_t dither_fs_scratch_bytes(int width, int height);

// DITHER_NONE / DITHER_SIMPLE over tiles [t0, t1) of one image only, for
// pipelined callers that launch an image's tiles in order, range by range, on
// one stream (each range's look-back reaches into the earlier ranges).
// `scratch` holds dither_scratch_bytes for the whole image; the first range
// must start at tile 0.
cudaError_t launch_dither_range(DitherArgs a, int dither, uint8_t* scratch, long long t0, long long t1,
                                cudaStream_t s);

// Runs the reference's rgb565_image for `dither` (DI_NONE, DI_SIMPLE or
// DI_FLOYDSTEINBERG) on stream `s`.  `scratch` must hold the larger of the two
// scratch sizes above.
cudaError_t launch_dither(DitherArgs a, int dither, uint8_t* scratch, cudaStream_t s);
cudaError_t launch_dither_fs(DitherArgs a, uint8_t* scratch, cudaStream_t s);
// Batched NONE / SIMPLE dither (`dither` DI_NONE or DI_SIMPLE); `w.status`,
// `w.aggs` and `w.ticket` point into `scratch` once this returns.
cudaError_t launch_dither_batch(DitherWork w, int dither, uint8_t* scratch, cudaStream_t s);

}  // namespace s2tc
