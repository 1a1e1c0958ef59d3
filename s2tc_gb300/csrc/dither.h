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

// Scratch bytes that launch_dither needs for an image of `npx` texels.
size_t dither_scratch_bytes(long long npx);
size_t dither_fs_scratch_bytes(int width, int height);

// Runs the reference's rgb565_image for `dither` (DI_NONE, DI_SIMPLE or
// DI_FLOYDSTEINBERG) on stream `s`.  `scratch` must hold the larger of the two
// scratch sizes above.
cudaError_t launch_dither(DitherArgs a, int dither, uint8_t* scratch, cudaStream_t s);
cudaError_t launch_dither_fs(DitherArgs a, uint8_t* scratch, cudaStream_t s);

}  // namespace s2tc
