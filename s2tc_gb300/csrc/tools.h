// tools.h -- kernels behind the reference's command-line tools (tools.cu):
// mip reduction and the "any alpha below 255" test of s2tc_compress, the
// texel decoder of s2tc_decompress, and the block rewrite of s2tc_from_s3tc.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace s2tc {

// One Image_MipReduce32 step towards 1x1 on RGBA8 texels (out of place):
// (w, h) -> (w > 1 ? w/2 : 1, h > 1 ? h/2 : 1).
cudaError_t launch_mip_reduce(const uint8_t* in, int w, int h, uint8_t* out, cudaStream_t s);

// *flag |= 1 if any of the `npx` RGBA8 texels has alpha != 255.
cudaError_t launch_any_alpha(const uint8_t* rgba, long long npx, int* flag, cudaStream_t s);

// The size of one mip step.
inline void mip_next(int& w, int& h) {
  if (w > 1) w >>= 1;
  if (h > 1) h >>= 1;
}

}  // namespace s2tc
