// encode.h -- launch interface of the block encoder kernels (encode.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace s2tc {

struct EncodeArgs {
  const uint32_t* t565;  // 5:6:5 texel words, row length `width`
  int width, height;     // image size in texels
  int bw, bh;            // image size in blocks
  uint8_t* dst;          // first block
  long long pitch;       // bytes between block rows
  int aligned;           // dst and pitch allow 8/16-byte vector stores
  int by0, nby;          // block rows [by0, by0 + nby) are encoded by this launch
  int nrandom;           // S2TC_RANDOM_COLORS
  const uint32_t* rnd;   // replayed rand() words, nrandom*(3|4) per block in raster
                         // order, starting at block row by0
  int prev_a1_first;     // second alpha endpoint left by the block before block 0
                         // (-1: none); see encode.cu
  int* leftover_out;     // if set, receives the last block's leftover alpha endpoint
};

cudaError_t launch_encode_m0(const EncodeArgs&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m1(const EncodeArgs&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m2(const EncodeArgs&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m3(const EncodeArgs&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m4(const EncodeArgs&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m5(const EncodeArgs&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m6(const EncodeArgs&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m7(const EncodeArgs&, int dxt, bool normal, int refine, cudaStream_t);

// Dispatch on the metric; `normal` selects the all-candidates search
// (nrandom >= 0), which NORMALMAP always uses.
inline cudaError_t launch_encode(const EncodeArgs& a, int dxt, int metric, bool normal, int refine,
                                 cudaStream_t s) {
  switch (metric) {
    case 0: return launch_encode_m0(a, dxt, normal, refine, s);
    case 1: return launch_encode_m1(a, dxt, normal, refine, s);
    case 2: return launch_encode_m2(a, dxt, normal, refine, s);
    case 3: return launch_encode_m3(a, dxt, normal, refine, s);
    case 4: return launch_encode_m4(a, dxt, normal, refine, s);
    case 6: return launch_encode_m6(a, dxt, normal, refine, s);
    case 7: return launch_encode_m7(a, dxt, normal, refine, s);
    default: return launch_encode_m5(a, dxt, normal, refine, s);
  }
}

}  // namespace s2tc
