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
  const int* prev_a1_dev;  // if set, that value is read from device memory instead
                           // (it may be this launch's own leftover_out)
  int* leftover_out;     // if set, receives the last block's leftover alpha endpoint
};

// Blocks to encode: one image (`single`, items == null) or many images of the
// same format whose blocks are numbered consecutively (`offsets[i]` = first
// block of image i; every image has at least one block).  All images share
// nrandom (the knobs of a launch are uniform).
struct EncodeWork {
  const EncodeArgs* items;   // device array, or null
  const long long* offsets;  // device array, nitems entries
  int nitems;
  long long total;           // blocks in all images
  int nrandom;               // S2TC_RANDOM_COLORS of every image
  EncodeArgs single;
};

// Launch layout of the encoder kernels for one mode (the autotuner's knobs;
// no effect on the bytes).
enum { kLayoutQuick = 0, kLayoutFull = 1, kLayoutRand = 2 };
struct EncodeLayout {
  int threads;           // threads per CTA of the thread-per-block kernels (32..128)
  int rand_warps;        // warps per CTA of the random-candidate kernel (1..4)
  int rand_ctas_per_sm;  // its persistent grid: CTAs per SM
};
EncodeLayout encode_layout(int metric, int dxt, int refine, int kind);
void set_encode_layout(int metric, int dxt, int refine, int kind, EncodeLayout layout);

cudaError_t launch_encode_m0(const EncodeWork&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m1(const EncodeWork&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m2(const EncodeWork&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m3(const EncodeWork&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m4(const EncodeWork&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m5(const EncodeWork&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m6(const EncodeWork&, int dxt, bool normal, int refine, cudaStream_t);
cudaError_t launch_encode_m7(const EncodeWork&, int dxt, bool normal, int refine, cudaStream_t);

// Dispatch on the metric; `normal` selects the all-candidates search
// (nrandom >= 0), which NORMALMAP always uses.
inline cudaError_t launch_encode(const EncodeWork& w, int dxt, int metric, bool normal, int refine,
                                 cudaStream_t s) {
  switch (metric) {
    case 0: return launch_encode_m0(w, dxt, normal, refine, s);
    case 1: return launch_encode_m1(w, dxt, normal, refine, s);
    case 2: return launch_encode_m2(w, dxt, normal, refine, s);
    case 3: return launch_encode_m3(w, dxt, normal, refine, s);
    case 4: return launch_encode_m4(w, dxt, normal, refine, s);
    case 6: return launch_encode_m6(w, dxt, normal, refine, s);
    case 7: return launch_encode_m7(w, dxt, normal, refine, s);
    default: return launch_encode_m5(w, dxt, normal, refine, s);
  }
}

// One image: block rows [a.by0, a.by0 + a.nby).
inline cudaError_t launch_encode(const EncodeArgs& a, int dxt, int metric, bool normal, int refine,
                                 cudaStream_t s) {
  EncodeWork w{};
  w.items = nullptr;
  w.offsets = nullptr;
  w.nitems = 1;
  w.total = (long long)a.bw * a.nby;
  w.nrandom = a.nrandom;
  w.single = a;
  return launch_encode(w, dxt, metric, normal, refine, s);
}

}  // namespace s2tc
