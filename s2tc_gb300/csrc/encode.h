// encode.h -- launch interface of the block encoder kernels (encode.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "dither.h"

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

// Fused strip kernel of the quick mode (encode.cu, k_strip_quick): the NONE
// or SIMPLE dither and the quick encoder in one launch, one CTA of 256
// threads per band of `rows_per_band` whole block rows, the texel words kept
// in shared memory.  A thread scans `seg` texels: 65, or 17 where 65 would
// leave the GPU with fewer bands than it holds CTAs (small images: more,
// shorter bands).  Rows of at most kStripMaxWidth texels; wider images take
// the two kernels, which were faster there (a 512-thread variant for 8192-wide
// rows ran 16% slower than the separate dither and encoder launches).
constexpr int kStripThreads = 256;
constexpr int kStripMaxWidth = kStripThreads * 65 / 4;  // 4160
constexpr long long kStripFullBands = 2 * 152;          // bands that fill the GPU (two CTAs per SM)

struct StripPlan {
  int seg;            // texels per thread of the scan (17 or 65)
  int rows_per_band;  // block rows per band
  long long bands;
};
inline bool strip_plan(int width, int height, StripPlan& p) {
  if (width <= 0 || height <= 0 || width > kStripMaxWidth) return false;
  const long long four_w = 4ll * width, bh = (height + 3) / 4;
  for (int seg : {65, 17}) {
    if (four_w > kStripThreads * seg) break;
    p.seg = seg;
    p.rows_per_band = int(kStripThreads * seg / four_w);
    p.bands = (bh + p.rows_per_band - 1) / p.rows_per_band;
    if (p.bands >= kStripFullBands) break;
  }
  return true;
}

struct StripArgs {
  const uint8_t* src;   // packed RGB8/RGBA8
  int width, height, srccomps, alphabits;
  int dither;           // DI_NONE or DI_SIMPLE
  uint8_t* dst;         // first block
  long long pitch;      // bytes between block rows
  int aligned;          // dst and pitch allow 8/16-byte stores
  int seg, rows_per_band;
  long long band_base;  // bands [band_base, band_base + nbands) of the image
  long long nbands;
  long long image_bands;  // bands of the whole image (the scan state's layout)
  int single_band;      // one band in all: the CTA takes band 0 without a ticket
  int use_tma;          // RGBA8 rows through the tensor map (16-byte aligned source)
  long long tma_rows;   // 256-texel rows the tensor map covers (texels / 256)
  DitherWork scan;      // scan state: status, aggs, ticket (zeroed by the launcher), error
  // optional: the CTA that finishes last sets *done_flag (host memory) after
  // every block is written; *done_count (zeroed) counts finished bands
  unsigned int* done_count;
  int* done_flag;
};

// Launches k_strip_quick over a.nbands bands; `scratch` holds
// dither_batch_scratch_bytes(a.image_bands) (the launch zeroes the status
// words of its bands and its ticket; ranges of one image launched in order
// on one stream chain through it).  With `scratch` null the scan state is
// a.scan.status / aggs / ticket as given, already zeroed by the caller (one
// launch per image).  `tmap` is the CUtensorMap of
// the source (ignored unless a.use_tma).  Returns cudaErrorNotSupported for a
// metric without the quick selection (NORMALMAP).
cudaError_t launch_strip_m0(StripArgs, const void* tmap, int dxt, int refine, uint8_t* scratch, cudaStream_t);
cudaError_t launch_strip_m1(StripArgs, const void* tmap, int dxt, int refine, uint8_t* scratch, cudaStream_t);
cudaError_t launch_strip_m2(StripArgs, const void* tmap, int dxt, int refine, uint8_t* scratch, cudaStream_t);
cudaError_t launch_strip_m3(StripArgs, const void* tmap, int dxt, int refine, uint8_t* scratch, cudaStream_t);
cudaError_t launch_strip_m4(StripArgs, const void* tmap, int dxt, int refine, uint8_t* scratch, cudaStream_t);
cudaError_t launch_strip_m5(StripArgs, const void* tmap, int dxt, int refine, uint8_t* scratch, cudaStream_t);
cudaError_t launch_strip_m6(StripArgs, const void* tmap, int dxt, int refine, uint8_t* scratch, cudaStream_t);
cudaError_t launch_strip_m7(StripArgs, const void* tmap, int dxt, int refine, uint8_t* scratch, cudaStream_t);
inline cudaError_t launch_strip(const StripArgs& a, const void* tmap, int dxt, int metric, int refine,
                                uint8_t* scratch, cudaStream_t s) {
  switch (metric) {
    case 0: return launch_strip_m0(a, tmap, dxt, refine, scratch, s);
    case 1: return launch_strip_m1(a, tmap, dxt, refine, scratch, s);
    case 2: return launch_strip_m2(a, tmap, dxt, refine, scratch, s);
    case 3: return launch_strip_m3(a, tmap, dxt, refine, scratch, s);
    case 4: return launch_strip_m4(a, tmap, dxt, refine, scratch, s);
    case 6: return launch_strip_m6(a, tmap, dxt, refine, scratch, s);
    case 7: return launch_strip_m7(a, tmap, dxt, refine, scratch, s);
    default: return launch_strip_m5(a, tmap, dxt, refine, scratch, s);
  }
}

// Builds NORMALMAP's table of prepared colours on the current device and
// waits for it (once per device, outside any stream capture; kernels compute
// the form themselves until the table is ready, so calling it is optional).
cudaError_t nm_table_init(cudaStream_t s);

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
