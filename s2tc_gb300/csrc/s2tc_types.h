// s2tc_types.h -- enums and launch descriptors shared by the host layer and the
// CUDA kernels.  Enum values equal the reference's (s2tc_algorithm.h:31-63).
#pragma once
#include <cstdint>

namespace s2tc {

enum Dxt { DXT1 = 0, DXT3 = 1, DXT5 = 2 };
enum Metric {
  CD_RGB = 0,
  CD_YUV = 1,
  CD_SRGB = 2,
  CD_SRGB_MIXED = 3,
  CD_AVG = 4,
  CD_WAVG = 5,
  CD_W0AVG = 6,
  CD_NORMALMAP = 7
};
enum Refine { RF_NEVER = 0, RF_ALWAYS = 1, RF_LOOP = 2 };
enum Dither { DI_NONE = 0, DI_SIMPLE = 1, DI_FLOYDSTEINBERG = 2 };

// Status codes of the extension API (0 = success).
enum Status {
  ST_OK = 0,
  ST_BAD_ARGUMENT = 1,
  ST_BAD_FORMAT = 2,
  ST_CUDA_ERROR = 3,
  ST_OUT_OF_MEMORY = 4,
  ST_TIMEOUT = 5,
  ST_TOO_LARGE = 6
};

inline int block_bytes(int dxt) { return dxt == DXT1 ? 8 : 16; }
inline int alpha_bits(int dxt) { return dxt == DXT1 ? 1 : dxt == DXT3 ? 4 : 8; }

}  // namespace s2tc
