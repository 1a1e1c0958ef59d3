// rand_glibc.h -- libc rand() words for the random-candidate mode, generated
// on the GPU (rand_glibc.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace s2tc {

// A position in libc's rand() stream: the additive generator's last 31 values
// v[-31..-1] followed by the next 30, v[0..29].  The outputs are v[k] >> 1.
struct RandWindow {
  uint32_t ext[61];
};

// Takes the next `n` rand() outputs of this process: fills `w` with the
// stream's current position and advances libc's generator by n outputs, as n
// calls of rand() would, without generating them.  Returns false (and leaves
// the generator alone) when libc's generator is not glibc's default additive
// one; callers then call rand() n times themselves.
bool rand_take(long long n, RandWindow* w);

// Whether rand_take works here (glibc's default generator in use);
// S2TC_HOST_RAND=1 in the environment makes it false, so that callers take
// the host loop instead.
bool rand_usable();

// Uploads the generator's jump table (once; call before any stream capture).
cudaError_t rand_prepare();

// out[k] = the k-th output after window `d_w` (a device copy), k < n.
cudaError_t rand_fill(const RandWindow* d_w, uint32_t* d_out, long long n, cudaStream_t s);

// Below this many words the host loop is cheaper than a launch.
constexpr long long kRandDeviceMin = 1 << 14;

}  // namespace s2tc
