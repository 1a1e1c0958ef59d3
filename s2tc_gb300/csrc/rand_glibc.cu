// rand_glibc.cu -- the random-candidate mode's rand() words on the GPU.
//
// The reference draws libc rand() for every random candidate
// (s2tc_algorithm.cpp:986-990), and byte parity needs exactly that stream.
// glibc's rand() is srandom's additive feedback generator (TYPE_3: a ring of
// 31 words, separation 3): every call adds the word 3 places behind, so the
// sequence of ring values obeys
//   v[t] = v[t-31] + v[t-3]   (mod 2^32),  output = v[t] >> 1.
// The recurrence is linear over Z/2^32, so for any m,
//   v[t+m] = sum_i a_i v[t+i]  where  x^m = sum_i a_i x^i  mod  x^31 - x^28 - 1,
// and a chunk of the stream starting m values ahead is reached with
// O(log m) products of degree-30 polynomials.  Each GPU thread jumps to its
// chunk this way and then runs the recurrence for its values; the host
// jumps libc's own state ahead by the words consumed, so a later rand() in
// the process continues exactly where the reference's encoder would have
// left it.
//
// libc's state is read and written through the standard setstate() call:
// switching to a scratch state array makes glibc record the current ring
// position in its own array (word -1 = 5 * rear index + generator type), whose
// words 0..30 are the ring; the updated ring and position are put back by
// switching to that array again.  Another thread calling rand() between the
// two setstate() calls would see the scratch state; the reference's encoder
// is not thread-safe with respect to rand() either.
#include <cuda_runtime.h>

#include <cstdlib>
#include <cstring>
#include <mutex>

#include "dither.h"
#include "rand_glibc.h"

namespace s2tc {
namespace {

constexpr int kDeg = 31, kSep = 3, kTypes = 5, kType3 = 3;
constexpr int kPowers = 63;            // x^(2^k) mod f for k < 63

// Polynomials mod f(x) = x^31 - x^28 - 1 over Z/2^32, 31 coefficients.
__host__ __device__ inline void poly_mulmod(const uint32_t* a, const uint32_t* b, uint32_t* out) {
  uint32_t c[2 * kDeg - 1];
#pragma unroll
  for (int k = 0; k < 2 * kDeg - 1; ++k) c[k] = 0;
#pragma unroll
  for (int i = 0; i < kDeg; ++i) {
    const uint32_t ai = a[i];
#pragma unroll
    for (int j = 0; j < kDeg; ++j) c[i + j] += ai * b[j];
  }
  // x^k = x^(k-3) + x^(k-31), highest degree first
#pragma unroll
  for (int k = 2 * kDeg - 2; k >= kDeg; --k) {
    c[k - 3] += c[k];
    c[k - kDeg] += c[k];
  }
#pragma unroll
  for (int i = 0; i < kDeg; ++i) out[i] = c[i];
}

struct PowerTable {
  uint32_t t[kPowers][kDeg];
};

const PowerTable& host_powers() {
  static PowerTable* p = [] {
    auto* q = new PowerTable();
    std::memset(q, 0, sizeof(*q));
    q->t[0][1] = 1;  // x
    for (int k = 1; k < kPowers; ++k) poly_mulmod(q->t[k - 1], q->t[k - 1], q->t[k]);
    return q;
  }();
  return *p;
}

// x^m mod f.
__host__ __device__ inline void poly_pow(const uint32_t (*T)[kDeg], unsigned long long m, uint32_t* out) {
#pragma unroll
  for (int i = 0; i < kDeg; ++i) out[i] = 0;
  out[0] = 1;
  for (int k = 0; m; ++k, m >>= 1)
    if (m & 1) {
      uint32_t t[kDeg], r[kDeg];
#pragma unroll
      for (int i = 0; i < kDeg; ++i) t[i] = T[k][i];
      poly_mulmod(out, t, r);
#pragma unroll
      for (int i = 0; i < kDeg; ++i) out[i] = r[i];
    }
}

// Kernel layout: a CTA of kFillThreads threads covers kSuper consecutive
// values; thread t owns the kSub values at t * kSub.  Warp 0 computes the
// CTA's jump x^(CTA start) cooperatively (lane k owns coefficients k and
// k + 31 of each product); every thread then multiplies by its own offset's
// power, taken from a table of x^(t * kSub), forms its 31-value window and
// runs the recurrence.  Values go out through shared memory, one 31-value
// pass at a time, so that a warp's stores cover whole runs of consecutive
// words.
constexpr int kFillThreads = 128;
constexpr int kPasses = 8;
constexpr int kSub = kDeg * kPasses;           // 248 values per thread
constexpr int kSuper = kSub * kFillThreads;    // 31744 values per CTA

struct OffsetTable {
  uint32_t t[kFillThreads][kDeg];  // x^(t * kSub) mod f
};

// out = a * b mod f by one warp; a, b, out in shared memory (out may alias a).
__device__ void warp_mulmod(const uint32_t* a, const uint32_t* b, uint32_t* out, uint32_t* tmp, int lane) {
  // tmp[0..60] = the product's coefficients
  for (int k = lane; k < 2 * kDeg - 1; k += 32) {
    uint32_t s = 0;
    const int lo = k < kDeg ? 0 : k - (kDeg - 1), hi = k < kDeg ? k : kDeg - 1;
    for (int i = lo; i <= hi; ++i) s += a[i] * b[k - i];
    tmp[k] = s;
  }
  __syncwarp();
  if (lane == 0) {
    // the reduction mod f in registers
    uint32_t c[2 * kDeg - 1];
#pragma unroll
    for (int k = 0; k < 2 * kDeg - 1; ++k) c[k] = tmp[k];
#pragma unroll
    for (int k = 2 * kDeg - 2; k >= kDeg; --k) {
      c[k - 3] += c[k];
      c[k - kDeg] += c[k];
    }
#pragma unroll
    for (int k = 0; k < kDeg; ++k) out[k] = c[k];
  }
  __syncwarp();
}

__global__ void __launch_bounds__(kFillThreads) k_rand_fill(const RandWindow* __restrict__ win,
                                                             const PowerTable* __restrict__ pw,
                                                             const OffsetTable* __restrict__ offs,
                                                             uint32_t* __restrict__ out, long long n) {
  __shared__ uint32_t s_a[kDeg], s_b[kDeg], s_tmp[2 * kDeg];
  __shared__ uint32_t s_ext[61];
  __shared__ uint32_t s_pass[kFillThreads / 32][32][kDeg + 2];  // odd row stride: no bank conflicts
  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const long long cta0 = (long long)blockIdx.x * kSuper;
  if (t < 61) s_ext[t] = __ldg(win->ext + t);
  if (warp == 0) {
    // x^cta0 by square-and-multiply over the table of x^(2^k)
    if (lane < kDeg) s_a[lane] = lane == 0 ? 1u : 0u;
    __syncwarp();
    unsigned long long m = (unsigned long long)cta0;
    for (int k = 0; m; ++k, m >>= 1) {
      if (!(m & 1)) continue;
      if (lane < kDeg) s_b[lane] = __ldg(&pw->t[k][lane]);
      __syncwarp();
      warp_mulmod(s_a, s_b, s_a, s_tmp, lane);
    }
  }
  __syncthreads();
  const long long start = cta0 + (long long)t * kSub;
  // a = x^start = x^cta0 * x^(t * kSub)
  uint32_t a[kDeg];
  {
    uint32_t x0[kDeg], x1[kDeg];
#pragma unroll
    for (int i = 0; i < kDeg; ++i) {
      x0[i] = s_a[i];
      x1[i] = __ldg(&offs->t[t][i]);
    }
    poly_mulmod(x0, x1, a);
  }
  // w[j] = v[start - 31 + j] = sum_i a_i v[-31 + j + i]
  uint32_t w[kDeg];
  {
    uint32_t e[61];
#pragma unroll
    for (int k = 0; k < 61; ++k) e[k] = s_ext[k];
#pragma unroll
    for (int j = 0; j < kDeg; ++j) {
      uint32_t s = 0;
#pragma unroll
      for (int i = 0; i < kDeg; ++i) s += a[i] * e[j + i];
      w[j] = s;
    }
  }
  uint32_t(*pass)[kDeg + 2] = s_pass[warp];
  for (int p = 0; p < kPasses; ++p) {
#pragma unroll
    for (int j = 0; j < kDeg; ++j) {
      w[j] += w[(j + kDeg - kSep) % kDeg];
      pass[lane][j] = w[j] >> 1;
    }
    __syncwarp();
    // the warp writes each lane's 31 values as one run (lanes 0..30 cover a run)
    for (int r = 0; r < 32; ++r) {
      const long long base = cta0 + (long long)(warp * 32 + r) * kSub + (long long)p * kDeg;
      if (lane < kDeg && base + lane < n) out[base + lane] = pass[r][lane];
    }
    __syncwarp();
  }
}

std::mutex g_mu;
PowerTable* g_dev_powers = nullptr;  // one copy (single-device library)
OffsetTable* g_dev_offsets = nullptr;

}  // namespace

bool rand_take(long long n, RandWindow* w) {
  std::lock_guard<std::mutex> lock(g_mu);
  // a scratch TYPE_3 state (word 0: rear index 0, type 3) to switch to
  int32_t scratch[kDeg + 1];
  std::memset(scratch, 0, sizeof(scratch));
  scratch[0] = kType3;
  scratch[1] = 1;
  int32_t* os = reinterpret_cast<int32_t*>(setstate(reinterpret_cast<char*>(scratch)));
  if (!os) return false;
  const int type = os[0] % kTypes, rear = os[0] / kTypes;
  if (type != kType3 || rear < 0 || rear >= kDeg) {
    setstate(reinterpret_cast<char*>(os));
    return false;
  }
  uint32_t* ring = reinterpret_cast<uint32_t*>(os + 1);
  const int front = (rear + kSep) % kDeg;
  // v[-31 + j] sits at ring[(front + j) % 31]
  for (int j = 0; j < kDeg; ++j) w->ext[j] = ring[(front + j) % kDeg];
  for (int t = 0; t < 30; ++t) w->ext[kDeg + t] = w->ext[t] + w->ext[kDeg + t - kSep];
  // the ring after n more outputs: v[n - 31 + j] = sum_i a_i v[-31 + j + i], a = x^n mod f
  uint32_t a[kDeg];
  poly_pow(host_powers().t, (unsigned long long)n, a);
  const int front2 = int((front + n) % kDeg), rear2 = int((rear + n) % kDeg);
  for (int j = 0; j < kDeg; ++j) {
    uint32_t s = 0;
    for (int i = 0; i < kDeg; ++i) s += a[i] * w->ext[j + i];
    ring[(front2 + j) % kDeg] = s;
  }
  os[0] = kTypes * rear2 + kType3;
  setstate(reinterpret_cast<char*>(os));
  return true;
}

bool rand_usable() {
  static const bool forced_host = [] {
    const char* v = std::getenv("S2TC_HOST_RAND");
    return v && *v == '1';
  }();
  if (forced_host) return false;
  RandWindow w;
  return rand_take(0, &w);
}

cudaError_t rand_prepare() {
  std::lock_guard<std::mutex> lock(g_mu);
  if (g_dev_powers) return cudaSuccess;
  OffsetTable* offs = new OffsetTable();
  for (int t = 0; t < kFillThreads; ++t) poly_pow(host_powers().t, (unsigned long long)t * kSub, offs->t[t]);
  PowerTable* dp = nullptr;
  OffsetTable* doffs = nullptr;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&dp), sizeof(PowerTable));
  if (e == cudaSuccess) e = cudaMalloc(reinterpret_cast<void**>(&doffs), sizeof(OffsetTable));
  if (e == cudaSuccess) e = cudaMemcpy(dp, &host_powers(), sizeof(PowerTable), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(doffs, offs, sizeof(OffsetTable), cudaMemcpyHostToDevice);
  delete offs;
  if (e != cudaSuccess) {
    cudaFree(dp);
    cudaFree(doffs);
    return e;
  }
  g_dev_powers = dp;
  g_dev_offsets = doffs;
  return e;
}

cudaError_t rand_fill(const RandWindow* d_w, uint32_t* d_out, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const cudaError_t e = rand_prepare();
  if (e != cudaSuccess) return e;
  const long long ctas = (n + kSuper - 1) / kSuper;
  count_launches(1);
  k_rand_fill<<<unsigned(ctas), kFillThreads, 0, s>>>(d_w, g_dev_powers, g_dev_offsets, d_out, n);
  return cudaGetLastError();
}

}  // namespace s2tc
