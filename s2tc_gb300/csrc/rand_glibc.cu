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
// chunk this way and then runs the recurrence for kChunk values; the host
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
constexpr int kChunk = kDeg * 128;     // values per thread (a multiple of 31)

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

// One thread per chunk of kChunk values: jump, then run the recurrence.
__global__ void __launch_bounds__(128) k_rand_fill(const RandWindow* __restrict__ win,
                                                    const PowerTable* __restrict__ pw, uint32_t* __restrict__ out,
                                                    long long n) {
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long start = c * kChunk;
  if (start >= n) return;
  uint32_t a[kDeg];
  poly_pow(pw->t, (unsigned long long)start, a);
  // w[j] = v[start - 31 + j] = sum_i a_i v[-31 + j + i]
  uint32_t w[kDeg];
#pragma unroll
  for (int j = 0; j < kDeg; ++j) {
    uint32_t s = 0;
#pragma unroll 1
    for (int i = 0; i < kDeg; ++i) s += a[i] * __ldg(win->ext + j + i);
    w[j] = s;
  }
  const long long end = start + kChunk < n ? start + kChunk : n;
  uint32_t* o = out + start;
  long long t = start;
  while (t + kDeg <= end) {
#pragma unroll
    for (int j = 0; j < kDeg; ++j) {
      w[j] += w[(j + kDeg - kSep) % kDeg];
      o[j] = w[j] >> 1;
    }
    o += kDeg;
    t += kDeg;
  }
#pragma unroll
  for (int j = 0; j < kDeg; ++j) {
    if (t + j >= end) break;
    w[j] += w[(j + kDeg - kSep) % kDeg];
    o[j] = w[j] >> 1;
  }
}

std::mutex g_mu;
PowerTable* g_dev_powers = nullptr;  // one copy (single-device library)

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
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&g_dev_powers), sizeof(PowerTable));
  if (e == cudaSuccess) e = cudaMemcpy(g_dev_powers, &host_powers(), sizeof(PowerTable), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(g_dev_powers);
    g_dev_powers = nullptr;
  }
  return e;
}

cudaError_t rand_fill(const RandWindow* d_w, uint32_t* d_out, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const cudaError_t e = rand_prepare();
  if (e != cudaSuccess) return e;
  const long long chunks = (n + kChunk - 1) / kChunk;
  count_launches(1);
  k_rand_fill<<<unsigned((chunks + 127) / 128), 128, 0, s>>>(d_w, g_dev_powers, d_out, n);
  return cudaGetLastError();
}

}  // namespace s2tc
