// Sampling and global reductions for the callers of the response: the mock
// data of jubik/data.py:138-159 (Poisson draws of the expected counts), the
// Gaussian draws of an MGVI linear sample, and the FP64 dot products that set
// the step sizes of its conjugate-gradient solve.
//
// Random numbers come from the counter-based Philox4x32-10 generator
// (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
// SC'11): a bijection of a 128-bit counter under a 64-bit key, so every
// output element has its own counter and the result does not depend on the
// launch shape.  Normal deviates use the Box-Muller transform; Poisson
// deviates use inversion for lam < 10 and Hormann's transformed rejection with
// squeeze (PTRS; W. Hormann, "The transformed rejection method for generating
// Poisson random variables", Insurance: Mathematics and Economics 12, 1993)
// above.
#include <cmath>
#include <cstdio>

#include "internal.h"
#include "jubik_common.cuh"

namespace jubik {
namespace {

constexpr int kThreads = 256;
constexpr int kDotBlocks = 1024;  // fixed grid: the reduction order never changes

// ------------------------------------------------------------------ Philox
constexpr uint32_t kPhM0 = 0xD2511F53u, kPhM1 = 0xCD9E8D57u;
constexpr uint32_t kPhW0 = 0x9E3779B9u, kPhW1 = 0xBB67AE85u;

__host__ __device__ inline uint32_t mulhi32(uint32_t a, uint32_t b) {
  return (uint32_t)(((uint64_t)a * (uint64_t)b) >> 32);
}

__host__ __device__ inline uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint32_t hi0 = mulhi32(kPhM0, c.x), lo0 = kPhM0 * c.x;
    const uint32_t hi1 = mulhi32(kPhM1, c.z), lo1 = kPhM1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += kPhW0;
    k.y += kPhW1;
  }
  return c;
}

// uniform in (0, 1): 23 bits plus a half (exact in float) or 53 bits from two
// words (double)
__device__ __forceinline__ float u01f(uint32_t x) {
  return ((float)(x >> 9) + 0.5f) * (1.0f / 8388608.0f);
}
__device__ __forceinline__ double u01d(uint32_t hi, uint32_t lo) {
  const uint64_t m = ((uint64_t)(hi >> 5) << 26) | (uint64_t)(lo >> 6);  // 27 + 26 bits
  return ((double)m + 0.5) * (1.0 / 9007199254740992.0);
}

// ------------------------------------------------------------------ normal
// FP32: one counter per 4 elements (two Box-Muller pairs); FP64: one counter
// per 2 elements (one pair from two 53-bit uniforms).
__global__ void k_normal_f32(float* out, int64_t n, uint2 key, uint32_t off_lo, uint32_t off_hi) {
  const int64_t groups = (n + 3) / 4;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const uint4 r = philox4x32_10(make_uint4((uint32_t)g, (uint32_t)(g >> 32), off_lo, off_hi),
                                  key);
    float z[4];
    {
      const float rad = sqrtf(-2.0f * logf(u01f(r.x)));
      float s, c;
      sincospif(2.0f * u01f(r.y), &s, &c);
      z[0] = rad * c;
      z[1] = rad * s;
    }
    {
      const float rad = sqrtf(-2.0f * logf(u01f(r.z)));
      float s, c;
      sincospif(2.0f * u01f(r.w), &s, &c);
      z[2] = rad * c;
      z[3] = rad * s;
    }
    const int64_t i0 = 4 * g;
#pragma unroll
    for (int t = 0; t < 4; ++t)
      if (i0 + t < n) out[i0 + t] = z[t];
  }
}

__global__ void k_normal_f64(double* out, int64_t n, uint2 key, uint32_t off_lo, uint32_t off_hi) {
  const int64_t groups = (n + 1) / 2;
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < groups;
       g += (int64_t)gridDim.x * blockDim.x) {
    const uint4 r = philox4x32_10(make_uint4((uint32_t)g, (uint32_t)(g >> 32), off_lo, off_hi),
                                  key);
    const double rad = sqrt(-2.0 * log(u01d(r.x, r.y)));
    double s, c;
    sincospi(2.0 * u01d(r.z, r.w), &s, &c);
    const int64_t i0 = 2 * g;
    out[i0] = rad * c;
    if (i0 + 1 < n) out[i0 + 1] = rad * s;
  }
}

// ------------------------------------------------------------------ Poisson
// Element i draws from counters (i, offset, attempt): every attempt of the
// rejection loop has its own pair of 53-bit uniforms.
constexpr int kMaxAttempts = 256;  // PTRS accepts > 85 % of attempts for lam >= 10

__device__ int32_t poisson_one(double lam, uint64_t i, uint32_t off, uint2 key) {
  if (!(lam >= 0.0)) return -1;  // negative or NaN
  if (lam == 0.0) return 0;
  if (lam >= 2.0e9) return -1;   // counts beyond int32
  if (lam < 10.0) {
    // inversion: smallest k with F(k) >= u
    const uint4 r = philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), off, 0u), key);
    const double u = u01d(r.x, r.y);
    double p = exp(-lam), F = p;
    int32_t k = 0;
    while (u > F && k < 1000) {
      ++k;
      p *= lam / (double)k;
      F += p;
      if (p == 0.0) break;
    }
    return k;
  }
  const double slam = sqrt(lam), loglam = log(lam);
  const double b = 0.931 + 2.53 * slam;
  const double a = -0.059 + 0.02483 * b;
  const double inv_alpha = 1.1239 + 1.1328 / (b - 3.4);
  const double vr = 0.9277 - 3.6224 / (b - 2.0);
  for (uint32_t att = 0; att < (uint32_t)kMaxAttempts; ++att) {
    const uint4 r =
        philox4x32_10(make_uint4((uint32_t)i, (uint32_t)(i >> 32), off, att + 1u), key);
    const double U = u01d(r.x, r.y) - 0.5;
    const double V = u01d(r.z, r.w);
    const double us = 0.5 - fabs(U);
    const double kd = floor((2.0 * a / us + b) * U + lam + 0.43);
    if (us >= 0.07 && V <= vr) return (int32_t)kd;
    if (kd < 0.0 || (us < 0.013 && V > us)) continue;
    if (log(V) + log(inv_alpha) - log(a / (us * us) + b) <= -lam + kd * loglam - lgamma(kd + 1.0))
      return (int32_t)kd;
  }
  return (int32_t)floor(lam + 0.5);  // not reached in practice (probability < 1e-200)
}

template <typename T>
__global__ void k_poisson_sample(const T* __restrict__ lam, int64_t n, uint2 key, uint32_t off,
                                 int32_t* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = poisson_one((double)lam[i], (uint64_t)i, off, key);
}

// ------------------------------------------------------------------ dot
// Sum of a[i] b[i] into FP64 in a fixed order.  FP64 operands: one FP64 fma
// each.  FP32 operands: the FP64 pipe of this GPU is far too narrow to convert
// and fma every element at HBM speed, so each thread sums its products on the
// FP32 pipe with the compensated dot product "Dot2" of Ogita, Rump & Oishi
// (SIAM J. Sci. Comput. 26, 2005): the product split exactly into p + e
// (p = fl(x y), e = fma(x, y, -p)), p added with Knuth's TwoSum, the two error
// terms gathered in a second word.  Every kDotFlush elements the two words go
// into the thread's FP64 total.  A group whose words are not finite (an inf or
// NaN operand or an overflow), or whose products are all tiny while some pair
// of operands is nonzero (an underflowed product, or an error term below about
// 2^-102 that is not exact), is summed again in FP64.
constexpr int kDotFlush = 32;  // float4 chunks (128 elements) per FP64 flush

struct Dot2 {
  float s = 0.0f, c = 0.0f;  // sum and the gathered error terms
  float pmax = 0.0f;         // largest |fl(x y)|
  float zmax = 0.0f;         // largest min(|x|, |y|): positive when some pair is nonzero
  __device__ __forceinline__ void add(float x, float y);
  // the two words hold the group's sum to about 2^-48 of its terms
  __device__ __forceinline__ bool exact() const {
    return isfinite(s) && isfinite(c) && (pmax >= 0x1p-60f || zmax == 0.0f);
  }
};

__device__ __forceinline__ void Dot2::add(float x, float y) {
  const float p = __fmul_rn(x, y);  // no contraction into the sum below
  const float e = fmaf(x, y, -p);
  const float t = __fadd_rn(s, p);
  const float bp = __fsub_rn(t, s);
  const float sg = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  s = t;
  c = __fadd_rn(c, __fadd_rn(e, sg));
  pmax = fmaxf(pmax, fabsf(p));
  zmax = fmaxf(zmax, fminf(fabsf(x), fabsf(y)));
}

__device__ __forceinline__ double dot_f32_share(const float* __restrict__ a,
                                                const float* __restrict__ b, int64_t n) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const bool vec = ((reinterpret_cast<uintptr_t>(a) | reinterpret_cast<uintptr_t>(b)) & 15) == 0;
  double acc = 0.0;
  int64_t nv = 0;  // elements covered by float4 chunks
  if (vec) {
    const float4* a4 = reinterpret_cast<const float4*>(a);
    const float4* b4 = reinterpret_cast<const float4*>(b);
    const int64_t n4 = n >> 2;
    nv = n4 << 2;
    for (int64_t j0 = tid; j0 < n4; j0 += stride * kDotFlush) {
      Dot2 d;
      int64_t j = j0;
      for (int g = 0; g < kDotFlush && j < n4; ++g, j += stride) {
        const float4 x = __ldcs(a4 + j), y = __ldcs(b4 + j);
        d.add(x.x, y.x);
        d.add(x.y, y.y);
        d.add(x.z, y.z);
        d.add(x.w, y.w);
      }
      if (d.exact()) {
        acc += (double)d.s;
        acc += (double)d.c;
      } else {  // the same chunks again in FP64
        j = j0;
        for (int g = 0; g < kDotFlush && j < n4; ++g, j += stride)
          for (int q = 0; q < 4; ++q) acc = fma((double)a[4 * j + q], (double)b[4 * j + q], acc);
      }
    }
  }
  // the rest (everything when the operands are not 16-byte aligned), element-wise
  for (int64_t i0 = nv + tid; i0 < n; i0 += stride * (4 * kDotFlush)) {
    Dot2 d;
    int64_t i = i0;
    for (int g = 0; g < 4 * kDotFlush && i < n; ++g, i += stride) d.add(a[i], b[i]);
    if (d.exact()) {
      acc += (double)d.s;
      acc += (double)d.c;
    } else {
      i = i0;
      for (int g = 0; g < 4 * kDotFlush && i < n; ++g, i += stride)
        acc = fma((double)a[i], (double)b[i], acc);
    }
  }
  return acc;
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_dot(const T* __restrict__ a, const T* __restrict__ b, int64_t n, double* partials,
          unsigned int* counter, double* out) {
  double acc = 0.0;
  if constexpr (sizeof(T) == 4) {
    acc = dot_f32_share(a, b, n);
  } else {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
      acc = fma(a[i], b[i], acc);
  }
  __shared__ double red[kThreads];
  __shared__ bool last;
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = red[0];
    __threadfence();
    last = atomicAdd(counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double p = 0.0;
  for (unsigned int i = threadIdx.x; i < gridDim.x; i += blockDim.x) p += __ldcg(partials + i);
  red[threadIdx.x] = p;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    out[0] = red[0];
    *counter = 0u;
  }
}

unsigned grid_of(int64_t work) {
  int64_t b = (work + kThreads - 1) / kThreads;
  if (b > 65536) b = 65536;
  if (b < 1) b = 1;
  return (unsigned)b;
}

uint2 key_of(uint64_t seed) { return make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)); }

}  // namespace

// host-side Philox for the known-answer check of the C ABI
void philox_host(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
  const uint4 r = philox4x32_10(make_uint4(ctr[0], ctr[1], ctr[2], ctr[3]),
                                make_uint2(key[0], key[1]));
  out[0] = r.x;
  out[1] = r.y;
  out[2] = r.z;
  out[3] = r.w;
}

}  // namespace jubik

using namespace jubik;

extern "C" {

int jubik_philox4x32_10(const uint32_t* counter, const uint32_t* key, uint32_t* out) {
  if (!counter || !key || !out) {
    set_error("philox: null argument");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  philox_host(counter, key, out);
  return JUBIK_OK;
}

int jubik_random_normal(void* out, int64_t n, int32_t dtype, uint64_t seed, uint64_t offset,
                        void* stream) {
  if (!out || n < 0 || (dtype != JUBIK_F32 && dtype != JUBIK_F64)) {
    set_error("random_normal: invalid argument");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (n == 0) return JUBIK_OK;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t lo = (uint32_t)offset, hi = (uint32_t)(offset >> 32);
  if (dtype == JUBIK_F32)
    k_normal_f32<<<grid_of((n + 3) / 4), kThreads, 0, s>>>((float*)out, n, key_of(seed), lo, hi);
  else
    k_normal_f64<<<grid_of((n + 1) / 2), kThreads, 0, s>>>((double*)out, n, key_of(seed), lo, hi);
  return cuda_status(cudaGetLastError(), "k_normal");
}

int jubik_random_poisson(const void* lam, int64_t n, int32_t dtype, uint64_t seed,
                         uint32_t offset, int32_t* out, void* stream) {
  if (!lam || !out || n < 0 || (dtype != JUBIK_F32 && dtype != JUBIK_F64)) {
    set_error("random_poisson: invalid argument");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (n == 0) return JUBIK_OK;
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == JUBIK_F32)
    k_poisson_sample<float><<<grid_of(n), kThreads, 0, s>>>((const float*)lam, n, key_of(seed),
                                                             offset, out);
  else
    k_poisson_sample<double><<<grid_of(n), kThreads, 0, s>>>((const double*)lam, n,
                                                              key_of(seed), offset, out);
  return cuda_status(cudaGetLastError(), "k_poisson_sample");
}

int jubik_dot(const void* a, const void* b, int64_t n, int32_t dtype, double* out, void* stream) {
  if (!out || n < 0 || (n > 0 && (!a || !b)) || (dtype != JUBIK_F32 && dtype != JUBIK_F64)) {
    set_error("dot: invalid argument");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (n == 0) return cuda_status(cudaMemsetAsync(out, 0, sizeof(double), s), "dot (empty)");
  double* partials = nullptr;
  unsigned int* counter = nullptr;
  JUBIK_TRY_CUDA(cudaMallocAsync((void**)&partials, kDotBlocks * sizeof(double), s));
  JUBIK_TRY_CUDA(cudaMallocAsync((void**)&counter, sizeof(unsigned int), s));
  JUBIK_TRY_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), s));
  if (dtype == JUBIK_F32)
    k_dot<float><<<kDotBlocks, kThreads, 0, s>>>((const float*)a, (const float*)b, n, partials,
                                                  counter, out);
  else
    k_dot<double><<<kDotBlocks, kThreads, 0, s>>>((const double*)a, (const double*)b, n,
                                                   partials, counter, out);
  const int st = cuda_status(cudaGetLastError(), "k_dot");
  cudaFreeAsync(partials, s);
  cudaFreeAsync(counter, s);
  return st;
}

}  // extern "C"
