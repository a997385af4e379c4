// Correlated-field log-sky: the field-sized part of the diffuse sky model
// that feeds the response (jubik/sky_models.py:205-225 builds the fields with
// NIFTy.re's CorrelatedFieldMaker, :306-341 combines and exponentiates them).
//
// One correlated field on a padded grid s0 x s1 is
//     field = offset + hartley(amp[pindex] * xi),
//     hartley(p) = Re(fftn(p)) + Im(fftn(p))            (unnormalised),
// with amp the amplitude spectrum over the distinct Fourier-mode lengths and
// pindex the mode-length index of each pixel (NIFTy.re's harmonic transform and
// power distributor).  The amplitude spectrum itself (a 1-D function of a few
// scalar parameters) stays with the caller.  J-UBIK's diffuse log-sky adds a
// spatial field and a spectral-index field times the log energy-bin centres
// (_apply_slope, sky_models.py:593-602) and keeps the unpadded corner:
//     logsky[e] = sum_b ecoef[e, b] * field_b[:nx, :ny].
//
// Layout: the fields are transformed two per complex array (z = x0 + i x1).
// For real x0, x1 with Z = F z, the Hartley transforms are
//     H x0 [k] = (Re Z[k] + Re Z[-k] + Im Z[k] - Im Z[-k]) / 2,
//     H x1 [k] = (Im Z[k] + Im Z[-k] + Re Z[-k] - Re Z[k]) / 2,
// read in one pass over Z.  The Hartley matrix is symmetric, so the
// vector-Jacobian product runs the same transform on the cotangent:
//     dxi_b = amp_b[pindex] * H g_b,   doffset_b = sum g_b = (H g_b)[0],
//     damp_b[m] = sum over pixels of mode m of xi_b * H g_b,
// the last as a deterministic segmented sum over a mode-sorted pixel list
// built once on the host: the list is cut into chunks of at most kChunk
// pixels of one mode, each chunk is summed in list order, then each mode's
// chunk sums in order (short critical paths however uneven the mode sizes).
// No atomics: results are bitwise reproducible.
#include <algorithm>
#include <new>
#include <vector>

#include "internal.h"
#include "jubik_common.cuh"

namespace jubik {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxFields = 4;
constexpr int kMaxEnergies = 32;
constexpr int kChunk = 16;

struct ECoef {
  int E, nx, ny;
  double c[kMaxEnergies * kMaxFields];  // c[e * nf + b]
};

unsigned blocks_for(int64_t n) {
  const int64_t b = (n + kThreads - 1) / kThreads;
  return (unsigned)std::min<int64_t>(std::max<int64_t>(b, 1), (int64_t)sm_count() * 16);
}

// The per-pixel kernels run a 2-D grid: blockIdx.y is the row y of the padded
// grid, x = blockIdx.x * kThreads + threadIdx.x its column.  NF (the number
// of fields) is a template parameter, so every per-field value stays in a
// register.
__device__ __forceinline__ bool pixel(int s1, int& y, int& x) {
  y = blockIdx.y;
  x = blockIdx.x * kThreads + threadIdx.x;
  return x < s1;
}

// z_p = amp_{2p}[pindex] xi_{2p} + i amp_{2p+1}[pindex] xi_{2p+1}
template <typename T, int NF>
__global__ void __launch_bounds__(kThreads)
    k_cf_pack(const T* __restrict__ amp, const T* __restrict__ xi, const int32_t* __restrict__ pd,
              int s0, int s1, int n_modes, cx<T>* __restrict__ work) {
  int y, x;
  if (!pixel(s1, y, x)) return;
  const int64_t npix = (int64_t)s0 * s1, i = (int64_t)y * s1 + x;
  const int m = pd[i];
#pragma unroll
  for (int p = 0; p < (NF + 1) / 2; ++p) {
    const T a = amp[(2 * p) * n_modes + m] * xi[(2 * p) * npix + i];
    const T b = 2 * p + 1 < NF ? amp[(2 * p + 1) * n_modes + m] * xi[(2 * p + 1) * npix + i]
                               : (T)0;
    work[p * npix + i] = mkc<T>(a, b);
  }
}

// cotangent packing: g_b from g_fields, or from g_logsky through the energy
// coefficients (zero outside the nx x ny corner)
template <typename T, int NF>
__global__ void __launch_bounds__(kThreads)
    k_cf_pack_cot(const T* __restrict__ g_fields, const T* __restrict__ g_logsky, ECoef ec,
                  int s0, int s1, cx<T>* __restrict__ work) {
  int y, x;
  if (!pixel(s1, y, x)) return;
  const int64_t npix = (int64_t)s0 * s1, i = (int64_t)y * s1 + x;
  T g[NF + 1];
#pragma unroll
  for (int b = 0; b <= NF; ++b) g[b] = (T)0;
  if (g_fields) {
#pragma unroll
    for (int b = 0; b < NF; ++b) g[b] = g_fields[b * npix + i];
  } else if (y < ec.nx && x < ec.ny) {
    const int64_t plane = (int64_t)ec.nx * ec.ny, o = (int64_t)y * ec.ny + x;
    for (int e = 0; e < ec.E; ++e) {
      const T v = g_logsky[e * plane + o];
#pragma unroll
      for (int b = 0; b < NF; ++b) g[b] += (T)ec.c[e * NF + b] * v;
    }
  }
#pragma unroll
  for (int p = 0; p < (NF + 1) / 2; ++p) work[p * npix + i] = mkc<T>(g[2 * p], g[2 * p + 1]);
}

// Hartley transforms of the pair packed in Z at a pixel (z) and its mirror (zm)
template <typename T>
__device__ __forceinline__ void hartley_pair(cx<T> z, cx<T> zm, T& h0, T& h1) {
  h0 = (T)0.5 * ((z.x + zm.x) + (z.y - zm.y));
  h1 = (T)0.5 * ((z.y + zm.y) + (zm.x - z.x));
}

template <typename T, int NF>
__device__ __forceinline__ void hartley_all(const cx<T>* __restrict__ work, int64_t npix,
                                            int64_t i, int64_t j, T (&h)[NF + 1]) {
#pragma unroll
  for (int p = 0; p < (NF + 1) / 2; ++p)
    hartley_pair<T>(work[p * npix + i], work[p * npix + j], h[2 * p], h[2 * p + 1]);
}

template <typename T, int NF>
__global__ void __launch_bounds__(kThreads)
    k_cf_unpack(const cx<T>* __restrict__ work, const T* __restrict__ offsets, int s0, int s1,
                T* __restrict__ fields, ECoef ec, T* __restrict__ logsky) {
  int y, x;
  if (!pixel(s1, y, x)) return;
  const int64_t npix = (int64_t)s0 * s1, i = (int64_t)y * s1 + x;
  const int64_t j = (int64_t)(y ? s0 - y : 0) * s1 + (x ? s1 - x : 0);
  T f[NF + 1];
  hartley_all<T, NF>(work, npix, i, j, f);
#pragma unroll
  for (int b = 0; b < NF; ++b) f[b] += offsets[b];
  if (fields) {
#pragma unroll
    for (int b = 0; b < NF; ++b) fields[b * npix + i] = f[b];
  }
  if (logsky && y < ec.nx && x < ec.ny) {
    const int64_t plane = (int64_t)ec.nx * ec.ny, o = (int64_t)y * ec.ny + x;
    for (int e = 0; e < ec.E; ++e) {
      T v = (T)ec.c[e * NF] * f[0];
#pragma unroll
      for (int b = 1; b < NF; ++b) v += (T)ec.c[e * NF + b] * f[b];
      logsky[e * plane + o] = v;
    }
  }
}

// h_b = H g_b: dxi_b = amp_b[pindex] h_b, prod_b = xi_b h_b, doffset_b = h_b[0]
template <typename T, int NF>
__global__ void __launch_bounds__(kThreads)
    k_cf_unpack_vjp(const cx<T>* __restrict__ work, const T* __restrict__ amp,
                    const T* __restrict__ xi, const int32_t* __restrict__ pd,
                    int s0, int s1, int n_modes,
                    T* __restrict__ dxi, T* __restrict__ prod, T* __restrict__ doffsets) {
  int y, x;
  if (!pixel(s1, y, x)) return;
  const int64_t npix = (int64_t)s0 * s1, i = (int64_t)y * s1 + x;
  const int64_t j = (int64_t)(y ? s0 - y : 0) * s1 + (x ? s1 - x : 0);
  const int m = pd[i];
  T h[NF + 1];
  hartley_all<T, NF>(work, npix, i, j, h);
#pragma unroll
  for (int b = 0; b < NF; ++b) {
    dxi[b * npix + i] = amp[b * n_modes + m] * h[b];
    prod[b * npix + i] = xi[b * npix + i] * h[b];
    if (i == 0) doffsets[b] = h[b];
  }
}

// part_b[c] = sum over chunk c (at most kChunk list entries) of prod_b[idx[q]]
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_cf_chunk_sum(const T* __restrict__ prod, const int32_t* __restrict__ idx,
                   const int32_t* __restrict__ chunk_beg, int nf, int nchunks, int64_t npix,
                   double* __restrict__ part) {
  const int64_t total = (int64_t)nf * nchunks;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(t / nchunks), c = (int)(t - (int64_t)b * nchunks);
    const T* pb = prod + (int64_t)b * npix;
    const int q0 = chunk_beg[c], n = chunk_beg[c + 1] - q0;
    int j[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u) j[u] = u < n ? idx[q0 + u] : -1;
    T v[kChunk];
#pragma unroll
    for (int u = 0; u < kChunk; ++u) v[u] = j[u] >= 0 ? pb[j[u]] : (T)0;
    double s = 0.0;
#pragma unroll
    for (int u = 0; u < kChunk; ++u) s += (double)v[u];
    part[t] = s;
  }
}

// damp_b[m] = sum of mode m's chunk sums in order
template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_cf_mode_sum(const double* __restrict__ part, const int32_t* __restrict__ mode_chunk, int nf,
                  int n_modes, int nchunks, T* __restrict__ damp) {
  const int64_t total = (int64_t)nf * n_modes;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int b = (int)(t / n_modes), m = (int)(t - (int64_t)b * n_modes);
    const double* pb = part + (int64_t)b * nchunks;
    double s = 0.0;
    for (int c = mode_chunk[m]; c < mode_chunk[m + 1]; ++c) s += pb[c];
    damp[t] = (T)s;
  }
}

}  // namespace
}  // namespace jubik

using namespace jubik;

struct jubik_cf {
  int nf = 0, s0 = 0, s1 = 0, n_modes = 0, dtype = 0;
  Fft1D f0, f1;
  int32_t* pindex = nullptr;
  int nchunks = 0;
  int32_t* idx = nullptr;         // pixels in mode-sorted order (npix)
  int32_t* chunk_beg = nullptr;   // list position where chunk c starts (nchunks + 1)
  int32_t* mode_chunk = nullptr;  // first chunk of mode m (n_modes + 1)
  double* part = nullptr;         // chunk sums (nf, nchunks)
  void* work = nullptr;  // ((nf + 1) / 2, s0, s1) complex
  void* prod = nullptr;  // (nf, s0, s1) real
  ~jubik_cf() {
    fft1d_free(&f0);
    fft1d_free(&f1);
    cudaFree(pindex);
    cudaFree(idx);
    cudaFree(chunk_beg);
    cudaFree(mode_chunk);
    cudaFree(part);
    cudaFree(work);
    cudaFree(prod);
  }
};

namespace {

int fill_coef(const jubik_cf* cf, const double* ecoef, int32_t E, int32_t nx, int32_t ny,
              ECoef* ec) {
  ec->E = 0;
  ec->nx = 0;
  ec->ny = 0;
  if (!ecoef) return JUBIK_OK;
  if (E < 1 || E > kMaxEnergies || nx < 1 || ny < 1 || nx > cf->s0 || ny > cf->s1) {
    set_error("cf: need 1 <= E <= %d and a crop 1 <= nx <= %d, 1 <= ny <= %d (got E=%d, %d x %d)",
              kMaxEnergies, cf->s0, cf->s1, E, nx, ny);
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  ec->E = E;
  ec->nx = nx;
  ec->ny = ny;
  for (int i = 0; i < E * cf->nf; ++i) ec->c[i] = ecoef[i];
  return JUBIK_OK;
}

template <typename T, int NF>
int cf_apply_nf(jubik_cf* cf, const void* amp, const void* xi, const void* offsets, void* fields,
                const ECoef& ec, void* logsky, cudaStream_t s) {
  const dim3 grid((unsigned)((cf->s1 + kThreads - 1) / kThreads), (unsigned)cf->s0);
  k_cf_pack<T, NF><<<grid, kThreads, 0, s>>>((const T*)amp, (const T*)xi, cf->pindex, cf->s0,
                                             cf->s1, cf->n_modes, (cx<T>*)cf->work);
  JUBIK_TRY_CUDA(cudaGetLastError());
  JUBIK_TRY(fft2_batched<T>(cf->f0, cf->f1, cf->work, (NF + 1) / 2, false, s));
  k_cf_unpack<T, NF><<<grid, kThreads, 0, s>>>((const cx<T>*)cf->work, (const T*)offsets,
                                               cf->s0, cf->s1, (T*)fields, ec, (T*)logsky);
  return cuda_status(cudaGetLastError(), "k_cf_unpack");
}

template <typename T, int NF>
int cf_vjp_nf(jubik_cf* cf, const void* amp, const void* xi, const void* g_fields,
              const ECoef& ec, const void* g_logsky, void* dxi, void* damp, void* doffsets,
              cudaStream_t s) {
  const int64_t npix = (int64_t)cf->s0 * cf->s1;
  const dim3 grid((unsigned)((cf->s1 + kThreads - 1) / kThreads), (unsigned)cf->s0);
  k_cf_pack_cot<T, NF><<<grid, kThreads, 0, s>>>((const T*)g_fields, (const T*)g_logsky, ec,
                                                 cf->s0, cf->s1, (cx<T>*)cf->work);
  JUBIK_TRY_CUDA(cudaGetLastError());
  JUBIK_TRY(fft2_batched<T>(cf->f0, cf->f1, cf->work, (NF + 1) / 2, false, s));
  k_cf_unpack_vjp<T, NF><<<grid, kThreads, 0, s>>>(
      (const cx<T>*)cf->work, (const T*)amp, (const T*)xi, cf->pindex, cf->s0, cf->s1,
      cf->n_modes, (T*)dxi, (T*)cf->prod, (T*)doffsets);
  JUBIK_TRY_CUDA(cudaGetLastError());
  k_cf_chunk_sum<T><<<blocks_for((int64_t)NF * cf->nchunks), kThreads, 0, s>>>(
      (const T*)cf->prod, cf->idx, cf->chunk_beg, NF, cf->nchunks, npix, cf->part);
  JUBIK_TRY_CUDA(cudaGetLastError());
  k_cf_mode_sum<T><<<blocks_for((int64_t)NF * cf->n_modes), kThreads, 0, s>>>(
      cf->part, cf->mode_chunk, NF, cf->n_modes, cf->nchunks, (T*)damp);
  return cuda_status(cudaGetLastError(), "k_cf_mode_sum");
}

template <typename T>
int cf_apply(jubik_cf* cf, const void* amp, const void* xi, const void* offsets, void* fields,
             const ECoef& ec, void* logsky, cudaStream_t s) {
  switch (cf->nf) {
    case 1: return cf_apply_nf<T, 1>(cf, amp, xi, offsets, fields, ec, logsky, s);
    case 2: return cf_apply_nf<T, 2>(cf, amp, xi, offsets, fields, ec, logsky, s);
    case 3: return cf_apply_nf<T, 3>(cf, amp, xi, offsets, fields, ec, logsky, s);
    default: return cf_apply_nf<T, 4>(cf, amp, xi, offsets, fields, ec, logsky, s);
  }
}

template <typename T>
int cf_vjp(jubik_cf* cf, const void* amp, const void* xi, const void* g_fields, const ECoef& ec,
           const void* g_logsky, void* dxi, void* damp, void* doffsets, cudaStream_t s) {
  switch (cf->nf) {
    case 1: return cf_vjp_nf<T, 1>(cf, amp, xi, g_fields, ec, g_logsky, dxi, damp, doffsets, s);
    case 2: return cf_vjp_nf<T, 2>(cf, amp, xi, g_fields, ec, g_logsky, dxi, damp, doffsets, s);
    case 3: return cf_vjp_nf<T, 3>(cf, amp, xi, g_fields, ec, g_logsky, dxi, damp, doffsets, s);
    default:
      return cf_vjp_nf<T, 4>(cf, amp, xi, g_fields, ec, g_logsky, dxi, damp, doffsets, s);
  }
}

}  // namespace

extern "C" {

int jubik_cf_create(int32_t n_fields, int32_t s0, int32_t s1, const int32_t* pindex,
                    int32_t n_modes, int32_t dtype, jubik_cf** out) {
  if (!out || !pindex || n_fields < 1 || n_fields > kMaxFields || s0 < 1 || s1 < 1 ||
      n_modes < 1 || (dtype != JUBIK_F32 && dtype != JUBIK_F64)) {
    set_error("cf_create: invalid arguments (1 <= n_fields <= %d, positive shape and modes)",
              kMaxFields);
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  if (!fft_length_supported(s0) || !fft_length_supported(s1)) {
    set_error("cf_create: FFT size %d x %d unsupported", s0, s1);
    return JUBIK_ERR_UNSUPPORTED;
  }
  const int64_t npix = (int64_t)s0 * s1;
  if (npix > 0x7fffffffLL || s0 > 65535) {
    set_error("cf_create: %d x %d grid too large (at most 65535 rows and 2^31 - 1 pixels)", s0,
              s1);
    return JUBIK_ERR_UNSUPPORTED;
  }
  // mode-sorted pixel list (a counting sort keeps ascending pixels per mode),
  // cut into chunks of at most kChunk entries of one mode
  std::vector<int32_t> off((size_t)n_modes + 1, 0), idx((size_t)npix);
  for (int64_t i = 0; i < npix; ++i) {
    const int32_t m = pindex[i];
    if (m < 0 || m >= n_modes) {
      set_error("cf_create: pindex[%lld] = %d outside [0, %d)", (long long)i, m, n_modes);
      return JUBIK_ERR_INVALID_ARGUMENT;
    }
    ++off[(size_t)m + 1];
  }
  for (int m = 0; m < n_modes; ++m) off[(size_t)m + 1] += off[(size_t)m];
  {
    std::vector<int32_t> pos(off.begin(), off.end() - 1);
    for (int64_t i = 0; i < npix; ++i) idx[(size_t)pos[(size_t)pindex[i]]++] = (int32_t)i;
  }
  std::vector<int32_t> chunk_beg, mode_chunk((size_t)n_modes + 1);
  for (int m = 0; m < n_modes; ++m) {
    mode_chunk[(size_t)m] = (int32_t)chunk_beg.size();
    for (int32_t q = off[(size_t)m]; q < off[(size_t)m + 1]; q += kChunk) chunk_beg.push_back(q);
  }
  mode_chunk[(size_t)n_modes] = (int32_t)chunk_beg.size();
  const int nchunks = (int)chunk_beg.size();
  chunk_beg.push_back((int32_t)npix);
  auto* cf = new (std::nothrow) jubik_cf();
  if (!cf) {
    set_error("cf_create: out of host memory");
    return JUBIK_ERR_ALLOC;
  }
  cf->nf = n_fields;
  cf->s0 = s0;
  cf->s1 = s1;
  cf->n_modes = n_modes;
  cf->nchunks = nchunks;
  cf->dtype = dtype;
  const size_t rsz = dtype == JUBIK_F32 ? sizeof(float) : sizeof(double);
  const int np = (n_fields + 1) / 2;
  auto fail = [&](int st) {
    delete cf;
    return st;
  };
  int st = fft1d_init(&cf->f0, s0);
  if (st == JUBIK_OK) st = fft1d_init(&cf->f1, s1);
  if (st != JUBIK_OK) return fail(st);
  if (cudaMalloc(&cf->pindex, sizeof(int32_t) * npix) != cudaSuccess ||
      cudaMalloc(&cf->idx, sizeof(int32_t) * npix) != cudaSuccess ||
      cudaMalloc(&cf->chunk_beg, sizeof(int32_t) * chunk_beg.size()) != cudaSuccess ||
      cudaMalloc(&cf->mode_chunk, sizeof(int32_t) * mode_chunk.size()) != cudaSuccess ||
      cudaMalloc(&cf->part, sizeof(double) * n_fields * nchunks) != cudaSuccess ||
      cudaMalloc(&cf->work, 2 * rsz * np * npix) != cudaSuccess ||
      cudaMalloc(&cf->prod, rsz * n_fields * npix) != cudaSuccess) {
    cudaGetLastError();
    set_error("cf_create: device allocation failed");
    return fail(JUBIK_ERR_ALLOC);
  }
  if (cudaMemcpy(cf->pindex, pindex, sizeof(int32_t) * npix, cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(cf->idx, idx.data(), sizeof(int32_t) * npix, cudaMemcpyHostToDevice) !=
          cudaSuccess ||
      cudaMemcpy(cf->chunk_beg, chunk_beg.data(), sizeof(int32_t) * chunk_beg.size(),
                 cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(cf->mode_chunk, mode_chunk.data(), sizeof(int32_t) * mode_chunk.size(),
                 cudaMemcpyHostToDevice) != cudaSuccess) {
    return fail(cuda_status(cudaGetLastError(), "cf_create upload"));
  }
  *out = cf;
  return JUBIK_OK;
}

int jubik_cf_apply(jubik_cf* cf, const void* amp, const void* xi, const void* offsets,
                   void* fields, const double* ecoef, int32_t E, int32_t nx, int32_t ny,
                   void* logsky, void* stream) {
  if (!cf || !amp || !xi || !offsets || (!fields && !logsky) || (logsky && !ecoef)) {
    set_error("cf_apply: need amp, xi, offsets and an output (logsky needs ecoef)");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  ECoef ec;
  JUBIK_TRY(fill_coef(cf, logsky ? ecoef : nullptr, E, nx, ny, &ec));
  cudaStream_t s = (cudaStream_t)stream;
  return cf->dtype == JUBIK_F32 ? cf_apply<float>(cf, amp, xi, offsets, fields, ec, logsky, s)
                                : cf_apply<double>(cf, amp, xi, offsets, fields, ec, logsky, s);
}

int jubik_cf_vjp(jubik_cf* cf, const void* amp, const void* xi, const void* g_fields,
                 const double* ecoef, int32_t E, int32_t nx, int32_t ny, const void* g_logsky,
                 void* dxi, void* damp, void* doffsets, void* stream) {
  if (!cf || !amp || !xi || !dxi || !damp || !doffsets || (!g_fields == !g_logsky) ||
      (g_logsky && !ecoef)) {
    set_error("cf_vjp: need amp, xi, outputs and exactly one cotangent (g_logsky needs ecoef)");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  ECoef ec;
  JUBIK_TRY(fill_coef(cf, g_logsky ? ecoef : nullptr, E, nx, ny, &ec));
  cudaStream_t s = (cudaStream_t)stream;
  return cf->dtype == JUBIK_F32
             ? cf_vjp<float>(cf, amp, xi, g_fields, ec, g_logsky, dxi, damp, doffsets, s)
             : cf_vjp<double>(cf, amp, xi, g_fields, ec, g_logsky, dxi, damp, doffsets, s);
}

int jubik_cf_destroy(jubik_cf* cf) {
  delete cf;
  return JUBIK_OK;
}

}  // extern "C"
