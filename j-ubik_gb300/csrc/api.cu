// C ABI of libjubik_gb300: plans, workspace, dispatch of the fused and the
// unfused (plain) paths, readout index map, likelihood entry points.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "internal.h"
#include "jubik_common.cuh"

namespace jubik {

namespace {
thread_local char g_err[1024] = "";
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_status(cudaError_t err, const char* what) {
  if (err == cudaSuccess) return JUBIK_OK;
  set_error("%s: %s", what, cudaGetErrorString(err));
  return err == cudaErrorMemoryAllocation ? JUBIK_ERR_ALLOC : JUBIK_ERR_CUDA;
}

namespace {

constexpr int kScanBlock = 1024;  // elements per scan block

// per-block counts of the read-out mask
__global__ void k_mask_counts(const uint8_t* __restrict__ mask, int64_t n, int32_t* counts) {
  __shared__ int32_t red[256];
  const int64_t base = (int64_t)blockIdx.x * kScanBlock;
  int32_t c = 0;
  for (int i = threadIdx.x; i < kScanBlock; i += blockDim.x) {
    const int64_t p = base + i;
    if (p < n && mask[p]) ++c;
  }
  red[threadIdx.x] = c;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) counts[blockIdx.x] = red[0];
}

// exclusive scan of the block counts (single thread; one-off set-up work)
__global__ void k_scan_counts(const int32_t* counts, int64_t nb, int64_t* offsets) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  int64_t acc = 0;
  for (int64_t i = 0; i < nb; ++i) {
    offsets[i] = acc;
    acc += counts[i];
  }
  offsets[nb] = acc;
}

// C-order compaction: ridx[p] = readout position or -1; list[pos] = p
__global__ void k_mask_compact(const uint8_t* __restrict__ mask, int64_t n,
                               const int64_t* __restrict__ offsets, int32_t* __restrict__ ridx,
                               int64_t* __restrict__ list) {
  __shared__ int32_t flags[kScanBlock];
  const int64_t base = (int64_t)blockIdx.x * kScanBlock;
  for (int i = threadIdx.x; i < kScanBlock; i += blockDim.x) {
    const int64_t p = base + i;
    flags[i] = (p < n && mask[p]) ? 1 : 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {  // serial prefix inside the block (1024 entries)
    int32_t acc = 0;
    for (int i = 0; i < kScanBlock; ++i) {
      const int32_t f = flags[i];
      flags[i] = f ? acc : -1;
      acc += f;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < kScanBlock; i += blockDim.x) {
    const int64_t p = base + i;
    if (p >= n) continue;
    const int32_t loc = flags[i];
    if (loc < 0) {
      ridx[p] = -1;
    } else {
      const int64_t pos = offsets[blockIdx.x] + loc;
      ridx[p] = (int32_t)pos;
      list[pos] = p;
    }
  }
}

__global__ void k_iota(int32_t* ridx, int64_t* list, int64_t n) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
       p += (int64_t)gridDim.x * blockDim.x) {
    ridx[p] = (int32_t)p;
    list[p] = p;
  }
}

template <typename T>
__global__ void k_to_cplx(const T* __restrict__ a, int64_t n, cx<T>* __restrict__ z) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    z[i] = mkc<T>(a[i], (T)0);
}

template <typename T>
__global__ void k_mul_bcast(const cx<T>* __restrict__ zk, int64_t bk, cx<T>* __restrict__ zs,
                            int64_t bs, int64_t hw) {
  const int64_t total = bs * hw;
  const int64_t rep = bs / bk;  // signal planes per kernel plane
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t plane = i / hw, r = i - plane * hw;
    zs[i] = cmul<T>(zk[(plane / rep) * hw + r], zs[i]);
  }
}

template <typename T>
__global__ void k_real_out(const cx<T>* __restrict__ z, int64_t n, T scale, T* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    out[i] = scale * z[i].x;
}

// sky = exp(s) on the (E, nx, ny) crop of a log-sky array s with plane
// stride ps and row stride rs (the unfused path reads a materialised sky)
template <typename T>
__global__ void k_exp_crop(const T* __restrict__ s, int E, int nx, int ny, int64_t ps,
                           int64_t rs, T* __restrict__ x) {
  const int64_t n = (int64_t)E * nx * ny;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = i / ((int64_t)nx * ny), r = (i / ny) % nx, c = i % ny;
    x[i] = exp(s[e * ps + r * rs + c]);
  }
}

// chain rule through sky = exp(s[:E, :nx, :ny]): grad_s = exp(s) * grad_x on the
// crop, 0 on the rest of the (Ep, n0p, n1p) log-sky array
// (gx_lo: the low words of a two-word gradient, or nullptr)
template <typename T>
__global__ void k_logsky_grad(const T* __restrict__ s, const T* __restrict__ gx,
                              const T* __restrict__ gx_lo, int E, int nx, int ny, int Ep, int n0p,
                              int n1p, T* __restrict__ gs) {
  const int64_t n = (int64_t)Ep * n0p * n1p;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = i / ((int64_t)n0p * n1p), r = (i / n1p) % n0p, c = i % n1p;
    if (e < E && r < nx && c < ny) {
      const int64_t j = (e * nx + r) * ny + c;
      gs[i] = exp(s[i]) * (gx_lo ? gx[j] + gx_lo[j] : gx[j]);
    } else {
      gs[i] = (T)0;
    }
  }
}

inline unsigned blocks_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  if (b > 1048576) b = 1048576;
  return (unsigned)(b < 1 ? 1 : b);
}

// numpy.linspace(0, 1, h) for the bilinear weights of jubik/convolve.py:18-25:
// step = 1/(h-1), a_i = i*step, last element exactly 1.
std::vector<double> bilinear_vector(int K) {
  const int h = K / 2;
  std::vector<double> a(h);
  if (h == 1) {
    a[0] = 0.0;
  } else {
    const double step = 1.0 / (double)(h - 1);
    for (int i = 0; i < h; ++i) a[i] = (double)i * step;
    a[h - 1] = 1.0;
  }
  std::vector<double> b(K);
  for (int i = 0; i < h; ++i) {
    b[i] = a[i];
    b[K - 1 - i] = a[i];
  }
  return b;
}

}  // namespace

template <typename T>
int convolve2d_run(const void* kernel, int64_t bk, const void* signal, int64_t bs, int64_t hw,
                   double dvol, const Fft1D& fh, const Fft1D& fw, void* zk, void* zs, void* out,
                   cudaStream_t s) {
  k_to_cplx<T><<<blocks_for(bk * hw), 256, 0, s>>>((const T*)kernel, bk * hw, (cx<T>*)zk);
  k_to_cplx<T><<<blocks_for(bs * hw), 256, 0, s>>>((const T*)signal, bs * hw, (cx<T>*)zs);
  JUBIK_TRY(fft2_batched<T>(fh, fw, zk, bk, false, s));
  JUBIK_TRY(fft2_batched<T>(fh, fw, zs, bs, false, s));
  k_mul_bcast<T><<<blocks_for(bs * hw), 256, 0, s>>>((const cx<T>*)zk, bk, (cx<T>*)zs, bs, hw);
  JUBIK_TRY(fft2_batched<T>(fh, fw, zs, bs, true, s));
  k_real_out<T><<<blocks_for(bs * hw), 256, 0, s>>>((const cx<T>*)zs, bs * hw,
                                                    (T)(dvol / (double)hw), (T*)out);
  return cuda_status(cudaGetLastError(), "convolve2d");
}


template int convolve2d_run<float>(const void*, int64_t, const void*, int64_t, int64_t, double,
                                   const Fft1D&, const Fft1D&, void*, void*, void*, cudaStream_t);
template int convolve2d_run<double>(const void*, int64_t, const void*, int64_t, int64_t, double,
                                    const Fft1D&, const Fft1D&, void*, void*, void*,
                                    cudaStream_t);

}  // namespace jubik

using namespace jubik;

struct jubik_plan {
  jubik_plan_desc desc{};
  Geom g;
  int path = JUBIK_PATH_PLAIN;
  int dtype = JUBIK_F32;
  size_t esz = 4;
  int device = 0;
  size_t bytes = 0;
  // constants
  void* wt = nullptr;  // (K) bilinear weights
  void* tw = nullptr;  // (P) fused twiddles
  Fft1D fft;           // plain transforms of length P
  // PSF spectra
  void* hmain = nullptr;
  void* hnyq = nullptr;
  void* hfull = nullptr;
  void* spec = nullptr;  // per-(energy, patch) spectra shared by the modules
  bool pdl = true;       // programmatic dependent launch between the kernels of a call
  int fwd_run = 0;       // module-shared forward: patches per run (0: the library's choice)
  void* acc = nullptr;   // per-(energy, patch) adjoint sums over modules (written whole by
                         // the ordered adjoint; grouped launches clear it before they add)
  // exact two-word accumulation (fused path): low-word planes of the images and
  // the gradient, the input-magnitude maxima that bound their terms, the spill
  // slots and grid of the ordered adjoint, and the largest sum of |kernel| over
  // the units (the PSF's share of the bounds)
  void* conv_lo = nullptr;
  void* conv_v_lo = nullptr;
  void* grad_lo = nullptr;
  void* bnd_f = nullptr;
  void* bnd_a = nullptr;
  void* spill = nullptr;
  int64_t adj_grid = 0;
  double kmax = 1.0;
  // images (M,E,nx,ny)
  void* conv = nullptr;
  void* conv_v = nullptr;
  void* resid = nullptr;
  void* wts = nullptr;  // metric weights eps^2 / lam of the last lam (image space)
  void* eps = nullptr;
  void* xsky = nullptr;   // (E,nx,ny) sky from a log-sky input (unfused path)
  void* xgrad = nullptr;  // (E,nx,ny) sky gradient before the chain rule to a log-sky
  int32_t* ridx = nullptr;
  int64_t* rlist = nullptr;
  int32_t* data = nullptr;
  int32_t* dimg = nullptr;  // per-pixel counts, -1 where not read out
  double* partials = nullptr;
  unsigned int* counter = nullptr;
  // unfused work buffers
  void* zs = nullptr;
  void* zu = nullptr;
  int zu_modules = 0;
  // state
  bool psf_set = false, exposure_set = false, data_set = false, lam_valid = false;
  // bumped whenever a buffer address or the readout map that a group copied in
  // jubik_group_set_io changes (exposure set or dropped, data buffers allocated)
  uint64_t layout_gen = 0;
  std::vector<int64_t> readout_sizes;
  int64_t readout_total = 0;
  std::vector<void*> allocs;
  // profiling
  bool prof = false;
  cudaEvent_t ev_a[JUBIK_PHASES] = {}, ev_b[JUBIK_PHASES] = {};
  double prof_ms[JUBIK_PHASES] = {0};
  int64_t prof_n[JUBIK_PHASES] = {0};

  int alloc(void** p, size_t n) {
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(p, n);
    if (e != cudaSuccess) return cuda_status(e, "cudaMalloc (plan workspace)");
    allocs.push_back(*p);
    bytes += n;
    return JUBIK_OK;
  }
  ~jubik_plan() {
    for (int i = 0; i < JUBIK_PHASES; ++i) {
      if (ev_a[i]) cudaEventDestroy(ev_a[i]);
      if (ev_b[i]) cudaEventDestroy(ev_b[i]);
    }
    for (void* p : allocs) cudaFree(p);
    fft1d_free(&fft);
  }
};

namespace {

inline cudaStream_t S(void* s) { return (cudaStream_t)s; }

// NVTX range named after the entry point (visible in Nsight timelines; a
// no-op unless a tool is attached)
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
};

// Brackets one kernel phase with events when the plan profiles.
struct Phase {
  jubik_plan* p;
  int k;
  cudaStream_t s;
  Phase(jubik_plan* p_, int k_, cudaStream_t s_) : p(p_), k(k_), s(s_) {
    if (p->prof) cudaEventRecord(p->ev_a[k], s);
  }
  ~Phase() {
    if (!p->prof) return;
    cudaEventRecord(p->ev_b[k], s);
    if (cudaEventSynchronize(p->ev_b[k]) == cudaSuccess) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, p->ev_a[k], p->ev_b[k]);
      p->prof_ms[k] += ms;
      p->prof_n[k] += 1;
    }
  }
};


int check_plan(const jubik_plan* p) {
  if (!p) {
    set_error("plan is NULL");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  return JUBIK_OK;
}

int64_t image_elems(const jubik_plan* p) { return (int64_t)p->g.M * p->g.E * p->g.pixels(); }

// forward of the PSF operator: out (M,E,nx,ny) = scale * sum_k patch convolutions
// `also_zero` (module-shared path only): a buffer of `also_zero_bytes` for the
// sky-spectrum kernel to clear as well -- the gradient that a later do_adjoint
// with out_zeroed adds into.  Returns whether it was cleared.
// How the forward reads its sky: the field itself (default), or exp of the
// (E, nx, ny) crop of a log-sky array with plane stride ps and row stride rs.
struct SkyView {
  int64_t ps = 0, rs = 0;
  bool exp = false;
};

// log2 of the most terms the two-word sums add per element: the patches that
// overlap a forward pixel (side P at stride dx, one more for clamped starts),
// and, for the gradient, the windows (side 2 dx) over a pixel times the modules.
int terms_log2(int64_t terms) {
  int L = 0;
  while ((int64_t(1) << L) < terms) ++L;
  return L;
}
int fwd_terms_log2(const Geom& g) {
  const int64_t per = (g.P + g.dx - 1) / g.dx + 1;
  return terms_log2(per * per);
}
int adj_terms_log2(const Geom& g) {
  const int64_t per = (g.K + g.dx - 1) / g.dx + 1;
  return terms_log2(per * per * g.M);
}

// row pass of the unfused path's 2-D transforms over batch P x P arrays
template <typename T>
int plain_rows(jubik_plan* p, void* data, int64_t batch, bool inverse, cudaStream_t s) {
  const int64_t P = p->g.P;
  return fft_batched<T>(p->fft, data, batch * P, (int)P, P * P, P, 1, inverse, 1.0, s);
}

int do_forward(jubik_plan* p, const void* x, void* out, void* out_lo, double scale,
               cudaStream_t s, void* also_zero = nullptr, int64_t also_zero_bytes = 0,
               bool* zeroed = nullptr, SkyView view = SkyView()) {
  const Geom& g = p->g;
  if (zeroed) *zeroed = false;
  if (view.exp && p->path != JUBIK_PATH_FUSED) {  // materialise the sky for the unfused path
    const int64_t n = (int64_t)g.E * g.pixels();
    if (p->dtype == JUBIK_F32)
      k_exp_crop<float><<<blocks_for(n), 256, 0, s>>>((const float*)x, g.E, g.nx, g.ny, view.ps,
                                                       view.rs, (float*)p->xsky);
    else
      k_exp_crop<double><<<blocks_for(n), 256, 0, s>>>((const double*)x, g.E, g.nx, g.ny,
                                                        view.ps, view.rs, (double*)p->xsky);
    JUBIK_TRY(cuda_status(cudaGetLastError(), "k_exp_crop"));
    x = p->xsky;
  }
  if (p->path == JUBIK_PATH_FUSED) {
    FusedLaunch a{x, out, p->hmain, p->hnyq, p->tw, p->wt, scale, p->spec};
    a.pdl = p->pdl;
    a.fwd_run = p->fwd_run;
    a.in_ps = view.ps;
    a.in_rs = view.rs;
    a.in_exp = view.exp;
    // the overlap-add is exact in two words: every partial sum of a pixel is
    // bounded by (terms) x (kernel gain) x |scale| x the largest weighted sky value
    a.out_lo = out_lo;
    const int L = fwd_terms_log2(g);
    a.bnd_log2 = L;
    a.bnd_scale = 2.0 * (double)(int64_t(1) << L) * p->kmax * std::fabs(scale);
    if (p->spec && also_zero) {
      a.aux = also_zero;
      a.aux_bytes = also_zero_bytes;
      if (zeroed) *zeroed = true;
    }
    if (!p->spec) {
      {
        Phase ph(p, 3, s);
        JUBIK_TRY_CUDA(cudaMemsetAsync(out, 0, image_elems(p) * p->esz, s));
        JUBIK_TRY_CUDA(cudaMemsetAsync(out_lo, 0, image_elems(p) * p->esz, s));
      }
      Phase ph(p, 0, s);
      int nb = 0;
      const int64_t ps = view.ps > 0 ? view.ps : g.pixels(), rs = view.rs > 0 ? view.rs : g.ny;
      JUBIK_TRY(p->dtype == JUBIK_F32
                    ? absmax_blocks<float>(x, g.E, g.nx, g.ny, ps, rs, view.exp, p->bnd_f, &nb,
                                           p->pdl, s)
                    : absmax_blocks<double>(x, g.E, g.nx, g.ny, ps, rs, view.exp, p->bnd_f, &nb,
                                            p->pdl, s));
      a.bnd_in = p->bnd_f;
      a.bnd_n = nb;
      return fused_run(g, p->dtype, a, FUSED_FWD_UNITS, s);
    }
    {  // the sky-spectrum kernel also clears `out` (both words) for the overlap-add
      // and records each window's largest weighted sky value
      Phase ph(p, 4, s);
      a.bnd_out = p->bnd_f;
      JUBIK_TRY(fused_run(g, p->dtype, a, FUSED_FWD_SKY, s));
    }
    Phase ph(p, 0, s);
    a.bnd_out = nullptr;
    a.bnd_in = p->bnd_f;
    a.bnd_n = (int)((int64_t)g.E * g.n * g.n);
    return fused_run(g, p->dtype, a, FUSED_FWD_FROM_SPEC, s);
  }
  Phase ph(p, 0, s);
  const bool f32 = p->dtype == JUBIK_F32;
  if (plain_cols_supported(g.P)) {
    // row pass over the weighted sky windows; per module chunk: column stage
    // with the PSF product, inverse row pass, overlap gather
    const void* tw = f32 ? p->fft.tw32 : p->fft.tw64;
    JUBIK_TRY(f32 ? fft_rows_windows<float>(p->fft, g, x, false, p->wt, 0, 1, p->zs, s)
                  : fft_rows_windows<double>(p->fft, g, x, false, p->wt, 0, 1, p->zs, s));
    for (int m0 = 0; m0 < g.M; m0 += p->zu_modules) {
      const int nm = std::min(p->zu_modules, g.M - m0);
      JUBIK_TRY(f32 ? plain_cols_forward<float>(g, p->zs, p->hfull, tw, m0, nm, p->zu, s)
                    : plain_cols_forward<double>(g, p->zs, p->hfull, tw, m0, nm, p->zu, s));
      const int64_t batch = (int64_t)nm * plain_pairs(g);
      JUBIK_TRY(f32 ? plain_rows<float>(p, p->zu, batch, true, s)
                    : plain_rows<double>(p, p->zu, batch, true, s));
      JUBIK_TRY(f32 ? plain_overlap_gather<float>(g, p->zu, m0, nm, scale, out, s)
                    : plain_overlap_gather<double>(g, p->zu, m0, nm, scale, out, s));
    }
    return JUBIK_OK;
  }
  JUBIK_TRY(f32 ? plain_sky_patches<float>(g, x, p->wt, p->zs, s)
                : plain_sky_patches<double>(g, x, p->wt, p->zs, s));
  JUBIK_TRY(f32 ? fft2_batched<float>(p->fft, p->fft, p->zs, plain_pairs(g), false, s)
                : fft2_batched<double>(p->fft, p->fft, p->zs, plain_pairs(g), false, s));
  for (int m0 = 0; m0 < g.M; m0 += p->zu_modules) {
    const int nm = std::min(p->zu_modules, g.M - m0);
    JUBIK_TRY(f32 ? plain_mul_modules<float>(g, p->zs, p->hfull, m0, nm, p->zu, s)
                  : plain_mul_modules<double>(g, p->zs, p->hfull, m0, nm, p->zu, s));
    const int64_t batch = (int64_t)nm * plain_pairs(g);
    JUBIK_TRY(f32 ? fft2_batched<float>(p->fft, p->fft, p->zu, batch, true, s)
                  : fft2_batched<double>(p->fft, p->fft, p->zu, batch, true, s));
    JUBIK_TRY(f32 ? plain_overlap_gather<float>(g, p->zu, m0, nm, scale, out, s)
                  : plain_overlap_gather<double>(g, p->zu, m0, nm, scale, out, s));
  }
  return JUBIK_OK;
}

// transpose: out_x (E,nx,ny) = scale * sum_m psf_m^T cot[m]; on the fused path
// in two words (out_x, out_lo), the caller adding them (combine_words)
// bnd_n: block maxima of |cot| that the kernel which wrote cot left in
// p->bnd_a (0: none, a pass over cot records them)
int do_adjoint(jubik_plan* p, const void* cot, void* out_x, void* out_lo, double scale,
               cudaStream_t s, bool out_zeroed = false, int bnd_n = 0) {
  const Geom& g = p->g;
  if (p->path == JUBIK_PATH_FUSED) {
    const int L = adj_terms_log2(g);
    // every partial sum of a gradient pixel is bounded by (windows x modules) x
    // (kernel gain) x |scale| x the largest cotangent magnitude
    const double bscale = 2.0 * (double)(int64_t(1) << L) * p->kmax * std::fabs(scale);
    if (bnd_n <= 0) {
      Phase ph(p, 3, s);
      JUBIK_TRY(p->dtype == JUBIK_F32
                    ? absmax_blocks<float>(cot, g.M * g.E, g.nx, g.ny, g.pixels(), g.ny, false,
                                           p->bnd_a, &bnd_n, p->pdl, s)
                    : absmax_blocks<double>(cot, g.M * g.E, g.nx, g.ny, g.pixels(), g.ny, false,
                                            p->bnd_a, &bnd_n, p->pdl, s));
    }
    if (!p->spec) {
      {
        Phase ph(p, 3, s);
        JUBIK_TRY_CUDA(cudaMemsetAsync(out_x, 0, (size_t)g.E * g.pixels() * p->esz, s));
        JUBIK_TRY_CUDA(cudaMemsetAsync(out_lo, 0, (size_t)g.E * g.pixels() * p->esz, s));
      }
      FusedLaunch a{cot, out_x, p->hmain, p->hnyq, p->tw, p->wt, scale, nullptr};
      a.pdl = p->pdl;
      a.out_lo = out_lo;
      a.bnd_log2 = L;
      a.bnd_scale = bscale;
      a.bnd_in = p->bnd_a;
      a.bnd_n = bnd_n;
      Phase ph(p, 1, s);
      return fused_run(g, p->dtype, a, FUSED_ADJ_UNITS, s);
    }
    // ordered per-unit kernel: clears out_x (unless zeroed) and out_lo, sums each
    // patch over modules in module order; per-patch kernel: accumulator plus
    // spill slots -> gradient in two words
    FusedLaunch a{cot, out_x, p->hmain, p->hnyq, p->tw, p->wt, scale, p->acc};
    a.zero_out = !out_zeroed;
    a.pdl = p->pdl;
    a.out_lo = out_lo;
    a.spill = p->spill;
    a.loop_grid = p->adj_grid;
    a.bnd_log2 = L;
    a.bnd_scale = bscale;
    {
      Phase ph(p, 1, s);
      JUBIK_TRY(fused_run(g, p->dtype, a, FUSED_ADJ_TO_SPEC, s));
    }
    Phase ph(p, 5, s);
    a.bnd_in = p->bnd_a;
    a.bnd_n = bnd_n;
    return fused_run(g, p->dtype, a, FUSED_ADJ_FROM_SPEC, s);
  }
  Phase ph(p, 1, s);
  const bool f32 = p->dtype == JUBIK_F32;
  if (plain_cols_supported(g.P)) {
    // per module chunk: row pass over the cotangent windows, column stage summing
    // the conjugate-PSF products over modules; then the inverse row pass and the
    // gradient gather
    const void* tw = f32 ? p->fft.tw32 : p->fft.tw64;
    for (int m0 = 0; m0 < g.M; m0 += p->zu_modules) {
      const int nm = std::min(p->zu_modules, g.M - m0);
      const bool first = m0 == 0, last = m0 + nm == g.M;
      JUBIK_TRY(f32 ? fft_rows_windows<float>(p->fft, g, cot, true, nullptr, m0, nm, p->zu, s)
                    : fft_rows_windows<double>(p->fft, g, cot, true, nullptr, m0, nm, p->zu, s));
      JUBIK_TRY(f32 ? plain_cols_adjoint<float>(g, p->zu, p->hfull, tw, m0, nm, first, last,
                                                p->zs, s)
                    : plain_cols_adjoint<double>(g, p->zu, p->hfull, tw, m0, nm, first, last,
                                                 p->zs, s));
    }
    JUBIK_TRY(f32 ? plain_rows<float>(p, p->zs, plain_pairs(g), true, s)
                  : plain_rows<double>(p, p->zs, plain_pairs(g), true, s));
    return f32 ? plain_grad_gather<float>(g, p->zs, p->wt, scale, out_x, s)
               : plain_grad_gather<double>(g, p->zs, p->wt, scale, out_x, s);
  }
  for (int m0 = 0; m0 < g.M; m0 += p->zu_modules) {
    const int nm = std::min(p->zu_modules, g.M - m0);
    JUBIK_TRY(f32 ? plain_cot_patches<float>(g, cot, m0, nm, p->zu, s)
                  : plain_cot_patches<double>(g, cot, m0, nm, p->zu, s));
    const int64_t batch = (int64_t)nm * plain_pairs(g);
    JUBIK_TRY(f32 ? fft2_batched<float>(p->fft, p->fft, p->zu, batch, false, s)
                  : fft2_batched<double>(p->fft, p->fft, p->zu, batch, false, s));
    JUBIK_TRY(f32 ? plain_mulconj_accum<float>(g, p->zu, p->hfull, m0, nm, m0 == 0, p->zs, s)
                  : plain_mulconj_accum<double>(g, p->zu, p->hfull, m0, nm, m0 == 0, p->zs, s));
  }
  JUBIK_TRY(f32 ? fft2_batched<float>(p->fft, p->fft, p->zs, plain_pairs(g), true, s)
                : fft2_batched<double>(p->fft, p->fft, p->zs, plain_pairs(g), true, s));
  return f32 ? plain_grad_gather<float>(g, p->zs, p->wt, scale, out_x, s)
             : plain_grad_gather<double>(g, p->zs, p->wt, scale, out_x, s);
}

// hi += lo where the fused path left a two-word result
int finish_words(jubik_plan* p, void* hi, const void* lo, int64_t n, cudaStream_t s) {
  if (p->path != JUBIK_PATH_FUSED) return JUBIK_OK;
  return p->dtype == JUBIK_F32 ? combine_words<float>(hi, lo, n, p->pdl, s)
                               : combine_words<double>(hi, lo, n, p->pdl, s);
}

int need(bool ok, const char* what) {
  if (!ok) {
    set_error("%s not set on this plan", what);
    return JUBIK_ERR_STATE;
  }
  return JUBIK_OK;
}

}  // namespace

extern "C" {

int jubik_abi_version(void) { return JUBIK_ABI_VERSION; }

const char* jubik_last_error(void) { return g_err; }

int jubik_fused_supported(int32_t P, int32_t dtype) { return fused_supported(P, dtype) ? 1 : 0; }

int jubik_fft_length_supported(int32_t L) { return fft_length_supported(L) ? 1 : 0; }

int jubik_plan_create(const jubik_plan_desc* d, jubik_plan** out) {
  NvtxRange nvtx_("jubik_plan_create");
  if (!d || !out) {
    set_error("NULL argument");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  *out = nullptr;
  if (d->dtype != JUBIK_F32 && d->dtype != JUBIK_F64) {
    set_error("dtype must be JUBIK_F32 or JUBIK_F64");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (d->n_modules < 1 || d->n_energies < 1 || d->nx < 1 || d->ny < 1 || d->n_patches < 1) {
    set_error("modules, energies, field and n_patches must be >= 1");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (d->margin < 1) {
    set_error("margin must be >= 1 (the reference crops [margin:-margin])");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  Geom g;
  g.M = d->n_modules;
  g.E = d->n_energies;
  g.nx = d->nx;
  g.ny = d->ny;
  g.n = d->n_patches;
  g.dx = d->nx / d->n_patches;
  const int dy = d->ny / d->n_patches;
  if (g.dx < 1 || dy != g.dx) {
    set_error("patch stride must be >= 1 and equal on both axes (got %d and %d): the "
              "bilinear weights of convolve.py:18-25 are square",
              g.dx, dy);
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  g.margin = d->margin;
  g.half = g.dx / 2;
  g.K = 2 * g.dx;
  g.P = g.K + 2 * g.margin;
  g.sr_max = g.nx + 2 * g.half - g.K;
  g.sc_max = g.ny + 2 * g.half - g.K;
  if (g.sr_max < 0 || g.sc_max < 0) {
    set_error("patch window does not fit the padded field");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (!fft_length_supported(g.P)) {
    set_error("FFT side P=%d unsupported", g.P);
    return JUBIK_ERR_UNSUPPORTED;
  }
  jubik_plan* p = new (std::nothrow) jubik_plan();
  if (!p) {
    set_error("host allocation failed");
    return JUBIK_ERR_ALLOC;
  }
  p->desc = *d;
  p->g = g;
  p->dtype = d->dtype;
  p->esz = d->dtype == JUBIK_F32 ? 4 : 8;
  cudaGetDevice(&p->device);
  const bool fused_ok = fused_supported(g.P, d->dtype);
  if (d->path == JUBIK_PATH_FUSED && !fused_ok) {
    delete p;
    set_error("fused path does not cover P=%d in this dtype", g.P);
    return JUBIK_ERR_UNSUPPORTED;
  }
  if (d->path < JUBIK_PATH_AUTO || d->path > JUBIK_PATH_FUSED_UNIT) {
    delete p;
    set_error("unknown path %d", d->path);
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (d->path == JUBIK_PATH_FUSED_UNIT && !fused_ok) {
    delete p;
    set_error("fused path does not cover P=%d in this dtype", g.P);
    return JUBIK_ERR_UNSUPPORTED;
  }
  p->path = (d->path == JUBIK_PATH_PLAIN || !fused_ok) ? JUBIK_PATH_PLAIN : JUBIK_PATH_FUSED;
  // modules share the patch spectra (sky forward, summed adjoint) when there are several
  const bool share = p->path == JUBIK_PATH_FUSED && d->path != JUBIK_PATH_FUSED_UNIT && g.M >= 2;

  int st = JUBIK_OK;
  auto fail = [&](int s) {
    delete p;
    return s;
  };
  const size_t csz = 2 * p->esz;
  const int64_t units = g.units();
  const int64_t img = (int64_t)g.M * g.E * g.pixels();
  // constants
  {
    std::vector<double> b = bilinear_vector(g.K);
    if ((st = p->alloc(&p->wt, g.K * p->esz))) return fail(st);
    if (p->dtype == JUBIK_F32) {
      std::vector<float> bf(b.begin(), b.end());
      if ((st = cuda_status(cudaMemcpy(p->wt, bf.data(), g.K * 4, cudaMemcpyHostToDevice),
                            "upload weights")))
        return fail(st);
    } else {
      if ((st = cuda_status(cudaMemcpy(p->wt, b.data(), g.K * 8, cudaMemcpyHostToDevice),
                            "upload weights")))
        return fail(st);
    }
  }
  if ((st = fft1d_init(&p->fft, g.P))) return fail(st);
  p->tw = p->dtype == JUBIK_F32 ? p->fft.tw32 : p->fft.tw64;
  if (p->path == JUBIK_PATH_FUSED) {
    if ((st = p->alloc(&p->hmain, (size_t)units * g.P * (g.P / 2) * csz))) return fail(st);
    if ((st = p->alloc(&p->hnyq, (size_t)units * g.P * csz))) return fail(st);
    if (share && (st = p->alloc(&p->spec, fused_spec_bytes(g, p->dtype)))) return fail(st);
    if (share && (st = p->alloc(&p->acc, fused_spec_bytes(g, p->dtype)))) return fail(st);
    if (share && (st = cuda_status(cudaMemset(p->acc, 0, fused_spec_bytes(g, p->dtype)),
                                   "memset accumulator")))
      return fail(st);
    const int64_t patches = (int64_t)g.E * g.n * g.n;
    if (share) {
      p->adj_grid = fused_adj_grid(g, p->dtype);
      if (p->adj_grid <= 0) {
        delete p;
        set_error("no launch configuration for the ordered adjoint at P=%d", g.P);
        return JUBIK_ERR_UNSUPPORTED;
      }
      if ((st = p->alloc(&p->spill, (size_t)p->adj_grid * g.P * (g.P / 2) * csz)))
        return fail(st);
    }
    if ((st = p->alloc(&p->conv_lo, img * p->esz))) return fail(st);
    if ((st = p->alloc(&p->conv_v_lo, img * p->esz))) return fail(st);
    if ((st = p->alloc(&p->grad_lo, (size_t)g.E * g.pixels() * p->esz))) return fail(st);
    if ((st = p->alloc(&p->bnd_f, sizeof(uint64_t) * std::max<int64_t>(patches,
                                                                        kMaxBoundBlocks))))
      return fail(st);
    if ((st = p->alloc(&p->bnd_a, sizeof(uint64_t) *
                                      std::max<int64_t>(energy_partials_count(), kMaxBoundBlocks))))
      return fail(st);
  } else {
    if ((st = p->alloc(&p->hfull, (size_t)units * g.P * (g.P / 2 + 1) * csz))) return fail(st);
    if ((st = p->alloc(&p->zs, (size_t)plain_pairs(g) * g.P * g.P * csz))) return fail(st);
    // bound the per-chunk unit buffer to ~2 GiB; JUBIK_PLAIN_CHUNK_MODULES, when
    // set to a positive count, bounds the modules per chunk further
    const size_t per_module = (size_t)plain_pairs(g) * g.P * g.P * csz;
    size_t chunk = std::min<size_t>(g.M, (2ull << 30) / per_module);
    if (const char* env = std::getenv("JUBIK_PLAIN_CHUNK_MODULES")) {
      const long v = std::strtol(env, nullptr, 10);
      if (v >= 1) chunk = std::min<size_t>(chunk, (size_t)v);
    }
    p->zu_modules = (int)std::max<size_t>(1, chunk);
    if ((st = p->alloc(&p->zu, per_module * p->zu_modules))) return fail(st);
  }
  if ((st = p->alloc(&p->conv, img * p->esz))) return fail(st);
  if ((st = p->alloc(&p->conv_v, img * p->esz))) return fail(st);
  if ((st = p->alloc(&p->resid, img * p->esz))) return fail(st);
  if ((st = p->alloc(&p->wts, img * p->esz))) return fail(st);
  if ((st = p->alloc(&p->xsky, (size_t)g.E * g.pixels() * p->esz))) return fail(st);
  if ((st = p->alloc(&p->xgrad, (size_t)g.E * g.pixels() * p->esz))) return fail(st);
  if ((st = p->alloc((void**)&p->ridx, img * sizeof(int32_t)))) return fail(st);
  if ((st = p->alloc((void**)&p->rlist, img * sizeof(int64_t)))) return fail(st);
  if ((st = p->alloc((void**)&p->partials, 2 * energy_partials_count() * sizeof(double))))
    return fail(st);
  if ((st = p->alloc((void**)&p->counter, sizeof(unsigned int)))) return fail(st);
  if ((st = cuda_status(cudaMemset(p->counter, 0, sizeof(unsigned int)), "memset counter")))
    return fail(st);
  if (img > 0x7fffffffLL) {
    delete p;
    set_error("more than 2^31 image pixels per plan");
    return JUBIK_ERR_UNSUPPORTED;
  }
  // default: everything read out, unit exposure
  k_iota<<<blocks_for(img), 256>>>(p->ridx, p->rlist, img);
  if ((st = cuda_status(cudaGetLastError(), "k_iota"))) return fail(st);
  if ((st = cuda_status(cudaDeviceSynchronize(), "plan set-up"))) return fail(st);
  p->readout_sizes.assign(g.M, (int64_t)g.E * g.pixels());
  p->readout_total = img;
  *out = p;
  return JUBIK_OK;
}

int jubik_plan_destroy(jubik_plan* plan) {
  if (!plan) return JUBIK_OK;
  cudaDeviceSynchronize();
  delete plan;
  return JUBIK_OK;
}

int jubik_plan_workspace_bytes(const jubik_plan* plan, int64_t* bytes) {
  JUBIK_TRY(check_plan(plan));
  if (bytes) *bytes = (int64_t)plan->bytes;
  return JUBIK_OK;
}

int jubik_plan_path(const jubik_plan* plan, int32_t* path) {
  JUBIK_TRY(check_plan(plan));
  if (path) *path = plan->path;
  return JUBIK_OK;
}

int jubik_plan_set_dependent_launch(jubik_plan* p, int32_t on) {
  JUBIK_TRY(check_plan(p));
  p->pdl = on != 0;
  return JUBIK_OK;
}

int jubik_plan_set_forward_run(jubik_plan* p, int32_t run_len) {
  JUBIK_TRY(check_plan(p));
  if (run_len != 0 && run_len != 1 && run_len != 2 && run_len != 4) {
    set_error("set_forward_run: run length %d is not 0, 1, 2 or 4", run_len);
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (run_len > 1 && (p->path != JUBIK_PATH_FUSED || !p->spec ||
                      fused_fwd_run_len(p->g, p->dtype, run_len) < 0)) {
    set_error("set_forward_run: runs of %d patches need the module-shared FP32 kernels at FFT "
              "side 192 with 64-pixel strides, a 32-pixel margin and %d | n", run_len, run_len);
    return JUBIK_ERR_UNSUPPORTED;
  }
  p->fwd_run = run_len;
  return JUBIK_OK;
}

int jubik_plan_forward_run(const jubik_plan* p, int32_t* run_len) {
  JUBIK_TRY(check_plan(p));
  if (!run_len) {
    set_error("forward_run: null output");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  *run_len = (p->path == JUBIK_PATH_FUSED && p->spec)
                 ? fused_fwd_run_len(p->g, p->dtype, p->fwd_run) : 1;
  return JUBIK_OK;
}

int jubik_plan_set_profiling(jubik_plan* p, int32_t on) {
  JUBIK_TRY(check_plan(p));
  if (on && !p->ev_a[0]) {
    for (int i = 0; i < JUBIK_PHASES; ++i) {
      JUBIK_TRY_CUDA(cudaEventCreate(&p->ev_a[i]));
      JUBIK_TRY_CUDA(cudaEventCreate(&p->ev_b[i]));
    }
  }
  p->prof = on != 0;
  for (int i = 0; i < JUBIK_PHASES; ++i) {
    p->prof_ms[i] = 0.0;
    p->prof_n[i] = 0;
  }
  return JUBIK_OK;
}

int jubik_plan_profile(const jubik_plan* p, double* ms, int64_t* launches) {
  JUBIK_TRY(check_plan(p));
  for (int i = 0; i < JUBIK_PHASES; ++i) {
    if (ms) ms[i] = p->prof_ms[i];
    if (launches) launches[i] = p->prof_n[i];
  }
  return JUBIK_OK;
}

int jubik_plan_set_psf(jubik_plan* p, const void* psf, int32_t layout, int32_t e_broadcast,
                       void* stream) {
  NvtxRange nvtx_("jubik_plan_set_psf");
  JUBIK_TRY(check_plan(p));
  if (!psf || (layout != JUBIK_PSF_PRECUT && layout != JUBIK_PSF_FULL)) {
    set_error("psf must be non-NULL with a valid layout");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  const Geom& g = p->g;
  if (layout == JUBIK_PSF_FULL) {
    const int kcx = (g.nx - 2 * g.dx) / 2, kcy = (g.ny - 2 * g.dx) / 2;
    if (kcx <= 0 || kcy <= 0 || g.nx - 2 * kcx != g.K || g.ny - 2 * kcy != g.K) {
      set_error("the kernel cut [%d:-%d] of convolve.py:107-111 does not give a %d x %d window "
                "(needs n_patches >= 3 and an even field-minus-window)",
                kcx, kcx, g.K, g.K);
      return JUBIK_ERR_INVALID_ARGUMENT;
    }
  }
  cudaStream_t s = S(stream);
  const int64_t units = g.units();
  const size_t per = (size_t)g.P * g.P * sizeof(double2);
  int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(units, (int64_t)((512ull << 20) / per)));
  void* buf = nullptr;
  double* sums = nullptr;
  JUBIK_TRY_CUDA(cudaMallocAsync(&buf, per * chunk, s));
  JUBIK_TRY_CUDA(cudaMallocAsync((void**)&sums, 2 * sizeof(double) * chunk, s));
  int st = JUBIK_OK;
  double kmax = 0.0;
  std::vector<double> hs(2 * chunk);
  for (int64_t u0 = 0; u0 < units && st == JUBIK_OK; u0 += chunk) {
    const int64_t nu = std::min(chunk, units - u0);
    st = p->dtype == JUBIK_F32
             ? psf_to_cplx<float>(g, psf, layout, e_broadcast, u0, nu, sums, buf, s)
             : psf_to_cplx<double>(g, psf, layout, e_broadcast, u0, nu, sums, buf, s);
    if (st) break;
    // sum |k| / |sum k| of each unit's window: the magnitude gain of its
    // normalised kernel, which the output bounds of the two-word sums use
    st = cuda_status(cudaMemcpyAsync(hs.data(), sums, 2 * sizeof(double) * nu,
                                     cudaMemcpyDeviceToHost, s), "copy kernel sums");
    if (!st) st = cuda_status(cudaStreamSynchronize(s), "copy kernel sums");
    if (st) break;
    for (int64_t i = 0; i < nu; ++i) {
      const double r = std::fabs(hs[2 * i + 1] / hs[2 * i]);
      kmax = (r > kmax || r != r) ? r : kmax;
    }
    st = fft2_batched<double>(p->fft, p->fft, buf, nu, false, s);
    if (st) break;
    st = p->dtype == JUBIK_F32
             ? spectra_store<float>(g, buf, u0, nu, p->hfull, p->hmain, p->hnyq, s)
             : spectra_store<double>(g, buf, u0, nu, p->hfull, p->hmain, p->hnyq, s);
  }
  cudaFreeAsync(buf, s);
  cudaFreeAsync(sums, s);
  JUBIK_TRY(st);
  p->kmax = kmax;
  p->psf_set = true;
  p->lam_valid = false;
  return cuda_status(cudaGetLastError(), "set_psf");
}

int jubik_plan_set_exposure(jubik_plan* p, const void* exposure, const uint8_t* readmask,
                            void* stream) {
  NvtxRange nvtx_("jubik_plan_set_exposure");
  JUBIK_TRY(check_plan(p));
  cudaStream_t s = S(stream);
  const Geom& g = p->g;
  const int64_t img = image_elems(p);
  if (exposure) {
    if (!p->eps) JUBIK_TRY(p->alloc(&p->eps, img * p->esz));
    JUBIK_TRY_CUDA(cudaMemcpyAsync(p->eps, exposure, img * p->esz, cudaMemcpyDeviceToDevice, s));
  } else if (p->eps) {
    // back to unit exposure
    for (auto it = p->allocs.begin(); it != p->allocs.end(); ++it)
      if (*it == p->eps) {
        p->allocs.erase(it);
        break;
      }
    cudaFree(p->eps);
    p->eps = nullptr;
  }
  std::vector<int64_t> sizes(g.M, 0);
  if (!readmask) {
    k_iota<<<blocks_for(img), 256, 0, s>>>(p->ridx, p->rlist, img);
    JUBIK_TRY_CUDA(cudaGetLastError());
    for (int m = 0; m < g.M; ++m) sizes[m] = (int64_t)g.E * g.pixels();
  } else {
    const int64_t nb = (img + kScanBlock - 1) / kScanBlock;
    int32_t* counts = nullptr;
    int64_t* offsets = nullptr;
    JUBIK_TRY_CUDA(cudaMallocAsync((void**)&counts, sizeof(int32_t) * nb, s));
    JUBIK_TRY_CUDA(cudaMallocAsync((void**)&offsets, sizeof(int64_t) * (nb + 1), s));
    k_mask_counts<<<(unsigned)nb, 256, 0, s>>>(readmask, img, counts);
    k_scan_counts<<<1, 1, 0, s>>>(counts, nb, offsets);
    k_mask_compact<<<(unsigned)nb, 256, 0, s>>>(readmask, img, offsets, p->ridx, p->rlist);
    JUBIK_TRY_CUDA(cudaGetLastError());
    // per-module sizes (host count of the uploaded mask; one-off set-up work)
    const int64_t per_module = (int64_t)g.E * g.pixels();
    JUBIK_TRY_CUDA(cudaStreamSynchronize(s));
    std::vector<uint8_t> hmask(img);
    JUBIK_TRY_CUDA(cudaMemcpy(hmask.data(), readmask, img, cudaMemcpyDeviceToHost));
    for (int m = 0; m < g.M; ++m) {
      int64_t c = 0;
      const uint8_t* mm = hmask.data() + m * per_module;
      for (int64_t i = 0; i < per_module; ++i) c += mm[i] ? 1 : 0;
      sizes[m] = c;
    }
    cudaFreeAsync(counts, s);
    cudaFreeAsync(offsets, s);
  }
  JUBIK_TRY_CUDA(cudaStreamSynchronize(s));
  p->readout_sizes = sizes;
  p->readout_total = 0;
  for (int64_t v : sizes) p->readout_total += v;
  p->exposure_set = true;
  p->data_set = false;
  p->lam_valid = false;
  ++p->layout_gen;
  return JUBIK_OK;
}

int jubik_plan_readout_sizes(const jubik_plan* p, int64_t* per_module, int64_t* total) {
  JUBIK_TRY(check_plan(p));
  if (per_module)
    for (int m = 0; m < p->g.M; ++m) per_module[m] = p->readout_sizes[m];
  if (total) *total = p->readout_total;
  return JUBIK_OK;
}

int jubik_plan_readout_index(const jubik_plan* p, const int64_t** device_index) {
  JUBIK_TRY(check_plan(p));
  if (device_index) *device_index = p->rlist;
  return JUBIK_OK;
}

int jubik_plan_set_data(jubik_plan* p, const int32_t* counts, void* stream) {
  NvtxRange nvtx_("jubik_plan_set_data");
  JUBIK_TRY(check_plan(p));
  if (!counts) {
    set_error("counts is NULL");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (!p->data || !p->dimg) ++p->layout_gen;
  if (!p->data) JUBIK_TRY(p->alloc((void**)&p->data, image_elems(p) * sizeof(int32_t)));
  if (!p->dimg) JUBIK_TRY(p->alloc((void**)&p->dimg, image_elems(p) * sizeof(int32_t)));
  JUBIK_TRY_CUDA(cudaMemcpyAsync(p->data, counts, p->readout_total * sizeof(int32_t),
                                 cudaMemcpyDeviceToDevice, S(stream)));
  JUBIK_TRY(count_image(p->ridx, p->data, image_elems(p), p->dimg, S(stream)));
  p->data_set = true;
  return JUBIK_OK;
}

int jubik_psf_forward(jubik_plan* p, const void* x, void* out, void* stream) {
  NvtxRange nvtx_("jubik_psf_forward");
  JUBIK_TRY(check_plan(p));
  JUBIK_TRY(need(p->psf_set, "PSF"));
  cudaStream_t s = S(stream);
  JUBIK_TRY(do_forward(p, x, out, p->conv_lo, 1.0, s));
  return finish_words(p, out, p->conv_lo, image_elems(p), s);
}

int jubik_psf_adjoint(jubik_plan* p, const void* cot, void* out_x, void* stream) {
  NvtxRange nvtx_("jubik_psf_adjoint");
  JUBIK_TRY(check_plan(p));
  JUBIK_TRY(need(p->psf_set, "PSF"));
  cudaStream_t s = S(stream);
  JUBIK_TRY(do_adjoint(p, cot, out_x, p->grad_lo, 1.0, s));
  return finish_words(p, out_x, p->grad_lo, (int64_t)p->g.E * p->g.pixels(), s);
}

int jubik_response_forward(jubik_plan* p, const void* x, void* out_readout, void* stream) {
  NvtxRange nvtx_("jubik_response_forward");
  JUBIK_TRY(check_plan(p));
  JUBIK_TRY(need(p->psf_set, "PSF"));
  cudaStream_t s = S(stream);
  JUBIK_TRY(do_forward(p, x, p->conv, p->conv_lo, p->desc.pixel_area, s));
  const void* lo = p->path == JUBIK_PATH_FUSED ? p->conv_lo : nullptr;
  Phase ph(p, 2, s);
  return p->dtype == JUBIK_F32
             ? readout_gather<float>(p->conv, p->eps, p->rlist, p->readout_total, out_readout, s,
                                     lo)
             : readout_gather<double>(p->conv, p->eps, p->rlist, p->readout_total, out_readout,
                                      s, lo);
}

int jubik_response_jvp(jubik_plan* p, const void* t, void* out_readout, void* stream) {
  NvtxRange nvtx_("jubik_response_jvp");
  return jubik_response_forward(p, t, out_readout, stream);
}

int jubik_response_vjp(jubik_plan* p, const void* cot_readout, void* out_x, void* stream) {
  NvtxRange nvtx_("jubik_response_vjp");
  JUBIK_TRY(check_plan(p));
  JUBIK_TRY(need(p->psf_set, "PSF"));
  cudaStream_t s = S(stream);
  {
    Phase ph(p, 2, s);
    JUBIK_TRY_CUDA(cudaMemsetAsync(p->resid, 0, image_elems(p) * p->esz, s));
    JUBIK_TRY(p->dtype == JUBIK_F32
                  ? readout_scatter<float>(cot_readout, p->eps, p->rlist, p->readout_total,
                                           p->resid, s)
                  : readout_scatter<double>(cot_readout, p->eps, p->rlist, p->readout_total,
                                            p->resid, s));
  }
  JUBIK_TRY(do_adjoint(p, p->resid, out_x, p->grad_lo, p->desc.pixel_area, s));
  return finish_words(p, out_x, p->grad_lo, (int64_t)p->g.E * p->g.pixels(), s);
}

int jubik_poisson_energy_grad(jubik_plan* p, const void* x, double* energy, void* grad_x,
                              void* stream) {
  NvtxRange nvtx_("jubik_poisson_energy_grad");
  JUBIK_TRY(check_plan(p));
  JUBIK_TRY(need(p->psf_set, "PSF"));
  JUBIK_TRY(need(p->data_set, "data"));
  cudaStream_t s = S(stream);
  bool grad_zeroed = false;
  JUBIK_TRY(do_forward(p, x, p->conv, p->conv_lo, p->desc.pixel_area, s, grad_x,
                       (int64_t)p->g.E * p->g.pixels() * (int64_t)p->esz, &grad_zeroed));
  const int64_t img = image_elems(p);
  const void* lo = p->path == JUBIK_PATH_FUSED ? p->conv_lo : nullptr;
  {
  Phase ph(p, 2, s);
  JUBIK_TRY(p->dtype == JUBIK_F32
                ? poisson_image<float>(p->conv, lo, p->eps, p->dimg, img, p->wts,
                                       grad_x ? p->resid : nullptr, p->partials, p->counter,
                                       energy, p->pdl, s, grad_x ? p->bnd_a : nullptr)
                : poisson_image<double>(p->conv, lo, p->eps, p->dimg, img, p->wts,
                                        grad_x ? p->resid : nullptr, p->partials, p->counter,
                                        energy, p->pdl, s, grad_x ? p->bnd_a : nullptr));
  }
  p->lam_valid = true;
  if (!grad_x) return JUBIK_OK;
  JUBIK_TRY(do_adjoint(p, p->resid, grad_x, p->grad_lo, p->desc.pixel_area, s, grad_zeroed,
                       energy_partials_count()));
  Phase ph(p, 6, s);
  return finish_words(p, grad_x, p->grad_lo, (int64_t)p->g.E * p->g.pixels(), s);
}

int jubik_poisson_energy_grad_logsky(jubik_plan* p, const void* s_log, int32_t e_pad,
                                     int32_t nx_pad, int32_t ny_pad, double* energy,
                                     void* grad_s, void* stream) {
  NvtxRange nvtx_("jubik_poisson_energy_grad_logsky");
  JUBIK_TRY(check_plan(p));
  JUBIK_TRY(need(p->psf_set, "PSF"));
  JUBIK_TRY(need(p->data_set, "data"));
  const Geom& g = p->g;
  if (!s_log || !energy || e_pad < g.E || nx_pad < g.nx || ny_pad < g.ny) {
    set_error("log-sky array (%d, %d, %d) must cover the (%d, %d, %d) sky", e_pad, nx_pad,
              ny_pad, g.E, g.nx, g.ny);
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = S(stream);
  SkyView view;
  view.rs = ny_pad;
  view.ps = (int64_t)nx_pad * ny_pad;
  view.exp = true;
  bool grad_zeroed = false;
  JUBIK_TRY(do_forward(p, s_log, p->conv, p->conv_lo, p->desc.pixel_area, s,
                       grad_s ? p->xgrad : nullptr, (int64_t)g.E * g.pixels() * (int64_t)p->esz,
                       &grad_zeroed, view));
  const int64_t img = image_elems(p);
  const void* lo = p->path == JUBIK_PATH_FUSED ? p->conv_lo : nullptr;
  {
    Phase ph(p, 2, s);
    JUBIK_TRY(p->dtype == JUBIK_F32
                  ? poisson_image<float>(p->conv, lo, p->eps, p->dimg, img, p->wts,
                                         grad_s ? p->resid : nullptr, p->partials, p->counter,
                                         energy, p->pdl, s, grad_s ? p->bnd_a : nullptr)
                  : poisson_image<double>(p->conv, lo, p->eps, p->dimg, img, p->wts,
                                          grad_s ? p->resid : nullptr, p->partials,
                                          p->counter, energy, p->pdl, s,
                                          grad_s ? p->bnd_a : nullptr));
  }
  p->lam_valid = true;
  if (!grad_s) return JUBIK_OK;
  JUBIK_TRY(do_adjoint(p, p->resid, p->xgrad, p->grad_lo, p->desc.pixel_area, s, grad_zeroed,
                       energy_partials_count()));
  const void* glo = p->path == JUBIK_PATH_FUSED ? p->grad_lo : nullptr;
  const int64_t n = (int64_t)e_pad * nx_pad * ny_pad;
  if (p->dtype == JUBIK_F32)
    k_logsky_grad<float><<<blocks_for(n), 256, 0, s>>>((const float*)s_log,
                                                        (const float*)p->xgrad, (const float*)glo,
                                                        g.E, g.nx, g.ny, e_pad, nx_pad, ny_pad,
                                                        (float*)grad_s);
  else
    k_logsky_grad<double><<<blocks_for(n), 256, 0, s>>>((const double*)s_log,
                                                         (const double*)p->xgrad,
                                                         (const double*)glo, g.E, g.nx, g.ny,
                                                         e_pad, nx_pad, ny_pad, (double*)grad_s);
  return cuda_status(cudaGetLastError(), "k_logsky_grad");
}

int jubik_metric_apply(jubik_plan* p, const void* x, const void* v, void* out, void* stream) {
  NvtxRange nvtx_("jubik_metric_apply");
  JUBIK_TRY(check_plan(p));
  JUBIK_TRY(need(p->psf_set, "PSF"));
  cudaStream_t s = S(stream);
  const int64_t img = image_elems(p);
  const bool two = p->path == JUBIK_PATH_FUSED;
  if (x) {  // weights eps^2 / lam of a new lam = R(x), as the likelihood pass leaves them
    JUBIK_TRY(do_forward(p, x, p->conv, p->conv_lo, p->desc.pixel_area, s));
    JUBIK_TRY(p->dtype == JUBIK_F32
                  ? metric_weights<float>(p->conv, two ? p->conv_lo : nullptr, p->eps, p->ridx,
                                          img, p->wts, s)
                  : metric_weights<double>(p->conv, two ? p->conv_lo : nullptr, p->eps, p->ridx,
                                           img, p->wts, s));
    p->lam_valid = true;
  }
  JUBIK_TRY(need(p->lam_valid, "lambda (call with x or after poisson_energy_grad)"));
  // R v, weighted in the pass that adds its two words, then the adjoint
  bool out_zeroed = false;
  JUBIK_TRY(do_forward(p, v, p->conv_v, p->conv_v_lo, p->desc.pixel_area, s, out,
                       (int64_t)p->g.E * p->g.pixels() * (int64_t)p->esz, &out_zeroed));
  int nb = 0;
  {
    Phase ph(p, 2, s);
    JUBIK_TRY(p->dtype == JUBIK_F32
                  ? apply_weights<float>(p->conv_v, two ? p->conv_v_lo : nullptr, p->wts, img,
                                         p->resid, p->pdl, s, p->bnd_a, &nb)
                  : apply_weights<double>(p->conv_v, two ? p->conv_v_lo : nullptr, p->wts, img,
                                          p->resid, p->pdl, s, p->bnd_a, &nb));
  }
  JUBIK_TRY(do_adjoint(p, p->resid, out, p->grad_lo, p->desc.pixel_area, s, out_zeroed, nb));
  Phase ph(p, 6, s);
  return finish_words(p, out, p->grad_lo, (int64_t)p->g.E * p->g.pixels(), s);
}

int jubik_plan_set_metric_lambda(jubik_plan* p, const void* lam, int32_t lam_dtype,
                                 void* stream) {
  NvtxRange nvtx_("jubik_plan_set_metric_lambda");
  JUBIK_TRY(check_plan(p));
  if (!lam || (lam_dtype != JUBIK_F32 && lam_dtype != JUBIK_F64)) {
    set_error("set_metric_lambda: need a device lam vector of dtype JUBIK_F32 or JUBIK_F64");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = S(stream);
  const int64_t img = image_elems(p);
  JUBIK_TRY(p->dtype == JUBIK_F32
                ? weights_from_lambda<float>(lam, lam_dtype, p->eps, p->ridx, img, p->wts, s)
                : weights_from_lambda<double>(lam, lam_dtype, p->eps, p->ridx, img, p->wts, s));
  p->lam_valid = true;
  return JUBIK_OK;
}

int jubik_poisson_energy(const void* lam, const int32_t* data, int64_t n, int32_t dtype,
                         double* energy, void* grad, void* stream) {
  NvtxRange nvtx_("jubik_poisson_energy");
  if (!lam || !data || !energy || n < 0) {
    set_error("invalid argument");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = S(stream);
  const int nb = energy_partials_count();
  double* partials = nullptr;
  unsigned int* counter = nullptr;
  JUBIK_TRY_CUDA(cudaMallocAsync((void**)&partials, 2 * nb * sizeof(double), s));
  JUBIK_TRY_CUDA(cudaMallocAsync((void**)&counter, sizeof(unsigned int), s));
  JUBIK_TRY_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned int), s));
  int st = dtype == JUBIK_F32 ? poisson_vec<float>(lam, data, n, partials, counter, energy, grad, s)
                              : poisson_vec<double>(lam, data, n, partials, counter, energy, grad,
                                                    s);
  cudaFreeAsync(partials, s);
  cudaFreeAsync(counter, s);
  return st;
}

int jubik_elementwise(int32_t op, const void* a, const void* b, const int32_t* data, int64_t n,
                      int32_t dtype, void* out, void* stream) {
  if (op < 0 || op > 3 || !a || !out || (op != 2 && !b) || (op == 2 && !data)) {
    set_error("invalid elementwise arguments");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  return dtype == JUBIK_F32 ? elementwise_op<float>(op, a, b, data, n, out, S(stream))
                            : elementwise_op<double>(op, a, b, data, n, out, S(stream));
}

int jubik_readout_gather(const void* img, const void* eps, const int64_t* idx, int64_t nread,
                         int32_t dtype, void* out, void* stream) {
  return dtype == JUBIK_F32 ? readout_gather<float>(img, eps, idx, nread, out, S(stream))
                            : readout_gather<double>(img, eps, idx, nread, out, S(stream));
}

int jubik_readout_scatter(const void* vec, const void* eps, const int64_t* idx, int64_t nread,
                          int32_t dtype, void* img, void* stream) {
  return dtype == JUBIK_F32 ? readout_scatter<float>(vec, eps, idx, nread, img, S(stream))
                            : readout_scatter<double>(vec, eps, idx, nread, img, S(stream));
}

int jubik_slice_patches(const void* x, int64_t batch, int32_t nx, int32_t ny, int32_t n,
                        int32_t additional_margin, int32_t dtype, void* out, void* stream) {
  return dtype == JUBIK_F32
             ? slice_patches_op<float>(x, batch, nx, ny, n, additional_margin, out, S(stream))
             : slice_patches_op<double>(x, batch, nx, ny, n, additional_margin, out, S(stream));
}

int jubik_slice_patches_adjoint(const void* patches, int64_t batch, int32_t nx, int32_t ny,
                                int32_t n, int32_t additional_margin, int32_t dtype, void* out,
                                void* stream) {
  return dtype == JUBIK_F32 ? slice_patches_adjoint_op<float>(patches, batch, nx, ny, n,
                                                              additional_margin, out, S(stream))
                            : slice_patches_adjoint_op<double>(patches, batch, nx, ny, n,
                                                               additional_margin, out, S(stream));
}

int jubik_convolve2d(const void* kernel, int64_t bk, const void* signal, int64_t bs, int32_t h,
                     int32_t w, double dvol, int32_t dtype, void* out, void* stream) {
  NvtxRange nvtx_("jubik_convolve2d");
  if (!kernel || !signal || !out || bk < 1 || bs < 1 || h < 1 || w < 1 || bs % bk != 0) {
    set_error("convolve2d: invalid shapes (kernel batch must divide the signal batch)");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (dtype != JUBIK_F32 && dtype != JUBIK_F64) {
    set_error("convolve2d: dtype must be JUBIK_F32 or JUBIK_F64");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = S(stream);
  Fft1D fh, fw;
  JUBIK_TRY(fft1d_init(&fh, h));
  int st = fft1d_init(&fw, w);
  if (st) {
    fft1d_free(&fh);
    return st;
  }
  const size_t csz = dtype == JUBIK_F32 ? 8 : 16;
  const int64_t hw = (int64_t)h * w;
  void* zk = nullptr;
  void* zs = nullptr;
  st = cuda_status(cudaMallocAsync(&zk, csz * bk * hw, s), "cudaMallocAsync");
  if (!st) st = cuda_status(cudaMallocAsync(&zs, csz * bs * hw, s), "cudaMallocAsync");
  if (!st)
    st = dtype == JUBIK_F32 ? convolve2d_run<float>(kernel, bk, signal, bs, hw, dvol, fh, fw, zk, zs, out, s)
                            : convolve2d_run<double>(kernel, bk, signal, bs, hw, dvol, fh, fw, zk, zs, out, s);
  if (zk) cudaFreeAsync(zk, s);
  if (zs) cudaFreeAsync(zs, s);
  cudaStreamSynchronize(s);
  fft1d_free(&fh);
  fft1d_free(&fw);
  return st;
}

}  // extern "C"

// ---------------------------------------------------------------- groups
// Independent problems evaluated together: per FFT side one grouped launch of
// each per-unit stage, one grouped likelihood pass and one grouped clearing
// kernel, instead of a launch sequence per problem.
struct GroupClass {
  int P = 0;
  bool shared = false;       // module-shared plans: 4 launches per pass, else 2
  std::vector<int> members;  // indices into the group's plans
  int64_t blocks = 0;        // units of all members
  int64_t items = 0;         // (energy, patch) items of all members (shared)
  void* fwd_list = nullptr;  // device Args per member: forward stages
  void* adj_list = nullptr;  // device Args per member: adjoint stages
  int* starts = nullptr;     // device: first unit of each member, then the total
  int* item_starts = nullptr;  // device: first item of each member, then the total
  int* ord_starts = nullptr;   // device (shared): first CTA of each member's ordered adjoint
  int64_t ord_blocks = 0;      // CTAs of the ordered adjoint over all members
};

struct jubik_group {
  std::vector<jubik_plan*> plans;
  std::vector<uint64_t> gens;  // each plan's layout_gen when set_io copied its buffers
  int dtype = JUBIK_F32;
  std::vector<GroupClass> classes;
  PoissonJob* pjobs = nullptr;
  int* pstarts = nullptr;
  int64_t pblocks = 0;
  ZeroJob* zjobs = nullptr;
  int* zstarts = nullptr;
  int64_t zblocks = 0;
  int nzero = 0;
  // exact two-word sums: one forward-bound slot per problem (the largest |sky|),
  // the grouped maxima pass that fills them, and the final hi + lo pass
  unsigned long long* bslots = nullptr;
  AbsmaxJob* ajobs = nullptr;
  int* astarts = nullptr;
  int64_t ablocks = 0;
  CombineJob* cjobs = nullptr;
  int* cstarts = nullptr;
  int64_t cblocks = 0;
  bool io_set = false;
  std::vector<void*> allocs;
  int alloc(void** p, size_t n) {
    JUBIK_TRY_CUDA(cudaMalloc(p, n));
    allocs.push_back(*p);
    return JUBIK_OK;
  }
  void free_io() {
    for (void* p : allocs) cudaFree(p);
    allocs.clear();
    for (auto& c : classes) {
      c.fwd_list = c.adj_list = nullptr;
      c.starts = c.item_starts = c.ord_starts = nullptr;
    }
    pjobs = nullptr;
    zjobs = nullptr;
    pstarts = zstarts = astarts = cstarts = nullptr;
    bslots = nullptr;
    ajobs = nullptr;
    cjobs = nullptr;
    io_set = false;
  }
  ~jubik_group() { free_io(); }
};

namespace {
template <typename V>
int upload(jubik_group* g, const std::vector<V>& host, V** dev) {
  JUBIK_TRY(g->alloc((void**)dev, sizeof(V) * std::max<size_t>(1, host.size())));
  return cuda_status(cudaMemcpy(*dev, host.data(), sizeof(V) * host.size(),
                                cudaMemcpyHostToDevice),
                     "group upload");
}
}  // namespace

extern "C" {

int jubik_group_create(jubik_plan* const* plans, int32_t n, jubik_group** out) {
  if (!plans || n < 1 || !out) {
    set_error("group: need at least one plan");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  auto* g = new (std::nothrow) jubik_group();
  if (!g) {
    set_error("group: out of host memory");
    return JUBIK_ERR_ALLOC;
  }
  for (int i = 0; i < n; ++i) {
    jubik_plan* p = plans[i];
    int st = JUBIK_OK;
    if (!p) {
      set_error("group: plan %d is NULL", i);
      st = JUBIK_ERR_INVALID_ARGUMENT;
    } else if (p->path != JUBIK_PATH_FUSED) {
      set_error("group: plan %d does not run the fused kernels (its FFT side or dtype takes the "
                "unfused path)", i);
      st = JUBIK_ERR_UNSUPPORTED;
    } else if (i > 0 && p->dtype != plans[0]->dtype) {
      set_error("group: plans of different dtypes");
      st = JUBIK_ERR_INVALID_ARGUMENT;
    } else if (!p->psf_set || !p->data_set) {
      set_error("group: plan %d needs its PSF and data set", i);
      st = JUBIK_ERR_STATE;
    }
    if (st) {
      delete g;
      return st;
    }
    g->plans.push_back(p);
  }
  g->dtype = plans[0]->dtype;
  for (int i = 0; i < n; ++i) {
    const int P = g->plans[i]->g.P;
    const bool shared = g->plans[i]->spec != nullptr;
    auto it = std::find_if(g->classes.begin(), g->classes.end(), [&](const GroupClass& c) {
      return c.P == P && c.shared == shared;
    });
    if (it == g->classes.end()) {
      g->classes.emplace_back();
      g->classes.back().P = P;
      g->classes.back().shared = shared;
      it = g->classes.end() - 1;
    }
    it->members.push_back(i);
  }
  *out = g;
  return JUBIK_OK;
}

int jubik_group_set_io(jubik_group* g, const void* const* x, void* const* grad,
                       double* energies) {
  if (!g || !x || !grad || !energies) {
    set_error("group: invalid arguments");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  const int n = (int)g->plans.size();
  for (int i = 0; i < n; ++i) {
    if (!x[i] || !grad[i]) {
      set_error("group: problem %d has no sky or gradient buffer", i);
      return JUBIK_ERR_INVALID_ARGUMENT;
    }
  }
  g->free_io();
  const size_t asz = fused_args_size();
  // forward-bound slots, one per problem (16-byte multiple for the clearing pass)
  const int64_t slot_bytes = ((int64_t)n * 8 + 15) & ~(int64_t)15;
  JUBIK_TRY(g->alloc((void**)&g->bslots, slot_bytes));
  for (auto& c : g->classes) {
    std::vector<unsigned char> fwd(asz * c.members.size()), adj(asz * c.members.size());
    std::vector<int> starts, item_starts, ord_starts;
    int64_t b = 0, items = 0, ob = 0;
    // module-shared classes: each problem's ordered adjoint gets CTAs in
    // proportion to its units (at most its spill slots), about as many in all as
    // the GPU holds at once
    int64_t per_cta = 1;
    auto ord_ctas = [&](int i) {
      const jubik_plan* p = g->plans[i];
      return std::max<int64_t>(
          1, std::min<int64_t>(p->adj_grid, (p->g.units() + per_cta - 1) / per_cta));
    };
    if (c.shared) {
      int64_t total = 0;
      for (int i : c.members) total += g->plans[i]->g.units();
      const int64_t cap = std::max<int64_t>(1, fused_ord_capacity(c.P, g->dtype));
      per_cta = std::max<int64_t>(1, (total + cap - 1) / cap);
      // all ranges in one wave: a CTA that waits for a free SM doubles the critical path
      for (;;) {
        int64_t ctas = 0;
        for (int i : c.members) ctas += ord_ctas(i);
        if (ctas <= cap || ctas <= (int64_t)c.members.size()) break;
        ++per_cta;
      }
    }
    for (size_t k = 0; k < c.members.size(); ++k) {
      const int i = c.members[k];
      jubik_plan* p = g->plans[i];
      const Geom& pg = p->g;
      starts.push_back((int)b);
      item_starts.push_back((int)items);
      b += pg.units();
      items += (int64_t)pg.E * pg.n * pg.n;
      const double area = std::fabs(p->desc.pixel_area);
      // forward: overlap-add exact in two words, bounded by the problem's largest |sky|
      FusedLaunch f{x[i], p->conv, p->hmain, p->hnyq, p->tw, p->wt, p->desc.pixel_area,
                    c.shared ? p->spec : nullptr};
      f.clear = false;
      f.out_lo = p->conv_lo;
      f.bnd_in = g->bslots + i;
      f.bnd_n = 1;
      f.bnd_log2 = fwd_terms_log2(pg);
      f.bnd_scale = 2.0 * (double)(int64_t(1) << f.bnd_log2) * p->kmax * area;
      fused_args_fill(pg, p->dtype, f, c.shared ? FUSED_FWD_SKY : FUSED_FWD_UNITS,
                      fwd.data() + k * asz);
      // adjoint: gradient exact in two words, bounded by the residual's block maxima
      // that the grouped likelihood pass leaves in the plan's bnd_a
      FusedLaunch r{p->resid, grad[i], p->hmain, p->hnyq, p->tw, p->wt, p->desc.pixel_area,
                    c.shared ? p->acc : nullptr};
      r.zero_out = false;
      r.clear = false;
      r.out_lo = p->grad_lo;
      r.bnd_in = p->bnd_a;
      r.bnd_n = poisson_group_blocks(image_elems(p));
      r.bnd_log2 = adj_terms_log2(pg);
      r.bnd_scale = 2.0 * (double)(int64_t(1) << r.bnd_log2) * p->kmax * area;
      if (c.shared) {  // module sums in module order (ordered adjoint, spill slots)
        const int64_t G = ord_ctas(i);
        ord_starts.push_back((int)ob);
        ob += G;
        r.spill = p->spill;
        r.loop_grid = G;
      }
      fused_args_fill(pg, p->dtype, r, c.shared ? FUSED_ADJ_TO_SPEC : FUSED_ADJ_UNITS,
                      adj.data() + k * asz);
    }
    if (b > 0x7fffffffLL) {
      set_error("group: too many patch units");
      return JUBIK_ERR_UNSUPPORTED;
    }
    starts.push_back((int)b);
    item_starts.push_back((int)items);
    c.blocks = b;
    c.items = items;
    JUBIK_TRY(upload(g, fwd, (unsigned char**)&c.fwd_list));
    JUBIK_TRY(upload(g, adj, (unsigned char**)&c.adj_list));
    JUBIK_TRY(upload(g, starts, &c.starts));
    if (c.shared) {
      ord_starts.push_back((int)ob);
      c.ord_blocks = ob;
      JUBIK_TRY(upload(g, item_starts, &c.item_starts));
      JUBIK_TRY(upload(g, ord_starts, &c.ord_starts));
    }
  }
  std::vector<PoissonJob> pj;
  std::vector<ZeroJob> zj;
  std::vector<AbsmaxJob> aj;
  std::vector<CombineJob> cj;
  std::vector<int> ps, zs, as, cs;
  int64_t pb = 0, zb = 0, ab = 0, cb = 0;
  auto add_zero = [&](void* ptr, int64_t bytes) {
    zj.push_back(ZeroJob{ptr, bytes});
    zs.push_back((int)zb);
    zb += std::max<int64_t>(1, std::min<int64_t>(1024, bytes / (256 * 16 * 8)));
  };
  add_zero(g->bslots, slot_bytes);
  for (int i = 0; i < n; ++i) {
    jubik_plan* p = g->plans[i];
    const int64_t img = image_elems(p);
    const int64_t sky = (int64_t)p->g.E * p->g.pixels();
    pj.push_back(PoissonJob{p->conv, p->conv_lo, p->eps, p->dimg, img, p->wts, p->resid,
                            p->partials, p->counter, energies + i,
                            (unsigned long long*)p->bnd_a});
    ps.push_back((int)pb);
    pb += poisson_group_blocks(img);
    aj.push_back(AbsmaxJob{x[i], sky, g->bslots + i});
    as.push_back((int)ab);
    ab += group_blocks(sky);
    cj.push_back(CombineJob{grad[i], p->grad_lo, sky});
    cs.push_back((int)cb);
    cb += group_blocks(sky);
    // both words of each problem's image and gradient start from zero (the
    // module sums of the ordered adjoint are written whole)
    add_zero(p->conv, img * (int64_t)p->esz);
    add_zero(p->conv_lo, img * (int64_t)p->esz);
    add_zero(grad[i], sky * (int64_t)p->esz);
    add_zero(p->grad_lo, sky * (int64_t)p->esz);
  }
  ps.push_back((int)pb);
  zs.push_back((int)zb);
  as.push_back((int)ab);
  cs.push_back((int)cb);
  g->pblocks = pb;
  g->zblocks = zb;
  g->ablocks = ab;
  g->cblocks = cb;
  g->nzero = (int)zj.size();
  JUBIK_TRY(upload(g, pj, &g->pjobs));
  JUBIK_TRY(upload(g, ps, &g->pstarts));
  JUBIK_TRY(upload(g, zj, &g->zjobs));
  JUBIK_TRY(upload(g, zs, &g->zstarts));
  JUBIK_TRY(upload(g, aj, &g->ajobs));
  JUBIK_TRY(upload(g, as, &g->astarts));
  JUBIK_TRY(upload(g, cj, &g->cjobs));
  JUBIK_TRY(upload(g, cs, &g->cstarts));
  g->gens.clear();
  for (jubik_plan* p : g->plans) g->gens.push_back(p->layout_gen);
  g->io_set = true;
  return JUBIK_OK;
}

int jubik_group_energy_grad(jubik_group* g, void* stream) {
  NvtxRange nvtx_("jubik_group_energy_grad");
  if (!g || !g->io_set) {
    set_error("group: set the sky, gradient and energy buffers first");
    return JUBIK_ERR_STATE;
  }
  cudaStream_t s = S(stream);
  const int n = (int)g->plans.size();
  for (int i = 0; i < n; ++i) {
    const jubik_plan* p = g->plans[i];
    if (p->layout_gen != g->gens[i] || !p->data_set) {
      set_error("group: plan %d changed its exposure, readout or data buffers since "
                "jubik_group_set_io (or has no data); call jubik_group_set_io again", i);
      return JUBIK_ERR_STATE;
    }
  }
  JUBIK_TRY(zero_group_run(g->zjobs, g->zstarts, g->nzero, g->zblocks, true, s));
  JUBIK_TRY(absmax_group_run(g->dtype, g->ajobs, g->astarts, n, g->ablocks, true, s));
  for (auto& c : g->classes) {
    const int m = (int)c.members.size();
    if (c.shared) {
      JUBIK_TRY(fused_group_shared_run(c.P, g->dtype, c.fwd_list, c.item_starts, m, c.items,
                                       FUSED_FWD_SKY, true, s));
      JUBIK_TRY(fused_group_shared_run(c.P, g->dtype, c.fwd_list, c.starts, m, c.blocks,
                                       FUSED_FWD_FROM_SPEC, true, s));
    } else {
      JUBIK_TRY(fused_group_run(c.P, g->dtype, c.fwd_list, c.starts, m, c.blocks, false, true,
                                s));
    }
  }
  JUBIK_TRY(poisson_group_run(g->dtype, g->pjobs, g->pstarts, n, g->pblocks, true, s));
  for (auto& c : g->classes) {
    const int m = (int)c.members.size();
    if (c.shared) {
      JUBIK_TRY(fused_group_shared_run(c.P, g->dtype, c.adj_list, c.ord_starts, m, c.ord_blocks,
                                       FUSED_ADJ_TO_SPEC, true, s));
      JUBIK_TRY(fused_group_shared_run(c.P, g->dtype, c.adj_list, c.item_starts, m, c.items,
                                       FUSED_ADJ_FROM_SPEC, true, s));
    } else {
      JUBIK_TRY(fused_group_run(c.P, g->dtype, c.adj_list, c.starts, m, c.blocks, true, true,
                                s));
    }
  }
  JUBIK_TRY(combine_group_run(g->dtype, g->cjobs, g->cstarts, n, g->cblocks, true, s));
  for (jubik_plan* p : g->plans) p->lam_valid = true;
  return JUBIK_OK;
}

int jubik_group_launches(const jubik_group* g, int32_t* launches) {
  if (!g || !launches) {
    set_error("group: invalid arguments");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  int32_t k = 4;  // clearing, sky maxima, likelihood, combine
  for (const auto& c : g->classes) k += c.shared ? 4 : 2;
  *launches = k;
  return JUBIK_OK;
}

int jubik_group_destroy(jubik_group* g) {
  if (g) delete g;
  return JUBIK_OK;
}

}  // extern "C"
