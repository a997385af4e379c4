// Internal declarations shared by the translation units of libjubik_gb300.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "jubik_gb300.h"

namespace jubik {

// ------------------------------------------------------------------ errors
void set_error(const char* fmt, ...);
int cuda_status(cudaError_t err, const char* what);

#define JUBIK_TRY_CUDA(expr)                                   \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if (_e != cudaSuccess) return ::jubik::cuda_status(_e, #expr); \
  } while (0)

#define JUBIK_TRY(expr)              \
  do {                               \
    int _s = (expr);                 \
    if (_s != JUBIK_OK) return _s;   \
  } while (0)

// Streaming multiprocessors of the current device (cached per device).
int sm_count();

// ------------------------------------------------------------------ geometry
// Patch geometry of jubik/convolve.py:43-63 / :102-143 (square patches).
struct Geom {
  int M = 0, E = 0, nx = 0, ny = 0, n = 0;
  int dx = 0, margin = 0, half = 0;  // half = dx // 2 (the slice pad)
  int K = 0, P = 0;                  // window 2*dx, FFT side 2*dx + 2*margin
  int sr_max = 0, sc_max = 0;        // clamp of dynamic_slice starts
  int64_t units() const { return (int64_t)M * E * n * n; }
  int64_t pixels() const { return (int64_t)nx * ny; }
};
// unfused path: real patches are transformed two per complex array
inline int64_t plain_pairs(const Geom& g) { return ((int64_t)g.E * g.n * g.n + 1) / 2; }

// Multiply-high constant for dividing numerators 0 <= u < bound by d on the
// device: floor(u / d) = high word of u * (floor(2^32 / d) + 1), exact while
// u d < 2^32 (the product exceeds u / d by less than 1 / d).  0 when d < 2 or
// the bound is too large: the kernel then divides.
inline uint32_t mulhi_divisor(int64_t d, int64_t bound) {
  if (d < 2 || bound <= 0 || bound * d >= (int64_t(1) << 32)) return 0;
  return (uint32_t)((uint64_t(1) << 32) / (uint64_t)d + 1);
}


// ------------------------------------------------------------------ plain FFT
constexpr int kMaxStages = 24;
constexpr int kMaxGenericRadix = 64;
struct FftStages {
  int n = 0;
  int r[kMaxStages] = {0};
};

// Mixed-radix Stockham plan for complex length-L transforms.  Twiddles
// w_L^t = exp(-2 pi i t / L) are evaluated once in long double on the host
// and rounded once to each precision.
struct Fft1D {
  int L = 0;
  FftStages st;
  void* tw32 = nullptr;  // float2[L]
  void* tw64 = nullptr;  // double2[L]
};
int fft1d_init(Fft1D* f, int L);
void fft1d_free(Fft1D* f);
// Fills f for length L with twiddle tables in caller-provided device memory
// (L float2 at tw32, L double2 at tw64) computed on the device: no allocation.
int fft1d_init_external(Fft1D* f, int L, void* tw32, void* tw64, cudaStream_t s);
bool fft_length_supported(int L);

// In-place batched complex FFT of nseq sequences of length f.L; sequence q
// starts at (q / nb) * sa + (q % nb) * sb, element i at + i * se (elements).
template <typename T>
int fft_batched(const Fft1D& f, void* data, int64_t nseq, int nb, int64_t sa, int64_t sb,
                int64_t se, bool inverse, double scale, cudaStream_t s);

// 2-D FFT over the last two axes of a (batch, h, w) complex array.
template <typename T>
int fft2_batched(const Fft1D& fh, const Fft1D& fw, void* data, int64_t batch, bool inverse,
                 cudaStream_t s);

// Forward row pass of the unfused path reading its rows from the images: pair
// j's row y holds row y of patch 2j's and 2j+1's P x P windows (real and
// imaginary parts), zero outside the field.  module_axis: img is (M, E, nx, ny)
// and the nm modules from m0 are transformed; else img is (E, nx, ny) (nm = 1).
// wt != nullptr applies the sky's window weights.  out: (nm, pairs, P, P).
// FFT sides P = 16 L1 with L1 in {10, 12, 16, 20, 24, 32}.
template <typename T>
int fft_rows_windows(const Fft1D& f, const Geom& g, const void* img, bool module_axis,
                     const void* wt, int m0, int nm, void* out, cudaStream_t s);

// ------------------------------------------------------------------ fused path
bool fused_supported(int P, int dtype);
size_t fused_smem_bytes(int P, int dtype);
struct FusedLaunch {
  const void* in;       // forward: sky (E,nx,ny); adjoint: cotangent (M,E,nx,ny)
  void* out;            // forward: (M,E,nx,ny) accumulator; adjoint: (E,nx,ny)
  const void* hmain;    // (units, P, P/2) complex, rows in 4-step order
  const void* hnyq;     // (units, P) complex: the kx = P/2 column
  const void* tw;       // (P) complex twiddles
  const void* wt;       // (2*dx) bilinear weight vector
  double scale;
  void* spec = nullptr; // (E n^2, P, P/2) shared spectra: module-shared kernels when set
  void* aux = nullptr;  // module-shared forward: a further buffer the sky-spectrum kernel clears
  int64_t aux_bytes = 0;
  bool zero_out = true; // module-shared adjoint: the per-unit kernel clears `out` first
  bool pdl = true;      // launch with programmatic stream serialisation
  // forward input as a crop of a larger (E', N0', N1') array: row and plane
  // strides (0 = the field's own), and whether it holds log-sky values
  int64_t in_rs = 0, in_ps = 0;
  bool in_exp = false;
  bool clear = true;    // false: the kernels clear nothing (grouped launches clear first)
  // One-problem launches accumulate their output exactly in two words: `out`
  // and its low-word plane out_lo (same layout).  The terms are bounded by
  // bnd_scale * the largest of the bnd_n magnitude maxima at bnd_in (device
  // doubles' bits), at most 2^bnd_log2 terms per element.  bnd_out receives
  // the maxima a kernel records (sky spectra: one per (energy, patch); ordered
  // adjoint: one per CTA).
  void* out_lo = nullptr;
  const void* bnd_in = nullptr;
  int bnd_n = 0, bnd_log2 = 0;
  double bnd_scale = 0.0;
  void* bnd_out = nullptr;
  // ordered module-shared adjoint: spill slots (loop_grid x P x P/2 complex)
  // and its grid (fused_adj_grid)
  void* spill = nullptr;
  int64_t loop_grid = 0;
  // module-shared forward: patches per run of the run-ordered kernel (0: the
  // library's choice, 1: one unit at a time; see fused_fwd_run_len)
  int fwd_run = 0;
};
// CTAs of the ordered module-shared adjoint for geometry g (0 where the fused
// path does not cover g.P): the count of its unit ranges and spill slots.
int64_t fused_adj_grid(const Geom& g, int dtype);
// Run length of the module-shared forward for a request (0 = the library's
// choice): 1, 2 or 4, or -1 where geometry g cannot take the request.
int fused_fwd_run_len(const Geom& g, int dtype, int requested);
// CTAs of the ordered module-shared adjoint at FFT side P that fit on the GPU
// at once (0 where the fused path does not cover P).
int64_t fused_ord_capacity(int P, int dtype);
size_t fused_spec_bytes(const Geom& g, int dtype);
// Grouped per-unit launches over independent problems of one FFT side: the
// kernel-argument block of one problem's stage (fused_args_size() bytes,
// written by fused_args_fill), and one launch of FUSED_FWD_UNITS (adj false)
// or FUSED_ADJ_UNITS (adj true) over nprob problems, problem p owning blocks
// [starts[p], starts[p + 1]) of `blocks` (list and starts in device memory).
// Grouped likelihood pass and grouped clearing over independent problems.
struct PoissonJob {
  const void* conv;
  const void* conv_lo;  // low words of the exact overlap-add (the image is conv + conv_lo)
  const void* eps;
  const int32_t* dimg;
  int64_t npix;
  void* wts;  // metric weights eps^2 / lam (image space)
  void* resid;
  double* partials;
  unsigned int* counter;
  double* energy;
  unsigned long long* rmax;  // per-block maxima of |resid| (the adjoint's bound), or nullptr
};
struct ZeroJob {
  void* ptr;
  int64_t bytes;
};
// Grouped maxima of |in[0 .. n)| into one slot per job (atomicMax of the bits).
struct AbsmaxJob {
  const void* in;
  int64_t n;
  unsigned long long* slot;
};
// Grouped two-word combine: hi[i] += lo[i], i < n.
struct CombineJob {
  void* hi;
  const void* lo;
  int64_t n;
};
// Blocks of one job of the grouped maxima and combine passes (<= 1024).
int group_blocks(int64_t n);
int absmax_group_run(int dtype, const AbsmaxJob* jobs, const int* starts, int njobs,
                     int64_t blocks, bool pdl, cudaStream_t s);
int combine_group_run(int dtype, const CombineJob* jobs, const int* starts, int njobs,
                      int64_t blocks, bool pdl, cudaStream_t s);
int poisson_group_blocks(int64_t npix);
int poisson_group_run(int dtype, const PoissonJob* jobs, const int* starts, int njobs,
                      int64_t blocks, bool pdl, cudaStream_t s);
int zero_group_run(const ZeroJob* jobs, const int* starts, int njobs, int64_t blocks, bool pdl,
                   cudaStream_t s);
size_t fused_args_size();
void fused_args_fill(const Geom& g, int dtype, const FusedLaunch& f, int which, void* dst);
// One module-shared stage (FUSED_FWD_SKY, FUSED_FWD_FROM_SPEC, FUSED_ADJ_TO_SPEC,
// FUSED_ADJ_FROM_SPEC) over nprob problems of FFT side P: starts (device, nprob + 1)
// index the (energy, patch) items of the per-patch stages or the units of the
// per-unit stages, count of them in all.
int fused_group_shared_run(int P, int dtype, const void* list, const int* starts, int nprob,
                           int64_t count, int which, bool pdl, cudaStream_t s);
int fused_group_run(int P, int dtype, const void* list, const int* starts, int nprob,
                    int64_t blocks, bool adj, bool pdl, cudaStream_t s);
enum FusedStage {
  FUSED_FWD_UNITS = 0,     // one kernel per unit, forward
  FUSED_ADJ_UNITS = 1,     // one kernel per unit, adjoint
  FUSED_FWD_SKY = 2,       // per (energy, patch): sky spectrum -> spec
  FUSED_FWD_FROM_SPEC = 3, // per unit: spec * H -> inverse -> overlap-add
  FUSED_ADJ_TO_SPEC = 4,   // per unit: cotangent spectrum * conj(H) -> spec (sum)
  FUSED_ADJ_FROM_SPEC = 5  // per (energy, patch): spec -> inverse -> gradient
};
int fused_run(const Geom& g, int dtype, const FusedLaunch& a, int which, cudaStream_t s);

// ------------------------------------------------------------------ ops
template <typename T>
int psf_to_cplx(const Geom& g, const void* psf, int layout, int e_broadcast, int64_t u0,
                int64_t nu, double* sums, void* buf, cudaStream_t s);
template <typename T>
int spectra_store(const Geom& g, const void* buf, int64_t u0, int64_t nu, void* hfull,
                  void* hmain, void* hnyq, cudaStream_t s);
template <typename T>
int plain_sky_patches(const Geom& g, const void* x, const void* wt, void* zs, cudaStream_t s);
template <typename T>
int plain_mul_modules(const Geom& g, const void* zs, const void* hfull, int m0, int nm, void* zu,
                      cudaStream_t s);
template <typename T>
int plain_overlap_gather(const Geom& g, const void* zu, int m0, int nm, double scale, void* out,
                         cudaStream_t s);
template <typename T>
int plain_cot_patches(const Geom& g, const void* cot, int m0, int nm, void* zu, cudaStream_t s);
template <typename T>
int plain_mulconj_accum(const Geom& g, const void* zu, const void* hfull, int m0, int nm,
                        bool first, void* zs, cudaStream_t s);
template <typename T>
int plain_grad_gather(const Geom& g, const void* zs, const void* wt, double scale, void* out,
                      cudaStream_t s);

// Column stage of the unfused path fused with the PSF product (plain_cols.cu),
// for FFT sides P = 16 L1 with L1 in {10, 12, 16, 20, 24, 32}.  Forward: zs
// holds the row-transformed sky pairs; zu gets, per module of the chunk
// [m0, m0 + nm), the products with their columns transformed back (the inverse
// row pass follows).  Adjoint: zu holds the chunk's row-transformed cotangent
// pairs; zs gets their conjugate-PSF products summed over modules, added to
// the sum of earlier chunks (first: none) and transformed back (last).
bool plain_cols_supported(int P);
template <typename T>
int plain_cols_forward(const Geom& g, const void* zs, const void* hfull, const void* tw, int m0,
                       int nm, void* zu, cudaStream_t s);
template <typename T>
int plain_cols_adjoint(const Geom& g, const void* zu, const void* hfull, const void* tw, int m0,
                       int nm, bool first, bool last, void* zs, cudaStream_t s);

template <typename T>
int slice_patches_op(const void* x, int64_t batch, int nx, int ny, int n, int dr, void* out,
                     cudaStream_t s);
template <typename T>
int slice_patches_adjoint_op(const void* patches, int64_t batch, int nx, int ny, int n, int dr,
                             void* out, cudaStream_t s);

// response epilogues / prologues over the (M,E,nx,ny) image
template <typename T>
int readout_gather(const void* img, const void* eps, const int64_t* idx, int64_t nread,
                   void* out, cudaStream_t s, const void* img_lo = nullptr);
template <typename T>
int readout_scatter(const void* vec, const void* eps, const int64_t* idx, int64_t nread,
                    void* img, cudaStream_t s);
// (rmax: energy_partials_count() block maxima of |resid|, the bound of an
// adjoint of resid, or nullptr)
template <typename T>
int poisson_image(const void* conv, const void* conv_lo, const void* eps, const int32_t* dimg,
                  int64_t npix, void* wts, void* resid, double* partials,
                  unsigned int* counter, double* energy, bool pdl, cudaStream_t s,
                  void* rmax = nullptr);
// Largest magnitude of an (E, rows, cols) array with plane stride ps and row
// stride rs (of exp(value) when exp_of), as nb <= kMaxBoundBlocks maxima
// (bits of non-negative doubles) at out; returns nb.
constexpr int kMaxBoundBlocks = 1024;
template <typename T>
int absmax_blocks(const void* in, int E, int rows, int cols, int64_t ps, int64_t rs, bool exp_of,
                  void* out, int* nb, bool pdl, cudaStream_t s);
// hi[i] += lo[i] for n elements: the value of a two-word accumulation
template <typename T>
int combine_words(void* hi, const void* lo, int64_t n, bool pdl, cudaStream_t s);
int count_image(const int32_t* ridx, const int32_t* data, int64_t npix, int32_t* dimg,
                cudaStream_t s);
// wts = eps^2 / lam with lam = eps * conv (conv_lo: the low words of a
// two-word conv, or nullptr) at read-out pixels (ridx >= 0), 0 elsewhere
template <typename T>
int metric_weights(const void* conv, const void* conv_lo, const void* eps, const int32_t* ridx,
                   int64_t npix, void* wts, cudaStream_t s);
// The same from a caller's lam in readout order (lam_dtype JUBIK_F32 or
// JUBIK_F64): w = eps^2 / lam formed in FP64, rounded once to T.
template <typename T>
int weights_from_lambda(const void* lam, int lam_dtype, const void* eps, const int32_t* ridx,
                        int64_t npix, void* wts, cudaStream_t s);
// out = w * (hi + lo) (lo nullptr: w * hi), n elements; *nb block maxima of
// |out| at rmax (nullptr: none)
template <typename T>
int apply_weights(const void* hi, const void* lo, const void* w, int64_t n, void* out, bool pdl,
                  cudaStream_t s, void* rmax = nullptr, int* nb = nullptr);
template <typename T>
int poisson_vec(const void* lam, const int32_t* data, int64_t n, double* partials,
                unsigned int* counter, double* energy, void* grad, cudaStream_t s);
template <typename T>
int elementwise_op(int op, const void* a, const void* b, const int32_t* d, int64_t n, void* out,
                   cudaStream_t s);
int energy_partials_count();

// out (bs,h,w) = dvol * Re(ifft2(fft2(kernel) * fft2(signal))) with complex work
// buffers zk (bk*h*w) and zs (bs*h*w) supplied by the caller.
template <typename T>
int convolve2d_run(const void* kernel, int64_t bk, const void* signal, int64_t bs, int64_t hw,
                   double dvol, const Fft1D& fh, const Fft1D& fw, void* zk, void* zs, void* out,
                   cudaStream_t s);

}  // namespace jubik
