/*
 * jubik_gb300.h -- C ABI of the GB300 (sm_103a) implementation of J-UBIK's
 * spatially-variant instrument response and its Poisson likelihood.
 *
 * Conventions
 *  - Every function returns an int status: JUBIK_OK (0) or a negative code;
 *    jubik_last_error() gives a message for the calling thread.  Nothing
 *    aborts or throws across this boundary.
 *  - Array arguments are DEVICE pointers owned by the caller, C-contiguous,
 *    of the plan's dtype (float or double) unless stated otherwise.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default).
 *  - A plan owns its device workspace; calls on one plan must not overlap
 *    (the plan is not thread-safe across concurrent calls).
 *  - Shapes: M telescope modules, E energy bins, field nx x ny, n patches
 *    per axis (stride dx = nx / n), margin m; window K = 2 dx; FFT side
 *    P = K + 2 m (jubik/convolve.py:43-44, :87-101).
 */
#ifndef JUBIK_GB300_H
#define JUBIK_GB300_H

#include <stdint.h>

#if defined(__GNUC__)
#define JUBIK_API __attribute__((visibility("default")))
#else
#define JUBIK_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define JUBIK_ABI_VERSION 1

enum jubik_status {
  JUBIK_OK = 0,
  JUBIK_ERR_INVALID_ARGUMENT = -1, /* the reference raises ValueError here */
  JUBIK_ERR_UNSUPPORTED = -2,      /* shape outside what the kernels cover */
  JUBIK_ERR_CUDA = -3,
  JUBIK_ERR_ALLOC = -4,
  JUBIK_ERR_STATE = -5 /* e.g. PSF / exposure / data not set yet */
};

enum jubik_dtype { JUBIK_F32 = 0, JUBIK_F64 = 1 };

enum jubik_path {
  JUBIK_PATH_AUTO = 0,  /* fused when the FFT side and dtype allow it */
  JUBIK_PATH_FUSED = 1, /* one kernel per patch unit: FFT, PSF product, overlap-add */
  JUBIK_PATH_PLAIN = 2, /* unfused: batched FFT kernels + gather kernels.  For FFT sides
                           160, 192, 256, 320, 384 and 512 the row passes read the
                           windows from the images and one kernel does the column
                           passes with the PSF product.  The per-module buffer is cut
                           into module chunks of at most ~2 GiB; the environment
                           variable JUBIK_PLAIN_CHUNK_MODULES (a positive count, read
                           at plan creation) bounds the modules per chunk further.
                           Results do not depend on the chunking. */
  JUBIK_PATH_FUSED_UNIT = 3 /* fused, one kernel per (module, energy, patch) unit with no
                               sharing of patch spectra across modules */
};

enum jubik_psf_layout {
  JUBIK_PSF_PRECUT = 0, /* (M, n*n, E, K, K): the window convolve.py:107-111 cuts */
  JUBIK_PSF_FULL = 1    /* (M, n*n, E, nx, ny): full-field kernels as passed to
                           linpatch_convolve (convolve.py:66, erosita_response.py:209) */
};

typedef struct jubik_plan jubik_plan;

typedef struct {
  int32_t n_modules;  /* M: the vmapped module axis, erosita_response.py:209-212 */
  int32_t n_energies; /* E */
  int32_t nx, ny;     /* spatial field shape (Domain.shape[-2:], data.py:19-29) */
  int32_t n_patches;  /* n_patches_per_axis */
  int32_t margin;     /* margin (>= 1; the reference crops [m:-m]) */
  int32_t dtype;      /* jubik_dtype */
  int32_t path;       /* jubik_path */
  double pixel_area;  /* x * pixel_area before the PSF, erosita_response.py:307,350 */
} jubik_plan_desc;

/* Library info. */
JUBIK_API int jubik_abi_version(void);
JUBIK_API const char* jubik_last_error(void);
/* 1 if the fused single-kernel path covers FFT side P in dtype. */
JUBIK_API int jubik_fused_supported(int32_t P, int32_t dtype);
/* 1 if the plain batched FFT covers length L. */
JUBIK_API int jubik_fft_length_supported(int32_t L);

/* Plan lifetime.  Replaces the per-call set-up inside linpatch_convolve
 * (jubik/convolve.py:66-131) and the response builders
 * (erosita_response.py:217-358, chandra_response.py:20-149). */
JUBIK_API int jubik_plan_create(const jubik_plan_desc* desc, jubik_plan** out);
JUBIK_API int jubik_plan_destroy(jubik_plan* plan);
/* Device bytes held by the plan's workspace. */
JUBIK_API int jubik_plan_workspace_bytes(const jubik_plan* plan, int64_t* bytes);
/* Effective path of the plan (JUBIK_PATH_FUSED or JUBIK_PATH_PLAIN). */
JUBIK_API int jubik_plan_path(const jubik_plan* plan, int32_t* path);

/* PSF kernels -> normalised spectra, computed once per plan (FP64 FFTs,
 * rounded once to the plan dtype).  Restates the kernel preparation of
 * jubik/convolve.py:104-131 (fftshift, cut, pad, ifftshift, / sum*dvol).
 * psf has the plan dtype; e_broadcast = 1 when the psf has no E axis
 * (the broadcast branch of convolve.py:167-171). */
JUBIK_API int jubik_plan_set_psf(jubik_plan* plan, const void* psf, int32_t layout, int32_t e_broadcast,
                       void* stream);

/* Exposure and readout mask.  exposure (M,E,nx,ny) in plan dtype or NULL
 * for ones (response.py:12-45, already thresholded and multiplied by any
 * effective area); readmask (M,E,nx,ny) uint8, nonzero = read out, or NULL
 * for all (the ~mask of response.py:87,110).  Readout order is C order per
 * module, modules concatenated. */
JUBIK_API int jubik_plan_set_exposure(jubik_plan* plan, const void* exposure, const uint8_t* readmask,
                            void* stream);
/* Host: number of read-out pixels per module (length M) and in total. */
JUBIK_API int jubik_plan_readout_sizes(const jubik_plan* plan, int64_t* per_module, int64_t* total);
/* Host: readout index map, total entries of flat (M,E,nx,ny) indices (device ptr). */
JUBIK_API int jubik_plan_readout_index(const jubik_plan* plan, const int64_t** device_index);

/* Poisson counts in readout order (int32, length total), the masked_data
 * of erosita_likelihood.py:89 / chandra_likelihood.py:37. */
JUBIK_API int jubik_plan_set_data(jubik_plan* plan, const int32_t* counts, void* stream);

/* PSF operator: out (M,E,nx,ny) = linpatch_convolve(x, domain, kernel[m], n, margin)
 * for every module m (jubik/convolve.py:66-145 vmapped as in
 * erosita_response.py:209-212).  x: (E,nx,ny).  No pixel_area. */
JUBIK_API int jubik_psf_forward(jubik_plan* plan, const void* x, void* out, void* stream);
/* Its transpose: out_x (E,nx,ny) = sum_m linpatch_convolve^T(cot[m]). */
JUBIK_API int jubik_psf_adjoint(jubik_plan* plan, const void* cot, void* out_x, void* stream);

/* Full response R(x) = mask(exposure(psf(x * pixel_area)))
 * (erosita_response.py:349-350, chandra_response.py:138-142).
 * out_readout: total elements, readout order. */
JUBIK_API int jubik_response_forward(jubik_plan* plan, const void* x, void* out_readout, void* stream);
/* JVP of the (linear) response: R(t). */
JUBIK_API int jubik_response_jvp(jubik_plan* plan, const void* t, void* out_readout, void* stream);
/* VJP: out_x = R^T cot (pixel_area * psf^T(exposure * mask^T(cot))). */
JUBIK_API int jubik_response_vjp(jubik_plan* plan, const void* cot_readout, void* out_x, void* stream);

/* Poisson energy and gradient through the response, one fused pass:
 * lam = R(x); energy = sum(lam) - sum(d * log(lam)) (NIFTy.re Poissonian,
 * demos/x-ray-imaging.py:312-315), accumulated in FP64; grad_x = R^T(1 - d/lam).
 * energy: device double[1]; grad_x may be NULL (energy only).  lam is kept
 * in the plan for jubik_metric_apply. */
JUBIK_API int jubik_poisson_energy_grad(jubik_plan* plan, const void* x, double* energy, void* grad_x,
                              void* stream);
/* The same for a sky given as the exp of the (E, nx, ny) crop of a log-sky
 * array s (e_pad, nx_pad, ny_pad): sky = exp(s[:E, :nx, :ny]), the
 * exp_padding of J-UBIK's diffuse sky model (jubik/sky_models.py:340-341).
 * The exp and the crop happen inside the response's first kernel;
 * grad_s (shape of s, may be NULL) = exp(s) * R^T(1 - d/lam) on the crop and 0
 * elsewhere. */
JUBIK_API int jubik_poisson_energy_grad_logsky(jubik_plan* plan, const void* s, int32_t e_pad,
                                               int32_t nx_pad, int32_t ny_pad, double* energy,
                                               void* grad_s, void* stream);
/* MGVI metric product out = R^T diag(1/lam) R v, lam = R(x).  x == NULL
 * reuses lam from the last jubik_poisson_energy_grad call. */
JUBIK_API int jubik_metric_apply(jubik_plan* plan, const void* x, const void* v, void* out,
                       void* stream);

/* Profiling: when on, every kernel phase of a plan call is bracketed by CUDA
 * events on the call's stream and its duration accumulated (the call then
 * synchronises on the phase's end event).  Phases: 0 forward per-unit PSF
 * kernel, 1 adjoint per-unit PSF kernel, 2 likelihood / readout kernels,
 * 3 memsets, 4 forward per-patch sky-spectrum kernel, 5 adjoint per-patch
 * inverse kernel (4 and 5 run when modules share patch spectra), 6 the pass
 * that adds the low words of the gradient's exact two-word sum (fused path). */
#define JUBIK_PHASES 7
/* Programmatic dependent launch between the kernels of one plan call (default
 * on; no counterpart in the reference): each kernel may be scheduled onto the
 * SMs the previous kernel's last wave frees, and waits there for that kernel's
 * results.  Plans whose calls run side by side on several streams (e.g. the
 * branches of one CUDA graph) may switch it off, so that waiting kernels do
 * not hold SMs the other streams could use. */
JUBIK_API int jubik_plan_set_dependent_launch(jubik_plan* plan, int32_t on);
/* Schedule of the module-shared FP32 forward at FFT side 192 (no counterpart in
 * the reference): a CTA takes runs of run_len vertically adjacent patches of
 * one module and sums the field rows they share in tensor memory before they
 * leave the CTA.  run_len 4 reduces fewest rows, 2 or 1 (one patch at a time)
 * give more work items for small fields; 0 (the default) lets the library
 * choose from the field size and the SM count.  Results agree to FP32 rounding
 * across run lengths and are the same bits for a given one.  Returns
 * JUBIK_ERR_UNSUPPORTED for runs the plan's geometry cannot take. */
JUBIK_API int jubik_plan_set_forward_run(jubik_plan* plan, int32_t run_len);
/* The run length the plan's forward uses (1 where it does not run in runs). */
JUBIK_API int jubik_plan_forward_run(const jubik_plan* plan, int32_t* run_len);
JUBIK_API int jubik_plan_set_profiling(jubik_plan* plan, int32_t on);
/* ms and launch counts per phase accumulated since profiling was switched on. */
JUBIK_API int jubik_plan_profile(const jubik_plan* plan, double* ms, int64_t* launches);

/* Metric weights from a caller's expected counts (no counterpart in the
 * reference): lam (device, readout order, readout_total values, dtype
 * JUBIK_F32 or JUBIK_F64) replaces the plan's cached lam for the next
 * jubik_metric_apply calls with x = NULL; the weights eps^2 / lam are formed in
 * FP64 and rounded once.  An FP32 plan's own lam carries the FP32 forward's
 * error, which the metric's 1/lam amplifies at faint pixels; a lam from an FP64
 * plan, computed once per linearisation point, leaves the FP32 metric products
 * only their own rounding.  The next energy or metric call with an x replaces
 * the weights again. */
JUBIK_API int jubik_plan_set_metric_lambda(jubik_plan* plan, const void* lam, int32_t lam_dtype,
                                           void* stream);

/* Stand-alone Poisson likelihood on readout vectors (jft.Poissonian(data)):
 * energy (device double[1]) = sum(lam - d log lam); grad (may be NULL) = 1 - d/lam. */
JUBIK_API int jubik_poisson_energy(const void* lam, const int32_t* data, int64_t n, int32_t dtype,
                         double* energy, void* grad, void* stream);
/* Elementwise Poisson helpers: op 0 metric t/lam, 1 left-sqrt-metric t/sqrt(lam),
 * 2 normalised residual (d - lam)/sqrt(lam) (b unused, uses data),
 * 3 exposure product a*b (response.py:44). */
JUBIK_API int jubik_elementwise(int32_t op, const void* a, const void* b, const int32_t* data, int64_t n,
                      int32_t dtype, void* out, void* stream);

/* Readout (response.py:110) and its transpose with an explicit index map
 * (flat int64 indices into the image, ascending).  gather: out[i] = img[idx[i]]
 * (eps may be NULL or multiplies); scatter: img[idx[i]] = eps[idx[i]]*vec[i]
 * (img must be zeroed by the caller). */
JUBIK_API int jubik_readout_gather(const void* img, const void* eps, const int64_t* idx, int64_t nread,
                         int32_t dtype, void* out, void* stream);
JUBIK_API int jubik_readout_scatter(const void* vec, const void* eps, const int64_t* idx, int64_t nread,
                          int32_t dtype, void* img, void* stream);

/* slice_patches (jubik/convolve.py:28-63) over x (batch, nx, ny):
 * out (n*n, batch, 2dx+2dr, 2dy+2dr).  Bit-exact gather. */
JUBIK_API int jubik_slice_patches(const void* x, int64_t batch, int32_t nx, int32_t ny, int32_t n,
                        int32_t additional_margin, int32_t dtype, void* out, void* stream);
/* Its transpose (jax.linear_transpose at convolve.py:138-143): overlap-add of
 * patches (n*n, batch, 2dx+2dr, 2dy+2dr) into out (batch, nx, ny). */
JUBIK_API int jubik_slice_patches_adjoint(const void* patches, int64_t batch, int32_t nx, int32_t ny,
                                int32_t n, int32_t additional_margin, int32_t dtype, void* out,
                                void* stream);

/* convolve (jubik/convolve.py:148-176) over the last two axes:
 * out (bs, h, w) = dvol * Re(ifft2(fft2(kernel) * fft2(signal))), kernel
 * (bk, h, w) with bk == bs, or bk dividing bs (kernel broadcast over the
 * trailing signal batch, the branch of convolve.py:167-171). */
JUBIK_API int jubik_convolve2d(const void* kernel, int64_t bk, const void* signal, int64_t bs, int32_t h,
                     int32_t w, double dvol, int32_t dtype, void* out, void* stream);

/* eROSITA PSF patches interpolated from gridded PSFs at a few off-axis radii
 * (psf_interpolator of jubik/instruments/erosita/erosita_psf_utils.py:198-264,
 * with get_psf :90-172).  Device arrays, float64, radii ascending per energy:
 * psfs (E, R, psf_h, psf_w), rs (E, R), center_ids (E, R, 2), deltas (E, 2),
 * pointing (E, 2).  Field nx x ny with pixel distances (dist_x, dist_y),
 * npatch patches per axis.  layout JUBIK_PSF_FULL: out (npatch^2, E, nx, ny),
 * the reference's rolled full-field array; JUBIK_PSF_PRECUT: out (npatch^2,
 * E, 2 nx/npatch, 2 ny/npatch), the windows jubik_plan_set_psf takes, without
 * forming the full field.  out in `dtype`; arithmetic in FP64.  At most 2048
 * radii (JUBIK_ERR_INVALID_ARGUMENT beyond). */
JUBIK_API int jubik_psf_interpolate(const double* psfs, const double* rs,
                                    const double* center_ids, const double* deltas,
                                    const double* pointing, int32_t n_energies, int32_t n_radii,
                                    int32_t psf_h, int32_t psf_w, int32_t nx, int32_t ny,
                                    double dist_x, double dist_y, int32_t npatch, int32_t layout,
                                    int32_t dtype, void* out, void* stream);

/* Independent problems evaluated together (no counterpart in the reference,
 * which evaluates one likelihood per call): plans of one dtype on a fused FFT
 * side, grouped by FFT side and kind (per-unit kernels, or module-shared patch
 * spectra for plans with several modules).  One energy+gradient call of the
 * group is one grouped clearing kernel and one pass over the skies' largest
 * magnitudes; per side, one forward and one adjoint launch over all of that
 * side's per-unit problems, or two of each (patch spectra, then units) for its
 * module-shared problems; one grouped likelihood pass; and one pass that adds
 * the low words of the gradients -- the work of jubik_poisson_energy_grad on
 * every plan.  As there, the overlap-adds and gradients are exact two-word
 * sums and the module sums run in module order, so results are the same bits
 * on every call (each problem's bound comes from its own sky and residual, so
 * they can differ from a one-plan call's in the last bit).  The
 * plans must outlive the group, and none of them may run another call while a
 * group call is in flight.  set_io copies the plans' buffer addresses; after a
 * plan's jubik_plan_set_exposure (or its first jubik_plan_set_data) the group's
 * calls return JUBIK_ERR_STATE until set_io runs again.
 * set_io: the device sky and gradient buffer of each problem (x[i], grad[i],
 * shaped (E,nx,ny) of plan i) and a device double[n] for the energies; they
 * are read at every later call. */
typedef struct jubik_group jubik_group;
JUBIK_API int jubik_group_create(jubik_plan* const* plans, int32_t n, jubik_group** out);
JUBIK_API int jubik_group_set_io(jubik_group* group, const void* const* x, void* const* grad,
                                 double* energies);
JUBIK_API int jubik_group_energy_grad(jubik_group* group, void* stream);
/* Kernel launches per jubik_group_energy_grad call. */
JUBIK_API int jubik_group_launches(const jubik_group* group, int32_t* launches);
JUBIK_API int jubik_group_destroy(jubik_group* group);

/* Correlated-field log-sky: the field-sized work of J-UBIK's diffuse sky
 * model (jubik/sky_models.py:205-225 and :306-341; the fields come from
 * NIFTy.re's CorrelatedFieldMaker, whose amplitude spectrum -- a 1-D function
 * of a few scalars -- the caller computes).  On a padded s0 x s1 grid,
 *     field_b = offsets[b] + hartley(amp[b][pindex] * xi[b]),
 *     hartley(p) = Re(fftn(p)) + Im(fftn(p)),
 * for n_fields <= 4 fields sharing one mode-length index pindex (s0 * s1
 * int32 values in [0, n_modes), host memory, copied at creation).  The
 * J-UBIK log-sky (spatial field plus spectral index times the log energy-bin
 * centres, _apply_slope at sky_models.py:593-602, cropped as at :340) is
 *     logsky[e][y][x] = sum_b ecoef[e * n_fields + b] * field_b[y][x],
 *     y < nx, x < ny, E <= 32 (ecoef: host doubles).
 * Device arrays in the cf's dtype: amp (n_fields, n_modes), xi and fields
 * (n_fields, s0, s1), offsets (n_fields), logsky (E, nx, ny). */
typedef struct jubik_cf jubik_cf;
JUBIK_API int jubik_cf_create(int32_t n_fields, int32_t s0, int32_t s1, const int32_t* pindex,
                              int32_t n_modes, int32_t dtype, jubik_cf** out);
/* fields and/or logsky (either may be NULL, not both; logsky needs ecoef). */
JUBIK_API int jubik_cf_apply(jubik_cf* cf, const void* amp, const void* xi, const void* offsets,
                             void* fields, const double* ecoef, int32_t E, int32_t nx, int32_t ny,
                             void* logsky, void* stream);
/* Vector-Jacobian product for one cotangent: g_fields (n_fields, s0, s1), or
 * g_logsky (E, nx, ny) with ecoef (pass NULL for the other).  Writes dxi
 * (n_fields, s0, s1), damp (n_fields, n_modes) and doffsets (n_fields);
 * deterministic (no atomics). */
JUBIK_API int jubik_cf_vjp(jubik_cf* cf, const void* amp, const void* xi, const void* g_fields,
                           const double* ecoef, int32_t E, int32_t nx, int32_t ny,
                           const void* g_logsky, void* dxi, void* damp, void* doffsets,
                           void* stream);
JUBIK_API int jubik_cf_destroy(jubik_cf* cf);

/* Sampling and global reductions for the callers of the response.
 * Random numbers: counter-based Philox4x32-10 (Salmon et al., SC'11) keyed by
 * `seed`; element i of a call uses its own counter, so results do not depend
 * on the launch shape, and `offset` selects an independent stream.
 *
 * One Philox4x32-10 block on the host (for known-answer checks). */
JUBIK_API int jubik_philox4x32_10(const uint32_t* counter, const uint32_t* key, uint32_t* out);
/* n standard normal deviates (Box-Muller) into out (dtype): the xi ~ N(0, 1)
 * draws of an MGVI linear sample (jax.random.normal inside NIFTy.re's
 * draw_linear_residual, configured at jubik/minimization_parser.py:337-420). */
JUBIK_API int jubik_random_normal(void* out, int64_t n, int32_t dtype, uint64_t seed,
                                  uint64_t offset, void* stream);
/* Poisson deviates of expected counts lam (dtype, length n) into out (int32):
 * inversion below 10, transformed rejection (PTRS) above; -1 where lam is
 * negative, NaN or >= 2e9.  The mock-data draw of jubik/data.py:143-146
 * (jax.random.poisson of each module's masked expected counts). */
JUBIK_API int jubik_random_poisson(const void* lam, int64_t n, int32_t dtype, uint64_t seed,
                                   uint32_t offset, int32_t* out, void* stream);
/* out (device double[1]) = sum_i a[i] b[i] in a fixed order (deterministic): the
 * global dot products of the conjugate-gradient solve of an MGVI linear sample.
 * FP64 operands accumulate in FP64; FP32 operands as exact FP32 product splits
 * in compensated FP32 sums (about 48 bits) flushed into FP64 every 128 elements.
 * n = 0 writes 0 (a, b may then be NULL). */
JUBIK_API int jubik_dot(const void* a, const void* b, int64_t n, int32_t dtype, double* out,
                        void* stream);

/* jubik_convolve2d without any device allocation (no counterpart in the reference).
 * For callers that cannot allocate device memory -- code under a framework that owns
 * all device memory through its own pool (e.g. an XLA FFI handler), or a loop where
 * cudaMalloc/cudaFree would synchronise the device.  All scratch (twiddles and the
 * complex spectra of kernel and signal) comes from one static device array of
 * JUBIK_NOALLOC_SCRATCH_BYTES per GPU, held until the process exits; inputs needing
 * more scratch are rejected with JUBIK_ERR_INVALID_ARGUMENT.  The first call on a
 * device looks up the array's address (set-up work: make it before any stream
 * capture); the address is cached for the device's context, so a process that
 * destroys that context (cudaDeviceReset) must not call this entry point again.
 * Every call shares the array: calls that overlap on the GPU race. */
#define JUBIK_NOALLOC_SCRATCH_BYTES (16 * 1024 * 1024)
JUBIK_API int jubik_convolve2d_noalloc(const void* kernel, int64_t bk, const void* signal,
                                       int64_t bs, int32_t h, int32_t w, double dvol,
                                       int32_t dtype, void* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* JUBIK_GB300_H */
