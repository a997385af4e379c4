// PSF patches of the eROSITA instrument model, interpolated on the GPU
// (jubik/instruments/erosita/erosita_psf_utils.py:90-264).
//
// For patch k of an n x n grid over an N0 x N1 field, the PSF is the
// radius-weighted sum of gridded PSFs measured at a few off-axis radii: the
// patch centre's distance r from the pointing centre gives linear weights
// over the radii (:40-71), and each gridded PSF is sampled by bilinear
// interpolation with clamped indices (map_coordinates(order=1,
// mode='nearest')) at the pixel offsets rotated by the patch's angle about
// the pointing centre (:132-172).  Patch centres, offset grid and patch order
// follow psf_interpolator (:217-258).
//
// The reference evaluates every patch on the full N0 x N1 field and rolls it
// by half the field (:259-262); the response then keeps only the 2dx x 2dy
// window around the centre (jubik/convolve.py:107-111).  Layout PRECUT
// evaluates that window directly -- window pixel a sits at offset a - dx --
// so the full-field array (n^2 E N0 N1 values, 45 GB in float64 for seven
// modules at 1024^2) is never formed.  Layout FULL writes the reference's
// array.  All arithmetic in FP64.
//
// A block row (blockIdx.y) takes one (patch, energy) item at a time: the
// patch's radial weights and its rotation (cos, sin of the angle phi) are
// computed once per item, and each pixel offset (dra, ddec) is rotated by
// phi directly -- x = dra cos phi + ddec sin phi, y = ddec cos phi - dra sin phi,
// the same point as the reference's ri cos(th - phi), ri sin(th - phi) with
// th = atan2(ddec, dra), to rounding -- so no trigonometric function runs per
// pixel (on this GPU the FP64 pipe is narrow).  Likewise the grid coordinate
// (x + c d) / d is formed as x (1 / d) + c, and only the radii with a nonzero
// weight (at most two for ascending radii) are visited, in ascending order.
#include <cmath>
#include <cstdio>

#include "internal.h"
#include "jubik_common.cuh"

namespace jubik {
namespace {

constexpr int kThreads = 256;
constexpr double kHalfPi = 1.57079632679489661923;

struct InterpArgs {
  const double* psfs;     // (E, R, h, w), radii ascending per energy
  const double* rs;       // (E, R)
  const double* cids;     // (E, R, 2)
  const double* deltas;   // (E, 2)
  const double* pointing; // (E, 2)
  int E, R, h, w, n0, n1, npatch, layout, out0, out1;
  double dist0, dist1;
};

// order-1 interpolation with indices clamped to the grid
__device__ double bilinear_nearest(const double* img, int h, int w, double q0, double q1) {
  q0 = fmin(fmax(q0, -1.0), (double)h);
  q1 = fmin(fmax(q1, -1.0), (double)w);
  const double f0 = floor(q0), f1 = floor(q1);
  const double t0 = q0 - f0, t1 = q1 - f1;
  const int i0 = (int)f0, i1 = (int)f1;
  const int a0 = min(max(i0, 0), h - 1), b0 = min(max(i0 + 1, 0), h - 1);
  const int a1 = min(max(i1, 0), w - 1), b1 = min(max(i1 + 1, 0), w - 1);
  return (1.0 - t0) * (1.0 - t1) * img[(int64_t)a0 * w + a1] +
         (1.0 - t0) * t1 * img[(int64_t)a0 * w + b1] + t0 * (1.0 - t1) * img[(int64_t)b0 * w + a1] +
         t0 * t1 * img[(int64_t)b0 * w + b1];
}

constexpr int kMaxRadii = 2048;  // radial weights and nonzero list of one item in shared memory

template <typename T>
__global__ void __launch_bounds__(kThreads) k_psf_interp(InterpArgs a, T* __restrict__ out) {
  extern __shared__ double s_w[];  // radial weight of each gridded PSF for this item
  __shared__ double s_rot[2];      // cos phi, sin phi
  __shared__ int s_nz;             // radii with a nonzero weight, listed in s_j
  int* s_j = reinterpret_cast<int*>(s_w + a.R);
  const int64_t per = (int64_t)a.out0 * a.out1;
  const int64_t nke = (int64_t)a.npatch * a.npatch * a.E;
  const int ps0i = a.n0 / a.npatch, ps1i = a.n1 / a.npatch;
  for (int64_t ke = blockIdx.y; ke < nke; ke += gridDim.y) {
    const int e = (int)(ke % a.E);
    const int k = (int)(ke / a.E);
    // patch centre: dec along k % n, ra reversed along k / n
    const double ps0 = (double)ps0i, ps1 = (double)ps1i;
    const double c_dec = ((double)(k % a.npatch) * ps0 + ps0 / 2.0) * a.dist0;
    const double c_ra = ((double)(a.npatch - 1 - k / a.npatch) * ps1 + ps1 / 2.0) * a.dist1;
    const double cc0 = c_ra - a.pointing[2 * e], cc1 = c_dec - a.pointing[2 * e + 1];
    const double r = sqrt(cc0 * cc0 + cc1 * cc1);
    const double* rs = a.rs + (int64_t)e * a.R;
    __syncthreads();  // the previous item's pixels no longer read s_w, s_rot
    if (threadIdx.x == 0) {
      const double phi = atan2(cc1, cc0) - kHalfPi;
      s_rot[0] = cos(phi);
      s_rot[1] = sin(phi);
    }
    for (int j = threadIdx.x; j < a.R; j += blockDim.x) {
      // radial weight of PSF j (the clamp and the interval both count at r == rs[R-1])
      double wj = 0.0;
      if (j == 0 && r <= rs[0]) wj += 1.0;
      if (j == a.R - 1 && r >= rs[a.R - 1]) wj += 1.0;
      if (j + 1 < a.R && rs[j] < r && r <= rs[j + 1]) wj += 1.0 - (r - rs[j]) / (rs[j + 1] - rs[j]);
      if (j > 0 && rs[j - 1] < r && r <= rs[j]) wj += (r - rs[j - 1]) / (rs[j] - rs[j - 1]);
      s_w[j] = wj;
    }
    __syncthreads();
    if (threadIdx.x == 0) {  // the nonzero weights in ascending j (the order of the sum)
      int nz = 0;
      for (int j = 0; j < a.R; ++j)
        if (s_w[j] != 0.0) s_j[nz++] = j;
      s_nz = nz;
    }
    __syncthreads();
    const double cph = s_rot[0], sph = s_rot[1];
    const int nz = s_nz;
    const double d0 = a.deltas[2 * e], d1 = a.deltas[2 * e + 1];
    const double inv0 = 1.0 / d0, inv1 = 1.0 / d1;
    T* __restrict__ dst = out + ke * per;
    for (int64_t pix = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; pix < per;
         pix += (int64_t)gridDim.x * blockDim.x) {
      const int i0 = (int)(pix / a.out1), i1 = (int)(pix - (int64_t)i0 * a.out1);
      // pixel offset (dec, -ra) of this output pixel
      double g0, g1;
      if (a.layout == JUBIK_PSF_PRECUT) {
        g0 = (double)(i0 - ps0i) * a.dist0;
        g1 = (double)(i1 - ps1i) * a.dist1;
      } else {  // rolled by half the field
        g0 = ((double)((i0 + a.n0 / 2) % a.n0) - (double)a.n0 / 2.0) * a.dist0;
        g1 = ((double)((i1 + a.n1 / 2) % a.n1) - (double)a.n1 / 2.0) * a.dist1;
      }
      const double ddec = g0, dra = -1.0 * g1;
      const double x = dra * cph + ddec * sph, y = ddec * cph - dra * sph;
      double acc = 0.0;
      for (int t = 0; t < nz; ++t) {
        const int j = s_j[t];
        const double wj = s_w[j];
        const double* cid = a.cids + ((int64_t)e * a.R + j) * 2;
        const double q0 = fma(x, inv0, cid[0]), q1 = fma(y, inv1, cid[1]);
        acc += wj * bilinear_nearest(a.psfs + ((int64_t)e * a.R + j) * a.h * a.w, a.h, a.w, q0,
                                     q1);
      }
      dst[pix] = (T)acc;
    }
  }
}

}  // namespace
}  // namespace jubik

using namespace jubik;

extern "C" {

int jubik_psf_interpolate(const double* psfs, const double* rs, const double* center_ids,
                          const double* deltas, const double* pointing, int32_t n_energies,
                          int32_t n_radii, int32_t psf_h, int32_t psf_w, int32_t nx, int32_t ny,
                          double dist_x, double dist_y, int32_t npatch, int32_t layout,
                          int32_t dtype, void* out, void* stream) {
  if (!psfs || !rs || !center_ids || !deltas || !pointing || !out || n_energies < 1 ||
      n_radii < 1 || psf_h < 1 || psf_w < 1 || nx < 2 || ny < 2 || npatch < 1 ||
      (layout != JUBIK_PSF_PRECUT && layout != JUBIK_PSF_FULL) ||
      (dtype != JUBIK_F32 && dtype != JUBIK_F64)) {
    set_error("psf_interpolate: invalid argument");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  if (nx % npatch != 0 || ny % npatch != 0 || nx % 2 != 0 || ny % 2 != 0) {
    set_error("psf_interpolate: the field must be even and divisible by npatch");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  InterpArgs a;
  a.psfs = psfs;
  a.rs = rs;
  a.cids = center_ids;
  a.deltas = deltas;
  a.pointing = pointing;
  a.E = n_energies;
  a.R = n_radii;
  a.h = psf_h;
  a.w = psf_w;
  a.n0 = nx;
  a.n1 = ny;
  a.npatch = npatch;
  a.layout = layout;
  a.out0 = layout == JUBIK_PSF_PRECUT ? 2 * (nx / npatch) : nx;
  a.out1 = layout == JUBIK_PSF_PRECUT ? 2 * (ny / npatch) : ny;
  a.dist0 = dist_x;
  a.dist1 = dist_y;
  if (n_radii > kMaxRadii) {
    set_error("psf_interpolate: at most %d radii", kMaxRadii);
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  // x: pixels of one (patch, energy) item; y: the items (looped beyond 65535)
  const int64_t per = (int64_t)a.out0 * a.out1;
  const int64_t nke = (int64_t)npatch * npatch * n_energies;
  int64_t gx = (per + kThreads - 1) / kThreads;
  if (gx > 1024) gx = 1024;
  const int64_t gy = nke < 65535 ? nke : 65535;
  const dim3 grid((unsigned)gx, (unsigned)gy);
  const size_t smem = (size_t)n_radii * (sizeof(double) + sizeof(int));
  cudaStream_t s = (cudaStream_t)stream;
  if (dtype == JUBIK_F32)
    k_psf_interp<float><<<grid, kThreads, smem, s>>>(a, (float*)out);
  else
    k_psf_interp<double><<<grid, kThreads, smem, s>>>(a, (double*)out);
  return cuda_status(cudaGetLastError(), "k_psf_interp");
}

}  // extern "C"
