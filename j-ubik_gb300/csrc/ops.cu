// Gather/scatter, spectrum preparation, unfused-path and likelihood kernels.
#include <algorithm>
#include <cmath>
#include <cstdio>

#include "fft_codelets.cuh"
#include "internal.h"

namespace jubik {

namespace {

constexpr int kBlock = 256;
constexpr int kRedBlocks = 1024;  // fixed grid of the energy reductions

inline unsigned grid_for(int64_t n, int per = kBlock) {
  int64_t b = (n + per - 1) / per;
  if (b > 1048576) b = 1048576;  // grid-stride beyond this
  if (b < 1) b = 1;
  return (unsigned)b;
}

__device__ __forceinline__ int img_row_base(int p, int dx, int smax, int half, int margin) {
  return min(p * dx, smax) - half - margin;
}

// --------------------------------------------------------------- PSF prep
// One block per unit hu = (m*n^2 + k)*E + e.  Reads the (2dx)^2 window (from
// the pre-cut or the full-field kernel: fftshift + centre cut of
// convolve.py:107-111), sums it in FP64, and writes the normalised kernel
// into a P x P complex FP64 array at the ifftshift(pad) positions
// ((a - dx) mod P, (b - dx) mod P) of convolve.py:118-131.
template <typename T>
__global__ void k_psf_to_cplx(const T* __restrict__ psf, int layout, int e_bcast, int E, int n2p,
                              int nx, int ny, int dx, int P, int64_t u0, double* __restrict__ sums,
                              double2* __restrict__ buf) {
  const int64_t hu = u0 + blockIdx.x;
  const int e = (int)(hu % E);
  const int64_t mk = hu / E;
  const int esrc = e_bcast ? 0 : e;
  const int Esrc = e_bcast ? 1 : E;
  const int K = 2 * dx;
  __shared__ double red[kBlock];
  auto fetch = [&](int a, int b) -> double {
    if (layout == JUBIK_PSF_PRECUT) {
      return (double)psf[((mk * Esrc + esrc) * K + a) * (int64_t)K + b];
    }
    const int kcx = (nx - 2 * dx) / 2, kcy = (ny - 2 * dx) / 2;
    int ia = (kcx + a - nx / 2) % nx;
    if (ia < 0) ia += nx;
    int ib = (kcy + b - ny / 2) % ny;
    if (ib < 0) ib += ny;
    return (double)psf[((mk * Esrc + esrc) * nx + ia) * (int64_t)ny + ib];
  };
  double acc = 0.0, aacc = 0.0;
  for (int i = threadIdx.x; i < K * K; i += blockDim.x) {
    const double v = fetch(i / K, i % K);
    acc += v;
    aacc += fabs(v);
  }
  __shared__ double ared[kBlock];
  red[threadIdx.x] = acc;
  ared[threadIdx.x] = aacc;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      red[threadIdx.x] += red[threadIdx.x + w];
      ared[threadIdx.x] += ared[threadIdx.x + w];
    }
    __syncthreads();
  }
  const double sum = red[0];
  // (sum, sum of magnitudes) of the window: the normalisation and its gain
  if (threadIdx.x == 0) {
    sums[2 * blockIdx.x] = sum;
    sums[2 * blockIdx.x + 1] = ared[0];
  }
  double2* dst = buf + (int64_t)blockIdx.x * P * P;
  for (int i = threadIdx.x; i < P * P; i += blockDim.x) dst[i] = make_double2(0.0, 0.0);
  __syncthreads();
  for (int i = threadIdx.x; i < K * K; i += blockDim.x) {
    const int a = i / K, b = i % K;
    int y = (a - dx) % P;
    if (y < 0) y += P;
    int x = (b - dx) % P;
    if (x < 0) x += P;
    dst[y * P + x] = make_double2(fetch(a, b) / sum, 0.0);
  }
}

// Spectrum (FP64, natural order) -> plan storage in dtype T, scaled by 1/P^2
// (the 1/N of ifftn folded in).  hfull: (U,P,P/2+1), the half plane kx <= P/2, for the
// unfused path;
// hmain/hnyq: half-spectrum rows in the fused kernel's 4-step order.  The
// fused kernels carry the kx = 0 and kx = P/2 columns of a real signal packed
// as W = A + iN; their product with the PSF is W' = alpha W + beta conj(W(-ky))
// with alpha = (H0 + HN)/2 and beta = (H0 - HN)/2, which hmain column 0 and
// hnyq store instead of H0 and HN.
template <typename T>
__global__ void k_spectra_store(const double2* __restrict__ buf, int P, int64_t u0, int64_t nu,
                                cx<T>* __restrict__ hfull, cx<T>* __restrict__ hmain,
                                cx<T>* __restrict__ hnyq) {
  const int H = P / 2;
  const int L1 = P / 16;
  const double sc = 1.0 / ((double)P * (double)P);
  const int64_t total = nu * P * P;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ul = i / ((int64_t)P * P);
    const int rem = (int)(i - ul * P * P);
    const int ky = rem / P, kx = rem % P;
    const double2 v = buf[i];
    const cx<T> w = mkc<T>((T)(v.x * sc), (T)(v.y * sc));
    const int64_t hu = u0 + ul;
    if (hfull && kx <= H) hfull[(hu * P + ky) * (H + 1) + kx] = w;
    if (hmain && kx <= H) {
      const int slot = 16 * (ky % L1) + ky / L1;
      if (kx == 0 || kx == H) {
        const double2 h0 = kx == 0 ? v : buf[i - H];
        const double2 hn = kx == H ? v : buf[i + H];
        const double2 al = make_double2(0.5 * (h0.x + hn.x) * sc, 0.5 * (h0.y + hn.y) * sc);
        const double2 be = make_double2(0.5 * (h0.x - hn.x) * sc, 0.5 * (h0.y - hn.y) * sc);
        if (kx == 0)
          hmain[(hu * P + slot) * H] = mkc<T>((T)al.x, (T)al.y);
        else
          hnyq[hu * P + slot] = mkc<T>((T)be.x, (T)be.y);
      } else if (kx < H) {
        hmain[(hu * P + slot) * H + kx] = w;
      }
    }
  }
}

// --------------------------------------------------------------- plain path
// Real patches travel two per complex transform: patch p = e n^2 + k is the
// real part (p even) or the imaginary part (p odd) of pair p / 2.  With
// Z = FFT(a + i b), A = (Z(k) + conj Z(-k)) / 2 and i B = (Z(k) - conj Z(-k)) / 2
// are the spectra of the two real patches; products with the (Hermitian) PSF
// spectra stay Hermitian, so one inverse transform of A Ha + i B Hb returns
// both real results as its real and imaginary parts.
// PSF spectrum value at flat frequency index rem of unit hu, from the stored
// half plane kx <= P/2 (the spectrum of a real kernel is Hermitian).

// The unfused path's element-wise kernels run on 3-D grids -- z: a unit pair or
// an image plane, y: a row, x: the threads along it -- so that no element
// index is divided back into its coordinates.  Every element is computed with
// the same operations, in the same order, as a flat index would give.
constexpr int kRowBlock = 128;
constexpr int kRowsPerBlock = 8;  // rows a block takes (every gridDim.y-th): fewer, fuller blocks

inline dim3 row_grid(int64_t Z, int64_t Y, int64_t X) {
  return dim3((unsigned)std::min<int64_t>(64, std::max<int64_t>(1, (X + kRowBlock - 1) / kRowBlock)),
              (unsigned)std::min<int64_t>(
                  65535, std::max<int64_t>(1, (Y + kRowsPerBlock - 1) / kRowsPerBlock)),
              (unsigned)std::min<int64_t>(65535, std::max<int64_t>(1, Z)));
}

#define JUBIK_FOR_Z(var_, n_) for (int64_t var_ = blockIdx.z; var_ < (n_); var_ += gridDim.z)
#define JUBIK_FOR_Y(var_, n_) \
  for (int var_ = (int)blockIdx.y; var_ < (n_); var_ += (int)gridDim.y)
#define JUBIK_FOR_X(var_, n_)                                                  \
  for (int var_ = (int)(blockIdx.x * blockDim.x + threadIdx.x); var_ < (n_); \
       var_ += (int)(gridDim.x * blockDim.x))

template <typename T>
__global__ void __launch_bounds__(kRowBlock)
    k_plain_sky_patches(const T* __restrict__ x, const T* __restrict__ wt, int E, int n, int nx,
                        int ny, int dx, int margin, int half, int sr_max, int sc_max, int P,
                        cx<T>* __restrict__ zs) {
  const int n2p = n * n;
  const int np = E * n2p, nph = (np + 1) / 2;
  const int K = 2 * dx;
  JUBIK_FOR_Z(j, nph) {
    bool ok[2];
    int e2[2], rb[2], cb[2];
    for (int part = 0; part < 2; ++part) {  // the pair's two patches
      const int p = (int)(2 * j + part);
      ok[part] = p < np;
      const int k = ok[part] ? p % n2p : 0;
      e2[part] = ok[part] ? p / n2p : 0;
      rb[part] = img_row_base(k % n, dx, sr_max, half, margin);
      cb[part] = img_row_base(k / n, dx, sc_max, half, margin);
    }
    JUBIK_FOR_Y(y, P) {
      const int ya = y - margin;
      cx<T>* __restrict__ zrow = zs + (j * P + y) * (int64_t)P;
      JUBIK_FOR_X(xx, P) {
        T v[2] = {(T)0, (T)0};
        for (int part = 0; part < 2; ++part) {
          if (!ok[part]) break;
          const int xa = xx - margin, row = rb[part] + y, col = cb[part] + xx;
          if (ya >= 0 && ya < K && xa >= 0 && xa < K && row >= 0 && row < nx && col >= 0 &&
              col < ny)
            v[part] = (wt[ya] * wt[xa]) * x[((int64_t)e2[part] * nx + row) * ny + col];
        }
        zrow[xx] = mkc<T>(v[0], v[1]);
      }
    }
  }
}

// H at spectrum position (ky, kx) of unit hu from the Hermitian half plane
// (kx <= P/2); kym = (P - ky) mod P
template <typename T>
__device__ __forceinline__ cx<T> h_row(const cx<T>* __restrict__ hh, int64_t hu, int ky, int kym,
                                       int kx, int P) {
  const int H1 = P / 2 + 1;
  if (kx < H1) return hh[(hu * P + ky) * H1 + kx];
  return cconj<T>(hh[(hu * P + kym) * H1 + (P - kx)]);
}

template <typename T>
__global__ void __launch_bounds__(kRowBlock)
    k_plain_mul_modules(const cx<T>* __restrict__ zs, const cx<T>* __restrict__ hfull, int m0,
                        int nm, int E, int n2p, int P, cx<T>* __restrict__ zu) {
  const int64_t pp = (int64_t)P * P;
  const int np = E * n2p, nph = (np + 1) / 2;
  JUBIK_FOR_Z(up, (int64_t)nm * nph) {
    const int64_t j = up % nph;
    const int m = m0 + (int)(up / nph);
    const int pa = (int)(2 * j), pb = pa + 1;
    const int64_t ha = ((int64_t)m * n2p + pa % n2p) * E + pa / n2p;
    const int64_t hb = pb < np ? ((int64_t)m * n2p + pb % n2p) * E + pb / n2p : 0;
    const cx<T>* __restrict__ zj = zs + j * pp;
    JUBIK_FOR_Y(ky, P) {
      const int kym = ky == 0 ? 0 : P - ky;
      cx<T>* __restrict__ zrow = zu + up * pp + (int64_t)ky * P;
      JUBIK_FOR_X(kx, P) {
        const int kxm = kx == 0 ? 0 : P - kx;
        const cx<T> z = zj[(int64_t)ky * P + kx], zm = cconj<T>(zj[(int64_t)kym * P + kxm]);
        const cx<T> a = cscale<T>(cadd<T>(z, zm), (T)0.5);   // spectrum of patch 2j
        const cx<T> ib = cscale<T>(csub<T>(z, zm), (T)0.5);  // i x spectrum of patch 2j + 1
        cx<T> w = cmul<T>(a, h_row<T>(hfull, ha, ky, kym, kx, P));
        if (pb < np) w = cadd<T>(w, cmul<T>(ib, h_row<T>(hfull, hb, ky, kym, kx, P)));
        zrow[kx] = w;
      }
    }
  }
}

// Deterministic overlap-add (transpose of the margin slice, convolve.py:135-144):
// every output pixel sums the <= 9 patch outputs that cover it, in patch
// order, with Kahan compensation.
template <typename T>
__global__ void __launch_bounds__(kRowBlock)
    k_plain_overlap_gather(const cx<T>* __restrict__ zu, int m0, int nm, int E, int n, int nx,
                           int ny, int dx, int margin, int half, int sr_max, int sc_max, int P,
                           T scale, T* __restrict__ out) {
  const int n2p = n * n;
  const int nph = (E * n2p + 1) / 2;
  const int64_t pp = (int64_t)P * P;
  JUBIK_FOR_Z(me, (int64_t)nm * E) {  // (m - m0) * E + e
    const int64_t mm = me / E;
    const int e = (int)(me % E);
    const int64_t m = m0 + mm;
    JUBIK_FOR_Y(r, nx) {
      const int tr = r + half + margin;
      const int ri_hi = min(n - 1, tr / dx);
      const int ri_lo = tr - P + 1 <= 0 ? 0 : (tr - P + 1 + dx - 1) / dx;
      T* __restrict__ orow = out + ((m * E + e) * nx + r) * (int64_t)ny;
      JUBIK_FOR_X(c, ny) {
        const int tc = c + half + margin;
        const int ci_hi = min(n - 1, tc / dx);
        const int ci_lo = tc - P + 1 <= 0 ? 0 : (tc - P + 1 + dx - 1) / dx;
        T s = (T)0, comp = (T)0;
        auto visit = [&](int pi, int pj) {
          const int rb = img_row_base(pi, dx, sr_max, half, margin);
          const int cb = img_row_base(pj, dx, sc_max, half, margin);
          const int y = r - rb, xx = c - cb;
          if (y < 0 || y >= P || xx < 0 || xx >= P) return;
          const int p = e * n2p + pj * n + pi;
          const cx<T> z = zu[(mm * nph + (p >> 1)) * pp + (int64_t)y * P + xx];
          const T v = (p & 1) ? z.y : z.x;
          const T yk = v - comp;
          const T tt = s + yk;
          comp = (tt - s) - yk;
          s = tt;
        };
        for (int pj = ci_lo; pj <= ci_hi; ++pj) {
          for (int pi = ri_lo; pi <= ri_hi; ++pi) visit(pi, pj);
          if (ri_hi < n - 1) visit(n - 1, pj);
        }
        if (ci_hi < n - 1) {
          for (int pi = ri_lo; pi <= ri_hi; ++pi) visit(pi, n - 1);
          if (ri_hi < n - 1) visit(n - 1, n - 1);
        }
        orow[c] = scale * s;
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kRowBlock)
    k_plain_cot_patches(const T* __restrict__ cot, int m0, int nm, int E, int n, int nx, int ny,
                        int dx, int margin, int half, int sr_max, int sc_max, int P,
                        cx<T>* __restrict__ zu) {
  const int n2p = n * n;
  const int np = E * n2p, nph = (np + 1) / 2;
  const int64_t pp = (int64_t)P * P;
  JUBIK_FOR_Z(up, (int64_t)nm * nph) {
    const int64_t j = up % nph;
    const int64_t m = m0 + up / nph;
    bool ok[2];
    int e2[2], rb[2], cb[2];
    for (int part = 0; part < 2; ++part) {
      const int p = (int)(2 * j + part);
      ok[part] = p < np;
      const int k = ok[part] ? p % n2p : 0;
      e2[part] = ok[part] ? p / n2p : 0;
      rb[part] = img_row_base(k % n, dx, sr_max, half, margin);
      cb[part] = img_row_base(k / n, dx, sc_max, half, margin);
    }
    JUBIK_FOR_Y(y, P) {
      cx<T>* __restrict__ zrow = zu + up * pp + (int64_t)y * P;
      JUBIK_FOR_X(xx, P) {
        T v[2] = {(T)0, (T)0};
        for (int part = 0; part < 2; ++part) {
          if (!ok[part]) break;
          const int row = rb[part] + y, col = cb[part] + xx;
          if (row >= 0 && row < nx && col >= 0 && col < ny)
            v[part] = cot[((m * E + e2[part]) * nx + row) * (int64_t)ny + col];
        }
        zrow[xx] = mkc<T>(v[0], v[1]);
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kRowBlock)
    k_plain_mulconj_accum(const cx<T>* __restrict__ zu, const cx<T>* __restrict__ hfull, int m0,
                          int nm, int E, int n2p, int P, int first, cx<T>* __restrict__ zs) {
  const int64_t pp = (int64_t)P * P;
  const int np = E * n2p, nph = (np + 1) / 2;
  JUBIK_FOR_Z(j, nph) {
    const int pa = (int)(2 * j), pb = pa + 1;
    const int ka = pa % n2p, ea = pa / n2p, kb = pb % n2p, eb = pb / n2p;
    JUBIK_FOR_Y(ky, P) {
      const int kym = ky == 0 ? 0 : P - ky;
      JUBIK_FOR_X(kx, P) {
        const int kxm = kx == 0 ? 0 : P - kx;
        const int64_t rem = (int64_t)ky * P + kx, mrem = (int64_t)kym * P + kxm;
        const int64_t i = j * pp + rem;
        cx<T> acc = first ? mkc<T>((T)0, (T)0) : zs[i];
        for (int mm = 0; mm < nm; ++mm) {
          const int64_t base = ((int64_t)mm * nph + j) * pp;
          const cx<T> z = zu[base + rem], zm = cconj<T>(zu[base + mrem]);
          const cx<T> a = cscale<T>(cadd<T>(z, zm), (T)0.5);
          const cx<T> ib = cscale<T>(csub<T>(z, zm), (T)0.5);
          const int64_t ha = ((int64_t)(m0 + mm) * n2p + ka) * E + ea;
          acc = cadd<T>(acc, cmulc<T>(a, h_row<T>(hfull, ha, ky, kym, kx, P)));
          if (pb < np) {
            const int64_t hb = ((int64_t)(m0 + mm) * n2p + kb) * E + eb;
            acc = cadd<T>(acc, cmulc<T>(ib, h_row<T>(hfull, hb, ky, kym, kx, P)));
          }
        }
        zs[i] = acc;
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(kRowBlock)
    k_plain_grad_gather(const cx<T>* __restrict__ zs, const T* __restrict__ wt, int E, int n,
                        int nx, int ny, int dx, int margin, int half, int sr_max, int sc_max,
                        int P, T scale, T* __restrict__ out) {
  const int n2p = n * n;
  const int64_t pp = (int64_t)P * P;
  const int K = 2 * dx;
  JUBIK_FOR_Z(ez, (int64_t)E) {
    const int e = (int)ez;
    JUBIK_FOR_Y(r, nx) {
      const int tr = r + half + margin;
      const int ri_hi = min(n - 1, tr / dx);
      const int ri_lo = tr - P + 1 <= 0 ? 0 : (tr - P + 1 + dx - 1) / dx;
      T* __restrict__ orow = out + ((int64_t)e * nx + r) * ny;
      JUBIK_FOR_X(c, ny) {
        const int tc = c + half + margin;
        const int ci_hi = min(n - 1, tc / dx);
        const int ci_lo = tc - P + 1 <= 0 ? 0 : (tc - P + 1 + dx - 1) / dx;
        T s = (T)0, comp = (T)0;
        auto visit = [&](int pi, int pj) {
          const int rb = img_row_base(pi, dx, sr_max, half, margin);
          const int cb = img_row_base(pj, dx, sc_max, half, margin);
          const int ya = r - rb - margin, xa = c - cb - margin;
          if (ya < 0 || ya >= K || xa < 0 || xa >= K) return;
          const int p = e * n2p + pj * n + pi;
          const cx<T> z = zs[(int64_t)(p >> 1) * pp + (int64_t)(ya + margin) * P + (xa + margin)];
          const T v = (wt[ya] * wt[xa]) * ((p & 1) ? z.y : z.x);
          const T yk = v - comp;
          const T tt = s + yk;
          comp = (tt - s) - yk;
          s = tt;
        };
        for (int pj = ci_lo; pj <= ci_hi; ++pj) {
          for (int pi = ri_lo; pi <= ri_hi; ++pi) visit(pi, pj);
          if (ri_hi < n - 1) visit(n - 1, pj);
        }
        if (ci_hi < n - 1) {
          for (int pi = ri_lo; pi <= ri_hi; ++pi) visit(pi, n - 1);
          if (ri_hi < n - 1) visit(n - 1, n - 1);
        }
        orow[c] = scale * s;
      }
    }
  }
}

// --------------------------------------------------------------- slice_patches
struct SliceGeom {
  int n, nx, ny, dx, dy, hx, hy, sh, sw, rmax, cmax;
};

inline int make_slice_geom(int nx, int ny, int n, int dr, SliceGeom* g) {
  if (n < 1 || dr < 0) {
    set_error("n_patches_per_axis must be >= 1 and the margin >= 0");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  g->n = n;
  g->nx = nx;
  g->ny = ny;
  g->dx = (nx - 2 * dr) / n;
  g->dy = (ny - 2 * dr) / n;
  g->hx = g->dx / 2;
  g->hy = g->dy / 2;
  g->sh = 2 * g->dx + 2 * dr;
  g->sw = 2 * g->dy + 2 * dr;
  const int ph = nx + 2 * g->hx, pw = ny + 2 * g->hy;
  if (g->dx < 1 || g->dy < 1 || g->sh > ph || g->sw > pw) {
    set_error("slice window (%d x %d) does not fit the padded field (%d x %d)", g->sh, g->sw, ph,
              pw);
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  g->rmax = ph - g->sh;
  g->cmax = pw - g->sw;
  return JUBIK_OK;
}

template <typename T>
__global__ void k_slice_patches(const T* __restrict__ x, int64_t batch, SliceGeom g,
                                T* __restrict__ out) {
  const int n2p = g.n * g.n;
  const int64_t total = (int64_t)n2p * batch * g.sh * g.sw;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int xx = (int)(i % g.sw);
    int64_t t = i / g.sw;
    const int y = (int)(t % g.sh);
    t /= g.sh;
    const int64_t b = t % batch;
    const int k = (int)(t / batch);
    const int r0 = min((k % g.n) * g.dx, g.rmax), c0 = min((k / g.n) * g.dy, g.cmax);
    const int row = r0 + y - g.hx, col = c0 + xx - g.hy;
    out[i] = (row >= 0 && row < g.nx && col >= 0 && col < g.ny)
                 ? x[(b * g.nx + row) * (int64_t)g.ny + col]
                 : (T)0;
  }
}

template <typename T>
__global__ void k_slice_patches_adjoint(const T* __restrict__ pt, int64_t batch, SliceGeom g,
                                        T* __restrict__ out) {
  const int64_t total = batch * g.nx * g.ny;
  const int64_t ps = (int64_t)g.sh * g.sw;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % g.ny);
    const int64_t t = i / g.ny;
    const int r = (int)(t % g.nx);
    const int64_t b = t / g.nx;
    const int tr = r + g.hx, tc = c + g.hy;
    const int ri_hi = min(g.n - 1, tr / g.dx), ci_hi = min(g.n - 1, tc / g.dy);
    const int ri_lo = tr - g.sh + 1 <= 0 ? 0 : (tr - g.sh + 1 + g.dx - 1) / g.dx;
    const int ci_lo = tc - g.sw + 1 <= 0 ? 0 : (tc - g.sw + 1 + g.dy - 1) / g.dy;
    T s = (T)0;
    auto visit = [&](int pi, int pj) {
      const int r0 = min(pi * g.dx, g.rmax), c0 = min(pj * g.dy, g.cmax);
      const int y = tr - r0, xx = tc - c0;
      if (y < 0 || y >= g.sh || xx < 0 || xx >= g.sw) return;
      const int64_t k = (int64_t)pj * g.n + pi;
      s += pt[(k * batch + b) * ps + (int64_t)y * g.sw + xx];
    };
    for (int pj = ci_lo; pj <= ci_hi; ++pj) {
      for (int pi = ri_lo; pi <= ri_hi; ++pi) visit(pi, pj);
      if (ri_hi < g.n - 1) visit(g.n - 1, pj);
    }
    if (ci_hi < g.n - 1) {
      for (int pi = ri_lo; pi <= ri_hi; ++pi) visit(pi, g.n - 1);
      if (ri_hi < g.n - 1) visit(g.n - 1, g.n - 1);
    }
    out[i] = s;
  }
}

// --------------------------------------------------------------- readout
template <typename T>
__global__ void k_readout_gather(const T* __restrict__ img, const T* __restrict__ eps,
                                 const int64_t* __restrict__ idx, int64_t nread,
                                 T* __restrict__ out, const T* __restrict__ img_lo) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nread;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = idx[i];
    const T v = img_lo ? img[p] + img_lo[p] : img[p];  // a two-word image: hi + lo
    out[i] = eps ? eps[p] * v : v;
  }
}

template <typename T>
__global__ void k_readout_scatter(const T* __restrict__ vec, const T* __restrict__ eps,
                                  const int64_t* __restrict__ idx, int64_t nread,
                                  T* __restrict__ img) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nread;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = idx[i];
    img[p] = eps ? eps[p] * vec[i] : vec[i];
  }
}

// --------------------------------------------------------------- Poisson
// Compensated (Kahan) accumulation in the working precision per thread, FP64
// across threads and blocks; the last block sums the block partials in a
// fixed order, so the total is deterministic.
template <typename T>
struct Kahan {
  T s = (T)0, c = (T)0;
  __device__ __forceinline__ void add(T v) {
    const T y = v - c;
    const T t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Block sums of (a, b) into partials[bid]; the last of nblocks blocks to finish
// sums the partials in a fixed order (deterministic) and writes a - b.
__device__ __forceinline__ void block_reduce2_of(double a, double b, double* partials,
                                                 unsigned int* counter, double* energy,
                                                 unsigned int bid, unsigned int nblocks) {
  __shared__ double sa[kBlock], sb[kBlock];
  __shared__ bool last;
  sa[threadIdx.x] = a;
  sb[threadIdx.x] = b;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sa[threadIdx.x] += sa[threadIdx.x + w];
      sb[threadIdx.x] += sb[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[2 * bid] = sa[0];
    partials[2 * bid + 1] = sb[0];
    __threadfence();
    const unsigned int done = atomicAdd(counter, 1u);
    last = (done == nblocks - 1);
  }
  __syncthreads();
  if (!last) return;
  // the last block sums the block partials in a fixed order (deterministic)
  __threadfence();
  double p1 = 0.0, p2 = 0.0;
  for (unsigned int i = threadIdx.x; i < nblocks; i += blockDim.x) {
    p1 += __ldcg(partials + 2 * i);
    p2 += __ldcg(partials + 2 * i + 1);
  }
  sa[threadIdx.x] = p1;
  sb[threadIdx.x] = p2;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) {
      sa[threadIdx.x] += sa[threadIdx.x + w];
      sb[threadIdx.x] += sb[threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    // H = sum(lam) - vdot(d, log(lam))
    if (energy) energy[0] = sa[0] - sb[0];
    *counter = 0u;
  }
}

__device__ __forceinline__ void block_reduce2(double a, double b, double* partials,
                                              unsigned int* counter, double* energy) {
  block_reduce2_of(a, b, partials, counter, energy, blockIdx.x, gridDim.x);
}

// One pass over the (M,E,nx,ny) images: lam = eps * conv where a pixel is read
// out (count image >= 0), the energy terms, the residual eps * (1 - d/lam)
// (0 elsewhere) and, optionally, the metric weight eps^2 / lam (0 elsewhere)
// that later Fisher-metric products apply to R v: the image-space weights of
// R^T diag(1/lam) R (the exposure enters once from R and once from R^T).
template <typename T>
__device__ __forceinline__ void poisson_px(T conv, T ep, int32_t d, T& w_o, T& res_o,
                                           Kahan<T>& s_lam, Kahan<T>& s_dlog) {
  if (d < 0) {
    res_o = (T)0;
    w_o = (T)0;
    return;
  }
  const T lam = ep * conv;
  const T dd = (T)d;
  s_lam.add(lam);
  s_dlog.add(dd * log(lam));
  w_o = (ep * ep) / lam;
  res_o = ep * ((T)1 - dd / lam);
}

// Block maximum of per-thread magnitudes (float or double bits; a NaN sorts
// last), stored as the bits of a non-negative double at out[bid] by thread 0.
__device__ __forceinline__ void store_block_max(unsigned long long v, unsigned long long* out,
                                                unsigned int bid) {
  __shared__ unsigned long long red[kBlock / 32];
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
    v = t > v ? t : v;
  }
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long r = 0ull;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = red[w] > r ? red[w] : r;
    out[bid] = r;
  }
}
__device__ __forceinline__ unsigned long long mag64(float v) {
  return (unsigned long long)__double_as_longlong((double)fabsf(v));
}
__device__ __forceinline__ unsigned long long mag64(double v) {
  return (unsigned long long)__double_as_longlong(fabs(v));
}
template <typename T>
struct MagMax {  // running largest |v| of one thread, in T (a NaN is kept)
  T m = (T)0;
  bool nan = false;
  __device__ __forceinline__ void add(T v) {
    const T a = v < (T)0 ? -v : v;
    nan |= (a != a);
    m = a > m ? a : m;
  }
  __device__ __forceinline__ unsigned long long bits() const {
    return nan ? 0x7ff8000000000000ull : mag64(m);
  }
};

// One problem's pass over its (M,E,nx,ny) images by block bid of nblocks.
template <typename T>
__device__ __forceinline__ void poisson_image_body(const T* __restrict__ conv,
                                                   const T* __restrict__ conv_lo,
                                                   const T* __restrict__ eps,
                                                   const int32_t* __restrict__ dimg, int64_t npix,
                                                   T* __restrict__ wts, T* __restrict__ resid,
                                                   double* partials, unsigned int* counter,
                                                   double* energy, unsigned int bid,
                                                   unsigned int nblocks,
                                                   unsigned long long* rmax) {
  Kahan<T> s_lam, s_dlog;
  MagMax<T> mr;  // the residual's largest magnitude (bound of the adjoint's terms)
  const int64_t stride = (int64_t)nblocks * blockDim.x;
  int64_t p0 = 0;
  if constexpr (sizeof(T) == 4) {
    // 4 pixels per thread with 16-byte accesses (all image bases are 16-byte aligned)
    const int64_t n4 = npix / 4;
    const float4* c4 = reinterpret_cast<const float4*>(conv);
    const float4* e4 = reinterpret_cast<const float4*>(eps);
    const int4* d4 = reinterpret_cast<const int4*>(dimg);
    auto px4 = [&](int64_t g, float4 c, float4 ep, int4 d) {
      float4 l, r;
      poisson_px<T>(c.x, ep.x, d.x, l.x, r.x, s_lam, s_dlog);
      poisson_px<T>(c.y, ep.y, d.y, l.y, r.y, s_lam, s_dlog);
      poisson_px<T>(c.z, ep.z, d.z, l.z, r.z, s_lam, s_dlog);
      poisson_px<T>(c.w, ep.w, d.w, l.w, r.w, s_lam, s_dlog);
      if (resid) reinterpret_cast<float4*>(resid)[g] = r;
      if (rmax) {
        mr.add(r.x);
        mr.add(r.y);
        mr.add(r.z);
        mr.add(r.w);
      }
      if (wts) __stcs(reinterpret_cast<float4*>(wts) + g, l);
    };
    int64_t g = bid * (int64_t)blockDim.x + threadIdx.x;
    // a two-word image (exact overlap-add): the value is hi + lo
    const float4* l4 = reinterpret_cast<const float4*>(conv_lo);
    auto cval = [&](int64_t i) {
      float4 c = __ldcs(c4 + i);
      if (l4) {
        const float4 l = __ldcs(l4 + i);
        c = make_float4(c.x + l.x, c.y + l.y, c.z + l.z, c.w + l.w);
      }
      return c;
    };
    for (; g + stride < n4; g += 2 * stride) {
      const float4 ca = cval(g), cb = cval(g + stride);
      const float4 ea = eps ? __ldcs(e4 + g) : make_float4(1, 1, 1, 1);
      const float4 eb = eps ? __ldcs(e4 + g + stride) : make_float4(1, 1, 1, 1);
      const int4 da = __ldcs(d4 + g), db = __ldcs(d4 + g + stride);
      px4(g, ca, ea, da);
      px4(g + stride, cb, eb, db);
    }
    if (g < n4) px4(g, cval(g), eps ? __ldcs(e4 + g) : make_float4(1, 1, 1, 1), __ldcs(d4 + g));
    p0 = n4 * 4;
  }
  for (int64_t p = p0 + bid * (int64_t)blockDim.x + threadIdx.x; p < npix; p += stride) {
    T l, r;
    poisson_px<T>(conv_lo ? conv[p] + conv_lo[p] : conv[p], eps ? eps[p] : (T)1, dimg[p], l, r,
                  s_lam, s_dlog);
    if (resid) resid[p] = r;
    if (wts) wts[p] = l;
    if (rmax) mr.add(r);
  }
  if (rmax) store_block_max(mr.bits(), rmax, bid);
  block_reduce2_of(s_lam.value(), s_dlog.value(), partials, counter, energy, bid, nblocks);
}

template <typename T>
__global__ void __launch_bounds__(kBlock)
    k_poisson_image(const T* __restrict__ conv, const T* __restrict__ conv_lo,
                    const T* __restrict__ eps,
                    const int32_t* __restrict__ dimg, int64_t npix, T* __restrict__ wts,
                    T* __restrict__ resid, double* partials, unsigned int* counter,
                    double* energy, unsigned long long* rmax) {
  // launched with programmatic stream serialisation after the forward kernels:
  // let the adjoint be scheduled early, wait for the forward image
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  poisson_image_body<T>(conv, conv_lo, eps, dimg, npix, wts, resid, partials, counter,
                        energy, blockIdx.x, gridDim.x, rmax);
}

// Grouped launch: job j (one problem) owns blocks [starts[j], starts[j + 1]).
template <typename T>
__global__ void __launch_bounds__(kBlock)
    k_poisson_group(const PoissonJob* __restrict__ jobs, const int* __restrict__ starts,
                    int njobs) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  __shared__ int s_job;
  if (threadIdx.x == 0) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (starts[mid] <= (int)blockIdx.x)
        lo = mid;
      else
        hi = mid - 1;
    }
    s_job = lo;
  }
  __syncthreads();
  const PoissonJob jb = jobs[s_job];
  poisson_image_body<T>((const T*)jb.conv, (const T*)jb.conv_lo, (const T*)jb.eps, jb.dimg,
                        jb.npix, (T*)jb.wts, (T*)jb.resid, jb.partials, jb.counter, jb.energy,
                        blockIdx.x - starts[s_job], starts[s_job + 1] - starts[s_job], jb.rmax);
}

// The job that owns this block (the last whose first block is <= blockIdx.x).
__device__ __forceinline__ int block_job(const int* __restrict__ starts, int njobs) {
  __shared__ int s_job;
  __syncthreads();  // a previous call's readers are done with s_job
  if (threadIdx.x == 0) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (starts[mid] <= (int)blockIdx.x)
        lo = mid;
      else
        hi = mid - 1;
    }
    s_job = lo;
  }
  __syncthreads();
  return s_job;
}

// Grouped magnitude maxima: job j (one problem's sky) owns blocks [starts[j],
// starts[j + 1]).  Each block takes the largest |value| of its share and raises
// the job's slot to it by atomicMax on the bits of a non-negative double, which
// order as the values do (a NaN, stored as the canonical quiet NaN, sorts above
// +inf): the slot ends at the same value in any order of the blocks.
template <typename T>
__global__ void __launch_bounds__(kBlock)
    k_absmax_group(const AbsmaxJob* __restrict__ jobs, const int* __restrict__ starts,
                   int njobs) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int j = block_job(starts, njobs);
  const AbsmaxJob jb = jobs[j];
  const int64_t nb = starts[j + 1] - starts[j], b = blockIdx.x - starts[j];
  const int64_t stride = nb * blockDim.x;
  const T* in = (const T*)jb.in;
  MagMax<T> mm;
  int64_t i0 = 0;
  if constexpr (sizeof(T) == 4) {
    if ((reinterpret_cast<uintptr_t>(in) & 15) == 0) {
      const int64_t n4 = jb.n / 4;
      const float4* in4 = reinterpret_cast<const float4*>(in);
      for (int64_t i = b * blockDim.x + threadIdx.x; i < n4; i += stride) {
        const float4 q = __ldcs(in4 + i);
        mm.add(q.x);
        mm.add(q.y);
        mm.add(q.z);
        mm.add(q.w);
      }
      i0 = n4 * 4;
    }
  }
  for (int64_t i = i0 + b * blockDim.x + threadIdx.x; i < jb.n; i += stride) mm.add(in[i]);
  __shared__ unsigned long long red[1];
  store_block_max(mm.bits(), red, 0);
  if (threadIdx.x == 0) atomicMax(jb.slot, red[0]);
}

// Grouped two-word combine: hi[i] += lo[i] over every job's n values.
template <typename T>
__global__ void __launch_bounds__(kBlock)
    k_combine_group(const CombineJob* __restrict__ jobs, const int* __restrict__ starts,
                    int njobs) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int j = block_job(starts, njobs);
  const CombineJob jb = jobs[j];
  const int64_t nb = starts[j + 1] - starts[j], b = blockIdx.x - starts[j];
  const int64_t stride = nb * blockDim.x;
  T* hi = (T*)jb.hi;
  const T* lo = (const T*)jb.lo;
  int64_t i0 = 0;
  if constexpr (sizeof(T) == 4) {  // plan and batch buffers are 16-byte aligned
    const int64_t n4 = jb.n / 4;
    float4* h4 = reinterpret_cast<float4*>(hi);
    const float4* l4 = reinterpret_cast<const float4*>(lo);
    for (int64_t i = b * blockDim.x + threadIdx.x; i < n4; i += stride) {
      const float4 h = h4[i], l = __ldcs(l4 + i);
      h4[i] = make_float4(h.x + l.x, h.y + l.y, h.z + l.z, h.w + l.w);
    }
    i0 = n4 * 4;
  }
  for (int64_t i = i0 + b * blockDim.x + threadIdx.x; i < jb.n; i += stride)
    hi[i] = hi[i] + lo[i];
}

// Grouped clearing: job j owns blocks [starts[j], starts[j + 1]) and clears its
// buffer in 16-byte stores (all plan and batch buffers are 256-byte aligned).
__global__ void k_zero_group(const ZeroJob* __restrict__ jobs, const int* __restrict__ starts,
                             int njobs) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  __shared__ int s_job;
  if (threadIdx.x == 0) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (starts[mid] <= (int)blockIdx.x)
        lo = mid;
      else
        hi = mid - 1;
    }
    s_job = lo;
  }
  __syncthreads();
  const ZeroJob jb = jobs[s_job];
  const int64_t nb = starts[s_job + 1] - starts[s_job], b = blockIdx.x - starts[s_job];
  const int64_t n16 = jb.bytes >> 4;
  float4* q = reinterpret_cast<float4*>(jb.ptr);
  for (int64_t i = b * blockDim.x + threadIdx.x; i < n16; i += nb * blockDim.x)
    q[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  unsigned char* c = static_cast<unsigned char*>(jb.ptr);
  for (int64_t i = (n16 << 4) + b * blockDim.x + threadIdx.x; i < jb.bytes; i += nb * blockDim.x)
    c[i] = 0;
}

// Count image: d[ridx[p]] where the pixel is read out, -1 elsewhere.
__global__ void k_count_image(const int32_t* __restrict__ ridx, const int32_t* __restrict__ data,
                              int64_t npix, int32_t* __restrict__ dimg) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npix;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = ridx[p];
    dimg[p] = r < 0 ? -1 : data[r];
  }
}

template <typename T>
__global__ void __launch_bounds__(kBlock)
    k_poisson_vec(const T* __restrict__ lam, const int32_t* __restrict__ data, int64_t n,
                  double* partials, unsigned int* counter, double* energy, T* __restrict__ grad) {
  Kahan<T> s_lam, s_dlog;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T l = lam[i];
    const T d = (T)data[i];
    s_lam.add(l);
    s_dlog.add(d * log(l));
    if (grad) grad[i] = (T)1 - d / l;
  }
  block_reduce2(s_lam.value(), s_dlog.value(), partials, counter, energy);
}

// Metric weights eps^2 / lam of a fresh lam = eps * conv (conv in two words,
// conv_lo nullptr for one): the same expression as the likelihood pass.
template <typename T>
__global__ void k_metric_weights(const T* __restrict__ conv, const T* __restrict__ conv_lo,
                                 const T* __restrict__ eps, const int32_t* __restrict__ ridx,
                                 int64_t npix, T* __restrict__ wts) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npix;
       p += (int64_t)gridDim.x * blockDim.x) {
    if (ridx[p] < 0) {
      wts[p] = (T)0;
      continue;
    }
    const T ep = eps ? eps[p] : (T)1;
    const T c = conv_lo ? conv[p] + conv_lo[p] : conv[p];
    wts[p] = (ep * ep) / (ep * c);
  }
}

// Metric weights from a caller's expected counts in readout order (FP32 or
// FP64): w = eps^2 / lam on read-out pixels, formed in FP64 and rounded once.
template <typename T, typename L>
__global__ void k_weights_from_lambda(const L* __restrict__ lam, const T* __restrict__ eps,
                                      const int32_t* __restrict__ ridx, int64_t npix,
                                      T* __restrict__ wts) {
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < npix;
       p += (int64_t)gridDim.x * blockDim.x) {
    const int32_t r = ridx[p];
    if (r < 0) {
      wts[p] = (T)0;
      continue;
    }
    const double ep = eps ? (double)eps[p] : 1.0;
    wts[p] = (T)((ep * ep) / (double)lam[r]);
  }
}

// resid = w * (hi + lo): the weighted image a metric product hands to the
// adjoint, made in the same pass that adds the two words of R v.
template <typename T>
__global__ void __launch_bounds__(kBlock)
    k_apply_weights(const T* __restrict__ hi, const T* __restrict__ lo, const T* __restrict__ w,
                    int64_t n, T* __restrict__ out, unsigned long long* __restrict__ rmax) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  MagMax<T> mr;  // the weighted image's largest magnitude (bound of the adjoint's terms)
  int64_t i0 = 0;
  if constexpr (sizeof(T) == 4) {  // all plan buffers are 16-byte aligned
    const int64_t n4 = n / 4;
    const float4* h4 = reinterpret_cast<const float4*>(hi);
    const float4* l4 = reinterpret_cast<const float4*>(lo);
    const float4* w4 = reinterpret_cast<const float4*>(w);
    float4* o4 = reinterpret_cast<float4*>(out);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
      float4 h = __ldcs(h4 + i);
      if (lo) {
        const float4 l = __ldcs(l4 + i);
        h = make_float4(h.x + l.x, h.y + l.y, h.z + l.z, h.w + l.w);
      }
      const float4 ww = __ldg(w4 + i);
      const float4 o = make_float4(ww.x * h.x, ww.y * h.y, ww.z * h.z, ww.w * h.w);
      o4[i] = o;
      mr.add(o.x);
      mr.add(o.y);
      mr.add(o.z);
      mr.add(o.w);
    }
    i0 = n4 * 4;
  }
  for (int64_t i = i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
    out[i] = w[i] * (lo ? hi[i] + lo[i] : hi[i]);
    mr.add(out[i]);
  }
  if (rmax) store_block_max(mr.bits(), rmax, blockIdx.x);
}

template <typename T>
__global__ void k_elementwise(int op, const T* __restrict__ a, const T* __restrict__ b,
                              const int32_t* __restrict__ d, int64_t n, T* __restrict__ out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    switch (op) {
      case 0: out[i] = b[i] / a[i]; break;
      case 1: out[i] = b[i] / sqrt(a[i]); break;
      case 2: out[i] = ((T)d[i] - a[i]) / sqrt(a[i]); break;
      default: out[i] = a[i] * b[i]; break;
    }
  }
}

}  // namespace

int energy_partials_count() { return kRedBlocks; }

// blocks a grouped likelihood pass gives a problem of npix pixels
int poisson_group_blocks(int64_t npix) {
  const int64_t b = (npix + (int64_t)kBlock * 16 - 1) / ((int64_t)kBlock * 16);
  return (int)(b < 1 ? 1 : (b > kRedBlocks ? kRedBlocks : b));
}

int poisson_group_run(int dtype, const PoissonJob* jobs, const int* starts, int njobs,
                      int64_t blocks, bool pdl, cudaStream_t s) {
  if (blocks <= 0) return JUBIK_OK;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(kBlock);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cuda_status(dtype == JUBIK_F32
                         ? cudaLaunchKernelEx(&cfg, k_poisson_group<float>, jobs, starts, njobs)
                         : cudaLaunchKernelEx(&cfg, k_poisson_group<double>, jobs, starts, njobs),
                     "k_poisson_group");
}

int zero_group_run(const ZeroJob* jobs, const int* starts, int njobs, int64_t blocks, bool pdl,
                   cudaStream_t s) {
  if (blocks <= 0) return JUBIK_OK;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(kBlock);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cuda_status(cudaLaunchKernelEx(&cfg, k_zero_group, jobs, starts, njobs),
                     "k_zero_group");
}

int group_blocks(int64_t n) {
  const int64_t b = (n + (int64_t)kBlock * 16 - 1) / ((int64_t)kBlock * 16);
  return (int)(b < 1 ? 1 : (b > 1024 ? 1024 : b));
}

namespace {
cudaLaunchConfig_t group_cfg(int64_t blocks, bool pdl, cudaStream_t s,
                             cudaLaunchAttribute* attr) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)blocks);
  cfg.blockDim = dim3(kBlock);
  cfg.stream = s;
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cfg;
}
}  // namespace

int absmax_group_run(int dtype, const AbsmaxJob* jobs, const int* starts, int njobs,
                     int64_t blocks, bool pdl, cudaStream_t s) {
  if (blocks <= 0) return JUBIK_OK;
  cudaLaunchAttribute attr[1];
  const cudaLaunchConfig_t cfg = group_cfg(blocks, pdl, s, attr);
  return cuda_status(dtype == JUBIK_F32
                         ? cudaLaunchKernelEx(&cfg, k_absmax_group<float>, jobs, starts, njobs)
                         : cudaLaunchKernelEx(&cfg, k_absmax_group<double>, jobs, starts, njobs),
                     "k_absmax_group");
}

int combine_group_run(int dtype, const CombineJob* jobs, const int* starts, int njobs,
                      int64_t blocks, bool pdl, cudaStream_t s) {
  if (blocks <= 0) return JUBIK_OK;
  cudaLaunchAttribute attr[1];
  const cudaLaunchConfig_t cfg = group_cfg(blocks, pdl, s, attr);
  return cuda_status(dtype == JUBIK_F32
                         ? cudaLaunchKernelEx(&cfg, k_combine_group<float>, jobs, starts, njobs)
                         : cudaLaunchKernelEx(&cfg, k_combine_group<double>, jobs, starts, njobs),
                     "k_combine_group");
}

// --------------------------------------------------------------- host wrappers
template <typename T>
int psf_to_cplx(const Geom& g, const void* psf, int layout, int e_broadcast, int64_t u0,
                int64_t nu, double* sums, void* buf, cudaStream_t s) {
  if (nu <= 0) return JUBIK_OK;
  k_psf_to_cplx<T><<<(unsigned)nu, kBlock, 0, s>>>((const T*)psf, layout, e_broadcast, g.E,
                                                   g.n * g.n, g.nx, g.ny, g.dx, g.P, u0, sums,
                                                   (double2*)buf);
  return cuda_status(cudaGetLastError(), "k_psf_to_cplx");
}

template <typename T>
int spectra_store(const Geom& g, const void* buf, int64_t u0, int64_t nu, void* hfull,
                  void* hmain, void* hnyq, cudaStream_t s) {
  const int64_t total = nu * g.P * g.P;
  k_spectra_store<T><<<grid_for(total), kBlock, 0, s>>>((const double2*)buf, g.P, u0, nu,
                                                        (cx<T>*)hfull, (cx<T>*)hmain,
                                                        (cx<T>*)hnyq);
  return cuda_status(cudaGetLastError(), "k_spectra_store");
}

template <typename T>
int plain_sky_patches(const Geom& g, const void* x, const void* wt, void* zs, cudaStream_t s) {
  k_plain_sky_patches<T><<<row_grid(plain_pairs(g), g.P, g.P), kRowBlock, 0, s>>>(
      (const T*)x, (const T*)wt, g.E, g.n, g.nx, g.ny, g.dx, g.margin, g.half, g.sr_max, g.sc_max,
      g.P, (cx<T>*)zs);
  return cuda_status(cudaGetLastError(), "k_plain_sky_patches");
}

template <typename T>
int plain_mul_modules(const Geom& g, const void* zs, const void* hfull, int m0, int nm, void* zu,
                      cudaStream_t s) {
  k_plain_mul_modules<T><<<row_grid((int64_t)nm * plain_pairs(g), g.P, g.P), kRowBlock, 0, s>>>(
      (const cx<T>*)zs, (const cx<T>*)hfull, m0, nm, g.E, g.n * g.n, g.P, (cx<T>*)zu);
  return cuda_status(cudaGetLastError(), "k_plain_mul_modules");
}

template <typename T>
int plain_overlap_gather(const Geom& g, const void* zu, int m0, int nm, double scale, void* out,
                         cudaStream_t s) {
  k_plain_overlap_gather<T><<<row_grid((int64_t)nm * g.E, g.nx, g.ny), kRowBlock, 0, s>>>(
      (const cx<T>*)zu, m0, nm, g.E, g.n, g.nx, g.ny, g.dx, g.margin, g.half, g.sr_max, g.sc_max,
      g.P, (T)scale, (T*)out);
  return cuda_status(cudaGetLastError(), "k_plain_overlap_gather");
}

template <typename T>
int plain_cot_patches(const Geom& g, const void* cot, int m0, int nm, void* zu, cudaStream_t s) {
  k_plain_cot_patches<T><<<row_grid((int64_t)nm * plain_pairs(g), g.P, g.P), kRowBlock, 0, s>>>(
      (const T*)cot, m0, nm, g.E, g.n, g.nx, g.ny, g.dx, g.margin, g.half, g.sr_max, g.sc_max,
      g.P, (cx<T>*)zu);
  return cuda_status(cudaGetLastError(), "k_plain_cot_patches");
}

template <typename T>
int plain_mulconj_accum(const Geom& g, const void* zu, const void* hfull, int m0, int nm,
                        bool first, void* zs, cudaStream_t s) {
  k_plain_mulconj_accum<T><<<row_grid(plain_pairs(g), g.P, g.P), kRowBlock, 0, s>>>(
      (const cx<T>*)zu, (const cx<T>*)hfull, m0, nm, g.E, g.n * g.n, g.P, first ? 1 : 0,
      (cx<T>*)zs);
  return cuda_status(cudaGetLastError(), "k_plain_mulconj_accum");
}

template <typename T>
int plain_grad_gather(const Geom& g, const void* zs, const void* wt, double scale, void* out,
                      cudaStream_t s) {
  k_plain_grad_gather<T><<<row_grid(g.E, g.nx, g.ny), kRowBlock, 0, s>>>(
      (const cx<T>*)zs, (const T*)wt, g.E, g.n, g.nx, g.ny, g.dx, g.margin, g.half, g.sr_max,
      g.sc_max, g.P, (T)scale, (T*)out);
  return cuda_status(cudaGetLastError(), "k_plain_grad_gather");
}

template <typename T>
int slice_patches_op(const void* x, int64_t batch, int nx, int ny, int n, int dr, void* out,
                     cudaStream_t s) {
  SliceGeom g;
  JUBIK_TRY(make_slice_geom(nx, ny, n, dr, &g));
  const int64_t total = (int64_t)n * n * batch * g.sh * g.sw;
  if (total == 0) return JUBIK_OK;
  k_slice_patches<T><<<grid_for(total), kBlock, 0, s>>>((const T*)x, batch, g, (T*)out);
  return cuda_status(cudaGetLastError(), "k_slice_patches");
}

template <typename T>
int slice_patches_adjoint_op(const void* patches, int64_t batch, int nx, int ny, int n, int dr,
                             void* out, cudaStream_t s) {
  SliceGeom g;
  JUBIK_TRY(make_slice_geom(nx, ny, n, dr, &g));
  const int64_t total = batch * nx * ny;
  if (total == 0) return JUBIK_OK;
  k_slice_patches_adjoint<T><<<grid_for(total), kBlock, 0, s>>>((const T*)patches, batch, g,
                                                                (T*)out);
  return cuda_status(cudaGetLastError(), "k_slice_patches_adjoint");
}

template <typename T>
int readout_gather(const void* img, const void* eps, const int64_t* idx, int64_t nread,
                   void* out, cudaStream_t s, const void* img_lo) {
  if (nread <= 0) return JUBIK_OK;
  k_readout_gather<T><<<grid_for(nread), kBlock, 0, s>>>((const T*)img, (const T*)eps, idx,
                                                         nread, (T*)out, (const T*)img_lo);
  return cuda_status(cudaGetLastError(), "k_readout_gather");
}

template <typename T>
int readout_scatter(const void* vec, const void* eps, const int64_t* idx, int64_t nread,
                    void* img, cudaStream_t s) {
  if (nread <= 0) return JUBIK_OK;
  k_readout_scatter<T><<<grid_for(nread), kBlock, 0, s>>>((const T*)vec, (const T*)eps, idx,
                                                          nread, (T*)img);
  return cuda_status(cudaGetLastError(), "k_readout_scatter");
}

template <typename T>
int poisson_image(const void* conv, const void* conv_lo, const void* eps, const int32_t* dimg,
                  int64_t npix, void* wts, void* resid, double* partials,
                  unsigned int* counter, double* energy, bool pdl, cudaStream_t s, void* rmax) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(kRedBlocks);
  cfg.blockDim = dim3(kBlock);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cuda_status(cudaLaunchKernelEx(&cfg, k_poisson_image<T>, (const T*)conv,
                                        (const T*)conv_lo, (const T*)eps, dimg, npix,
                                        (T*)wts, (T*)resid, partials, counter, energy,
                                        (unsigned long long*)rmax),
                     "k_poisson_image");
}

int count_image(const int32_t* ridx, const int32_t* data, int64_t npix, int32_t* dimg,
                cudaStream_t s) {
  k_count_image<<<grid_for(npix), kBlock, 0, s>>>(ridx, data, npix, dimg);
  return cuda_status(cudaGetLastError(), "k_count_image");
}

template <typename T>
int metric_weights(const void* conv, const void* conv_lo, const void* eps, const int32_t* ridx,
                   int64_t npix, void* wts, cudaStream_t s) {
  k_metric_weights<T><<<grid_for(npix), kBlock, 0, s>>>((const T*)conv, (const T*)conv_lo,
                                                        (const T*)eps, ridx, npix, (T*)wts);
  return cuda_status(cudaGetLastError(), "k_metric_weights");
}

template <typename T>
int weights_from_lambda(const void* lam, int lam_dtype, const void* eps, const int32_t* ridx,
                        int64_t npix, void* wts, cudaStream_t s) {
  if (lam_dtype == JUBIK_F64)
    k_weights_from_lambda<T, double><<<grid_for(npix), kBlock, 0, s>>>(
        (const double*)lam, (const T*)eps, ridx, npix, (T*)wts);
  else
    k_weights_from_lambda<T, float><<<grid_for(npix), kBlock, 0, s>>>(
        (const float*)lam, (const T*)eps, ridx, npix, (T*)wts);
  return cuda_status(cudaGetLastError(), "k_weights_from_lambda");
}

template <typename T>
int apply_weights(const void* hi, const void* lo, const void* w, int64_t n, void* out, bool pdl,
                  cudaStream_t s, void* rmax, int* nb) {
  const unsigned grid = (unsigned)std::min<int64_t>(
      kRedBlocks, std::max<int64_t>(1, (n / 4 + kBlock - 1) / kBlock));
  if (nb) *nb = (int)grid;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(kBlock);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cuda_status(cudaLaunchKernelEx(&cfg, k_apply_weights<T>, (const T*)hi, (const T*)lo,
                                        (const T*)w, n, (T*)out, (unsigned long long*)rmax),
                     "k_apply_weights");
}

template <typename T>
int poisson_vec(const void* lam, const int32_t* data, int64_t n, double* partials,
                unsigned int* counter, double* energy, void* grad, cudaStream_t s) {
  k_poisson_vec<T><<<kRedBlocks, kBlock, 0, s>>>((const T*)lam, data, n, partials, counter,
                                                 energy, (T*)grad);
  return cuda_status(cudaGetLastError(), "k_poisson_vec");
}

template <typename T>
int elementwise_op(int op, const void* a, const void* b, const int32_t* d, int64_t n, void* out,
                   cudaStream_t s) {
  if (n <= 0) return JUBIK_OK;
  k_elementwise<T><<<grid_for(n), kBlock, 0, s>>>(op, (const T*)a, (const T*)b, d, n, (T*)out);
  return cuda_status(cudaGetLastError(), "k_elementwise");
}

// Largest magnitude of an (E, rows, cols) view (exp of the values when
// exp_of): one maximum per block, as the bits of a non-negative double (a NaN
// sorts above every number).  Grid-stride over the view.
template <typename T>
__global__ void __launch_bounds__(kBlock)
    k_absmax(const T* __restrict__ in, int E, int rows, int cols, int64_t ps, int64_t rs,
             int exp_of, unsigned long long* __restrict__ out) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int64_t n = (int64_t)E * rows * cols;
  // the largest value (exp_of: exp is increasing, applied once at the end) or magnitude
  T m = exp_of ? (T)-INFINITY : (T)0;
  bool nan = false;
  auto take = [&](T v) {
    const T a = exp_of ? v : (v < (T)0 ? -v : v);
    nan |= (a != a);
    m = a > m ? a : m;
  };
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  if (sizeof(T) == 4 && rs == cols && ps == (int64_t)rows * cols &&
      (reinterpret_cast<uintptr_t>(in) & 15) == 0) {
    // a contiguous array: 16-byte loads
    const int64_t n4 = n / 4;
    const float4* in4 = reinterpret_cast<const float4*>(in);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
      const float4 q = __ldcs(in4 + i);
      take((T)q.x);
      take((T)q.y);
      take((T)q.z);
      take((T)q.w);
    }
    for (int64_t i = n4 * 4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += stride)
      take(in[i]);
  } else {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride) {
      const int64_t e = i / ((int64_t)rows * cols), rc = i - e * rows * cols;
      const int64_t r = rc / cols, c = rc - r * cols;
      take(in[e * ps + r * rs + c]);
    }
  }
  __shared__ unsigned long long red[kBlock / 32];
  const double md = (double)(exp_of ? exp(m) : m);  // in T: exp(-inf) = 0 for an empty share
  unsigned long long b = nan ? 0x7ff8000000000000ull : (unsigned long long)__double_as_longlong(md);
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long t = __shfl_xor_sync(0xffffffffu, b, o);
    b = t > b ? t : b;
  }
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long r = 0ull;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = red[w] > r ? red[w] : r;
    out[blockIdx.x] = r;
  }
}

template <typename T>
int absmax_blocks(const void* in, int E, int rows, int cols, int64_t ps, int64_t rs, bool exp_of,
                  void* out, int* nb, bool pdl, cudaStream_t s) {
  const int64_t n = (int64_t)E * rows * cols;
  // at least 16 values per thread: every kernel that reads the bound reduces
  // these nb maxima once per CTA, so fewer, fuller blocks serve them better
  constexpr int64_t kPerBlock = (int64_t)kBlock * 16;
  int blocks = (int)std::min<int64_t>(kMaxBoundBlocks,
                                      std::max<int64_t>(1, (n + kPerBlock - 1) / kPerBlock));
  *nb = blocks;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(blocks);
  cfg.blockDim = dim3(kBlock);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cuda_status(cudaLaunchKernelEx(&cfg, k_absmax<T>, (const T*)in, E, rows, cols, ps, rs,
                                        exp_of ? 1 : 0, (unsigned long long*)out),
                     "k_absmax");
}

// hi[i] += lo[i]: the value of an exact two-word accumulation, rounded once.
template <typename T>
__global__ void __launch_bounds__(kBlock)
    k_combine(T* __restrict__ hi, const T* __restrict__ lo, int64_t n) {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  asm volatile("griddepcontrol.wait;" ::: "memory");
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  int64_t i0 = 0;
  if constexpr (sizeof(T) == 4) {  // all plan buffers are 16-byte aligned
    const int64_t n4 = n / 4;
    float4* h4 = reinterpret_cast<float4*>(hi);
    const float4* l4 = reinterpret_cast<const float4*>(lo);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4; i += stride) {
      float4 h = h4[i];
      const float4 l = __ldcs(l4 + i);
      h4[i] = make_float4(h.x + l.x, h.y + l.y, h.z + l.z, h.w + l.w);
    }
    i0 = n4 * 4;
  }
  for (int64_t i = i0 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += stride)
    hi[i] = hi[i] + lo[i];
}

template <typename T>
int combine_words(void* hi, const void* lo, int64_t n, bool pdl, cudaStream_t s) {
  if (n <= 0) return JUBIK_OK;
  if ((reinterpret_cast<uintptr_t>(hi) | reinterpret_cast<uintptr_t>(lo)) & 15) {
    set_error("combine_words: buffers must be 16-byte aligned");
    return JUBIK_ERR_INVALID_ARGUMENT;
  }
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)std::min<int64_t>(4096, std::max<int64_t>(1, (n / 4 + kBlock - 1) /
                                                                              kBlock)));
  cfg.blockDim = dim3(kBlock);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cuda_status(cudaLaunchKernelEx(&cfg, k_combine<T>, (T*)hi, (const T*)lo, n),
                     "k_combine");
}

#define JUBIK_INST(T)                                                                            \
  template int psf_to_cplx<T>(const Geom&, const void*, int, int, int64_t, int64_t, double*,     \
                              void*, cudaStream_t);                                              \
  template int spectra_store<T>(const Geom&, const void*, int64_t, int64_t, void*, void*, void*, \
                                cudaStream_t);                                                   \
  template int plain_sky_patches<T>(const Geom&, const void*, const void*, void*, cudaStream_t); \
  template int plain_mul_modules<T>(const Geom&, const void*, const void*, int, int, void*,      \
                                    cudaStream_t);                                               \
  template int plain_overlap_gather<T>(const Geom&, const void*, int, int, double, void*,        \
                                       cudaStream_t);                                            \
  template int plain_cot_patches<T>(const Geom&, const void*, int, int, void*, cudaStream_t);    \
  template int plain_mulconj_accum<T>(const Geom&, const void*, const void*, int, int, bool,     \
                                      void*, cudaStream_t);                                      \
  template int plain_grad_gather<T>(const Geom&, const void*, const void*, double, void*,        \
                                    cudaStream_t);                                               \
  template int slice_patches_op<T>(const void*, int64_t, int, int, int, int, void*,              \
                                   cudaStream_t);                                                \
  template int slice_patches_adjoint_op<T>(const void*, int64_t, int, int, int, int, void*,      \
                                           cudaStream_t);                                        \
  template int readout_gather<T>(const void*, const void*, const int64_t*, int64_t, void*,       \
                                 cudaStream_t, const void*);                                     \
  template int readout_scatter<T>(const void*, const void*, const int64_t*, int64_t, void*,      \
                                  cudaStream_t);                                                 \
  template int poisson_image<T>(const void*, const void*, const void*, const int32_t*, int64_t,  \
                                void*, void*, double*, unsigned int*, double*, bool,             \
                                cudaStream_t, void*);                                            \
  template int absmax_blocks<T>(const void*, int, int, int, int64_t, int64_t, bool, void*, int*,  \
                                bool, cudaStream_t);                                             \
  template int combine_words<T>(void*, const void*, int64_t, bool, cudaStream_t);                \
  template int metric_weights<T>(const void*, const void*, const void*, const int32_t*, int64_t, \
                                 void*, cudaStream_t);                                           \
  template int weights_from_lambda<T>(const void*, int, const void*, const int32_t*, int64_t,    \
                                      void*, cudaStream_t);                                      \
  template int apply_weights<T>(const void*, const void*, const void*, int64_t, void*, bool,     \
                                cudaStream_t, void*, int*);                                      \
  template int poisson_vec<T>(const void*, const int32_t*, int64_t, double*, unsigned int*,      \
                              double*, void*, cudaStream_t);                                     \
  template int elementwise_op<T>(int, const void*, const void*, const int32_t*, int64_t, void*,  \
                                 cudaStream_t);

JUBIK_INST(float)
JUBIK_INST(double)
#undef JUBIK_INST

}  // namespace jubik
