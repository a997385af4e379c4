// Fused per-patch-unit response kernels (one CTA per unit (module, energy, patch)).
//
// Forward (jubik/convolve.py:86-145 for one unit):
//   sky window (2dx x 2dx, at the slice_patches position of :55-63)
//   * bilinear weights (:89-90), zero margin (:92-101)
//   -> real 2-D FFT of side P (in shared memory)
//   * normalised PSF spectrum (kernel prep :104-131 done once per plan)
//   -> inverse real 2-D FFT -> overlap-add into the (M,E,nx,ny) image with
//   the crop of :144 applied by bounds (the transpose of slice_patches with
//   margin, :135-143).
// Adjoint: cotangent window (P x P) -> FFT -> * conj(spectrum) -> inverse
//   -> crop the margin -> * weights -> scatter into the sky gradient.
//
// Shared-memory tile: P*P/2 complex values.  Rows are first processed in
// pairs (two real rows packed as one complex row, "pair form": pair j,
// slot s in [0,P)); after the real-to-complex split the same storage is read
// as P rows of P/2 complex half-spectrum columns ("row form": row y, column
// c; column 0 packs the kx=0 and kx=P/2 values of the real rows).
// Every 1-D transform of side P = L1*16 is an in-place two-phase
// Cooley-Tukey (4-step) pass whose data never leaves its own slots:
//   variant A (natural -> permuted):  X[k1 + L1 k2] lands in slot 16 k1 + k2
//   variant B (permuted -> natural):  input x[n1 + L1 n2] in slot 16 n1 + n2
// so no reordering pass is needed: the spectrum stays in A-order, the PSF
// spectrum is stored in that order, and the inverse (B) returns to natural
// order.  An XOR swizzle on the low 4 bits of the slot keeps both the
// row-pair and the column accesses free of shared-memory bank conflicts.
#include <cstdio>

#include "fft_codelets.cuh"
#include "internal.h"

namespace jubik {

namespace {

template <int P> struct Cfg;
template <> struct Cfg<16> { static constexpr int NT = 64; };
template <> struct Cfg<32> { static constexpr int NT = 64; };
template <> struct Cfg<48> { static constexpr int NT = 96; };
template <> struct Cfg<64> { static constexpr int NT = 128; };
template <> struct Cfg<96> { static constexpr int NT = 192; };
template <> struct Cfg<128> { static constexpr int NT = 256; };
template <> struct Cfg<192> { static constexpr int NT = 384; };

template <int P>
__device__ __forceinline__ int swz(int j, int s) {
  return j * P + (s & ~15) + ((s & 15) ^ (((s >> 4) + j) & 15));
}
template <int P>
__device__ __forceinline__ int swr(int y, int c) {
  return swz<P>(y >> 1, (y & 1) * (P / 2) + c);
}
// Slot of index i in the permuted order shared by variants A (output) and B (input).
template <int P>
__device__ __forceinline__ int pslot(int i) {
  constexpr int L1 = P / 16;
  return 16 * (i % L1) + i / L1;
}

struct Args {
  const void* in;
  void* out;
  const void* hmain;
  const void* hnyq;
  const void* tw;
  const void* wt;
  double scale;
  int M, E, nx, ny, n, dx, margin, half, sr_max, sc_max;
};

// Real-to-complex split of one pair row (see header): slots {k, H-k, H+k, P-k}.
template <typename T, int P>
__device__ __forceinline__ void split_group(cx<T>* tile, int j, int k) {
  constexpr int H = P / 2;
  const T h = (T)0.5;
  if (k == 0) {
    const cx<T> z0 = tile[swz<P>(j, 0)], zh = tile[swz<P>(j, H)];
    tile[swz<P>(j, 0)] = mkc<T>(z0.x, zh.x);
    tile[swz<P>(j, H)] = mkc<T>(z0.y, zh.y);
    return;
  }
  auto A = [&](cx<T> a, cx<T> b) { return mkc<T>(h * (a.x + b.x), h * (a.y - b.y)); };
  auto B = [&](cx<T> a, cx<T> b) { return mkc<T>(h * (a.y + b.y), h * (b.x - a.x)); };
  if (4 * k == P) {
    const cx<T> za = tile[swz<P>(j, k)], zb = tile[swz<P>(j, P - k)];
    tile[swz<P>(j, k)] = A(za, zb);
    tile[swz<P>(j, P - k)] = B(za, zb);
    return;
  }
  const int k2 = H - k;
  const cx<T> za = tile[swz<P>(j, k)], zb = tile[swz<P>(j, P - k)];
  const cx<T> zc = tile[swz<P>(j, k2)], zd = tile[swz<P>(j, P - k2)];
  tile[swz<P>(j, k)] = A(za, zb);
  tile[swz<P>(j, H + k)] = B(za, zb);
  tile[swz<P>(j, k2)] = A(zc, zd);
  tile[swz<P>(j, H + k2)] = B(zc, zd);
}

// Inverse of split_group: two half-spectrum rows -> one Hermitian-extended pair row.
template <typename T, int P>
__device__ __forceinline__ void combine_group(cx<T>* tile, int j, int k) {
  constexpr int H = P / 2;
  if (k == 0) {
    const cx<T> a = tile[swz<P>(j, 0)], b = tile[swz<P>(j, H)];
    tile[swz<P>(j, 0)] = mkc<T>(a.x, b.x);
    tile[swz<P>(j, H)] = mkc<T>(a.y, b.y);
    return;
  }
  auto Zp = [&](cx<T> a, cx<T> b) { return mkc<T>(a.x - b.y, a.y + b.x); };  // a + i b
  auto Zm = [&](cx<T> a, cx<T> b) { return mkc<T>(a.x + b.y, b.x - a.y); };  // conj(a) + i conj(b)
  if (4 * k == P) {
    const cx<T> a = tile[swz<P>(j, k)], b = tile[swz<P>(j, H + k)];
    tile[swz<P>(j, k)] = Zp(a, b);
    tile[swz<P>(j, P - k)] = Zm(a, b);
    return;
  }
  const int k2 = H - k;
  const cx<T> ak = tile[swz<P>(j, k)], bk = tile[swz<P>(j, H + k)];
  const cx<T> ak2 = tile[swz<P>(j, k2)], bk2 = tile[swz<P>(j, H + k2)];
  tile[swz<P>(j, k)] = Zp(ak, bk);
  tile[swz<P>(j, P - k)] = Zm(ak, bk);
  tile[swz<P>(j, k2)] = Zp(ak2, bk2);
  tile[swz<P>(j, P - k2)] = Zm(ak2, bk2);
}

// Column 0 holds DC (re) and Nyquist (im) columns of the real rows; after its
// column FFT it is W = A + iN with A, N Hermitian spectra.  Unpack the pair
// (ky, -ky), multiply by the PSF spectrum columns kx = 0 and kx = P/2, repack.
template <typename T, int P, bool ADJ>
__device__ __forceinline__ void col0_product(cx<T>* tile, const cx<T>* __restrict__ hmain,
                                             const cx<T>* __restrict__ hnyq, int ky) {
  constexpr int H = P / 2;
  const int s1 = pslot<P>(ky);
  const cx<T> h0 = hmain[s1 * H];
  const cx<T> hn = hnyq[s1];
  const cx<T> w1 = tile[swr<P>(s1, 0)];
  auto mul = [&](cx<T> a, cx<T> b) { return ADJ ? cmulc<T>(a, b) : cmul<T>(a, b); };
  if (ky == 0 || ky == H) {
    const cx<T> A = mul(mkc<T>(w1.x, (T)0), h0);
    const cx<T> N = mul(mkc<T>(w1.y, (T)0), hn);
    tile[swr<P>(s1, 0)] = mkc<T>(A.x - N.y, A.y + N.x);
    return;
  }
  const int s2 = pslot<P>(P - ky);
  const cx<T> w2 = tile[swr<P>(s2, 0)];
  const T h = (T)0.5;
  cx<T> A = mkc<T>(h * (w1.x + w2.x), h * (w1.y - w2.y));
  cx<T> N = mkc<T>(h * (w1.y + w2.y), h * (w2.x - w1.x));
  A = mul(A, h0);
  N = mul(N, hn);
  tile[swr<P>(s1, 0)] = mkc<T>(A.x - N.y, A.y + N.x);  // A + iN
  tile[swr<P>(s2, 0)] = mkc<T>(A.x + N.y, N.x - A.y);  // conj(A) + i conj(N)
}

template <typename T, int P, bool ADJ>
__global__ void __launch_bounds__(Cfg<P>::NT) k_fused(Args a) {
  constexpr int L1 = P / 16;
  constexpr int H = P / 2;
  constexpr int NT = Cfg<P>::NT;
  constexpr int TILE = P * H;
  extern __shared__ unsigned char smem_raw[];
  cx<T>* tile = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* tw = tile + TILE;
  const int tid = threadIdx.x;

  // unit u = ((e * n^2 + k) * M + m): the modules of one sky window are adjacent
  const int n2p = a.n * a.n;
  int u = blockIdx.x;
  const int m = u % a.M;
  u /= a.M;
  const int k = u % n2p;
  const int e = u / n2p;
  const int sr = min((k % a.n) * a.dx, a.sr_max);
  const int sc = min((k / a.n) * a.dx, a.sc_max);
  const int rb = sr - a.half - a.margin;  // image row of FFT row 0
  const int cb = sc - a.half - a.margin;
  const int K = 2 * a.dx;
  const int64_t hu = ((int64_t)m * n2p + k) * a.E + e;
  const cx<T>* __restrict__ hmain = (const cx<T>*)a.hmain + hu * (int64_t)(P * H);
  const cx<T>* __restrict__ hnyq = (const cx<T>*)a.hnyq + hu * (int64_t)P;
  const T* __restrict__ wt = (const T*)a.wt;
  const int64_t npix = (int64_t)a.nx * a.ny;

  for (int i = tid; i < P; i += NT) tw[i] = ((const cx<T>*)a.tw)[i];

  // ---- 1. load the real P x P patch as pair rows, x in B-input (permuted) order
  if (!ADJ) {
    const T* __restrict__ src = (const T*)a.in + (int64_t)e * npix;
    for (int idx = tid; idx < H * P; idx += NT) {
      const int j = idx / P, x = idx - j * P;
      T v0 = (T)0, v1 = (T)0;
      const int xa = x - a.margin, col = cb + x;
      if (xa >= 0 && xa < K && col >= 0 && col < a.ny) {
        const T wx = wt[xa];
        const int y0 = 2 * j;
        int ya = y0 - a.margin, row = rb + y0;
        if (ya >= 0 && ya < K && row >= 0 && row < a.nx)
          v0 = (wt[ya] * wx) * src[(int64_t)row * a.ny + col];
        ++ya;
        ++row;
        if (ya >= 0 && ya < K && row >= 0 && row < a.nx)
          v1 = (wt[ya] * wx) * src[(int64_t)row * a.ny + col];
      }
      tile[swz<P>(j, pslot<P>(x))] = mkc<T>(v0, v1);
    }
  } else {
    const T* __restrict__ src = (const T*)a.in + ((int64_t)m * a.E + e) * npix;
    for (int idx = tid; idx < H * P; idx += NT) {
      const int j = idx / P, x = idx - j * P;
      T v0 = (T)0, v1 = (T)0;
      const int col = cb + x;
      if (col >= 0 && col < a.ny) {
        const int row = rb + 2 * j;
        if (row >= 0 && row < a.nx) v0 = src[(int64_t)row * a.ny + col];
        if (row + 1 >= 0 && row + 1 < a.nx) v1 = src[(int64_t)(row + 1) * a.ny + col];
      }
      tile[swz<P>(j, pslot<P>(x))] = mkc<T>(v0, v1);
    }
  }
  __syncthreads();

  // ---- 2. row FFT, variant B (forward): step A, items (j, n1)
  for (int it = tid; it < H * L1; it += NT) {
    const int j = it % H, n1 = it / H;
    cx<T> v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = tile[swz<P>(j, 16 * n1 + q)];
    Dft<16, false, T>::run(v);
#pragma unroll
    for (int q = 1; q < 16; ++q) v[q] = cmul<T>(v[q], tw[n1 * q]);
#pragma unroll
    for (int q = 0; q < 16; ++q) tile[swz<P>(j, 16 * n1 + q)] = v[q];
  }
  __syncthreads();
  // step B, items (j, k2)
  for (int it = tid; it < H * 16; it += NT) {
    const int j = it % H, k2 = it / H;
    cx<T> v[L1];
#pragma unroll
    for (int q = 0; q < L1; ++q) v[q] = tile[swz<P>(j, 16 * q + k2)];
    Dft<L1, false, T>::run(v);
#pragma unroll
    for (int q = 0; q < L1; ++q) tile[swz<P>(j, 16 * q + k2)] = v[q];
  }
  __syncthreads();

  // ---- 3. split pair rows into half-spectrum rows
  for (int it = tid; it < H * (P / 4 + 1); it += NT) split_group<T, P>(tile, it % H, it / H);
  __syncthreads();

  // ---- 4. column FFT, variant A (forward) phase 1: items (c, n2)
  for (int it = tid; it < H * 16; it += NT) {
    const int c = it % H, n2 = it / H;
    cx<T> v[L1];
#pragma unroll
    for (int q = 0; q < L1; ++q) v[q] = tile[swr<P>(n2 + 16 * q, c)];
    Dft<L1, false, T>::run(v);
#pragma unroll
    for (int q = 1; q < L1; ++q) v[q] = cmul<T>(v[q], tw[n2 * q]);
#pragma unroll
    for (int q = 0; q < L1; ++q) tile[swr<P>(n2 + 16 * q, c)] = v[q];
  }
  __syncthreads();

  // ---- 5. phase 2 + PSF product + inverse variant-B step A, items (c, k1)
  for (int it = tid; it < H * L1; it += NT) {
    const int c = it % H, k1 = it / H;
    cx<T> v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = tile[swr<P>(16 * k1 + q, c)];
    Dft<16, false, T>::run(v);
    if (c != 0) {
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const cx<T> h = hmain[(16 * k1 + q) * H + c];
        v[q] = ADJ ? cmulc<T>(v[q], h) : cmul<T>(v[q], h);
      }
      Dft<16, true, T>::run(v);
#pragma unroll
      for (int q = 1; q < 16; ++q) v[q] = cmulc<T>(v[q], tw[k1 * q]);
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) tile[swr<P>(16 * k1 + q, c)] = v[q];
  }
  __syncthreads();

  // ---- 6. column 0: unpack / product / repack, then its inverse step A
  for (int ky = tid; ky <= H; ky += NT) col0_product<T, P, ADJ>(tile, hmain, hnyq, ky);
  __syncthreads();
  for (int k1 = tid; k1 < L1; k1 += NT) {
    cx<T> v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = tile[swr<P>(16 * k1 + q, 0)];
    Dft<16, true, T>::run(v);
#pragma unroll
    for (int q = 1; q < 16; ++q) v[q] = cmulc<T>(v[q], tw[k1 * q]);
#pragma unroll
    for (int q = 0; q < 16; ++q) tile[swr<P>(16 * k1 + q, 0)] = v[q];
  }
  __syncthreads();

  // ---- 7. inverse column step B, items (c, q): rows 16 a + q -> natural rows
  for (int it = tid; it < H * 16; it += NT) {
    const int c = it % H, q = it / H;
    cx<T> v[L1];
#pragma unroll
    for (int i = 0; i < L1; ++i) v[i] = tile[swr<P>(16 * i + q, c)];
    Dft<L1, true, T>::run(v);
#pragma unroll
    for (int i = 0; i < L1; ++i) tile[swr<P>(16 * i + q, c)] = v[i];
  }
  __syncthreads();

  // ---- 8. half-spectrum rows -> Hermitian pair rows
  for (int it = tid; it < H * (P / 4 + 1); it += NT) combine_group<T, P>(tile, it % H, it / H);
  __syncthreads();

  // ---- 9. inverse row FFT, variant A: phase 1 items (j, n2)
  for (int it = tid; it < H * 16; it += NT) {
    const int j = it % H, n2 = it / H;
    cx<T> v[L1];
#pragma unroll
    for (int q = 0; q < L1; ++q) v[q] = tile[swz<P>(j, n2 + 16 * q)];
    Dft<L1, true, T>::run(v);
#pragma unroll
    for (int q = 1; q < L1; ++q) v[q] = cmulc<T>(v[q], tw[n2 * q]);
#pragma unroll
    for (int q = 0; q < L1; ++q) tile[swz<P>(j, n2 + 16 * q)] = v[q];
  }
  __syncthreads();
  // phase 2 items (j, k1): slot 16 k1 + k2 holds x = k1 + L1 k2
  for (int it = tid; it < H * L1; it += NT) {
    const int j = it % H, k1 = it / H;
    cx<T> v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = tile[swz<P>(j, 16 * k1 + q)];
    Dft<16, true, T>::run(v);
#pragma unroll
    for (int q = 0; q < 16; ++q) tile[swz<P>(j, 16 * k1 + q)] = v[q];
  }
  __syncthreads();

  // ---- 10. overlap-add / scatter (bounds = crop of convolve.py:144)
  const T scale = (T)a.scale;
  if (!ADJ) {
    T* __restrict__ dst = (T*)a.out + ((int64_t)m * a.E + e) * npix;
    for (int idx = tid; idx < H * P; idx += NT) {
      const int j = idx / P, x = idx - j * P;
      const int col = cb + x;
      if (col < 0 || col >= a.ny) continue;
      const cx<T> z = tile[swz<P>(j, pslot<P>(x))];
      const int row = rb + 2 * j;
      if (row >= 0 && row < a.nx) atomicAdd(dst + (int64_t)row * a.ny + col, scale * z.x);
      if (row + 1 >= 0 && row + 1 < a.nx)
        atomicAdd(dst + (int64_t)(row + 1) * a.ny + col, scale * z.y);
    }
  } else {
    T* __restrict__ dst = (T*)a.out + (int64_t)e * npix;
    for (int idx = tid; idx < H * P; idx += NT) {
      const int j = idx / P, x = idx - j * P;
      const int xa = x - a.margin, col = cb + x;
      if (xa < 0 || xa >= K || col < 0 || col >= a.ny) continue;
      const cx<T> z = tile[swz<P>(j, pslot<P>(x))];
      const T wx = wt[xa] * scale;
      const int y0 = 2 * j;
      int ya = y0 - a.margin, row = rb + y0;
      if (ya >= 0 && ya < K && row >= 0 && row < a.nx)
        atomicAdd(dst + (int64_t)row * a.ny + col, (wt[ya] * wx) * z.x);
      ++ya;
      ++row;
      if (ya >= 0 && ya < K && row >= 0 && row < a.nx)
        atomicAdd(dst + (int64_t)row * a.ny + col, (wt[ya] * wx) * z.y);
    }
  }
}

template <typename T, int P>
size_t smem_for() {
  return sizeof(cx<T>) * (size_t)(P * (P / 2) + P);
}

template <typename T, int P, bool ADJ>
int launch_one(const Geom& g, const FusedLaunch& f, cudaStream_t s) {
  Args a;
  a.in = f.in;
  a.out = f.out;
  a.hmain = f.hmain;
  a.hnyq = f.hnyq;
  a.tw = f.tw;
  a.wt = f.wt;
  a.scale = f.scale;
  a.M = g.M;
  a.E = g.E;
  a.nx = g.nx;
  a.ny = g.ny;
  a.n = g.n;
  a.dx = g.dx;
  a.margin = g.margin;
  a.half = g.half;
  a.sr_max = g.sr_max;
  a.sc_max = g.sc_max;
  const size_t smem = smem_for<T, P>();
  static bool attr_set = false;
  if (!attr_set) {
    JUBIK_TRY_CUDA(cudaFuncSetAttribute(k_fused<T, P, ADJ>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr_set = true;
  }
  const int64_t units = g.units();
  if (units <= 0) return JUBIK_OK;
  if (units > 0x7fffffffLL) {
    set_error("too many patch units for one launch");
    return JUBIK_ERR_UNSUPPORTED;
  }
  k_fused<T, P, ADJ><<<(unsigned)units, Cfg<P>::NT, smem, s>>>(a);
  return cuda_status(cudaGetLastError(), "k_fused launch");
}

template <typename T, bool ADJ>
int dispatch(const Geom& g, const FusedLaunch& f, cudaStream_t s) {
  switch (g.P) {
    case 16: return launch_one<T, 16, ADJ>(g, f, s);
    case 32: return launch_one<T, 32, ADJ>(g, f, s);
    case 48: return launch_one<T, 48, ADJ>(g, f, s);
    case 64: return launch_one<T, 64, ADJ>(g, f, s);
    case 96: return launch_one<T, 96, ADJ>(g, f, s);
    case 128: return launch_one<T, 128, ADJ>(g, f, s);
    case 192:
      if constexpr (sizeof(T) == 4) return launch_one<T, 192, ADJ>(g, f, s);
      break;
    default: break;
  }
  set_error("fused path does not cover P=%d for this dtype", g.P);
  return JUBIK_ERR_UNSUPPORTED;
}

}  // namespace

bool fused_supported(int P, int dtype) {
  switch (P) {
    case 16: case 32: case 48: case 64: case 96: case 128: return true;
    case 192: return dtype == JUBIK_F32;
    default: return false;
  }
}

size_t fused_smem_bytes(int P, int dtype) {
  const size_t c = dtype == JUBIK_F32 ? 8 : 16;
  return c * (size_t)(P * (P / 2) + P);
}

int fused_forward(const Geom& g, int dtype, const FusedLaunch& a, cudaStream_t s) {
  return dtype == JUBIK_F32 ? dispatch<float, false>(g, a, s) : dispatch<double, false>(g, a, s);
}

int fused_adjoint(const Geom& g, int dtype, const FusedLaunch& a, cudaStream_t s) {
  return dtype == JUBIK_F32 ? dispatch<float, true>(g, a, s) : dispatch<double, true>(g, a, s);
}

}  // namespace jubik
