// Fused per-patch-unit response kernels (one CTA per unit (module, energy, patch)).
//
// Forward (jubik/convolve.py:86-145 for one unit):
//   sky window (2dx x 2dx at the slice_patches position of :55-63)
//   * bilinear weights (:89-90), zero margin (:92-101)
//   -> real 2-D FFT of side P in shared memory
//   * normalised PSF spectrum (the kernel preparation of :104-131, done once per plan)
//   -> inverse real 2-D FFT -> overlap-add into the (M,E,nx,ny) image; the
//   crop of :144 is applied by bounds (transpose of slice_patches with margin, :135-143).
// Adjoint: cotangent window (P x P) -> FFT -> * conj(spectrum) -> inverse
//   -> crop the margin -> * weights -> scatter into the sky gradient.
//
// Layout.  The tile holds P*P/2 complex values as P/2 "pairs" of pitch P+1:
// pair j, slot s.  Rows are transformed two at a time (row 2j real, row 2j+1
// imaginary); after the real-to-complex split the same storage is read in
// "row form": row y = 2j + b, column c at slot b*(P/2) + c.  Column 0 packs the
// kx = 0 and kx = P/2 values of each real row.  The odd pitch keeps the
// pair-parallel row passes and the column-parallel column passes free of
// bank conflicts, and every element address inside an item is a base plus a
// compile-time offset.
//
// Each 1-D transform of side P = 16*L1 is an in-place two-phase Cooley-Tukey
// (4-step) pass on fixed slots:
//   variant A (natural -> permuted): X[k1 + L1 k2] ends in slot 16 k1 + k2
//   variant B (permuted -> natural): x[n1 + L1 n2] starts in slot 16 n1 + n2
// so no reordering pass is needed: the spectrum stays in A order, the PSF
// spectrum is stored in that order and the inverse B pass returns to natural
// order.  Every twiddle w_P^(c*q) is applied in a 16-point phase whose class c
// (the 16-slot block) is the warp index, so each thread keeps its 15 twiddles
// in registers.  The real-to-complex split is fused into the second row phase
// (classes kappa and 16-kappa form closed slot sets), the inverse combine
// into the first inverse row phase.
#include <cstdio>

#include "fft_codelets.cuh"
#include "internal.h"

namespace jubik {

namespace {

template <typename T, int P>
struct Tr {
  static constexpr int L1 = P / 16;
  static constexpr int H = P / 2;
  static constexpr int NW = L1;       // one warp per 16-point class
  static constexpr int NT = 32 * NW;
  static constexpr int TP = P + 1;    // pair pitch (complex elements)
  static constexpr int CH = H < 32 ? H : 32;  // staging chunk (pairs)
  static constexpr size_t TILE = (size_t)H * TP;
  static constexpr size_t STG = (size_t)CH * TP;
  static constexpr size_t SMEM = sizeof(cx<T>) * (TILE + STG);
};

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

__device__ __forceinline__ float2 ldg2(const float2* p) { return __ldg(p); }
__device__ __forceinline__ double2 ldg2(const double2* p) { return __ldg(p); }

__device__ __forceinline__ void prefetch_l2(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Asynchronous 4/8-byte global->shared copy; src_bytes = 0 writes zeros.
template <typename T>
__device__ __forceinline__ void cp_async(T* dst, const T* src, bool ok) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(T) == 4) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src),
                 "r"(ok ? 4 : 0)
                 : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src),
                 "r"(ok ? 8 : 0)
                 : "memory");
  }
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

// 4 consecutive floats added to global memory in one reduction (16-byte aligned)
__device__ __forceinline__ void red_add_v4(float* p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1,%2,%3,%4};" ::"l"(p), "f"(a), "f"(b), "f"(c),
               "f"(d)
               : "memory");
}

// (a + conj(b)) / 2 and (a - conj(b)) / (2i)
template <typename T>
__device__ __forceinline__ cx<T> sp_a(cx<T> a, cx<T> b) {
  return mkc<T>((T)0.5 * (a.x + b.x), (T)0.5 * (a.y - b.y));
}
template <typename T>
__device__ __forceinline__ cx<T> sp_b(cx<T> a, cx<T> b) {
  return mkc<T>((T)0.5 * (a.y + b.y), (T)0.5 * (b.x - a.x));
}
// a + i b and conj(a) + i conj(b)
template <typename T>
__device__ __forceinline__ cx<T> cb_p(cx<T> a, cx<T> b) {
  return mkc<T>(a.x - b.y, a.y + b.x);
}
template <typename T>
__device__ __forceinline__ cx<T> cb_m(cx<T> a, cx<T> b) {
  return mkc<T>(a.x + b.y, b.x - a.y);
}

// Row form address of (row y, column c).
template <int P>
__device__ __forceinline__ int rf(int y, int c) {
  return (y >> 1) * (P + 1) + (y & 1) * (P / 2) + c;
}

template <typename T, int P, bool ADJ>
__global__ void __launch_bounds__(Tr<T, P>::NT) k_fused(Args a) {
  using R = Tr<T, P>;
  constexpr int L1 = R::L1, H = R::H, NT = R::NT, TP = R::TP, CH = R::CH, HL = L1 / 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* tile = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* stg = tile + R::TILE;
  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int cls = warp;  // 16-point class of this warp

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
  const int cb = sc - a.half - a.margin;  // image column of FFT column 0
  const int K = 2 * a.dx;
  const int mg = a.margin;
  const int64_t hu = ((int64_t)m * n2p + k) * a.E + e;
  const cx<T>* __restrict__ hmain = (const cx<T>*)a.hmain + hu * (int64_t)(P * H);
  const cx<T>* __restrict__ hnyq = (const cx<T>*)a.hnyq + hu * (int64_t)P;
  const T* __restrict__ wt = (const T*)a.wt;
  const cx<T>* __restrict__ twg = (const cx<T>*)a.tw;
  const int64_t npix = (int64_t)a.nx * a.ny;

  if (tid == 0) {
    prefetch_l2(hmain, (unsigned)(sizeof(cx<T>) * P * H));
    prefetch_l2(hnyq, (unsigned)(sizeof(cx<T>) * P));
  }
  // this warp's twiddles w_P^(cls*q), q = 0..15
  cx<T> wq[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) wq[q] = ldg2(twg + cls * q);

  // pairs holding input rows (forward: the window rows only)
  const int jlo = ADJ ? 0 : mg / 2;
  const int jhi = ADJ ? H : (mg + K + 1) / 2;

  // ---- 1. input: staged chunks of pairs -> row step A (variant B forward)
  if (!ADJ) {
    // zero the pairs outside the window rows
    const int nz_lo = jlo, nz_hi = H - jhi;
    for (int i = tid; i < (nz_lo + nz_hi) * P; i += NT) {
      const int jj = i / P, s = i - jj * P;
      const int j = jj < nz_lo ? jj : jhi + (jj - nz_lo);
      tile[j * TP + s] = mkc<T>((T)0, (T)0);
    }
  }
  const int xoff = ADJ ? 0 : mg;     // staging column 0 = FFT column xoff
  const int width = ADJ ? P : K;     // staged columns
  // per-warp column weights of the 16 slots this class reads (forward)
  T wc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int xa = cls + L1 * q - mg;
    wc[q] = (!ADJ && xa >= 0 && xa < K) ? wt[xa] : (T)0;
  }
  for (int j0 = jlo; j0 < jhi; j0 += CH) {
    const int nch = min(CH, jhi - j0);
    {
      // raw window rows (zero outside the field / window) -> staging, asynchronously
      const T* __restrict__ src =
          (const T*)a.in + (ADJ ? ((int64_t)m * a.E + e) : (int64_t)e) * npix;
      for (int i = tid; i < nch * width; i += NT) {
        const int jj = i / width, xs = i - jj * width;
        const int col = cb + xoff + xs;
        const int y0 = 2 * (j0 + jj);
        const int row = rb + y0;
        const bool cok = col >= 0 && col < a.ny;
        const bool ok0 = cok && row >= 0 && row < a.nx && (ADJ || (y0 - mg >= 0 && y0 - mg < K));
        const bool ok1 = cok && row + 1 >= 0 && row + 1 < a.nx &&
                         (ADJ || (y0 + 1 - mg >= 0 && y0 + 1 - mg < K));
        T* d = reinterpret_cast<T*>(stg + jj * TP + xs);
        cp_async<T>(d, ok0 ? src + (int64_t)row * a.ny + col : src, ok0);
        cp_async<T>(d + 1, ok1 ? src + (int64_t)(row + 1) * a.ny + col : src, ok1);
      }
      cp_async_wait_all();
    }
    __syncthreads();
    // step A: items (pair, n1 = cls): x = cls + L1 q -> DFT16 -> twiddle -> slots 16 cls + k2
    for (int jj = lane; jj < nch; jj += 32) {
      const int y0 = 2 * (j0 + jj);
      const T wr0 = (!ADJ && y0 - mg >= 0 && y0 - mg < K) ? wt[y0 - mg] : (T)0;
      const T wr1 = (!ADJ && y0 + 1 - mg >= 0 && y0 + 1 - mg < K) ? wt[y0 + 1 - mg] : (T)0;
      cx<T> v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int xs = cls + L1 * q - xoff;
        if (xs >= 0 && xs < width) {
          const cx<T> t = stg[jj * TP + xs];
          // (w_row * w_col) * x, the order of weights * slices in convolve.py:89-90
          v[q] = ADJ ? t : mkc<T>((wr0 * wc[q]) * t.x, (wr1 * wc[q]) * t.y);
        } else {
          v[q] = mkc<T>((T)0, (T)0);
        }
      }
      Dft<16, false, T>::run(v);
      cx<T>* dst = tile + (j0 + jj) * TP + 16 * cls;
#pragma unroll
      for (int q = 0; q < 16; ++q) dst[q] = q ? cmul<T>(v[q], wq[q]) : v[q];
    }
    __syncthreads();
  }

  // ---- 2. row step B (DFT-L1 per class) fused with the real-to-complex split
  for (int it = tid; it < H * 8; it += NT) {
    const int j = it % H, kap = it / H;
    cx<T>* row = tile + j * TP;
    cx<T> va[L1], vb[L1];
    const int ca = kap == 0 ? 0 : kap, cbk = kap == 0 ? 8 : 16 - kap;
#pragma unroll
    for (int i = 0; i < L1; ++i) {
      va[i] = row[16 * i + ca];
      vb[i] = row[16 * i + cbk];
    }
    Dft<L1, false, T>::run(va);
    Dft<L1, false, T>::run(vb);
    if (kap == 0) {
      // class 0: DC / Nyquist packing and pairs (16 k1, 16 (L1 - k1))
      row[0] = mkc<T>(va[0].x, va[HL].x);
      row[H] = mkc<T>(va[0].y, va[HL].y);
#pragma unroll
      for (int k1 = 1; k1 < HL; ++k1) {
        row[16 * k1] = sp_a<T>(va[k1], va[L1 - k1]);
        row[16 * (k1 + HL)] = sp_b<T>(va[k1], va[L1 - k1]);
      }
      // class 8: pairs (8 + 16 k1, 8 + 16 (L1 - 1 - k1))
#pragma unroll
      for (int k1 = 0; k1 < HL; ++k1) {
        row[8 + 16 * k1] = sp_a<T>(vb[k1], vb[L1 - 1 - k1]);
        row[8 + 16 * (k1 + HL)] = sp_b<T>(vb[k1], vb[L1 - 1 - k1]);
      }
    } else {
#pragma unroll
      for (int k1 = 0; k1 < HL; ++k1) {
        row[kap + 16 * k1] = sp_a<T>(va[k1], vb[L1 - 1 - k1]);
        row[kap + 16 * (k1 + HL)] = sp_b<T>(va[k1], vb[L1 - 1 - k1]);
        row[16 - kap + 16 * k1] = sp_a<T>(vb[k1], va[L1 - 1 - k1]);
        row[16 - kap + 16 * (k1 + HL)] = sp_b<T>(vb[k1], va[L1 - 1 - k1]);
      }
    }
  }
  __syncthreads();

  // ---- 3. column phase 1 (variant A forward): items (c, n2), DFT-L1 over n1
  {
    const int ylo = 2 * jlo, yhi = 2 * jhi;
    for (int it = tid; it < H * 16; it += NT) {
      const int c = it % H, n2 = it / H;
      cx<T> v[L1];
#pragma unroll
      for (int i = 0; i < L1; ++i) {
        const int y = n2 + 16 * i;
        v[i] = (y >= ylo && y < yhi) ? tile[rf<P>(y, c)] : mkc<T>((T)0, (T)0);
      }
      Dft<L1, false, T>::run(v);
#pragma unroll
      for (int i = 0; i < L1; ++i) tile[rf<P>(n2 + 16 * i, c)] = v[i];
    }
  }
  __syncthreads();

  // ---- 4. phase 2 (class k1 = cls) + PSF product + inverse variant-B step A
  for (int c = lane; c < H; c += 32) {
    cx<T> hv[16];
    if (c != 0) {
#pragma unroll
      for (int q = 0; q < 16; ++q) hv[q] = ldg2(hmain + (16 * cls + q) * H + c);
    }
    cx<T> v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const cx<T> t = tile[rf<P>(16 * cls + q, c)];
      v[q] = q ? cmul<T>(t, wq[q]) : t;
    }
    Dft<16, false, T>::run(v);
    if (c != 0) {
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = ADJ ? cmulc<T>(v[q], hv[q]) : cmul<T>(v[q], hv[q]);
      Dft<16, true, T>::run(v);
#pragma unroll
      for (int q = 1; q < 16; ++q) v[q] = cmulc<T>(v[q], wq[q]);
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) tile[rf<P>(16 * cls + q, c)] = v[q];
  }
  __syncthreads();

  // ---- 5. column 0 (warp 0) || inverse variant-B step B for columns >= 1
  if (warp == 0) {
    // unpack W = A + iN into the kx = 0 and kx = P/2 spectra, multiply, repack
    for (int ky = lane; ky <= H; ky += 32) {
      const int s1 = 16 * (ky % L1) + ky / L1;
      const cx<T> h0 = ldg2(hmain + s1 * H), hn = ldg2(hnyq + s1);
      const cx<T> w1 = tile[rf<P>(s1, 0)];
      if (ky == 0 || ky == H) {
        const cx<T> A = ADJ ? cmulc<T>(mkc<T>(w1.x, (T)0), h0) : cmul<T>(mkc<T>(w1.x, (T)0), h0);
        const cx<T> N = ADJ ? cmulc<T>(mkc<T>(w1.y, (T)0), hn) : cmul<T>(mkc<T>(w1.y, (T)0), hn);
        tile[rf<P>(s1, 0)] = cb_p<T>(A, N);
      } else {
        const int km = P - ky;
        const int s2 = 16 * (km % L1) + km / L1;
        const cx<T> w2 = tile[rf<P>(s2, 0)];
        cx<T> A = sp_a<T>(w1, w2), N = sp_b<T>(w1, w2);
        A = ADJ ? cmulc<T>(A, h0) : cmul<T>(A, h0);
        N = ADJ ? cmulc<T>(N, hn) : cmul<T>(N, hn);
        tile[rf<P>(s1, 0)] = cb_p<T>(A, N);
        tile[rf<P>(s2, 0)] = cb_m<T>(A, N);
      }
    }
    __syncwarp();
    // inverse step A for column 0 (lane = class k1)
    if (lane < L1) {
      cx<T> v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = tile[rf<P>(16 * lane + q, 0)];
      Dft<16, true, T>::run(v);
#pragma unroll
      for (int q = 1; q < 16; ++q) v[q] = cmulc<T>(v[q], ldg2(twg + lane * q));
#pragma unroll
      for (int q = 0; q < 16; ++q) tile[rf<P>(16 * lane + q, 0)] = v[q];
    }
    __syncwarp();
    // inverse step B for column 0
    if (lane < 16) {
      cx<T> v[L1];
#pragma unroll
      for (int i = 0; i < L1; ++i) v[i] = tile[rf<P>(16 * i + lane, 0)];
      Dft<L1, true, T>::run(v);
#pragma unroll
      for (int i = 0; i < L1; ++i) tile[rf<P>(16 * i + lane, 0)] = v[i];
    }
  }
  if (NT > 32 || warp == 0) {
    // columns 1..H-1 by warps 1.. (all warps when there is only one)
    const int t0 = NT > 32 ? tid - 32 : tid;
    const int nt = NT > 32 ? NT - 32 : NT;
    if (t0 >= 0) {
      for (int it = t0; it < (H - 1) * 16; it += nt) {
        const int c = 1 + it % (H - 1), q = it / (H - 1);
        cx<T> v[L1];
#pragma unroll
        for (int i = 0; i < L1; ++i) v[i] = tile[rf<P>(16 * i + q, c)];
        Dft<L1, true, T>::run(v);
#pragma unroll
        for (int i = 0; i < L1; ++i) tile[rf<P>(16 * i + q, c)] = v[i];
      }
    }
  }
  __syncthreads();

  // ---- 6. combine (Hermitian pair rows) fused with inverse variant-A phase 1
  {
    const int jc_lo = ADJ ? mg / 2 : 0;
    const int jc_hi = ADJ ? (mg + K + 1) / 2 : H;
    const int ncp = jc_hi - jc_lo;
    for (int it = tid; it < ncp * 8; it += NT) {
      const int j = jc_lo + it % ncp, kap = it / ncp;
      cx<T>* row = tile + j * TP;
      cx<T> va[L1], vb[L1];
      if (kap == 0) {
        const cx<T> a0 = row[0], b0 = row[H];
        va[0] = mkc<T>(a0.x, b0.x);
        va[HL] = mkc<T>(a0.y, b0.y);
#pragma unroll
        for (int k1 = 1; k1 < HL; ++k1) {
          const cx<T> A = row[16 * k1], B = row[16 * (k1 + HL)];
          va[k1] = cb_p<T>(A, B);
          va[L1 - k1] = cb_m<T>(A, B);
        }
#pragma unroll
        for (int k1 = 0; k1 < HL; ++k1) {
          const cx<T> A = row[8 + 16 * k1], B = row[8 + 16 * (k1 + HL)];
          vb[k1] = cb_p<T>(A, B);
          vb[L1 - 1 - k1] = cb_m<T>(A, B);
        }
      } else {
#pragma unroll
        for (int k1 = 0; k1 < HL; ++k1) {
          const cx<T> A = row[kap + 16 * k1], B = row[kap + 16 * (k1 + HL)];
          va[k1] = cb_p<T>(A, B);
          vb[L1 - 1 - k1] = cb_m<T>(A, B);
          const cx<T> A2 = row[16 - kap + 16 * k1], B2 = row[16 - kap + 16 * (k1 + HL)];
          vb[k1] = cb_p<T>(A2, B2);
          va[L1 - 1 - k1] = cb_m<T>(A2, B2);
        }
      }
      Dft<L1, true, T>::run(va);
      Dft<L1, true, T>::run(vb);
      const int ca = kap == 0 ? 0 : kap, cbk = kap == 0 ? 8 : 16 - kap;
#pragma unroll
      for (int i = 0; i < L1; ++i) {
        row[ca + 16 * i] = va[i];
        row[cbk + 16 * i] = vb[i];
      }
    }
  }
  __syncthreads();

  // ---- 7. inverse variant-A phase 2 -> natural-order staging -> global
  const T scale = (T)a.scale;
  // 16-byte reductions need column groups aligned in memory and inside the field
  const bool vec4 = ((cb + (ADJ ? mg : 0)) % 4 == 0) && (a.ny % 4 == 0) &&
                    (((uintptr_t)a.out) % 16 == 0) && (ADJ ? K % 4 == 0 : true);
  const int jo_lo = ADJ ? mg / 2 : 0;
  const int jo_hi = ADJ ? (mg + K + 1) / 2 : H;
  for (int j0 = jo_lo; j0 < jo_hi; j0 += CH) {
    const int nch = min(CH, jo_hi - j0);
    for (int jj = lane; jj < nch; jj += 32) {
      const cx<T>* srcr = tile + (j0 + jj) * TP + 16 * cls;
      cx<T> v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = q ? cmulc<T>(srcr[q], wq[q]) : srcr[q];
      Dft<16, true, T>::run(v);
#pragma unroll
      for (int q = 0; q < 16; ++q) stg[jj * TP + cls + L1 * q] = v[q];
    }
    __syncthreads();
    if (!ADJ) {
      T* __restrict__ dst = (T*)a.out + ((int64_t)m * a.E + e) * npix;
      if (sizeof(T) == 4 && vec4) {
        // groups of 4 columns never straddle the field edge (cb, ny multiples of 4)
        for (int i = tid; i < nch * (P / 4); i += NT) {
          const int jj = i / (P / 4), x = 4 * (i - jj * (P / 4));
          const int col = cb + x;
          if (col < 0 || col >= a.ny) continue;
          const cx<T> z0 = stg[jj * TP + x], z1 = stg[jj * TP + x + 1];
          const cx<T> z2 = stg[jj * TP + x + 2], z3 = stg[jj * TP + x + 3];
          const int row = rb + 2 * (j0 + jj);
          if (row >= 0 && row < a.nx)
            red_add_v4((float*)(dst + (int64_t)row * a.ny + col), scale * z0.x, scale * z1.x,
                       scale * z2.x, scale * z3.x);
          if (row + 1 >= 0 && row + 1 < a.nx)
            red_add_v4((float*)(dst + (int64_t)(row + 1) * a.ny + col), scale * z0.y,
                       scale * z1.y, scale * z2.y, scale * z3.y);
        }
      } else {
        for (int i = tid; i < nch * P; i += NT) {
          const int jj = i / P, x = i - jj * P;
          const int col = cb + x;
          if (col < 0 || col >= a.ny) continue;
          const cx<T> z = stg[jj * TP + x];
          const int row = rb + 2 * (j0 + jj);
          if (row >= 0 && row < a.nx) atomicAdd(dst + (int64_t)row * a.ny + col, scale * z.x);
          if (row + 1 >= 0 && row + 1 < a.nx)
            atomicAdd(dst + (int64_t)(row + 1) * a.ny + col, scale * z.y);
        }
      }
    } else {
      T* __restrict__ dst = (T*)a.out + (int64_t)e * npix;
      if (sizeof(T) == 4 && vec4) {
        for (int i = tid; i < nch * (K / 4); i += NT) {
          const int jj = i / (K / 4), xa = 4 * (i - jj * (K / 4));
          const int x = xa + mg, col = cb + x;
          if (col < 0 || col >= a.ny) continue;
          const int y0 = 2 * (j0 + jj);
          const int ya = y0 - mg, row = rb + y0;
          cx<T> z[4];
          T w4[4];
#pragma unroll
          for (int t = 0; t < 4; ++t) {
            z[t] = stg[jj * TP + x + t];
            w4[t] = wt[xa + t] * scale;
          }
          if (ya >= 0 && ya < K && row >= 0 && row < a.nx) {
            const T wy = wt[ya];
            red_add_v4((float*)(dst + (int64_t)row * a.ny + col), (wy * w4[0]) * z[0].x,
                       (wy * w4[1]) * z[1].x, (wy * w4[2]) * z[2].x, (wy * w4[3]) * z[3].x);
          }
          if (ya + 1 >= 0 && ya + 1 < K && row + 1 >= 0 && row + 1 < a.nx) {
            const T wy = wt[ya + 1];
            red_add_v4((float*)(dst + (int64_t)(row + 1) * a.ny + col), (wy * w4[0]) * z[0].y,
                       (wy * w4[1]) * z[1].y, (wy * w4[2]) * z[2].y, (wy * w4[3]) * z[3].y);
          }
        }
      } else {
        for (int i = tid; i < nch * K; i += NT) {
          const int jj = i / K, xa = i - jj * K;
          const int x = xa + mg, col = cb + x;
          if (col < 0 || col >= a.ny) continue;
          const cx<T> z = stg[jj * TP + x];
          const T wx = wt[xa] * scale;
          const int y0 = 2 * (j0 + jj);
          const int ya = y0 - mg, row = rb + y0;
          if (ya >= 0 && ya < K && row >= 0 && row < a.nx)
            atomicAdd(dst + (int64_t)row * a.ny + col, (wt[ya] * wx) * z.x);
          if (ya + 1 >= 0 && ya + 1 < K && row + 1 >= 0 && row + 1 < a.nx)
            atomicAdd(dst + (int64_t)(row + 1) * a.ny + col, (wt[ya + 1] * wx) * z.y);
        }
      }
    }
    __syncthreads();
  }
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
  const size_t smem = Tr<T, P>::SMEM;
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
  k_fused<T, P, ADJ><<<(unsigned)units, Tr<T, P>::NT, smem, s>>>(a);
  return cuda_status(cudaGetLastError(), "k_fused launch");
}

template <typename T, bool ADJ>
int dispatch(const Geom& g, const FusedLaunch& f, cudaStream_t s) {
  switch (g.P) {
    case 32: return launch_one<T, 32, ADJ>(g, f, s);
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
    case 32: case 64: case 96: case 128: return true;
    case 192: return dtype == JUBIK_F32;
    default: return false;
  }
}

size_t fused_smem_bytes(int P, int dtype) {
  const size_t c = dtype == JUBIK_F32 ? 8 : 16;
  const size_t H = P / 2, TP = P + 1, CH = H < 32 ? H : 32;
  return c * (H * TP + CH * TP);
}

int fused_forward(const Geom& g, int dtype, const FusedLaunch& a, cudaStream_t s) {
  return dtype == JUBIK_F32 ? dispatch<float, false>(g, a, s) : dispatch<double, false>(g, a, s);
}

int fused_adjoint(const Geom& g, int dtype, const FusedLaunch& a, cudaStream_t s) {
  return dtype == JUBIK_F32 ? dispatch<float, true>(g, a, s) : dispatch<double, true>(g, a, s);
}

}  // namespace jubik
