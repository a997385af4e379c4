// Batched complex FFTs of arbitrary supported length (mixed radix 4/2/3 with
// generic odd radices up to 64), Stockham auto-sort in shared memory; lengths
// 16 L1 with a register codelet for L1 use a two-pass four-step kernel.
//
// This is the "plain" transform: it stands in for the jnp.fft.fftn / ifftn
// calls of jubik/convolve.py:165-174 (complex, full size, unnormalised
// forward; the caller applies the 1/N of ifftn through `scale`).  It is used
// by the unfused path, by the FP64 PSF-spectrum preparation of every plan and
// by the stand-alone convolve.  Stage s with radix r and running length Ns:
//   v_q = in[j + q L/r] * w^(q k),  k = j mod Ns,  w = exp(-2 pi i / (Ns r))
//   out[(j / Ns) Ns r + k + q Ns] = DFT_r(v)_q
#include <atomic>
#include <cmath>
#include <cstdio>
#include <vector>

#include "fft_codelets.cuh"
#include "internal.h"

namespace jubik {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxSeqPerBlock = 64;  // sequences one block transforms (spc <= 64)

// Division by a divisor d fixed for the kernel, as one multiply-high: with
// m = floor(2^32 / d) + 1, floor(n / d) = (n m) >> 32 exactly whenever n d < 2^32
// (here n < 2^18 and d <= 4096).  d = 1 passes n through.
struct Divider {
  uint32_t d, m;
  __device__ __forceinline__ explicit Divider(uint32_t div)
      : d(div), m(div > 1 ? (uint32_t)(0x100000000ull / div + 1) : 0u) {}
  __device__ __forceinline__ uint32_t div(uint32_t n) const { return d > 1 ? __umulhi(n, m) : n; }
};

// Asynchronous global -> shared copy of one complex value (8 or 16 bytes): the
// staging loops issue every load of a thread before any of them is waited for.
template <typename T>
__device__ __forceinline__ void cp_async_cx(cx<T>* smem, const cx<T>* gmem) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(cx<T>) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

template <int R, typename T>
__device__ __forceinline__ void bfly(const cx<T>* __restrict__ src, cx<T>* __restrict__ dst,
                                     int j, int Lr, int Ns, int tstep,
                                     const cx<T>* __restrict__ tw, bool inv) {
  const int k = j % Ns;
  cx<T> v[R];
#pragma unroll
  for (int q = 0; q < R; ++q) v[q] = src[j + q * Lr];
#pragma unroll
  for (int q = 1; q < R; ++q) {
    cx<T> w = tw[q * k * tstep];
    v[q] = inv ? cmulc<T>(v[q], w) : cmul<T>(v[q], w);
  }
  if (inv)
    Dft<R, true, T>::run(v);
  else
    Dft<R, false, T>::run(v);
  const int base = (j / Ns) * Ns * R + k;
#pragma unroll
  for (int q = 0; q < R; ++q) dst[base + q * Ns] = v[q];
}

// Generic radix r (odd prime up to kMaxGenericRadix): direct r-point DFT with
// the length-L twiddle table (w_r^t = tw[t * L / r]).
template <typename T>
__device__ void bfly_generic(const cx<T>* __restrict__ src, cx<T>* __restrict__ dst, int j,
                             int L, int r, int Ns, const cx<T>* __restrict__ tw, bool inv) {
  const int Lr = L / r;
  const int k = j % Ns;
  const int tstep = L / (Ns * r);
  cx<T> v[kMaxGenericRadix];
  for (int q = 0; q < r; ++q) {
    cx<T> a = src[j + q * Lr];
    if (q > 0) {
      cx<T> w = tw[q * k * tstep];
      a = inv ? cmulc<T>(a, w) : cmul<T>(a, w);
    }
    v[q] = a;
  }
  const int base = (j / Ns) * Ns * r + k;
  for (int kk = 0; kk < r; ++kk) {
    cx<T> acc = v[0];
    for (int q = 1; q < r; ++q) {
      cx<T> w = tw[((q * kk) % r) * Lr];
      acc = cadd<T>(acc, inv ? cmulc<T>(v[q], w) : cmul<T>(v[q], w));
    }
    dst[base + kk * Ns] = acc;
  }
}

template <typename T>
__global__ void __launch_bounds__(kThreads)
    k_fft_batched(cx<T>* __restrict__ data, int64_t nseq, int L, int nb, int64_t sa, int64_t sb,
                  int64_t se, const cx<T>* __restrict__ tw, FftStages st, int inv, T scale,
                  int spc) {
  extern __shared__ unsigned char smem_raw[];
  // odd pitch per sequence: staging strided sequences one lane per sequence
  // has no bank conflicts
  const int LP = L | 1;
  cx<T>* b0 = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* b1 = b0 + (size_t)spc * LP;
  const int64_t s0 = (int64_t)blockIdx.x * spc;
  const int ns = (int)min((int64_t)spc, nseq - s0);
  const bool seq_fast = (se != 1);
  const Divider dns((uint32_t)ns), dL((uint32_t)L);
  // start offset of each of the block's sequences (one 64-bit division per sequence)
  __shared__ int64_t seq_base[kMaxSeqPerBlock];
  for (int sq = threadIdx.x; sq < ns; sq += blockDim.x) {
    const int64_t q = s0 + sq;
    seq_base[sq] = (q / nb) * sa + (q % nb) * sb;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < ns * L; idx += blockDim.x) {
    int s, i;
    if (seq_fast) {
      i = (int)dns.div((uint32_t)idx);
      s = idx - i * ns;
    } else {
      s = (int)dL.div((uint32_t)idx);
      i = idx - s * L;
    }
    cp_async_cx<T>(b0 + s * LP + i, data + seq_base[s] + (int64_t)i * se);
  }
  cp_async_wait_all();
  __syncthreads();
  cx<T>* in = b0;
  cx<T>* out = b1;
  int Ns = 1;
  for (int stg = 0; stg < st.n; ++stg) {
    const int r = st.r[stg];
    const int Lr = L / r;
    const int tstep = L / (Ns * r);
    const Divider dLr((uint32_t)Lr);
    for (int b = threadIdx.x; b < ns * Lr; b += blockDim.x) {
      const int s = (int)dLr.div((uint32_t)b);
      const int j = b - s * Lr;
      const cx<T>* src = in + s * LP;
      cx<T>* dst = out + s * LP;
      switch (r) {
        case 2: bfly<2, T>(src, dst, j, Lr, Ns, tstep, tw, inv); break;
        case 3: bfly<3, T>(src, dst, j, Lr, Ns, tstep, tw, inv); break;
        case 4: bfly<4, T>(src, dst, j, Lr, Ns, tstep, tw, inv); break;
        case 5: bfly<5, T>(src, dst, j, Lr, Ns, tstep, tw, inv); break;
        case 7: bfly<7, T>(src, dst, j, Lr, Ns, tstep, tw, inv); break;
        case 8: bfly<8, T>(src, dst, j, Lr, Ns, tstep, tw, inv); break;
        case 9: bfly<9, T>(src, dst, j, Lr, Ns, tstep, tw, inv); break;
        case 11: bfly<11, T>(src, dst, j, Lr, Ns, tstep, tw, inv); break;
        default: bfly_generic<T>(src, dst, j, L, r, Ns, tw, inv); break;
      }
    }
    __syncthreads();
    cx<T>* t = in;
    in = out;
    out = t;
    Ns *= r;
  }
  for (int idx = threadIdx.x; idx < ns * L; idx += blockDim.x) {
    int s, i;
    if (seq_fast) {
      i = (int)dns.div((uint32_t)idx);
      s = idx - i * ns;
    } else {
      s = (int)dL.div((uint32_t)idx);
      i = idx - s * L;
    }
    cx<T> v = in[s * LP + i];
    data[seq_base[s] + (int64_t)i * se] = mkc<T>(v.x * scale, v.y * scale);
  }
}

// The two register passes of the four-step length-16 L1 transform of ns
// sequences staged at pitch L + 1 in bx (by: scratch of 16 Q per sequence);
// the result is back in bx, in natural order.
template <typename T, int L1, bool INV>
__device__ __forceinline__ void fft4_passes(cx<T>* bx, cx<T>* by, int ns,
                                            const cx<T>* __restrict__ tw) {
  constexpr int L = 16 * L1;
  constexpr int LP = L + 1;
  constexpr int Q = (L1 % 2 == 0) ? L1 + 1 : L1 + 2;
  constexpr int LY = 16 * Q;
  for (int it = threadIdx.x; it < ns * L1; it += blockDim.x) {
    const int sq = it / L1, n1 = it - sq * L1;
    const cx<T>* src = bx + sq * LP + n1;
    cx<T> v[16];
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) v[n2] = src[L1 * n2];
    Dft<16, INV, T>::run(v);
    cx<T>* dst = by + sq * LY + n1;
    dst[0] = v[0];
#pragma unroll
    for (int k2 = 1; k2 < 16; ++k2) {
      const cx<T> w = tw[n1 * k2];
      dst[Q * k2] = INV ? cmulc<T>(v[k2], w) : cmul<T>(v[k2], w);
    }
  }
  __syncthreads();
  for (int it = threadIdx.x; it < ns * 16; it += blockDim.x) {
    const int sq = it >> 4, k2 = it & 15;
    const cx<T>* src = by + sq * LY + Q * k2;
    cx<T> v[L1];
#pragma unroll
    for (int n1 = 0; n1 < L1; ++n1) v[n1] = src[n1];
    Dft<L1, INV, T>::run(v);
    cx<T>* dst = bx + sq * LP + k2;
#pragma unroll
    for (int k1 = 0; k1 < L1; ++k1) dst[16 * k1] = v[k1];
  }
  __syncthreads();
}

// Batched complex FFTs of length L = 16 L1 in two register passes (four-step),
// x[n1 + L1 n2]:
//   pass 1, per (sequence, n1): DFT-16 over n2, times w_L^(n1 k2)
//           -> Y[n1 + Q k2]  (row pitch Q = L1 + 1 or L1 + 2, odd: no bank conflicts)
//   pass 2, per (sequence, k2): DFT-L1 over n1 -> X[k2 + 16 k1]
// Each pass is compile-time indexed, against the generic kernel's log_r L
// passes with run-time radix and index arithmetic.
template <typename T, int L1, bool INV>
__global__ void __launch_bounds__(kThreads)
    k_fft4(cx<T>* __restrict__ data, int64_t nseq, int nb, int64_t sa, int64_t sb, int64_t se,
           const cx<T>* __restrict__ tw, T scale, int spc) {
  constexpr int L = 16 * L1;
  constexpr int LP = L + 1;  // odd pitch of a sequence in bx: the column-major staging of
                             // strided sequences (one lane per sequence) has no bank conflicts
  extern __shared__ unsigned char smem_raw[];
  cx<T>* bx = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* by = bx + (size_t)spc * LP;
  const int64_t s0 = (int64_t)blockIdx.x * spc;
  const int ns = (int)min((int64_t)spc, nseq - s0);
  const bool seq_fast = (se != 1);
  const Divider dns((uint32_t)ns), dL((uint32_t)L);
  __shared__ int64_t seq_base[kMaxSeqPerBlock];
  for (int sq = threadIdx.x; sq < ns; sq += blockDim.x) {
    const int64_t q = s0 + sq;
    seq_base[sq] = (q / nb) * sa + (q % nb) * sb;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < ns * L; idx += blockDim.x) {
    int sq, i;
    if (seq_fast) {
      i = (int)dns.div((uint32_t)idx);
      sq = idx - i * ns;
    } else {
      sq = (int)dL.div((uint32_t)idx);
      i = idx - sq * L;
    }
    cp_async_cx<T>(bx + sq * LP + i, data + seq_base[sq] + (int64_t)i * se);
  }
  cp_async_wait_all();
  __syncthreads();
  fft4_passes<T, L1, INV>(bx, by, ns, tw);
  for (int idx = threadIdx.x; idx < ns * L; idx += blockDim.x) {
    int sq, i;
    if (seq_fast) {
      i = (int)dns.div((uint32_t)idx);
      sq = idx - i * ns;
    } else {
      sq = (int)dL.div((uint32_t)idx);
      i = idx - sq * L;
    }
    const cx<T> v = bx[sq * LP + i];
    data[seq_base[sq] + (int64_t)i * se] = mkc<T>(v.x * scale, v.y * scale);
  }
}

template <typename T, int L1, bool INV>
int launch_fft4(void* data, int64_t nseq, int nb, int64_t sa, int64_t sb, int64_t se,
                const cx<T>* tw, double scale, int smax, cudaStream_t s) {
  constexpr int L = 16 * L1;
  constexpr int Q = (L1 % 2 == 0) ? L1 + 1 : L1 + 2;
  const size_t per = sizeof(cx<T>) * (size_t)(L + 1 + 16 * Q);
  // (1 KB of the block's shared memory stays for the static sequence offsets)
  int spc = (int)std::min<size_t>(16, (size_t)(smax - 1024) / per);
  if (spc < 1) {
    set_error("FFT length %d needs %zu bytes of shared memory", L, per);
    return JUBIK_ERR_UNSUPPORTED;
  }
  const size_t smem = per * spc;
  auto kern = k_fft4<T, L1, INV>;
  if (smem > 47 * 1024)
    JUBIK_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
  const int64_t blocks = (nseq + spc - 1) / spc;
  if (blocks > 0x7fffffffLL) {
    set_error("too many FFT sequences");
    return JUBIK_ERR_UNSUPPORTED;
  }
  kern<<<(unsigned)blocks, kThreads, smem, s>>>((cx<T>*)data, nseq, nb, sa, sb, se, tw, (T)scale,
                                                spc);
  return cuda_status(cudaGetLastError(), "k_fft4 launch");
}

// Forward row pass of the unfused path with its rows read straight from the
// images (the windows k_plain_sky_patches and k_plain_cot_patches write, without
// the round trip through a pair buffer).  Sequence q = (chunk module mm, pair j,
// row y): its real part is row y of patch 2j's P x P window, its imaginary part
// that of patch 2j + 1 (zero if there is none), both zero outside the field.
// Windows are cut as in convolve.py:86-104: the window of patch (r, c) starts at
// (min(r dx, sr_max) - half - margin, min(c dx, sc_max) - half - margin).
// module_axis: the image is (M, E, nx, ny) and the chunk starts at module m0;
// else (E, nx, ny).  wt != nullptr: the sky's window weights, (wt[ya] wt[xa]) x
// inside the 2dx window at offset margin (ya = y - margin, xa = x - margin), 0
// outside it.  Output: (nm, pairs, P, P), row-transformed.
struct RowWindows {
  int E, n, nx, ny, dx, margin, half, sr_max, sc_max, K;
  int m0, module_axis;
  int64_t nph;
};

template <typename T>
__device__ __forceinline__ void cp_async_real(T* smem, const T* gmem, bool ok) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
  const int n = ok ? (int)sizeof(T) : 0;  // 0: zero fill, nothing read
  if constexpr (sizeof(T) == 4)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(gmem), "r"(n)
                 : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(gmem), "r"(n)
                 : "memory");
}

template <typename T, int L1>
__global__ void __launch_bounds__(kThreads)
    k_fft4_rows_win(const T* __restrict__ img, const T* __restrict__ wt, RowWindows w,
                    int64_t nseq, const cx<T>* __restrict__ tw, int spc,
                    cx<T>* __restrict__ out) {
  constexpr int L = 16 * L1;
  constexpr int LP = L + 1;
  extern __shared__ unsigned char smem_raw[];
  cx<T>* bx = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* by = bx + (size_t)spc * LP;
  __shared__ int64_t row_off[2][kMaxSeqPerBlock];  // element offset of the image row, -1: zero
  __shared__ int col0[2][kMaxSeqPerBlock];         // image column of window column 0
  __shared__ T row_w[kMaxSeqPerBlock];             // wt[y - margin] (weighted rows)
  const int64_t s0 = (int64_t)blockIdx.x * spc;
  const int ns = (int)min((int64_t)spc, nseq - s0);
  const int n2p = w.n * w.n, np = w.E * n2p;
  for (int sq = threadIdx.x; sq < ns; sq += blockDim.x) {
    const int64_t q = s0 + sq;
    const int y = (int)(q % L);
    const int64_t up = q / L;
    const int64_t j = up % w.nph;
    const int64_t mm = up / w.nph;
    const int ya = y - w.margin;
    const bool row_in = wt == nullptr || (ya >= 0 && ya < w.K);
    row_w[sq] = (wt != nullptr && row_in) ? wt[ya] : (T)1;
    for (int part = 0; part < 2; ++part) {
      const int p = (int)(2 * j + part);
      int64_t off = -1;
      int c0 = 0;
      if (p < np && row_in) {
        const int k = p % n2p, e = p / n2p;
        const int rb = min((k % w.n) * w.dx, w.sr_max) - w.half - w.margin;
        c0 = min((k / w.n) * w.dx, w.sc_max) - w.half - w.margin;
        const int row = rb + y;
        if (row >= 0 && row < w.nx) {
          const int64_t plane = w.module_axis ? (int64_t)(w.m0 + mm) * w.E + e : (int64_t)e;
          off = (plane * w.nx + row) * (int64_t)w.ny;
        }
      }
      row_off[part][sq] = off;
      col0[part][sq] = c0;
    }
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < ns * L; idx += blockDim.x) {
    const int sq = idx / L, x = idx - sq * L;
    const bool col_in = wt == nullptr || (x - w.margin >= 0 && x - w.margin < w.K);
    T* dst = reinterpret_cast<T*>(bx + sq * LP + x);
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      const int64_t off = row_off[part][sq];
      const int col = col0[part][sq] + x;
      const bool ok = off >= 0 && col_in && col >= 0 && col < w.ny;
      cp_async_real<T>(dst + part, ok ? img + off + col : img, ok);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  if (wt != nullptr) {
    for (int idx = threadIdx.x; idx < ns * L; idx += blockDim.x) {
      const int sq = idx / L, x = idx - sq * L;
      const int xa = x - w.margin;
      cx<T>& v = bx[sq * LP + x];
      if (xa >= 0 && xa < w.K) {
        const T wgt = row_w[sq] * wt[xa];
        v = mkc<T>(wgt * v.x, wgt * v.y);
      } else {
        v = mkc<T>((T)0, (T)0);
      }
    }
    __syncthreads();
  }
  fft4_passes<T, L1, false>(bx, by, ns, tw);
  for (int idx = threadIdx.x; idx < ns * L; idx += blockDim.x) {
    const int sq = idx / L, x = idx - sq * L;
    out[(s0 + sq) * L + x] = bx[sq * LP + x];
  }
}

template <typename T, int L1>
int launch_rows_win(const Geom& g, const void* img, bool module_axis, const void* wt, int m0,
                    int nm, const cx<T>* tw, int smax, void* out, cudaStream_t s) {
  constexpr int L = 16 * L1;
  constexpr int Q = (L1 % 2 == 0) ? L1 + 1 : L1 + 2;
  const size_t per = sizeof(cx<T>) * (size_t)(L + 1 + 16 * Q);
  // (2 KB of the block's shared memory stay for the static per-sequence tables)
  const int spc = (int)std::min<size_t>(16, (size_t)(smax - 2048) / per);
  if (spc < 1) {
    set_error("FFT length %d needs %zu bytes of shared memory", L, per);
    return JUBIK_ERR_UNSUPPORTED;
  }
  RowWindows w{g.E, g.n, g.nx, g.ny, g.dx, g.margin, g.half, g.sr_max, g.sc_max, g.K,
               m0, module_axis ? 1 : 0, plain_pairs(g)};
  const int64_t nseq = (int64_t)nm * w.nph * L;
  const size_t smem = per * spc;
  auto kern = k_fft4_rows_win<T, L1>;
  if (smem > 47 * 1024)
    JUBIK_TRY_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smem));
  const int64_t blocks = (nseq + spc - 1) / spc;
  if (blocks > 0x7fffffffLL) {
    set_error("too many FFT sequences");
    return JUBIK_ERR_UNSUPPORTED;
  }
  kern<<<(unsigned)blocks, kThreads, smem, s>>>((const T*)img, (const T*)wt, w, nseq, tw, spc,
                                                (cx<T>*)out);
  return cuda_status(cudaGetLastError(), "k_fft4_rows_win launch");
}

// lengths 16 L1 with a DFT-L1 codelet take the two-pass kernel; 0 = not covered
template <typename T, bool INV>
int try_fft4(int L, void* data, int64_t nseq, int nb, int64_t sa, int64_t sb, int64_t se,
             const cx<T>* tw, double scale, int smax, cudaStream_t s, bool* done) {
  *done = true;
  switch (L) {
    case 32: return launch_fft4<T, 2, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 48: return launch_fft4<T, 3, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 64: return launch_fft4<T, 4, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 80: return launch_fft4<T, 5, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 96: return launch_fft4<T, 6, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 128: return launch_fft4<T, 8, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 160: return launch_fft4<T, 10, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 192: return launch_fft4<T, 12, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 256: return launch_fft4<T, 16, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 320: return launch_fft4<T, 20, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 384: return launch_fft4<T, 24, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    case 512: return launch_fft4<T, 32, INV>(data, nseq, nb, sa, sb, se, tw, scale, smax, s);
    default: *done = false; return JUBIK_OK;
  }
}

bool factorize(int L, FftStages* st) {
  st->n = 0;
  if (L < 1) return false;
  int rem = L;
  auto push = [&](int r) {
    if (st->n >= kMaxStages) return false;
    st->r[st->n++] = r;
    return true;
  };
  // larger register codelets first: fewer passes through shared memory
  while (rem % 8 == 0) {
    if (!push(8)) return false;
    rem /= 8;
  }
  while (rem % 4 == 0) {
    if (!push(4)) return false;
    rem /= 4;
  }
  while (rem % 2 == 0) {
    if (!push(2)) return false;
    rem /= 2;
  }
  while (rem % 9 == 0) {
    if (!push(9)) return false;
    rem /= 9;
  }
  while (rem % 3 == 0) {
    if (!push(3)) return false;
    rem /= 3;
  }
  for (int p = 5; rem > 1 && p <= kMaxGenericRadix; p += 2) {
    while (rem % p == 0) {
      if (!push(p)) return false;
      rem /= p;
    }
  }
  return rem == 1;
}

constexpr int kMaxL = 4096;

// Opt-in shared memory per block of the current device (cached per device).
int max_smem_optin() {
  constexpr int kMaxDev = 64;
  static std::atomic<int> cache[kMaxDev];  // 0 = not looked up yet
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return 48 * 1024;
  int v = cache[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess ||
        v <= 0) {
      cudaGetLastError();
      v = 48 * 1024;
    }
    cache[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

}  // namespace

bool fft_length_supported(int L) {
  FftStages st;
  return L >= 1 && L <= kMaxL && factorize(L, &st);
}

int fft1d_init(Fft1D* f, int L) {
  if (!fft_length_supported(L)) {
    set_error("FFT length %d unsupported (needs prime factors <= %d and L <= %d)", L,
              kMaxGenericRadix, kMaxL);
    return JUBIK_ERR_UNSUPPORTED;
  }
  f->L = L;
  factorize(L, &f->st);
  std::vector<float2> t32(L);
  std::vector<double2> t64(L);
  const long double twopi = 6.283185307179586476925286766559005768L;
  for (int t = 0; t < L; ++t) {
    const long double a = twopi * (long double)t / (long double)L;
    const long double c = cosl(a), s = -sinl(a);
    t64[t] = make_double2((double)c, (double)s);
    t32[t] = make_float2((float)c, (float)s);
  }
  f->tw32 = f->tw64 = nullptr;
  cudaError_t e = cudaMalloc(&f->tw32, sizeof(float2) * L);
  if (e == cudaSuccess) e = cudaMalloc(&f->tw64, sizeof(double2) * L);
  if (e == cudaSuccess)
    e = cudaMemcpy(f->tw32, t32.data(), sizeof(float2) * L, cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(f->tw64, t64.data(), sizeof(double2) * L, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {  // release whatever was allocated before the failure
    fft1d_free(f);
    return cuda_status(e, "fft1d_init");
  }
  return JUBIK_OK;
}

// Twiddles w_L^t = exp(-2 pi i t / L) computed on the device in FP64
// (sincospi) and rounded once to FP32.
__global__ void k_twiddles(float2* tw32, double2* tw64, int L) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < L; t += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(2.0 * (double)t / (double)L, &s, &c);
    tw64[t] = make_double2(c, -s);
    tw32[t] = make_float2((float)c, (float)-s);
  }
}

int fft1d_init_external(Fft1D* f, int L, void* tw32, void* tw64, cudaStream_t s) {
  if (!fft_length_supported(L)) {
    set_error("FFT length %d unsupported (needs prime factors <= %d and L <= %d)", L,
              kMaxGenericRadix, kMaxL);
    return JUBIK_ERR_UNSUPPORTED;
  }
  f->L = L;
  factorize(L, &f->st);
  f->tw32 = tw32;
  f->tw64 = tw64;
  k_twiddles<<<(L + 255) / 256, 256, 0, s>>>((float2*)tw32, (double2*)tw64, L);
  return cuda_status(cudaGetLastError(), "k_twiddles");
}

void fft1d_free(Fft1D* f) {
  if (f->tw32) cudaFree(f->tw32);
  if (f->tw64) cudaFree(f->tw64);
  f->tw32 = f->tw64 = nullptr;
  f->L = 0;
}

template <typename T>
int fft_batched(const Fft1D& f, void* data, int64_t nseq, int nb, int64_t sa, int64_t sb,
                int64_t se, bool inverse, double scale, cudaStream_t s) {
  if (nseq <= 0) return JUBIK_OK;
  const int L = f.L;
  const int smax = max_smem_optin();
  {
    const cx<T>* tw = (const cx<T>*)(sizeof(T) == 4 ? f.tw32 : f.tw64);
    bool done = false;
    const int st = inverse ? try_fft4<T, true>(L, data, nseq, nb, sa, sb, se, tw, scale, smax, s,
                                               &done)
                           : try_fft4<T, false>(L, data, nseq, nb, sa, sb, se, tw, scale, smax,
                                                s, &done);
    if (done) return st;
  }
  const size_t per = 2 * sizeof(cx<T>) * (size_t)(L | 1);
  // (1 KB of the block's shared memory stays for the static sequence offsets)
  int spc = (int)std::max<size_t>(1, std::min<size_t>(64, (size_t)(47 * 1024) / per));
  if (per + 1024 > (size_t)smax) {
    set_error("FFT length %d needs %zu bytes of shared memory", L, per);
    return JUBIK_ERR_UNSUPPORTED;
  }
  const size_t smem = per * spc;
  if (smem > 47 * 1024) {
    JUBIK_TRY_CUDA(cudaFuncSetAttribute(k_fft_batched<T>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  }
  const int64_t blocks = (nseq + spc - 1) / spc;
  if (blocks > 0x7fffffffLL) {
    set_error("too many FFT sequences");
    return JUBIK_ERR_UNSUPPORTED;
  }
  const cx<T>* tw = (const cx<T>*)(sizeof(T) == 4 ? f.tw32 : f.tw64);
  k_fft_batched<T><<<(unsigned)blocks, kThreads, smem, s>>>((cx<T>*)data, nseq, L, nb, sa, sb, se,
                                                           tw, f.st, inverse ? 1 : 0, (T)scale,
                                                           spc);
  return cuda_status(cudaGetLastError(), "k_fft_batched launch");
}

template <typename T>
int fft2_batched(const Fft1D& fh, const Fft1D& fw, void* data, int64_t batch, bool inverse,
                 cudaStream_t s) {
  const int64_t h = fh.L, w = fw.L;
  // rows: sequences (b, y), contiguous
  JUBIK_TRY(fft_batched<T>(fw, data, batch * h, (int)h, h * w, w, 1, inverse, 1.0, s));
  // columns: sequences (b, x), stride w
  JUBIK_TRY(fft_batched<T>(fh, data, batch * w, (int)w, h * w, 1, w, inverse, 1.0, s));
  return JUBIK_OK;
}

template <typename T>
int fft_rows_windows(const Fft1D& f, const Geom& g, const void* img, bool module_axis,
                     const void* wt, int m0, int nm, void* out, cudaStream_t s) {
  const cx<T>* tw = (const cx<T>*)(sizeof(T) == 4 ? f.tw32 : f.tw64);
  const int smax = max_smem_optin();
  switch (f.L) {
    case 160: return launch_rows_win<T, 10>(g, img, module_axis, wt, m0, nm, tw, smax, out, s);
    case 192: return launch_rows_win<T, 12>(g, img, module_axis, wt, m0, nm, tw, smax, out, s);
    case 256: return launch_rows_win<T, 16>(g, img, module_axis, wt, m0, nm, tw, smax, out, s);
    case 320: return launch_rows_win<T, 20>(g, img, module_axis, wt, m0, nm, tw, smax, out, s);
    case 384: return launch_rows_win<T, 24>(g, img, module_axis, wt, m0, nm, tw, smax, out, s);
    case 512: return launch_rows_win<T, 32>(g, img, module_axis, wt, m0, nm, tw, smax, out, s);
    default:
      set_error("no windowed row pass for FFT side %d", f.L);
      return JUBIK_ERR_UNSUPPORTED;
  }
}

template int fft_rows_windows<float>(const Fft1D&, const Geom&, const void*, bool, const void*,
                                     int, int, void*, cudaStream_t);
template int fft_rows_windows<double>(const Fft1D&, const Geom&, const void*, bool, const void*,
                                      int, int, void*, cudaStream_t);
template int fft_batched<float>(const Fft1D&, void*, int64_t, int, int64_t, int64_t, int64_t,
                                bool, double, cudaStream_t);
template int fft_batched<double>(const Fft1D&, void*, int64_t, int, int64_t, int64_t, int64_t,
                                 bool, double, cudaStream_t);
template int fft2_batched<float>(const Fft1D&, const Fft1D&, void*, int64_t, bool, cudaStream_t);
template int fft2_batched<double>(const Fft1D&, const Fft1D&, void*, int64_t, bool, cudaStream_t);

}  // namespace jubik
