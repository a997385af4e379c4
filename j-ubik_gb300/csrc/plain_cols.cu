// Column stage of the unfused path, fused with the PSF product
// (jubik/convolve.py:165-174 per patch: ifftn(fftn(x) * fftn(k))).
//
// The unfused path transforms real patches two per complex P x P array (patch
// 2j in the real part, 2j+1 in the imaginary part of pair j).  A 2-D transform
// is a row pass and a column pass.  The row passes stay batched FFT launches;
// everything that needs whole columns runs here, one CTA per set of columns of
// one pair.  The set is closed under the mirror c -> (P - c) mod P, so Z(k) and
// Z(-k) -- which separate the pair's transform into its two patches' spectra --
// sit in the same CTA:
//   forward: column FFT of the row-transformed sky pair, then per module the
//            PSF product A Ha + iB Hb and the inverse column FFT, written as
//            that module's pair (its inverse row pass follows);
//   adjoint: per module the column FFT of the row-transformed cotangent pair
//            and the product with the conjugate PSFs, summed over modules in
//            module order; the inverse column FFT of the sum.
// This replaces a column pass of the products, a product kernel and a column
// pass of the results -- three global round trips per module -- by one.
//
// Each column (P = 16 L1) is transformed in shared memory by an in-place
// four-step in a padded layout: y = n1 + L1 n2 lives at n1 + Q n2 (Q = L1 + 1
// or L1 + 2, odd, so the stride-Q and the stride-1 accesses are free of bank
// conflicts), and columns lie CP = 16 Q + 1 apart (odd as well: the slot-
// parallel loads and products are conflict free).
//   forward, natural -> permuted: per n1, DFT-16 over n2 times w_P^(n1 k2);
//            per k2, DFT-L1 over n1: X[k2 + 16 k1] at Q k2 + k1;
//   inverse, permuted -> natural: per k2, inverse DFT-L1 over k1 times
//            w_P^(-n1 k2); per n1, inverse DFT-16 over k2: x[n1 + L1 n2] at n1 + Q n2.
// The twiddles are the length-P table of the batched transforms.
#include "fft_codelets.cuh"
#include "internal.h"

namespace jubik {

namespace {

constexpr int kColThreads = 256;
constexpr int kColCtasPerSm = 2;

// left columns per CTA: 64-byte row segments, 32 bytes for P = 512 (the
// buffers then stay small enough for two CTAs per SM)
template <typename T, int L1>
constexpr int cols_left() {
  return (sizeof(T) == 4 ? 8 : 4) / (L1 > 24 ? 2 : 1);
}

template <typename T, int L1>
struct ColTile {
  static constexpr int P = 16 * L1;
  static constexpr int Q = (L1 % 2 == 0) ? L1 + 1 : L1 + 2;
  static constexpr int CP = 16 * Q + 1;
  static constexpr int C = cols_left<T, L1>();
  static constexpr int NC = 2 * C;  // slots: C left columns and their mirrors
  static constexpr int GROUPS = (P / 2) / C;
  static constexpr size_t kBufBytes = sizeof(cx<T>) * (size_t)NC * CP;
  // row y of a column -> its place in the padded layout
  __device__ static __forceinline__ int pos(int y) { return y + (y / L1) * (Q - L1); }
  // spectrum value X[k] (k = k2 + 16 k1) -> its place after the forward transform
  __device__ static __forceinline__ int spos(int k) { return Q * (k & 15) + (k >> 4); }
  // column of slot s in group g: left slots g C + s; mirror slots P - (g C + s - C),
  // group 0's first mirror slot holding the self-mirror column P / 2
  __device__ static __forceinline__ int col(int s, int g) {
    if (s < C) return g * C + s;
    const int t = g * C + (s - C);
    return t == 0 ? P / 2 : P - t;
  }
  // slot holding the mirror column of slot s
  __device__ static __forceinline__ int mirror(int s, int g) {
    if (g == 0 && (s == 0 || s == C)) return s;  // columns 0 and P / 2
    return s < C ? s + C : s - C;
  }
};

template <typename T>
__device__ __forceinline__ void cp_async_val(cx<T>* smem, const cx<T>* gmem) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (sizeof(cx<T>) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_drain() {
  asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;" ::: "memory");
}

// A thread's share of the slot-parallel loops (NC slots x P rows).  The CTA has
// kColThreads threads, a multiple of NC, so each thread keeps one slot s and
// takes the rows y0, y0 + YSTEP, ... (ROWS of them); everything that depends on
// the slot alone is computed once.
template <typename T, int L1>
struct Slot {
  using Tl = ColTile<T, L1>;
  static constexpr int YSTEP = kColThreads / Tl::NC;
  static constexpr int ROWS = Tl::P / YSTEP;
  static_assert(kColThreads % Tl::NC == 0 && Tl::P % YSTEP == 0, "slot loop shape");
  int s, y0;
  int col;     // the slot's column
  int mplace;  // start of the mirror slot's column in the tile
  int hcol;    // the stored PSF half-plane column this slot reads
  bool direct; // column <= P / 2: H(ky, col); else conj H(-ky, P - col)
  __device__ __forceinline__ explicit Slot(int g) {
    s = threadIdx.x % Tl::NC;
    y0 = threadIdx.x / Tl::NC;
    col = Tl::col(s, g);
    mplace = Tl::mirror(s, g) * Tl::CP;
    direct = col <= Tl::P / 2;
    hcol = direct ? col : Tl::P - col;
  }
};

// the CTA's NC columns of one P x P pair -> buf (padded layout)
template <typename T, int L1>
__device__ __forceinline__ void load_cols(cx<T>* buf, const cx<T>* __restrict__ src,
                                          const Slot<T, L1>& sl) {
  using Tl = ColTile<T, L1>;
  using Sl = Slot<T, L1>;
  cx<T>* b = buf + sl.s * Tl::CP;
  const cx<T>* g = src + sl.col;
#pragma unroll 4
  for (int i = 0; i < Sl::ROWS; ++i) {
    const int y = sl.y0 + i * Sl::YSTEP;
    cp_async_val<T>(b + Tl::pos(y), g + (int64_t)y * Tl::P);
  }
  cp_async_drain();
  __syncthreads();
}

template <typename T, int L1>
__device__ __forceinline__ void store_cols(const cx<T>* buf, cx<T>* __restrict__ dst,
                                           const Slot<T, L1>& sl) {
  using Tl = ColTile<T, L1>;
  using Sl = Slot<T, L1>;
  const cx<T>* b = buf + sl.s * Tl::CP;
  cx<T>* g = dst + sl.col;
#pragma unroll 4
  for (int i = 0; i < Sl::ROWS; ++i) {
    const int y = sl.y0 + i * Sl::YSTEP;
    g[(int64_t)y * Tl::P] = b[Tl::pos(y)];
  }
}

// forward column transform of every slot, natural -> permuted, in place
// (tw: the length-P twiddles, in shared memory).  The slot varies fastest across
// threads: a warp's lanes then read the same twiddle (a broadcast), and the
// odd column pitch keeps their tile accesses on distinct banks.
template <typename T, int L1>
__device__ __forceinline__ void cols_forward(cx<T>* buf, const cx<T>* tw) {
  using Tl = ColTile<T, L1>;
  constexpr int Q = Tl::Q;
  for (int it = threadIdx.x; it < Tl::NC * L1; it += blockDim.x) {
    const int s = it % Tl::NC, n1 = it / Tl::NC;
    cx<T>* c = buf + s * Tl::CP + n1;
    cx<T> v[16];
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) v[n2] = c[Q * n2];
    Dft<16, false, T>::run(v);
    c[0] = v[0];
#pragma unroll
    for (int k2 = 1; k2 < 16; ++k2) c[Q * k2] = cmul<T>(v[k2], tw[n1 * k2]);
  }
  __syncthreads();
  for (int it = threadIdx.x; it < Tl::NC * 16; it += blockDim.x) {
    const int s = it % Tl::NC, k2 = it / Tl::NC;
    cx<T>* c = buf + s * Tl::CP + Q * k2;
    cx<T> v[L1];
#pragma unroll
    for (int n1 = 0; n1 < L1; ++n1) v[n1] = c[n1];
    Dft<L1, false, T>::run(v);
#pragma unroll
    for (int k1 = 0; k1 < L1; ++k1) c[k1] = v[k1];
  }
  __syncthreads();
}

// inverse column transform (unnormalised), permuted -> natural, in place
template <typename T, int L1>
__device__ __forceinline__ void cols_inverse(cx<T>* buf, const cx<T>* tw) {
  using Tl = ColTile<T, L1>;
  constexpr int Q = Tl::Q;
  for (int it = threadIdx.x; it < Tl::NC * 16; it += blockDim.x) {
    const int s = it % Tl::NC, k2 = it / Tl::NC;
    cx<T>* c = buf + s * Tl::CP + Q * k2;
    cx<T> v[L1];
#pragma unroll
    for (int k1 = 0; k1 < L1; ++k1) v[k1] = c[k1];
    Dft<L1, true, T>::run(v);
    c[0] = v[0];
#pragma unroll
    for (int n1 = 1; n1 < L1; ++n1) c[n1] = cmulc<T>(v[n1], tw[n1 * k2]);
  }
  __syncthreads();
  for (int it = threadIdx.x; it < Tl::NC * L1; it += blockDim.x) {
    const int s = it % Tl::NC, n1 = it / Tl::NC;
    cx<T>* c = buf + s * Tl::CP + n1;
    cx<T> v[16];
#pragma unroll
    for (int k2 = 0; k2 < 16; ++k2) v[k2] = c[Q * k2];
    Dft<16, true, T>::run(v);
#pragma unroll
    for (int n2 = 0; n2 < 16; ++n2) c[Q * n2] = v[n2];
  }
  __syncthreads();
}

// The spectrum stage over the CTA's NC x P values: f(place, a, ib, Ha, Hb) with
// a and ib the pair's two patch spectra (a: patch 2j, ib: i x patch 2j + 1) at
// tile place `place`, and Ha, Hb the two patches' PSF spectra there (hb < 0: no
// second patch).  The PSF spectra come from the stored half plane kx <= P/2; a
// mirror slot's column P - t reads conj H(-ky, t).  Each thread issues the PSF
// loads of kBatch rows before it uses any, so that enough bytes are in flight
// to cover the latency of the global loads.
template <typename T, int L1, typename F>
__device__ __forceinline__ void spectrum_stage(const cx<T>* bz, const cx<T>* __restrict__ hfull,
                                               int64_t ha, int64_t hb, const Slot<T, L1>& sl,
                                               F&& f) {
  using Tl = ColTile<T, L1>;
  using Sl = Slot<T, L1>;
  constexpr int P = Tl::P, H1 = P / 2 + 1;
  constexpr int kBatch = sizeof(T) == 4 ? 8 : 4;
  const cx<T>* hA = hfull + ha * P * H1 + sl.hcol;
  const cx<T>* hB = hfull + (hb >= 0 ? hb : ha) * P * H1 + sl.hcol;
  const T hsign = sl.direct ? (T)1 : (T)-1;
  const int place0 = sl.s * Tl::CP;
  for (int i0 = 0; i0 < Sl::ROWS; i0 += kBatch) {
    cx<T> va[kBatch], vb[kBatch];
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      if (i0 + u < Sl::ROWS) {
        const int ky = sl.y0 + (i0 + u) * Sl::YSTEP;
        const int kym = ky == 0 ? 0 : P - ky;
        const int row = sl.direct ? ky : kym;
        va[u] = hA[(int64_t)row * H1];
        vb[u] = hB[(int64_t)row * H1];
      }
    }
#pragma unroll
    for (int u = 0; u < kBatch; ++u) {
      if (i0 + u < Sl::ROWS) {
        const int ky = sl.y0 + (i0 + u) * Sl::YSTEP;
        const int kym = ky == 0 ? 0 : P - ky;
        const int place = place0 + Tl::spos(ky);
        const cx<T> z = bz[place];
        const cx<T> zm = cconj<T>(bz[sl.mplace + Tl::spos(kym)]);
        const cx<T> a = cscale<T>(cadd<T>(z, zm), (T)0.5);
        const cx<T> ib = cscale<T>(csub<T>(z, zm), (T)0.5);
        f(place, a, ib, mkc<T>(va[u].x, hsign * va[u].y), mkc<T>(vb[u].x, hsign * vb[u].y));
      }
    }
  }
}

// PSF units of pair j's two patches for module m (hb < 0: no second patch)
__device__ __forceinline__ void pair_units(int64_t j, int m, int E, int n2p, int64_t* ha,
                                           int64_t* hb) {
  const int np = E * n2p;
  const int pa = (int)(2 * j), pb = pa + 1;
  *ha = ((int64_t)m * n2p + pa % n2p) * E + pa / n2p;
  *hb = pb < np ? ((int64_t)m * n2p + pb % n2p) * E + pb / n2p : -1;
}

// shared memory: two column tiles, then the length-P twiddles
template <typename T, int L1>
constexpr size_t cols_smem_bytes() {
  return 2 * ColTile<T, L1>::kBufBytes + sizeof(cx<T>) * (size_t)ColTile<T, L1>::P;
}

template <typename T, int L1>
__global__ void __launch_bounds__(kColThreads, kColCtasPerSm)
    k_plain_cols_fwd(const cx<T>* __restrict__ zs, const cx<T>* __restrict__ hfull,
                     const cx<T>* __restrict__ tw, int m0, int nm, int E, int n2p, int64_t nph,
                     cx<T>* __restrict__ zu) {
  using Tl = ColTile<T, L1>;
  constexpr int P = Tl::P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* bz = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* bw = bz + Tl::NC * Tl::CP;
  cx<T>* stw = bw + Tl::NC * Tl::CP;
  for (int i = threadIdx.x; i < P; i += blockDim.x) stw[i] = tw[i];  // (load_cols syncs)
  const Slot<T, L1> sl(blockIdx.x);
  const int64_t pp = (int64_t)P * P;
  for (int64_t j = blockIdx.y; j < nph; j += gridDim.y) {
    load_cols<T, L1>(bz, zs + j * pp, sl);
    cols_forward<T, L1>(bz, stw);
    for (int mm = 0; mm < nm; ++mm) {
      int64_t ha, hb;
      pair_units(j, m0 + mm, E, n2p, &ha, &hb);
      spectrum_stage<T, L1>(bz, hfull, ha, hb, sl,
                            [&](int place, cx<T> a, cx<T> ib, cx<T> h_a, cx<T> h_b) {
                              cx<T> w = cmul<T>(a, h_a);
                              if (hb >= 0) w = cadd<T>(w, cmul<T>(ib, h_b));
                              bw[place] = w;
                            });
      __syncthreads();
      cols_inverse<T, L1>(bw, stw);
      store_cols<T, L1>(bw, zu + ((int64_t)mm * nph + j) * pp, sl);
      __syncthreads();  // bw is rewritten by the next module
    }
  }
}

// first: the module sum starts at zero (else from zs, left in spectral order by
// the previous module chunk); last: the sum is transformed back and written in
// natural order (else written in spectral order for the next chunk)
template <typename T, int L1>
__global__ void __launch_bounds__(kColThreads, kColCtasPerSm)
    k_plain_cols_adj(const cx<T>* __restrict__ zu, const cx<T>* __restrict__ hfull,
                     const cx<T>* __restrict__ tw, int m0, int nm, int E, int n2p, int64_t nph,
                     int first, int last, cx<T>* __restrict__ zs) {
  using Tl = ColTile<T, L1>;
  constexpr int P = Tl::P;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  cx<T>* bz = reinterpret_cast<cx<T>*>(smem_raw);
  cx<T>* bw = bz + Tl::NC * Tl::CP;
  cx<T>* stw = bw + Tl::NC * Tl::CP;
  for (int i = threadIdx.x; i < P; i += blockDim.x) stw[i] = tw[i];  // (load_cols syncs)
  const Slot<T, L1> sl(blockIdx.x);
  const int64_t pp = (int64_t)P * P;
  for (int64_t j = blockIdx.y; j < nph; j += gridDim.y) {
    if (first) {
      for (int i = threadIdx.x; i < Tl::NC * Tl::CP; i += blockDim.x) bw[i] = mkc<T>((T)0, (T)0);
    } else {
      load_cols<T, L1>(bw, zs + j * pp, sl);
    }
    for (int mm = 0; mm < nm; ++mm) {
      load_cols<T, L1>(bz, zu + ((int64_t)mm * nph + j) * pp, sl);
      cols_forward<T, L1>(bz, stw);
      int64_t ha, hb;
      pair_units(j, m0 + mm, E, n2p, &ha, &hb);
      spectrum_stage<T, L1>(bz, hfull, ha, hb, sl,
                            [&](int place, cx<T> a, cx<T> ib, cx<T> h_a, cx<T> h_b) {
                              cx<T> acc = cadd<T>(bw[place], cmulc<T>(a, h_a));
                              if (hb >= 0) acc = cadd<T>(acc, cmulc<T>(ib, h_b));
                              bw[place] = acc;
                            });
      __syncthreads();  // bz is reloaded by the next module
    }
    if (last) cols_inverse<T, L1>(bw, stw);
    store_cols<T, L1>(bw, zs + j * pp, sl);
    __syncthreads();  // bw is reset by the next pair
  }
}

template <typename T, int L1>
int launch_cols(const Geom& g, bool adjoint, const void* zin, const void* hfull, const void* tw,
                int m0, int nm, bool first, bool last, void* zout, cudaStream_t s) {
  using Tl = ColTile<T, L1>;
  const size_t smem = cols_smem_bytes<T, L1>();
  const int64_t nph = plain_pairs(g);
  const dim3 grid(Tl::GROUPS, (unsigned)std::min<int64_t>(nph, 65535));
  const int n2p = g.n * g.n;
  if (adjoint) {
    auto kern = k_plain_cols_adj<T, L1>;
    JUBIK_TRY_CUDA(
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    kern<<<grid, kColThreads, smem, s>>>((const cx<T>*)zin, (const cx<T>*)hfull,
                                         (const cx<T>*)tw, m0, nm, g.E, n2p, nph, first ? 1 : 0,
                                         last ? 1 : 0, (cx<T>*)zout);
    return cuda_status(cudaGetLastError(), "k_plain_cols_adj");
  }
  auto kern = k_plain_cols_fwd<T, L1>;
  JUBIK_TRY_CUDA(
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<grid, kColThreads, smem, s>>>((const cx<T>*)zin, (const cx<T>*)hfull, (const cx<T>*)tw,
                                       m0, nm, g.E, n2p, nph, (cx<T>*)zout);
  return cuda_status(cudaGetLastError(), "k_plain_cols_fwd");
}

template <typename T>
int dispatch_cols(const Geom& g, bool adjoint, const void* zin, const void* hfull, const void* tw,
                  int m0, int nm, bool first, bool last, void* zout, cudaStream_t s) {
  switch (g.P) {
    case 160: return launch_cols<T, 10>(g, adjoint, zin, hfull, tw, m0, nm, first, last, zout, s);
    case 192: return launch_cols<T, 12>(g, adjoint, zin, hfull, tw, m0, nm, first, last, zout, s);
    case 256: return launch_cols<T, 16>(g, adjoint, zin, hfull, tw, m0, nm, first, last, zout, s);
    case 320: return launch_cols<T, 20>(g, adjoint, zin, hfull, tw, m0, nm, first, last, zout, s);
    case 384: return launch_cols<T, 24>(g, adjoint, zin, hfull, tw, m0, nm, first, last, zout, s);
    case 512: return launch_cols<T, 32>(g, adjoint, zin, hfull, tw, m0, nm, first, last, zout, s);
    default:
      set_error("no fused column stage for FFT side %d", g.P);
      return JUBIK_ERR_UNSUPPORTED;
  }
}

}  // namespace

bool plain_cols_supported(int P) {
  return P == 160 || P == 192 || P == 256 || P == 320 || P == 384 || P == 512;
}

template <typename T>
int plain_cols_forward(const Geom& g, const void* zs, const void* hfull, const void* tw, int m0,
                       int nm, void* zu, cudaStream_t s) {
  return dispatch_cols<T>(g, false, zs, hfull, tw, m0, nm, false, false, zu, s);
}

template <typename T>
int plain_cols_adjoint(const Geom& g, const void* zu, const void* hfull, const void* tw, int m0,
                       int nm, bool first, bool last, void* zs, cudaStream_t s) {
  return dispatch_cols<T>(g, true, zu, hfull, tw, m0, nm, first, last, zs, s);
}

template int plain_cols_forward<float>(const Geom&, const void*, const void*, const void*, int,
                                       int, void*, cudaStream_t);
template int plain_cols_forward<double>(const Geom&, const void*, const void*, const void*, int,
                                        int, void*, cudaStream_t);
template int plain_cols_adjoint<float>(const Geom&, const void*, const void*, const void*, int,
                                       int, bool, bool, void*, cudaStream_t);
template int plain_cols_adjoint<double>(const Geom&, const void*, const void*, const void*, int,
                                        int, bool, bool, void*, cudaStream_t);

}  // namespace jubik
