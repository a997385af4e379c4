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
#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

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
  void* spec;  // (E n^2, P, P/2) spectra shared by the modules of a patch
  double scale;
  int64_t zchunk;  // bytes of `out` each CTA clears (sky-spectrum and adjoint per-unit kernels)
  void* aux;       // sky-spectrum kernel: a further buffer to clear (aux_bytes, aux_chunk per CTA)
  int64_t aux_bytes, aux_chunk;
  int zero_out;    // adjoint per-unit kernel: clear `out` first
  int64_t in_rs, in_ps;  // forward input: row and plane strides (a crop of a larger array)
  int in_exp;            // forward input holds log-sky values: the sky is their exp
  int M, E, nx, ny, n, dx, margin, half, sr_max, sc_max;
  // exact two-word accumulation of the output (see Split2): the low words, and
  // the bound on its terms = bnd_scale * max(bnd_in[0 .. bnd_n)), at most
  // 2^bnd_log2 terms per element.  out_lo == nullptr: single-word reductions.
  void* out_lo;
  const unsigned long long* bnd_in;
  int bnd_n, bnd_log2;
  double bnd_scale;
  // input magnitude maxima this kernel records (per item or per CTA), or nullptr
  unsigned long long* bnd_out;
  // module-shared adjoint in unit order (one problem): partial module sums of
  // the patch a CTA continues (one slot per CTA of the loop grid `loop_grid`)
  void* spill;
  int loop_grid;
  int run_len;  // run-ordered forward: patches per run (2 or 4)
  // floor(u / d) for d = M, n^2, n and n / run_len as one multiply-high by these
  // constants (mulhi_divisor); 0: divide
  uint32_t div_M, div_n2, div_n, div_nq;
};

// floor(u / d) for 0 <= u: with mul = floor(2^32 / d) + 1 the high word of u mul
// is exact while u d < 2^32 (mul d exceeds 2^32 by at most d, so u mul / 2^32
// exceeds u / d by less than 1 / d).  mul = 0 divides.
__device__ __forceinline__ int div_by(int u, int d, uint32_t mul) {
  return mul ? (int)__umulhi((uint32_t)u, mul) : u / d;
}

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
// Unpredicated 4/8-byte global->shared copy (the source is known in bounds).
template <typename T>
__device__ __forceinline__ void cp_async_in(T* dst, const T* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(T) == 4) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
  }
}
// The same copy to a shared-memory address already in the shared window.
template <typename T>
__device__ __forceinline__ void cp_async_in_s(unsigned d, const T* src) {
  if constexpr (sizeof(T) == 4) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(d), "l"(src) : "memory");
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(d), "l"(src) : "memory");
  }
}

// Programmatic dependent launch: every kernel of a step lets the next one be
// scheduled as soon as all of its CTAs run (launch_dependents), and waits for
// the previous kernel's completion and memory (wait) before it touches
// anything that kernel, or one before it, writes or reads.
__device__ __forceinline__ void pdl_trigger() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// CTA blockIdx.x of the grid clears its share (chunk bytes, a multiple of 16,
// computed on the host) of nbytes at base (16-byte stores when base is
// 16-byte aligned).
__device__ __forceinline__ void zero_slice(void* base, int64_t nbytes, int64_t chunk) {
  const int64_t lo = (int64_t)blockIdx.x * chunk;
  const int64_t hi = lo + chunk < nbytes ? lo + chunk : nbytes;
  if (lo >= hi) return;
  unsigned char* p = static_cast<unsigned char*>(base);
  int64_t b = lo;
  if ((reinterpret_cast<uintptr_t>(p) & 15) == 0) {
    const int64_t n16 = (hi - lo) >> 4;
    float4* q = reinterpret_cast<float4*>(p + lo);
    for (int64_t i = threadIdx.x; i < n16; i += blockDim.x) q[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    b = lo + (n16 << 4);
  }
  for (int64_t i = b + threadIdx.x; i < hi; i += blockDim.x) p[i] = 0;
}

// 4 consecutive floats added to global memory in one reduction (16-byte aligned)
__device__ __forceinline__ void red_add_v4(float* p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1,%2,%3,%4};" ::"l"(p), "f"(a), "f"(b), "f"(c),
               "f"(d)
               : "memory");
}

// ---- exact, order-independent accumulation in two words
// Atomic reductions add in whatever order the patches arrive, and floating
// point addition rounds differently in different orders.  Each term v of an
// overlap-add is therefore split into two words whose sums are exact:
//   hi = v rounded to a multiple of Q1,   lo = (v - hi) rounded to a multiple of Q2,
// with Q1 = 2^(e - (D - 2)) for a bound 2^e > B on every term and partial sum
// (D = significand bits of T) and Q2 = Q1 * 2^(L + 1 - D) for at most 2^L terms
// per element.  Multiples of Q below 2^D * Q in magnitude add exactly in T, so the
// hi words and the lo words each reach the same bits in any order; the result
// hi + lo (one rounding) is within 2^L * Q2 / 2 of the exact sum of the terms,
// about B * 2^(2L + 2 - 2D) -- far below the rounding of the FFT that made them.
// Rounding to a grid is one add and one subtract of 1.5 * 2^(D-1) * Q.
template <typename T>
struct Split2 {
  T m1, m2;
  // The grid constants from the bits of the bound, in integer arithmetic (the
  // FP64 pipe of this GPU is narrow, and every thread runs this).
  __device__ __forceinline__ void init(double bound, int L) {
    constexpr int D = sizeof(T) == 4 ? 24 : 53;
    constexpr int EMIN = sizeof(T) == 4 ? -75 : -900, EMAX = sizeof(T) == 4 ? 120 : 1000;
    const unsigned long long b = (unsigned long long)__double_as_longlong(bound);
    const int be = (int)((b >> 52) & 0x7ff);
    if (be == 0x7ff || (b >> 63)) {  // a NaN, infinite or negative bound: results become NaN
      m1 = m2 = (T)NAN;
      return;
    }
    // bound < 2^e: e = unbiased exponent + 1 (a zero or subnormal bound takes EMIN)
    int e = be == 0 ? EMIN : be - 1023 + 1;
    e = e < EMIN ? EMIN : (e > EMAX ? EMAX : e);
    const int q1 = e - (D - 2), q2 = q1 + L + 1 - D;
    m1 = pow2_times_1_5(q1 + D - 1);
    m2 = pow2_times_1_5(q2 + D - 1);
  }
  // 1.5 * 2^k as T, built from its bits (k within T's normal range here)
  __device__ __forceinline__ static T pow2_times_1_5(int k) {
    if constexpr (sizeof(T) == 4) {
      return __uint_as_float(((unsigned)(k + 127) << 23) | 0x400000u);
    } else {
      return __longlong_as_double((long long)(((unsigned long long)(k + 1023) << 52) |
                                              0x8000000000000ull));
    }
  }
  __device__ __forceinline__ void split(T v, T& hi, T& lo) const {
    if constexpr (sizeof(T) == 4) {
      hi = __fsub_rn(__fadd_rn(v, m1), m1);
      lo = __fsub_rn(v, hi);
      lo = __fsub_rn(__fadd_rn(lo, m2), m2);
    } else {
      hi = __dsub_rn(__dadd_rn(v, m1), m1);
      lo = __dsub_rn(v, hi);
      lo = __dsub_rn(__dadd_rn(lo, m2), m2);
    }
  }
};

// Magnitude maxima travel as the bits of a non-negative double: unsigned
// comparison of those bits orders them, and a NaN sorts above every number.
__device__ __forceinline__ unsigned long long mag_bits(double v) {
  return (unsigned long long)__double_as_longlong(fabs(v));
}
__device__ __forceinline__ unsigned long long umax64(unsigned long long a, unsigned long long b) {
  return a > b ? a : b;
}
__device__ __forceinline__ unsigned umax32(unsigned a, unsigned b) { return a > b ? a : b; }
// U.mx of either width as the bits of a double magnitude
__device__ __forceinline__ unsigned long long mag_as_double_bits(unsigned v) {
  return mag_bits((double)__uint_as_float(v));
}
__device__ __forceinline__ unsigned long long mag_as_double_bits(unsigned long long v) {
  return v;
}
// CTA-wide maximum of one value per thread (every thread gets it); uses s_slot.
__device__ __forceinline__ unsigned long long cta_max(unsigned long long v,
                                                      unsigned long long* s_slot) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = umax64(v, __shfl_xor_sync(0xffffffffu, v, o));
  if (threadIdx.x == 0) *s_slot = 0ull;
  __syncthreads();
  if ((threadIdx.x & 31) == 0) atomicMax(s_slot, v);
  __syncthreads();
  const unsigned long long r = *s_slot;
  __syncthreads();
  return r;
}
// Maximum of n stored maxima, by the whole CTA.
__device__ __forceinline__ double reduce_bound(const unsigned long long* p, int n,
                                               unsigned long long* s_slot) {
  unsigned long long v = 0ull;
  for (int i = threadIdx.x; i < n; i += blockDim.x) v = umax64(v, __ldcg(p + i));
  return __longlong_as_double((long long)cta_max(v, s_slot));
}

// ---- tensor memory (TMEM) as a per-SM accumulator
// The adjoint keeps each patch's running sum over modules in tensor memory:
// 128 lanes x 512 columns of 32 bits per SM, which this kernel's arithmetic
// does not otherwise use.  Warp w reaches lanes 32 (w % 4) .. 32 (w % 4) + 31;
// thread (w, lane) owns TMEM lane 32 (w % 4) + lane and the column range of its
// warp.  Allocation, loads and stores are warp-collective (.sync.aligned).
__device__ __forceinline__ void tmem_alloc(uint32_t* smem_slot, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   (uint32_t)__cvta_generic_to_shared(smem_slot)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
               : "memory");
}
__device__ __forceinline__ void tmem_fence_before_sync() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tmem_fence_after_sync() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// 32 consecutive 32-bit columns of the thread's lane, from column taddr
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
      "%28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
        "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
        "=r"(r[31])
      : "r"(taddr)
      : "memory");
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_st32(uint32_t taddr, const uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, "
      "%11, %12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, "
      "%28, %29, %30, %31, %32};" ::"r"(taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
      "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]),
      "r"(r[15]), "r"(r[16]), "r"(r[17]), "r"(r[18]), "r"(r[19]), "r"(r[20]), "r"(r[21]),
      "r"(r[22]), "r"(r[23]), "r"(r[24]), "r"(r[25]), "r"(r[26]), "r"(r[27]), "r"(r[28]),
      "r"(r[29]), "r"(r[30]), "r"(r[31])
      : "memory");
}
__device__ __forceinline__ void tmem_wait_st() {
  asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
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
// Offset of row y0 + d from row y0 when y0 is even (d a compile-time constant).
template <int P>
__device__ __forceinline__ constexpr int rfd(int d) {
  return (d >> 1) * (P + 1) + (d & 1) * (P / 2);
}

// Per-CTA view of one unit: geometry, warp class and its register twiddles.
template <typename T, int P>
struct Unit {
  using R = Tr<T, P>;
  cx<T>* tile;
  cx<T>* stg;
  int tid, warp, lane, cls;
  int m, e, k, rb, cb, K, mg;
  int64_t npix;
  const cx<T>* hmain;
  const cx<T>* hnyq;
  cx<T>* spec;  // this patch's shared spectrum (P rows x P/2 columns, A order)
  const T* wt;
  const cx<T>* twg;
  cx<T> wq[16];
  // largest input magnitude staged so far (bits of |v|; a NaN sorts last)
  typename std::conditional<sizeof(T) == 4, unsigned, unsigned long long>::type mx;
  // module-shared adjoint in unit order: partial sums of this patch held by
  // the CTAs that continued it (nsp slots from sp0)
  const cx<T>* sp0;
  int nsp;

  // unit block index ub (the CTA's blockIdx.x unless a grouped launch maps it)
  // -> (m, e, k); per_module == false decodes (e, k) only
  __device__ __forceinline__ void init(const Args& a, unsigned char* smem, bool per_module,
                                       int ub = -1) {
    geom(a, smem, per_module, ub);
    mx = 0;
    sp0 = nullptr;
    nsp = 0;
    twg = (const cx<T>*)a.tw;
#pragma unroll
    for (int q = 0; q < 16; ++q) wq[q] = ldg2(twg + cls * q);
  }
  // everything but the twiddles (a loop over units keeps those)
  __device__ __forceinline__ void geom(const Args& a, unsigned char* smem, bool per_module,
                                       int ub) {
    tile = reinterpret_cast<cx<T>*>(smem);
    stg = tile + R::TILE;
    tid = threadIdx.x;
    warp = tid >> 5;
    lane = tid & 31;
    cls = warp;
    const int n2p = a.n * a.n;
    int u = ub >= 0 ? ub : (int)blockIdx.x;
    m = 0;
    if (per_module) {
      const int q = div_by(u, a.M, a.div_M);
      m = u - q * a.M;
      u = q;
    }
    e = div_by(u, n2p, a.div_n2);
    k = u - e * n2p;
    const int kc = div_by(k, a.n, a.div_n);
    const int sr = min((k - kc * a.n) * a.dx, a.sr_max);
    const int sc = min(kc * a.dx, a.sc_max);
    rb = sr - a.half - a.margin;
    cb = sc - a.half - a.margin;
    K = 2 * a.dx;
    mg = a.margin;
    npix = (int64_t)a.nx * a.ny;
    const int64_t hu = ((int64_t)m * n2p + k) * a.E + e;
    hmain = (const cx<T>*)a.hmain + hu * (int64_t)(P * R::H);
    hnyq = (const cx<T>*)a.hnyq + hu * (int64_t)P;
    spec = a.spec ? (cx<T>*)a.spec + ((int64_t)e * n2p + k) * (int64_t)(P * R::H) : nullptr;
    wt = (const T*)a.wt;
  }
};

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// ---- input rows -> staging (cp.async) -> row step A (variant B forward)
// forward: weighted sky window rows; adjoint: cotangent window rows.
// Chunks of CH pairs are double-buffered when a part of the tile that the
// current chunk does not write is free: the next chunk's loads then overlap
// the current chunk's transform.  Buffers are pair rows of pitch TP: chunk c
// uses the staging area (c even) or a tile region (c odd).
// Chunk layout of the input stage: pair rows [jlo, jhi) in chunks of CH.
template <typename T, int P, bool ADJ>
struct InChunks {
  using R = Tr<T, P>;
  int jlo, jhi, nchunks, nzero;
  bool db;
  __device__ __forceinline__ InChunks(const Unit<T, P>& U) {
    constexpr int H = R::H, CH = R::CH;
    jlo = ADJ ? 0 : U.mg / 2;
    jhi = ADJ ? H : (U.mg + U.K + 1) / 2;
    nchunks = (jhi - jlo + CH - 1) / CH;
    nzero = H - (jhi - jlo);
    // second buffer: adjoint with 3 full chunks -> the last chunk's tile pairs
    // [2 CH, 3 CH) (a short last chunk, as for P = 160, leaves too few);
    // forward with 2 chunks -> the zero pairs outside the window rows
    db = ADJ ? (nchunks == 3 && 3 * CH <= H) : (nchunks == 2 && nzero >= CH);
  }
  // tile pair holding row-pair jj of the odd chunk
  __device__ __forceinline__ int alt_pair(int jj) const {
    if (ADJ) return 2 * R::CH + jj;
    return jj < jlo ? jj : jhi + (jj - jlo);
  }
  __device__ __forceinline__ cx<T>* buf(const Unit<T, P>& U, int c, int jj) const {
    return (db && (c & 1)) ? U.tile + alt_pair(jj) * R::TP : U.stg + jj * R::TP;
  }
};

// cp.async of input chunk c (one commit group).  Chunk 0 goes to the staging
// area, so a loop over units may issue the next unit's chunk 0 while the
// current unit's later stages (which leave the staging area alone) run.
template <typename T, int P, bool ADJ>
__device__ __forceinline__ void input_issue(const Unit<T, P>& U, const Args& a,
                                            const InChunks<T, P, ADJ>& ch, int c) {
  using R = Tr<T, P>;
  constexpr int NT = R::NT, CH = R::CH;
  const int mg = U.mg, K = U.K;
  const int xoff = ADJ ? 0 : mg;
  const int width = ADJ ? P : K;
  // forward input: element (row, col) of energy e at e * in_ps + row * in_rs + col
  const int64_t rs = ADJ ? (int64_t)a.ny : a.in_rs;
  const T* __restrict__ src =
      (const T*)a.in + (ADJ ? ((int64_t)U.m * a.E + U.e) * U.npix : (int64_t)U.e * a.in_ps);
  // adjoint units whose P x P window lies inside the field need no bounds checks
  const bool interior = ADJ && U.rb >= 0 && U.rb + P <= a.nx && U.cb >= 0 && U.cb + P <= a.ny;
  const int j0 = ch.jlo + c * CH;
  const int nch = min(CH, ch.jhi - j0);
  if (ADJ && interior && NT % P == 0) {
    // a chunk's buffer is linear in its pair rows: walk both addresses by
    // increments instead of recomputing them per pair row
    constexpr int JSTEP = NT / P;
    const int xs = U.tid % P;
    int jj = U.tid / P;
    const T* g = src + (int64_t)(U.rb + 2 * (j0 + jj)) * rs + U.cb + xs;
    const int64_t gstep = 2 * JSTEP * rs;
    unsigned d = (unsigned)__cvta_generic_to_shared(ch.buf(U, c, jj) + xs);
#pragma unroll 4
    for (; jj < nch; jj += JSTEP) {
      cp_async_in_s<T>(d, g);
      cp_async_in_s<T>(d + (unsigned)sizeof(T), g + rs);
      g += gstep;
      d += (unsigned)(JSTEP * R::TP * sizeof(cx<T>));
    }
  } else if (NT % width == 0) {
    // each thread owns one staged column and every (NT / width)-th pair row;
    // the row, its element offset and the buffer address advance by increments
    const int xs = U.tid % width, jstep = NT / width;
    const int col = U.cb + xoff + xs;
    const bool cok = col >= 0 && col < a.ny;
    const T* gcol = src + (cok ? col : 0);
    int jj = U.tid / width;
    int y0 = 2 * (j0 + jj);
    int64_t off = (int64_t)(U.rb + y0) * rs;
    const int64_t ostep = 2 * (int64_t)jstep * rs;
    T* d = reinterpret_cast<T*>(ch.buf(U, c, jj) + xs);
    const int dstep = 2 * jstep * R::TP;
    // the forward's odd chunk in a second buffer skips the window's pair rows:
    // its buffer is not linear in jj
    const bool lin = ADJ || !(ch.db && (c & 1));
    for (; jj < nch; jj += jstep, y0 += 2 * jstep, off += ostep, d += dstep) {
      const int row = U.rb + y0;
      const bool ok0 = cok && row >= 0 && row < a.nx && (ADJ || (y0 - mg >= 0 && y0 - mg < K));
      const bool ok1 = cok && row + 1 >= 0 && row + 1 < a.nx &&
                       (ADJ || (y0 + 1 - mg >= 0 && y0 + 1 - mg < K));
      T* dd = lin ? d : reinterpret_cast<T*>(ch.buf(U, c, jj) + xs);
      cp_async<T>(dd, ok0 ? gcol + off : src, ok0);
      cp_async<T>(dd + 1, ok1 ? gcol + off + rs : src, ok1);
    }
  } else {
    for (int i = U.tid; i < nch * width; i += NT) {
      const int jj = i / width, xs = i - jj * width;
      const int col = U.cb + xoff + xs;
      const int y0 = 2 * (j0 + jj);
      const int row = U.rb + y0;
      const bool cok = col >= 0 && col < a.ny;
      const bool ok0 =
          cok && row >= 0 && row < a.nx && (ADJ || (y0 - mg >= 0 && y0 - mg < K));
      const bool ok1 = cok && row + 1 >= 0 && row + 1 < a.nx &&
                       (ADJ || (y0 + 1 - mg >= 0 && y0 + 1 - mg < K));
      T* d = reinterpret_cast<T*>(ch.buf(U, c, jj) + xs);
      cp_async<T>(d, ok0 ? src + (int64_t)row * rs + col : src, ok0);
      cp_async<T>(d + 1, ok1 ? src + (int64_t)(row + 1) * rs + col : src, ok1);
    }
  }
  cp_async_commit();
}

// ---- input rows -> staging (cp.async) -> row step A (variant B forward)
// forward: weighted sky window rows; adjoint: cotangent window rows.
// Chunks of CH pairs are double-buffered when a part of the tile that the
// current chunk does not write is free: the next chunk's loads then overlap
// the current chunk's transform.  Buffers are pair rows of pitch TP: chunk c
// uses the staging area (c even) or a tile region (c odd).  chunk0_issued:
// input_issue(c = 0) already ran for this unit (and nothing was committed since).
// TRACK: also record the largest magnitude of the staged (weighted) values in U.mx.
template <typename T, int P, bool ADJ, bool TRACK = false>
__device__ __forceinline__ void stage_input(Unit<T, P>& U, const Args& a,
                                            bool chunk0_issued = false) {
  using R = Tr<T, P>;
  constexpr int L1 = R::L1, NT = R::NT, TP = R::TP, CH = R::CH;
  cx<T>* tile = U.tile;
  const int mg = U.mg, K = U.K;
  const InChunks<T, P, ADJ> ch(U);
  const int jlo = ch.jlo, jhi = ch.jhi, nchunks = ch.nchunks, nzero = ch.nzero;
  const bool db = ch.db;
  auto bufp = [&](int c, int jj) -> cx<T>* { return ch.buf(U, c, jj); };
  const int xoff = ADJ ? 0 : mg;
  const int width = ADJ ? P : K;
  // column weights, zero outside the window and outside the field (where the
  // staged values are the zero fill, whose exp would not be zero)
  T wc[16];
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int xa = U.cls + L1 * q - mg;
    const int col = U.cb + U.cls + L1 * q;
    wc[q] = (!ADJ && xa >= 0 && xa < K && col >= 0 && col < a.ny) ? U.wt[xa] : (T)0;
  }
  auto issue = [&](int c) { input_issue<T, P, ADJ>(U, a, ch, c); };
  if (!ADJ && !db) {  // zero pairs outside the window rows (before step A writes)
    for (int i = U.tid; i < nzero * P; i += NT) {
      const int jj = i / P, sl = i - jj * P;
      const int j = jj < jlo ? jj : jhi + (jj - jlo);
      tile[j * TP + sl] = mkc<T>((T)0, (T)0);
    }
  }
  if (!chunk0_issued) issue(0);
  if (db && nchunks > 1) issue(1);
  for (int c = 0; c < nchunks; ++c) {
    const int j0 = jlo + c * CH;
    const int nch = min(CH, jhi - j0);
    if (db && c + 1 < nchunks)
      cp_async_wait<1>();
    else
      cp_async_wait<0>();
    __syncthreads();
    for (int jj = U.lane; jj < nch; jj += 32) {
      const int y0 = 2 * (j0 + jj);
      const int row0 = U.rb + y0;
      const T wr0 = (!ADJ && y0 - mg >= 0 && y0 - mg < K && row0 >= 0 && row0 < a.nx)
                        ? U.wt[y0 - mg] : (T)0;
      const T wr1 = (!ADJ && y0 + 1 - mg >= 0 && y0 + 1 - mg < K && row0 + 1 >= 0 &&
                     row0 + 1 < a.nx)
                        ? U.wt[y0 + 1 - mg] : (T)0;
      const cx<T>* bsrc = bufp(c, jj);
      cx<T> v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int xs = U.cls + L1 * q - xoff;
        // the adjoint stages whole P-wide rows: cls + L1 q is always inside
        if (ADJ || (xs >= 0 && xs < width)) {
          cx<T> t = bsrc[xs];
          if (!ADJ && a.in_exp) t = mkc<T>(exp(t.x), exp(t.y));
          // (w_row * w_col) * x, the order of weights * slices in convolve.py:89-90
          v[q] = ADJ ? t : mkc<T>((wr0 * wc[q]) * t.x, (wr1 * wc[q]) * t.y);
        } else {
          v[q] = mkc<T>((T)0, (T)0);
        }
        if constexpr (TRACK) {
          if constexpr (sizeof(T) == 4) {
            const unsigned b = umax32(__float_as_uint(fabsf(v[q].x)),
                                      __float_as_uint(fabsf(v[q].y)));
            U.mx = b > U.mx ? b : U.mx;
          } else {
            U.mx = umax64(U.mx, umax64(mag_bits(v[q].x), mag_bits(v[q].y)));
          }
        }
      }
      Dft<16, false, T>::run(v);
      cx<T>* dst = tile + (j0 + jj) * TP + 16 * U.cls;
#pragma unroll
      for (int q = 0; q < 16; ++q) dst[q] = q ? cmul<T>(v[q], U.wq[q]) : v[q];
    }
    __syncthreads();
    if (db) {
      if (c + 2 < nchunks) issue(c + 2);  // into the buffer chunk c just released
    } else if (c + 1 < nchunks) {
      issue(c + 1);
    }
  }
  if (!ADJ && db) {  // the zero pairs held chunk 1's rows; clear them now
    for (int i = U.tid; i < nzero * P; i += NT) {
      const int jj = i / P, sl = i - jj * P;
      const int j = jj < jlo ? jj : jhi + (jj - jlo);
      tile[j * TP + sl] = mkc<T>((T)0, (T)0);
    }
    __syncthreads();
  }
}

// ---- row step B (DFT-L1 per class) fused with the real-to-complex split
template <typename T, int P>
__device__ __forceinline__ void stage_split(Unit<T, P>& U) {
  using R = Tr<T, P>;
  constexpr int L1 = R::L1, H = R::H, NT = R::NT, TP = R::TP, HL = L1 / 2;
  for (int it = U.tid; it < H * 8; it += NT) {
    const int j = it % H, kap = it / H;
    cx<T>* row = U.tile + j * TP;
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
}

// ---- column phase 1 (variant A forward): items (c, n2), DFT-L1 over n1;
// rows outside [ylo, yhi) are known zeros (FULL: none are)
template <typename T, int P, bool FULL = false>
__device__ __forceinline__ void stage_col1(Unit<T, P>& U, int ylo, int yhi) {
  using R = Tr<T, P>;
  constexpr int L1 = R::L1, H = R::H, NT = R::NT;
  for (int it = U.tid; it < H * 16; it += NT) {
    const int c = it % H, n2 = it / H;
    cx<T> v[L1];
    cx<T>* base = U.tile + rf<P>(n2, c);  // row n2 + 16 i is 8 i pairs further
#pragma unroll
    for (int i = 0; i < L1; ++i) {
      const int y = n2 + 16 * i;
      v[i] = (FULL || (y >= ylo && y < yhi)) ? base[8 * i * (P + 1)] : mkc<T>((T)0, (T)0);
    }
    Dft<L1, false, T>::run(v);
#pragma unroll
    for (int i = 0; i < L1; ++i) base[8 * i * (P + 1)] = v[i];
  }
}

// ---- column phase 2 (class k1 = warp): the spectrum-side step
enum Mid { MID_FULL, MID_TO_SPEC, MID_FROM_SPEC, MID_FROM_ACC };

template <typename T, int P, int MODE, bool ADJ>
__device__ __forceinline__ void stage_mid(Unit<T, P>& U) {
  constexpr int L1 = Tr<T, P>::L1, H = Tr<T, P>::H;
  const int cls = U.cls;
  for (int c = U.lane; c < H; c += 32) {
    cx<T> v[16];
    cx<T> hv[16];
    const bool prod = MODE == MID_FULL || MODE == MID_FROM_SPEC;
    // column 0 carries the packed kx = 0 / kx = P/2 columns: alpha / beta products
    const bool col0 = c == 0 && MODE == MID_FROM_SPEC;
    if (prod && (c != 0 || col0)) {
#pragma unroll
      for (int q = 0; q < 16; ++q) hv[q] = ldg2(U.hmain + (16 * cls + q) * H + c);
    }
    cx<T>* tb = U.tile + rf<P>(16 * cls, c);  // rows 16 cls + q at rfd(q)
    if (MODE == MID_FROM_SPEC || MODE == MID_FROM_ACC) {
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = U.spec[(16 * cls + q) * H + c];
      if (MODE == MID_FROM_ACC) {
        // partial sums of the CTAs that continued this patch, in CTA order
        for (int j = 0; j < U.nsp; ++j) {
          const cx<T>* sq = U.sp0 + (int64_t)j * (P * H);
#pragma unroll
          for (int q = 0; q < 16; ++q) v[q] = cadd<T>(v[q], sq[(16 * cls + q) * H + c]);
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const cx<T> t = tb[rfd<P>(q)];
        v[q] = q ? cmul<T>(t, U.wq[q]) : t;
      }
      Dft<16, false, T>::run(v);
    }
    if (MODE == MID_TO_SPEC) {
#pragma unroll
      for (int q = 0; q < 16; ++q) U.spec[(16 * cls + q) * H + c] = v[q];
      continue;
    }
    if (col0 && MODE == MID_FROM_SPEC) {
      // W'(ky) = alpha W(ky) + beta conj(W(-ky)), W(-ky) read from the shared spectrum
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const int ky = cls + L1 * q, km = (P - ky) % P;
        const int sm = 16 * (km % L1) + km / L1;
        const cx<T> wm = U.spec[sm * H];
        const cx<T> be = ldg2(U.hnyq + 16 * cls + q);
        v[q] = cadd<T>(cmul<T>(v[q], hv[q]), cmul<T>(cconj<T>(wm), be));
      }
    } else if (prod && c != 0) {
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = ADJ ? cmulc<T>(v[q], hv[q]) : cmul<T>(v[q], hv[q]);
    }
    // inverse variant-B step A; in MID_FULL column 0 waits for its product (stage_col0)
    if (c != 0 || MODE != MID_FULL) {
      Dft<16, true, T>::run(v);
#pragma unroll
      for (int q = 1; q < 16; ++q) v[q] = cmulc<T>(v[q], U.wq[q]);
    }
#pragma unroll
    for (int q = 0; q < 16; ++q) tb[rfd<P>(q)] = v[q];
  }
}

// ---- column 0 of the per-unit kernel: W'(ky) = alpha W(ky) + beta conj(W(-ky))
// (conjugated coefficients for the adjoint), pairs (ky, -ky) per thread, then
// the inverse column transform of column 0.  One warp.
template <typename T, int P, bool ADJ>
__device__ __forceinline__ void stage_col0(Unit<T, P>& U) {
  using R = Tr<T, P>;
  constexpr int L1 = R::L1, H = R::H;
  const int lane = U.lane;
  cx<T>* tile = U.tile;
  auto mulc = [&](cx<T> a, cx<T> b) { return ADJ ? cmulc<T>(a, b) : cmul<T>(a, b); };
  for (int ky = lane; ky <= H; ky += 32) {
    const int s1 = 16 * (ky % L1) + ky / L1;
    const int km = (P - ky) % P;
    const int s2 = 16 * (km % L1) + km / L1;
    const cx<T> w1 = tile[rf<P>(s1, 0)], w2 = tile[rf<P>(s2, 0)];
    const cx<T> a1 = ldg2(U.hmain + s1 * H), b1 = ldg2(U.hnyq + s1);
    tile[rf<P>(s1, 0)] = cadd<T>(mulc(w1, a1), mulc(cconj<T>(w2), b1));
    if (s2 != s1) {
      const cx<T> a2 = ldg2(U.hmain + s2 * H), b2 = ldg2(U.hnyq + s2);
      tile[rf<P>(s2, 0)] = cadd<T>(mulc(w2, a2), mulc(cconj<T>(w1), b2));
    }
  }
  __syncwarp();
  if (lane < L1) {  // inverse step A, class = lane
    cx<T> v[16];
#pragma unroll
    for (int q = 0; q < 16; ++q) v[q] = tile[rf<P>(16 * lane + q, 0)];
    Dft<16, true, T>::run(v);
#pragma unroll
    for (int q = 1; q < 16; ++q) v[q] = cmulc<T>(v[q], ldg2(U.twg + lane * q));
#pragma unroll
    for (int q = 0; q < 16; ++q) tile[rf<P>(16 * lane + q, 0)] = v[q];
  }
  __syncwarp();
  if (lane < 16) {  // inverse step B
    cx<T> v[L1];
#pragma unroll
    for (int i = 0; i < L1; ++i) v[i] = tile[rf<P>(16 * i + lane, 0)];
    Dft<L1, true, T>::run(v);
#pragma unroll
    for (int i = 0; i < L1; ++i) tile[rf<P>(16 * i + lane, 0)] = v[i];
  }
}

// ---- inverse variant-B step B for columns [C0, H) by threads t0 of nt
template <typename T, int P, int C0>
__device__ __forceinline__ void stage_invB(Unit<T, P>& U, int t0, int nt) {
  using R = Tr<T, P>;
  constexpr int L1 = R::L1, H = R::H, NC = H - C0;
  for (int it = t0; it < NC * 16; it += nt) {
    const int c = C0 + it % NC, q = it / NC;
    cx<T>* base = U.tile + rf<P>(q, c);  // rows 16 i + q
    cx<T> v[L1];
#pragma unroll
    for (int i = 0; i < L1; ++i) v[i] = base[8 * i * (P + 1)];
    Dft<L1, true, T>::run(v);
#pragma unroll
    for (int i = 0; i < L1; ++i) base[8 * i * (P + 1)] = v[i];
  }
}

// ---- combine (Hermitian pair rows) fused with inverse variant-A phase 1
template <typename T, int P>
__device__ __forceinline__ void stage_combine(Unit<T, P>& U, int jc_lo, int jc_hi) {
  using R = Tr<T, P>;
  constexpr int L1 = R::L1, H = R::H, NT = R::NT, TP = R::TP, HL = L1 / 2;
  const int ncp = jc_hi - jc_lo;
  for (int it = U.tid; it < ncp * 8; it += NT) {
    const int j = jc_lo + it % ncp, kap = it / ncp;
    cx<T>* row = U.tile + j * TP;
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

// Accumulate into an output element (group): one reduction per word.  TWO:
// the exact two-word form (Split2), hi into the output, lo into its low plane.
template <bool TWO>
__device__ __forceinline__ void acc4(float* hi, float* lo, const Split2<float>& sp, float a,
                                     float b, float c, float d) {
  if constexpr (TWO) {
    float h0, h1, h2, h3, l0, l1, l2, l3;
    sp.split(a, h0, l0);
    sp.split(b, h1, l1);
    sp.split(c, h2, l2);
    sp.split(d, h3, l3);
    red_add_v4(hi, h0, h1, h2, h3);
    red_add_v4(lo, l0, l1, l2, l3);
  } else {
    red_add_v4(hi, a, b, c, d);
  }
}
template <bool TWO, typename T>
__device__ __forceinline__ void acc1(T* hi, T* lo, const Split2<T>& sp, T v) {
  if constexpr (TWO) {
    T h, l;
    sp.split(v, h, l);
    atomicAdd(hi, h);
    atomicAdd(lo, l);
  } else {
    atomicAdd(hi, v);
  }
}

// ---- inverse variant-A phase 2 -> natural-order staging -> global
// forward: overlap-add of the whole P x P patch into out[m][e];
// adjoint: crop to the window, bilinear weights, scatter into out[e].
// TWO: exact two-word accumulation into out / out_lo with the splitter sp.
template <typename T, int P, bool ADJ, bool TWO = false>
__device__ __forceinline__ void stage_output(Unit<T, P>& U, const Args& a,
                                             const Split2<T>& sp = Split2<T>{}) {
  using R = Tr<T, P>;
  constexpr int L1 = R::L1, H = R::H, NT = R::NT, TP = R::TP, CH = R::CH;
  const int mg = U.mg, K = U.K, cb = U.cb, rb = U.rb;
  const T scale = (T)a.scale;
  const bool vec4 = ((cb + (ADJ ? mg : 0)) % 4 == 0) && (a.ny % 4 == 0) &&
                    (((uintptr_t)a.out) % 16 == 0) && (!TWO || ((uintptr_t)a.out_lo) % 16 == 0) &&
                    (ADJ ? K % 4 == 0 : true);
  const int jo_lo = ADJ ? mg / 2 : 0;
  const int jo_hi = ADJ ? (mg + K + 1) / 2 : H;
  const T* wt = U.wt;
  // chunk c writes its natural-order rows into the staging area (c even) or
  // into the tile pairs of chunk c-1, which its inverse transform already read
  for (int j0 = jo_lo, c = 0; j0 < jo_hi; j0 += CH, ++c) {
    const int nch = min(CH, jo_hi - j0);
    cx<T>* stg = (c & 1) ? U.tile + (j0 - CH) * TP : U.stg;
    for (int jj = U.lane; jj < nch; jj += 32) {
      const cx<T>* srcr = U.tile + (j0 + jj) * TP + 16 * U.cls;
      cx<T> v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = q ? cmulc<T>(srcr[q], U.wq[q]) : srcr[q];
      Dft<16, true, T>::run(v);
#pragma unroll
      for (int q = 0; q < 16; ++q) stg[jj * TP + U.cls + L1 * q] = v[q];
    }
    __syncthreads();
    const int64_t plane = ADJ ? (int64_t)U.e * U.npix : ((int64_t)U.m * a.E + U.e) * U.npix;
    T* __restrict__ dst = (T*)a.out + plane;
    T* __restrict__ dlo = TWO ? (T*)a.out_lo + plane : nullptr;
    if (!ADJ) {
      if (sizeof(T) == 4 && vec4) {
        // groups of 4 columns never straddle the field edge (cb, ny multiples of 4).
        // A warp takes 8 pair rows x 4 groups: with the pitch P + 1 = 1 (mod 16)
        // the staging reads of a half-warp fall on 16 distinct 8-byte bank pairs
        // (16 consecutive groups of one row would share 4 of them).
        constexpr int GT = P / 16;  // warp tiles across one row
        const int ntile = ((nch + 7) / 8) * GT;
        if (rb >= 0 && rb + P <= a.nx && cb >= 0 && cb + P <= a.ny) {
          // the whole P x P patch lies inside the field: no bounds checks
          const int64_t o0 = (int64_t)(rb + 2 * j0) * a.ny + cb;
          for (int w = U.warp; w < ntile; w += R::NW) {
            const int jj = 8 * (w / GT) + (U.lane >> 2);
            const int x = 16 * (w % GT) + 4 * (U.lane & 3);
            if (jj >= nch) continue;
            const cx<T>* sq = stg + jj * TP + x;
            const cx<T> z0 = sq[0], z1 = sq[1], z2 = sq[2], z3 = sq[3];
            const int64_t o = o0 + (int64_t)(2 * jj) * a.ny + x;
            acc4<TWO>((float*)(dst + o), (float*)(dlo + o), (const Split2<float>&)sp,
                      scale * z0.x, scale * z1.x, scale * z2.x, scale * z3.x);
            acc4<TWO>((float*)(dst + o + a.ny), (float*)(dlo + o + a.ny),
                      (const Split2<float>&)sp, scale * z0.y, scale * z1.y, scale * z2.y,
                      scale * z3.y);
          }
        } else
        for (int w = U.warp; w < ntile; w += R::NW) {
          const int jj = 8 * (w / GT) + (U.lane >> 2);
          const int x = 16 * (w % GT) + 4 * (U.lane & 3);
          if (jj >= nch) continue;
          const int col = cb + x;
          if (col < 0 || col >= a.ny) continue;
          const cx<T> z0 = stg[jj * TP + x], z1 = stg[jj * TP + x + 1];
          const cx<T> z2 = stg[jj * TP + x + 2], z3 = stg[jj * TP + x + 3];
          const int row = rb + 2 * (j0 + jj);
          if (row >= 0 && row < a.nx) {
            const int64_t o = (int64_t)row * a.ny + col;
            acc4<TWO>((float*)(dst + o), (float*)(dlo + o), (const Split2<float>&)sp,
                      scale * z0.x, scale * z1.x, scale * z2.x, scale * z3.x);
          }
          if (row + 1 >= 0 && row + 1 < a.nx) {
            const int64_t o = (int64_t)(row + 1) * a.ny + col;
            acc4<TWO>((float*)(dst + o), (float*)(dlo + o), (const Split2<float>&)sp,
                      scale * z0.y, scale * z1.y, scale * z2.y, scale * z3.y);
          }
        }
      } else {
        for (int i = U.tid; i < nch * P; i += NT) {
          const int jj = i / P, x = i - jj * P;
          const int col = cb + x;
          if (col < 0 || col >= a.ny) continue;
          const cx<T> z = stg[jj * TP + x];
          const int row = rb + 2 * (j0 + jj);
          if (row >= 0 && row < a.nx) {
            const int64_t o = (int64_t)row * a.ny + col;
            acc1<TWO, T>(dst + o, dlo + o, sp, scale * z.x);
          }
          if (row + 1 >= 0 && row + 1 < a.nx) {
            const int64_t o = (int64_t)(row + 1) * a.ny + col;
            acc1<TWO, T>(dst + o, dlo + o, sp, scale * z.y);
          }
        }
      }
    } else {
      if (sizeof(T) == 4 && vec4) {
        // warp tiles of 8 pair rows x 4 column groups, as in the forward branch
        const int G = K / 4, GT = (G + 3) / 4;
        const int ntile = ((nch + 7) / 8) * GT;
        for (int w = U.warp; w < ntile; w += R::NW) {
          const int jj = 8 * (w / GT) + (U.lane >> 2);
          const int g = 4 * (w % GT) + (U.lane & 3);
          if (jj >= nch || g >= G) continue;
          const int xa = 4 * g;
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
            const int64_t o = (int64_t)row * a.ny + col;
            acc4<TWO>((float*)(dst + o), (float*)(dlo + o), (const Split2<float>&)sp,
                      (wy * w4[0]) * z[0].x, (wy * w4[1]) * z[1].x, (wy * w4[2]) * z[2].x,
                      (wy * w4[3]) * z[3].x);
          }
          if (ya + 1 >= 0 && ya + 1 < K && row + 1 >= 0 && row + 1 < a.nx) {
            const T wy = wt[ya + 1];
            const int64_t o = (int64_t)(row + 1) * a.ny + col;
            acc4<TWO>((float*)(dst + o), (float*)(dlo + o), (const Split2<float>&)sp,
                      (wy * w4[0]) * z[0].y, (wy * w4[1]) * z[1].y, (wy * w4[2]) * z[2].y,
                      (wy * w4[3]) * z[3].y);
          }
        }
      } else {
        for (int i = U.tid; i < nch * K; i += NT) {
          const int jj = i / K, xa = i - jj * K;
          const int x = xa + mg, col = cb + x;
          if (col < 0 || col >= a.ny) continue;
          const cx<T> z = stg[jj * TP + x];
          const T wx = wt[xa] * scale;
          const int y0 = 2 * (j0 + jj);
          const int ya = y0 - mg, row = rb + y0;
          if (ya >= 0 && ya < K && row >= 0 && row < a.nx) {
            const int64_t o = (int64_t)row * a.ny + col;
            acc1<TWO, T>(dst + o, dlo + o, sp, (wt[ya] * wx) * z.x);
          }
          if (ya + 1 >= 0 && ya + 1 < K && row + 1 >= 0 && row + 1 < a.nx) {
            const int64_t o = (int64_t)(row + 1) * a.ny + col;
            acc1<TWO, T>(dst + o, dlo + o, sp, (wt[ya + 1] * wx) * z.y);
          }
        }
      }
    }
  }
}

// ---- ordered module sum of the module-shared adjoint (one problem)
// Thread (warp w, lane) holds, for its NCI column iterations, 16 complex
// values of the patch's running sum in TMEM lane 32 (w % 4) + lane, columns
// (w / 4) * PER_WARP + i * WC ... + WC.
template <typename T, int P>
struct TmemGeom {
  static constexpr int H = P / 2, NW = P / 16;
  static constexpr int NCI = (H + 31) / 32;                   // column iterations per thread
  static constexpr int WC = 16 * (int)sizeof(cx<T>) / 4;      // 32-bit columns per iteration
  static constexpr int PER_WARP = NCI * WC;
  static constexpr int NEED = ((NW + 3) / 4) * PER_WARP;
  static constexpr int NCOLS = NEED <= 32 ? 32 : NEED <= 64 ? 64 : NEED <= 128 ? 128
                               : NEED <= 256 ? 256 : 512;
  static_assert(NEED <= 512, "the running sum must fit the 512 TMEM columns of an SM");
};

// v[q] += the 16 complex values at TMEM address ta (this thread's lane)
template <typename T>
__device__ __forceinline__ void tmem_add16(uint32_t ta, cx<T> (&v)[16]) {
  if constexpr (sizeof(T) == 4) {
    uint32_t r[32];
    tmem_ld32(ta, r);
#pragma unroll
    for (int q = 0; q < 16; ++q)
      v[q] = mkc<T>(v[q].x + __uint_as_float(r[2 * q]), v[q].y + __uint_as_float(r[2 * q + 1]));
  } else {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint32_t r[32];
      tmem_ld32(ta + 32 * h, r);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int q = 8 * h + j;
        v[q] = mkc<T>(v[q].x + __hiloint2double((int)r[4 * j + 1], (int)r[4 * j]),
                      v[q].y + __hiloint2double((int)r[4 * j + 3], (int)r[4 * j + 2]));
      }
    }
  }
}
template <typename T>
__device__ __forceinline__ void tmem_put16(uint32_t ta, const cx<T> (&v)[16]) {
  if constexpr (sizeof(T) == 4) {
    uint32_t r[32];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      r[2 * q] = __float_as_uint(v[q].x);
      r[2 * q + 1] = __float_as_uint(v[q].y);
    }
    tmem_st32(ta, r);
  } else {
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      uint32_t r[32];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int q = 8 * h + j;
        r[4 * j] = (uint32_t)__double2loint(v[q].x);
        r[4 * j + 1] = (uint32_t)__double2hiint(v[q].x);
        r[4 * j + 2] = (uint32_t)__double2loint(v[q].y);
        r[4 * j + 3] = (uint32_t)__double2hiint(v[q].y);
      }
      tmem_st32(ta + 32 * h, r);
    }
  }
}

// The cotangent spectrum of this unit times conj(PSF spectrum), added to the
// patch's running sum over modules in TMEM.  The first unit of a patch in the
// CTA's range starts the sum; the last writes it to `dest` (the patch's
// accumulator, or this CTA's spill slot when an earlier CTA holds module 0).
// Column 0 (the packed kx = 0 / P/2 columns) takes the scatter form, whose two
// terms land on rows of different warps: they meet in shared memory (c0own,
// c0mir) and column 0's sum stays there (c0acc).  Sums run in module order:
// the result does not depend on timing.
template <typename T, int P>
__device__ __forceinline__ void stage_acc_tmem(Unit<T, P>& U, uint32_t tbase, bool first,
                                               bool last, cx<T>* dest, cx<T>* c0own,
                                               cx<T>* c0mir, cx<T>* c0acc) {
  using TG = TmemGeom<T, P>;
  constexpr int L1 = Tr<T, P>::L1, H = TG::H, NT = Tr<T, P>::NT;
  const int cls = U.cls;
  const uint32_t trow = tbase + ((uint32_t)(32 * (U.warp & 3)) << 16) +
                        (uint32_t)((U.warp >> 2) * TG::PER_WARP);
#pragma unroll 1
  for (int i = 0; i < TG::NCI; ++i) {
    const int c = U.lane + 32 * i;
    const bool act = c < H;
    cx<T> v[16];
    if (act) {
      cx<T> hv[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) hv[q] = ldg2(U.hmain + (16 * cls + q) * H + c);
      const cx<T>* tb = U.tile + rf<P>(16 * cls, c);
#pragma unroll
      for (int q = 0; q < 16; ++q) {
        const cx<T> t = tb[rfd<P>(q)];
        v[q] = q ? cmul<T>(t, U.wq[q]) : t;
      }
      Dft<16, false, T>::run(v);
      if (c == 0) {
        // W(ky) adds conj(alpha(ky)) W(ky) to ky and conj(beta(-ky)) conj(W(ky)) to -ky
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const int ky = cls + L1 * q, km = (P - ky) % P;
          const int sm = 16 * (km % L1) + km / L1;
          c0own[16 * cls + q] = cmulc<T>(v[q], hv[q]);
          c0mir[sm] = cconj<T>(cmul<T>(v[q], ldg2(U.hnyq + sm)));
        }
      } else {
#pragma unroll
        for (int q = 0; q < 16; ++q) v[q] = cmulc<T>(v[q], hv[q]);
      }
    } else {
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = mkc<T>((T)0, (T)0);
    }
    // the running sum: warp-collective TMEM access, every lane takes part
    const uint32_t ta = trow + (uint32_t)(i * TG::WC);
    if (!first) tmem_add16<T>(ta, v);
    if (last) {
      if (act && c != 0) {
#pragma unroll
        for (int q = 0; q < 16; ++q) dest[(16 * cls + q) * H + c] = v[q];
      }
    } else {
      tmem_put16<T>(ta, v);
    }
  }
  if (!last) tmem_wait_st();
  __syncthreads();  // column 0 terms of every warp are in shared memory
  for (int sr = threadIdx.x; sr < P; sr += NT) {
    cx<T> t = cadd<T>(c0own[sr], c0mir[sr]);
    if (!first) t = cadd<T>(c0acc[sr], t);
    if (last)
      dest[sr * H] = t;
    else
      c0acc[sr] = t;
  }
}

// column 0 (warp 0) in parallel with the inverse step B of columns 1.. (other warps)
template <typename T, int P, bool ADJ>
__device__ __forceinline__ void stage_col0_and_invB(Unit<T, P>& U) {
  constexpr int NT = Tr<T, P>::NT;
  if (U.warp == 0) stage_col0<T, P, ADJ>(U);
  if (NT > 32) {
    if (U.warp > 0) stage_invB<T, P, 1>(U, U.tid - 32, NT - 32);
  } else {
    __syncwarp();
    stage_invB<T, P, 1>(U, U.tid, NT);
  }
}

__device__ __forceinline__ void prefetch_unit(const void* h, unsigned hb, const void* hn,
                                              unsigned nb) {
  if (threadIdx.x == 0) {
    prefetch_l2(h, hb);
    prefetch_l2(hn, nb);
  }
}

// Where a kernel's block (or loop) index g finds its arguments: one problem
// (the kernel parameter itself), or a list of independent problems, problem p
// owning indices [starts[p], starts[p + 1]) (grouped launches).
struct OneProblem {
  Args a;
  __device__ __forceinline__ const Args& at(int g, int& local) const {
    local = g;
    return a;
  }
};
// ProblemList::at returns a copy: the kernels then read the fields from
// registers or local memory, not through a pointer into global memory that
// their own stores could alias (which would keep every field access a load).
struct ProblemList {
  const Args* list;
  const int* starts;
  int n;
  __device__ __forceinline__ Args at(int g, int& local) const {
    int lo = 0, hi = n - 1;  // the last problem whose first index is <= g
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(starts + mid) <= g)
        lo = mid;
      else
        hi = mid - 1;
    }
    local = g - __ldg(starts + lo);
    return list[lo];
  }
};

// ================================================================= kernels
// The output bound of a kernel that accumulates in two words: bnd_scale times
// the largest stored input magnitude (read after the dependency wait).
template <typename T>
__device__ __forceinline__ Split2<T> output_splitter(const Args& a, unsigned long long* s_slot) {
  Split2<T> sp;
  const double m = reduce_bound(a.bnd_in, a.bnd_n, s_slot);
  sp.init(a.bnd_scale * m, a.bnd_log2);
  return sp;
}

// The same for a bound already reduced to one value (bnd_n == 1), per thread:
// no CTA-wide step, so a loop over the units of several problems can take
// each unit's problem's splitter.
template <typename T>
__device__ __forceinline__ Split2<T> splitter_one(const Args& a) {
  Split2<T> sp;
  sp.init(a.bnd_scale * __longlong_as_double((long long)__ldcg(a.bnd_in)), a.bnd_log2);
  return sp;
}

// One CTA per unit: the whole forward or adjoint of one patch.  TWO: the
// output accumulates in two words (one problem; its input bound was recorded
// by a pass before this kernel).
template <typename T, int P, bool ADJ, bool TWO>
__device__ __forceinline__ void fused_unit_body(const Args& a, int ub, unsigned char* smem_raw,
                                                unsigned long long* s_slot) {
  using R = Tr<T, P>;
  Unit<T, P> U;
  U.init(a, smem_raw, true, ub);
  prefetch_unit(U.hmain, sizeof(cx<T>) * P * R::H, U.hnyq, sizeof(cx<T>) * P);
  pdl_wait();
  Split2<T> sp{};
  if constexpr (TWO) sp = output_splitter<T>(a, s_slot);
  stage_input<T, P, ADJ>(U, a);
  stage_split<T, P>(U);
  __syncthreads();
  stage_col1<T, P, ADJ>(U, ADJ ? 0 : 2 * (U.mg / 2), ADJ ? P : 2 * ((U.mg + U.K + 1) / 2));
  __syncthreads();
  stage_mid<T, P, MID_FULL, ADJ>(U);
  __syncthreads();
  stage_col0_and_invB<T, P, ADJ>(U);
  __syncthreads();
  stage_combine<T, P>(U, ADJ ? U.mg / 2 : 0, ADJ ? (U.mg + U.K + 1) / 2 : R::H);
  __syncthreads();
  stage_output<T, P, ADJ, TWO>(U, a, sp);
}

template <typename T, int P, bool ADJ>
__global__ void __launch_bounds__(Tr<T, P>::NT) k_fused(Args a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long s_slot;
  pdl_trigger();
  fused_unit_body<T, P, ADJ, true>(a, (int)blockIdx.x, smem_raw, &s_slot);
}

// Grouped launch over independent problems of one FFT side: problem p owns
// blocks [starts[p], starts[p + 1]) and its own arguments list[p].  Each
// problem's output accumulates exactly in two words, with its own bound.
template <typename T, int P, bool ADJ>
__global__ void __launch_bounds__(Tr<T, P>::NT)
    k_fused_group(const Args* __restrict__ list, const int* __restrict__ starts, int nprob) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_prob;
  __shared__ unsigned long long s_slot;
  pdl_trigger();
  if (threadIdx.x == 0) {  // the last problem whose first block is <= blockIdx.x
    int lo = 0, hi = nprob - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (starts[mid] <= (int)blockIdx.x)
        lo = mid;
      else
        hi = mid - 1;
    }
    s_prob = lo;
  }
  __syncthreads();
  const int p = s_prob;
  const Args a = list[p];
  fused_unit_body<T, P, ADJ, true>(a, (int)blockIdx.x - starts[p], smem_raw, &s_slot);
}

// Forward, module-shared: the sky spectrum of each (energy, patch) once; the
// CTAs also clear the (M,E,nx,ny) output that the next kernel adds into, and
// (one problem) record the largest weighted sky magnitude of their window ...
template <typename T, int P, typename Src>
__global__ void __launch_bounds__(Tr<T, P>::NT) k_sky_spec(Src src) {
  constexpr bool ORD = std::is_same<Src, OneProblem>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long s_slot;
  Unit<T, P> U;
  pdl_trigger();
  int item;
  const Args& a = src.at((int)blockIdx.x, item);
  U.init(a, smem_raw, false, item);
  pdl_wait();
  const int64_t obytes = (int64_t)a.M * a.E * a.nx * a.ny * (int64_t)sizeof(T);
  zero_slice(a.out, obytes, a.zchunk);
  if (ORD && a.out_lo) zero_slice(a.out_lo, obytes, a.zchunk);
  if (a.aux) zero_slice(a.aux, a.aux_bytes, a.aux_chunk);
  stage_input<T, P, false, ORD>(U, a);
  if constexpr (ORD) {
    const unsigned long long m = cta_max(mag_as_double_bits(U.mx), &s_slot);
    if (threadIdx.x == 0 && a.bnd_out) a.bnd_out[item] = m;
  }
  stage_split<T, P>(U);
  __syncthreads();
  stage_col1<T, P>(U, 2 * (U.mg / 2), 2 * ((U.mg + U.K + 1) / 2));
  __syncthreads();
  stage_mid<T, P, MID_TO_SPEC, false>(U);
}

// ... then, per unit, spectrum * PSF spectrum -> inverse -> overlap-add, as a
// loop over units (CTA b takes units b, b + G, ...; G = gridDim.x, as many
// CTAs as fit on the GPU at once; one per SM at P = 192).  The next unit's PSF and shared spectra are prefetched into L2 when this
// unit's output stage starts: its reductions leave the HBM reads free, and the
// data is in L2 when the next unit's spectrum stage reads it.  (Prefetching a
// whole unit ahead was slower: the prefetches then compete with the current
// unit's spectrum loads.)  One problem: the overlap-add is exact in two words.
template <typename T, int P, typename Src>
__global__ void __launch_bounds__(Tr<T, P>::NT) k_fwd_from_spec(Src src, int units) {
  using R = Tr<T, P>;
  constexpr bool ORD = std::is_same<Src, OneProblem>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long s_slot;
  Unit<T, P> U;
  pdl_trigger();
  int g = blockIdx.x;
  {
    int lu;
    U.init(src.at(g, lu), smem_raw, true, lu);
  }
  prefetch_unit(U.hmain, sizeof(cx<T>) * P * R::H, U.hnyq, sizeof(cx<T>) * P);
  pdl_wait();
  if (threadIdx.x == 32) prefetch_l2(U.spec, sizeof(cx<T>) * P * R::H);
  Split2<T> sp{};
  if constexpr (ORD) {
    int lu;
    sp = output_splitter<T>(src.at(g, lu), &s_slot);
  }
  for (;;) {
    const int gn = g + (int)gridDim.x;
    if constexpr (!ORD) {  // each problem of a list has its own bound, reduced to one value
      int lu;
      sp = splitter_one<T>(src.at(g, lu));
    }
    stage_mid<T, P, MID_FROM_SPEC, false>(U);
    __syncthreads();
    stage_invB<T, P, 0>(U, U.tid, R::NT);
    __syncthreads();
    stage_combine<T, P>(U, 0, R::H);
    __syncthreads();
    if (gn < units) {  // the output stage's reductions leave HBM reads free
      int lun;
      Unit<T, P> N;
      N.geom(src.at(gn, lun), smem_raw, true, lun);
      prefetch_unit(N.hmain, sizeof(cx<T>) * P * R::H, N.hnyq, sizeof(cx<T>) * P);
      if (threadIdx.x == 32) prefetch_l2(N.spec, sizeof(cx<T>) * P * R::H);
    }
    {
      int lu;
      stage_output<T, P, false, true>(U, src.at(g, lu), sp);
    }
    if (gn >= units) break;
    __syncthreads();  // the output stage's last staging reads before the next mid writes
    g = gn;
    int lu;
    U.geom(src.at(g, lu), smem_raw, true, lu);
  }
}

// ---- forward of aligned geometries in runs of vertically adjacent patches
// When P = 3 dx with dx = 64 and margin dx / 2, a patch's P x P output covers
// exactly three block rows of dx field rows (i - 1, i, i + 1 for patch row i),
// and the staging chunks of the output stage (32 pair rows) are those block
// rows.  A CTA then takes runs of a.run_len (2 or 4) vertically adjacent
// patches of one module and adds the block rows they share in TMEM, in patch
// order, before they leave the CTA: each block row of a run is reduced into the
// image once (as an exact two-word sum), 6 block rows per run of 4 patches
// instead of 12.  The modules of a run are consecutive work items, which
// neighbouring CTAs run at the same time, so the shared sky spectra still meet
// in L2.  Longer runs mean fewer reductions but fewer work items: the run
// length is a schedule choice (auto_run_len, or set per plan).
constexpr int kRunCols = 96;  // TMEM columns of one pending block row (per lane)

// Output stage of patch s (0 .. run_len - 1) of a run: chunk c is block row
// i - 1 + c.  Thread (warp w, lane) owns, in every chunk, the warp tiles of
// the overlap-add (8 pair rows x 16 columns; the tile row tau = 0..3 gives pair
// rows 8 tau + lane / 4, columns 16 w + 4 (lane % 4) .. + 4): 32 values, kept for
// the pending block rows in its TMEM lane 32 (w % 4) + lane, columns
// 96 slot + 32 (w / 4) .. + 32 (slot = block row % 2).
template <typename T, int P>
__device__ __forceinline__ void stage_output_run(Unit<T, P>& U, const Args& a,
                                                 const Split2<T>& sp, uint32_t tbase, int s) {
  static_assert(sizeof(T) == 4 && P == 192, "runs cover FP32 patches of side 192");
  using R = Tr<T, P>;
  constexpr int L1 = R::L1, TP = R::TP, CH = R::CH;
  const T scale = (T)a.scale;
  const uint32_t tl = tbase + ((uint32_t)(32 * (U.warp & 3)) << 16) +
                      (uint32_t)((U.warp >> 2) * 32);
  const int64_t plane = ((int64_t)U.m * a.E + U.e) * U.npix;
  T* __restrict__ dst = (T*)a.out + plane;
  T* __restrict__ dlo = (T*)a.out_lo + plane;
  const int x = 16 * U.warp + 4 * (U.lane & 3);
  const int col = U.cb + x;  // a multiple of 4: the group lies wholly in or out of the field
  const bool col_in = col >= 0 && col + 4 <= a.ny;
  const int i = U.k % a.n;  // patch row
  for (int c = 0; c < 3; ++c) {
    const int j0 = c * CH;
    cx<T>* stg = (c & 1) ? U.tile + (j0 - CH) * TP : U.stg;
    {  // inverse variant-A phase 2 of the chunk's 32 pair rows -> natural order
      const int jj = U.lane;
      const cx<T>* srcr = U.tile + (j0 + jj) * TP + 16 * U.cls;
      cx<T> v[16];
#pragma unroll
      for (int q = 0; q < 16; ++q) v[q] = q ? cmulc<T>(srcr[q], U.wq[q]) : srcr[q];
      Dft<16, true, T>::run(v);
#pragma unroll
      for (int q = 0; q < 16; ++q) stg[jj * TP + U.cls + L1 * q] = v[q];
    }
    __syncthreads();
    T v[32];  // tile row tau: v[8 tau .. + 4] row 2 jj, v[8 tau + 4 .. + 4] row 2 jj + 1
#pragma unroll
    for (int tau = 0; tau < 4; ++tau) {
      const cx<T>* sq = stg + (8 * tau + (U.lane >> 2)) * TP + x;
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const cx<T> z = sq[t];
        v[8 * tau + t] = scale * z.x;
        v[8 * tau + 4 + t] = scale * z.y;
      }
    }
    const int br = i - 1 + c;  // block row of the field
    const uint32_t ta = tl + (uint32_t)(((br + 2) & 1) * kRunCols);
    // warp-uniform: pending rows exist from the run's previous patch; a row
    // leaves the CTA once no later patch of the run adds to it
    if (s > 0 && c < 2) {
      uint32_t r[32];
      tmem_ld32(ta, r);
#pragma unroll
      for (int j = 0; j < 32; ++j) v[j] += __uint_as_float(r[j]);
    }
    if (c == 0 || s == a.run_len - 1) {
      if (col_in) {
#pragma unroll
        for (int tau = 0; tau < 4; ++tau) {
          const int row = U.rb + 2 * (j0 + 8 * tau + (U.lane >> 2));
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            if (row + h < 0 || row + h >= a.nx) continue;
            const int64_t o = (int64_t)(row + h) * a.ny + col;
            const int q = 8 * tau + 4 * h;
            acc4<true>((float*)(dst + o), (float*)(dlo + o), (const Split2<float>&)sp, v[q],
                       v[q + 1], v[q + 2], v[q + 3]);
          }
        }
      }
    } else {
      uint32_t r[32];
#pragma unroll
      for (int j = 0; j < 32; ++j) r[j] = __float_as_uint(v[j]);
      tmem_st32(ta, r);
    }
  }
  tmem_wait_st();
}

// Work item w of the run-ordered forward: module fastest, then the run q of
// run_len patch rows, the patch column j, the energy e.  Returns unit (w, s).
__device__ __forceinline__ int run_unit(const Args& a, int w, int s) {
  const int nq = a.n / a.run_len;
  int t = div_by(w, a.M, a.div_M);
  const int m = w - t * a.M;
  const int t2 = div_by(t, nq, a.div_nq);
  const int q = t - t2 * nq;
  t = t2;
  const int e = div_by(t, a.n, a.div_n), j = t - e * a.n;
  const int k = a.run_len * q + s + a.n * j;
  return ((e * a.n * a.n + k) * a.M + m);
}

template <typename T, int P>
__global__ void __launch_bounds__(Tr<T, P>::NT) k_fwd_run(Args a, int items) {
  using R = Tr<T, P>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long s_slot;
  __shared__ uint32_t s_tmem;
  pdl_trigger();
  int w = blockIdx.x, s = 0;
  Unit<T, P> U;
  U.init(a, smem_raw, true, run_unit(a, w, 0));
  prefetch_unit(U.hmain, sizeof(cx<T>) * P * R::H, U.hnyq, sizeof(cx<T>) * P);
  if (U.warp == 0) tmem_alloc(&s_tmem, 2 * kRunCols <= 256 ? 256 : 512);
  tmem_fence_before_sync();
  __syncthreads();
  tmem_fence_after_sync();
  const uint32_t tbase = s_tmem;
  pdl_wait();
  if (threadIdx.x == 32) prefetch_l2(U.spec, sizeof(cx<T>) * P * R::H);
  const Split2<T> sp = output_splitter<T>(a, &s_slot);
  for (;;) {
    const int sn = s + 1 < a.run_len ? s + 1 : 0;
    const int wn = s + 1 < a.run_len ? w : w + (int)gridDim.x;
    const bool more = wn < items;
    stage_mid<T, P, MID_FROM_SPEC, false>(U);
    __syncthreads();
    stage_invB<T, P, 0>(U, U.tid, R::NT);
    __syncthreads();
    stage_combine<T, P>(U, 0, R::H);
    __syncthreads();
    if (more) {  // the output stage's reductions leave HBM reads free
      Unit<T, P> N;
      N.geom(a, smem_raw, true, run_unit(a, wn, sn));
      prefetch_unit(N.hmain, sizeof(cx<T>) * P * R::H, N.hnyq, sizeof(cx<T>) * P);
      if (threadIdx.x == 32) prefetch_l2(N.spec, sizeof(cx<T>) * P * R::H);
    }
    stage_output_run<T, P>(U, a, sp, tbase, s);
    if (!more) break;
    __syncthreads();  // the output stage's last staging reads before the next mid writes
    w = wn;
    s = sn;
    U.geom(a, smem_raw, true, run_unit(a, w, s));
  }
  tmem_fence_before_sync();
  __syncthreads();
  tmem_fence_after_sync();
  if (U.warp == 0) tmem_dealloc(tbase, 2 * kRunCols <= 256 ? 256 : 512);
}

// Shared memory of the ordered adjoint beyond the tile: column 0's two terms
// and running sum (3 P complex values).
template <typename T, int P>
constexpr size_t ord_extra_smem() { return 3 * (size_t)P * sizeof(cx<T>); }

// Unit schedule of the ordered adjoint over P patches of M modules on G CTAs:
// R = floor(P / G) full rounds in which CTA b takes patch b + r G with all its
// modules (neighbouring CTAs work on neighbouring patches at the same time, so
// the overlapping cotangent windows meet in L2), then the units of the
// remaining patches in Gt = min(G, tail units) non-empty contiguous ranges
// (CTAs b >= Gt have none).  Tail units are u = tail0 ... (unit u = patch * M +
// module).
struct OrdSchedule {
  int64_t G, M, rounds, tail0, tail_units, Gt;
  __device__ __forceinline__ OrdSchedule(int64_t g, int64_t m, int64_t patches)
      : G(g), M(m), rounds(patches / g), tail0((patches / g) * g * m),
        tail_units((patches - (patches / g) * g) * m),
        Gt(tail_units < g ? tail_units : g) {}
  __device__ __forceinline__ int64_t tail_lo(int64_t b) const {
    return b >= Gt ? tail0 + tail_units : tail0 + b * tail_units / Gt;
  }
  __device__ __forceinline__ int64_t count(int64_t b) const {
    return rounds * M + tail_lo(b + 1) - tail_lo(b);
  }
  __device__ __forceinline__ int64_t unit(int64_t b, int64_t t) const {
    if (t < rounds * M) return (b + (t / M) * G) * M + t % M;
    return tail_lo(b) + (t - rounds * M);
  }
};

// Adjoint, module-shared, one problem, in module order: each CTA takes its
// units from OrdSchedule -- the modules of a patch one after another -- and
// sums each patch's products over modules in TMEM in module order
// (stage_acc_tmem).  The CTA holding module 0 of a patch writes the patch's
// accumulator; a CTA whose tail range starts inside a patch writes its part to
// its spill slot, which the next kernel adds in CTA order.  No atomics, no
// clearing of the accumulator: the sums are the same bits on every run.  The
// CTAs clear the gradient's low words (and, when asked, the gradient); the
// bound of the gradient terms comes from the kernel that wrote the cotangent.
//
// Position in a CTA's unit sequence of OrdSchedule, advanced without divisions.
struct OrdCursor {
  int64_t t, r, m, g;
  __device__ __forceinline__ OrdCursor(const OrdSchedule& s, int64_t b)
      : t(0), r(0), m(0), g(s.unit(b, 0)) {}
  __device__ __forceinline__ void advance(const OrdSchedule& s, int64_t b, int64_t tlo) {
    ++t;
    if (t < s.rounds * s.M) {
      if (++m == s.M) {
        m = 0;
        ++r;
      }
      g = (b + r * s.G) * s.M + m;
    } else {
      g = tlo + (t - s.rounds * s.M);
    }
  }
};

// The ordered adjoint of one problem on CTA b of the G CTAs given to it.
template <typename T, int P>
__device__ __forceinline__ void ord_adjoint(const Args& a, int64_t b, int64_t G, int units,
                                            unsigned char* smem_raw, uint32_t* s_tmem) {
  using R = Tr<T, P>;
  using TG = TmemGeom<T, P>;
  cx<T>* c0 = reinterpret_cast<cx<T>*>(smem_raw + R::SMEM);
  const OrdSchedule sch(G, a.M, units / a.M);
  const int64_t cnt = sch.count(b), tlo = sch.tail_lo(b), tail_start = sch.rounds * sch.M;
  OrdCursor cur(sch, b);
  Unit<T, P> U;
  U.init(a, smem_raw, true, (int)cur.g);
  prefetch_unit(U.hmain, sizeof(cx<T>) * P * R::H, U.hnyq, sizeof(cx<T>) * P);
  if (U.warp == 0) tmem_alloc(s_tmem, TG::NCOLS);
  tmem_fence_before_sync();
  __syncthreads();
  tmem_fence_after_sync();
  const uint32_t tbase = *s_tmem;
  pdl_wait();
  const int64_t gbytes = (int64_t)a.E * a.nx * a.ny * (int64_t)sizeof(T);
  if (a.zero_out) zero_slice(a.out, gbytes, a.zchunk);
  if (a.out_lo) zero_slice(a.out_lo, gbytes, a.zchunk);
  bool pre = false;
  while (cur.t < cnt) {
    const int64_t t = cur.t, g = cur.g;
    stage_input<T, P, true>(U, a, pre);
    stage_split<T, P>(U);
    __syncthreads();
    stage_col1<T, P, true>(U, 0, P);
    __syncthreads();
    OrdCursor nx = cur;
    nx.advance(sch, b, tlo);
    Unit<T, P> N;
    if (nx.t < cnt) {  // the next unit's first input chunk, into the staging area
      N.geom(a, smem_raw, true, (int)nx.g);
      input_issue<T, P, true>(N, a, InChunks<T, P, true>(N), 0);
    }
    const bool first = U.m == 0 || t == tail_start;
    const bool last = U.m == a.M - 1 || t == cnt - 1;
    const bool owner = t < tail_start || g - U.m >= tlo;  // module 0 of this patch is ours
    cx<T>* dest = owner ? U.spec : (cx<T>*)a.spill + b * (int64_t)(P * R::H);
    stage_acc_tmem<T, P>(U, tbase, first, last, dest, c0, c0 + P, c0 + 2 * P);
    if (nx.t >= cnt) break;
    __syncthreads();
    cur = nx;
    U.geom(a, smem_raw, true, (int)cur.g);
    prefetch_unit(U.hmain, sizeof(cx<T>) * P * R::H, U.hnyq, sizeof(cx<T>) * P);
    pre = true;
  }
  tmem_fence_before_sync();
  __syncthreads();
  tmem_fence_after_sync();
  if (U.warp == 0) tmem_dealloc(tbase, TG::NCOLS);
}

template <typename T, int P>
__global__ void __launch_bounds__(Tr<T, P>::NT) k_adj_to_spec_ord(Args a, int units) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint32_t s_tmem;
  pdl_trigger();
  ord_adjoint<T, P>(a, blockIdx.x, gridDim.x, units, smem_raw, &s_tmem);
}

// The ordered adjoint over a list of independent problems: problem p takes CTAs
// [cta_starts[p], cta_starts[p + 1]) and runs its own schedule on them (its
// spill slots hold that many CTAs).  The grouped pass clears every output first.
template <typename T, int P>
__global__ void __launch_bounds__(Tr<T, P>::NT)
    k_adj_to_spec_ord_list(const Args* __restrict__ list, const int* __restrict__ cta_starts,
                           int nprob) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ uint32_t s_tmem;
  pdl_trigger();
  int lo = 0, hi = nprob - 1;  // the last problem whose first CTA is <= blockIdx.x
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(cta_starts + mid) <= (int)blockIdx.x)
      lo = mid;
    else
      hi = mid - 1;
  }
  const Args a = list[lo];
  const int64_t b0 = __ldg(cta_starts + lo), G = __ldg(cta_starts + lo + 1) - b0;
  ord_adjoint<T, P>(a, (int64_t)blockIdx.x - b0, G, a.M * a.E * a.n * a.n, smem_raw, &s_tmem);
}

// ... then, per (energy, patch), one inverse transform -> window -> gradient:
// the patch's module sum plus the continuing CTAs' spill slots (in CTA order),
// and the gradient accumulates exactly in two words (each problem with its own
// bound).
template <typename T, int P, typename Src>
__global__ void __launch_bounds__(Tr<T, P>::NT) k_adj_from_spec(Src src) {
  using R = Tr<T, P>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long s_slot;
  Unit<T, P> U;
  pdl_trigger();
  int item;
  const Args& a = src.at((int)blockIdx.x, item);
  U.init(a, smem_raw, false, item);
  {  // the module sums of the ordered adjoint: this patch's plus any spill slots
    // CTAs of the ordered adjoint whose tail range starts inside this patch:
    // tail_lo(b) in (u0, u0 + M) (none for the patches of the full rounds)
    const int64_t G = a.loop_grid, patches = (int64_t)a.E * a.n * a.n;
    const OrdSchedule sch(G, a.M, patches);
    const int64_t u0 = (int64_t)item * a.M;
    int n = 0;
    int64_t b = 0;
    if (u0 >= sch.tail0 && sch.tail_units > 0) {
      b = ((u0 + 1 - sch.tail0) * sch.Gt + sch.tail_units - 1) / sch.tail_units;
      while (b + n < sch.Gt && sch.tail_lo(b + n) < u0 + a.M) ++n;
    }
    U.sp0 = (const cx<T>*)a.spill + b * (int64_t)(P * R::H);
    U.nsp = n;
  }
  pdl_wait();
  // the module sum (written by the previous kernel, mostly evicted from L2 by its
  // PSF stream) is read in three rounds of loads: fetch all of it into L2 at once
  if (threadIdx.x == 0) {
    prefetch_l2(U.spec, sizeof(cx<T>) * P * R::H);
    for (int j = 0; j < U.nsp; ++j)
      prefetch_l2(U.sp0 + (int64_t)j * (P * R::H), sizeof(cx<T>) * P * R::H);
  }
  const Split2<T> sp = output_splitter<T>(a, &s_slot);  // the gradient is exact in two words
  stage_mid<T, P, MID_FROM_ACC, true>(U);
  __syncthreads();
  stage_invB<T, P, 0>(U, U.tid, R::NT);
  __syncthreads();
  stage_combine<T, P>(U, U.mg / 2, (U.mg + U.K + 1) / 2);
  __syncthreads();
  stage_output<T, P, true, true>(U, a, sp);
}

template <typename KernelT>
int set_smem(KernelT kern, size_t smem) {
  return cuda_status(
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
      "cudaFuncSetAttribute");
}

// Grid of a loop kernel over `count` items: as many CTAs as fit on the
// current device at once (the kernel's occupancy per SM from its shared
// memory, registers and block size -- one at P = 192, several at small P), at
// most one per item.  Cached per kernel and device.
struct OccEntry {
  const void* kern;
  int dev, per_sm;
};
std::mutex g_occ_mu;
std::vector<OccEntry> g_occ;

template <typename T, int P, typename KernelT>
int64_t loop_grid(KernelT kern, int64_t count, size_t smem = Tr<T, P>::SMEM) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) dev = 0;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lock(g_occ_mu);
    for (const OccEntry& e : g_occ)
      if (e.kern == (const void*)kern && e.dev == dev) per_sm = e.per_sm;
  }
  if (!per_sm) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, Tr<T, P>::NT, smem) !=
            cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    }
    std::lock_guard<std::mutex> lock(g_occ_mu);
    g_occ.push_back(OccEntry{(const void*)kern, dev, per_sm});
  }
  return std::max<int64_t>(1, std::min<int64_t>(count, (int64_t)sm_count() * per_sm));
}

// Kernel arguments of one stage of one plan (sizes in bytes use esz).
// numerators of the unit decompositions stay below the unit count
void set_div_consts(Args& a, int64_t units) {
  const int64_t bound = units + 1;
  a.div_M = mulhi_divisor(a.M, bound);
  a.div_n2 = mulhi_divisor((int64_t)a.n * a.n, bound);
  a.div_n = mulhi_divisor(a.n, bound);
  a.div_nq = a.run_len > 0 ? mulhi_divisor(a.n / a.run_len, bound) : 0;
}

Args make_args(const Geom& g, const FusedLaunch& f, int which, size_t esz) {
  Args a;
  a.in = f.in;
  a.out = f.out;
  a.hmain = f.hmain;
  a.hnyq = f.hnyq;
  a.tw = f.tw;
  a.wt = f.wt;
  a.spec = f.spec;
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
  const int64_t units = g.units();
  const int64_t patches = (int64_t)g.E * g.n * g.n;
  const int64_t grid = which == FUSED_FWD_SKY ? patches : units;
  const int64_t zbytes =
      (which == FUSED_FWD_SKY ? (int64_t)g.M : 1) * g.E * g.pixels() * (int64_t)esz;
  a.zchunk = grid > 0 ? ((zbytes + grid - 1) / grid + 15) & ~(int64_t)15 : 0;
  a.aux = f.aux;
  a.aux_bytes = f.aux ? f.aux_bytes : 0;
  a.aux_chunk = grid > 0 ? ((a.aux_bytes + grid - 1) / grid + 15) & ~(int64_t)15 : 0;
  a.zero_out = f.zero_out ? 1 : 0;
  if (!f.clear) {  // grouped launches clear every problem's buffers in one kernel
    a.zchunk = 0;
    a.aux = nullptr;
    a.aux_bytes = 0;
    a.aux_chunk = 0;
    a.zero_out = 0;
  }
  a.in_rs = f.in_rs > 0 ? f.in_rs : (int64_t)g.ny;
  a.in_ps = f.in_ps > 0 ? f.in_ps : g.pixels();
  a.in_exp = f.in_exp ? 1 : 0;
  a.out_lo = f.out_lo;
  a.bnd_in = (const unsigned long long*)f.bnd_in;
  a.bnd_n = f.bnd_n;
  a.bnd_log2 = f.bnd_log2;
  a.bnd_scale = f.bnd_scale;
  a.bnd_out = (unsigned long long*)f.bnd_out;
  a.spill = f.spill;
  a.loop_grid = (int)f.loop_grid;
  a.run_len = 0;
  set_div_consts(a, g.units());
  return a;
}

// Dynamic shared memory of the ordered adjoint: the tile, column 0's arrays,
// and -- where more CTAs would fit an SM than its 512 TMEM columns serve --
// enough extra that no more than that many CTAs share an SM.
template <typename T, int P>
size_t ord_smem_bytes() {
  const size_t s = Tr<T, P>::SMEM + ord_extra_smem<T, P>();
  const int cap = 512 / TmemGeom<T, P>::NCOLS;
  int dev = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) !=
          cudaSuccess ||
      per_sm <= 0) {
    cudaGetLastError();
    per_sm = 233472;
  }
  const size_t floor_s = (((size_t)per_sm / (size_t)(cap + 1) + 1) + 127) & ~(size_t)127;
  return std::max(s, floor_s);
}

// The shared-memory opt-in is a per-device function attribute: set it once per
// device before the first launch there (so never inside a stream capture that
// follows a warm-up call).
template <typename T, int P>
int ensure_smem_attrs() {
  const size_t smem = Tr<T, P>::SMEM;
  constexpr int kMaxDev = 64;
  static bool attr_set[kMaxDev] = {};
  int dev = 0;
  JUBIK_TRY_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDev) {
    set_error("device ordinal %d beyond %d", dev, kMaxDev);
    return JUBIK_ERR_UNSUPPORTED;
  }
  if (!attr_set[dev]) {
    JUBIK_TRY(set_smem(k_fused<T, P, false>, smem));
    JUBIK_TRY(set_smem(k_fused<T, P, true>, smem));
    JUBIK_TRY(set_smem(k_fused_group<T, P, false>, smem));
    JUBIK_TRY(set_smem(k_fused_group<T, P, true>, smem));
    JUBIK_TRY(set_smem(k_sky_spec<T, P, OneProblem>, smem));
    JUBIK_TRY(set_smem(k_adj_from_spec<T, P, OneProblem>, smem));
    JUBIK_TRY(set_smem(k_fwd_from_spec<T, P, OneProblem>, smem));
    JUBIK_TRY(set_smem(k_sky_spec<T, P, ProblemList>, smem));
    JUBIK_TRY(set_smem(k_adj_from_spec<T, P, ProblemList>, smem));
    JUBIK_TRY(set_smem(k_fwd_from_spec<T, P, ProblemList>, smem));
    JUBIK_TRY(set_smem(k_adj_to_spec_ord<T, P>, ord_smem_bytes<T, P>()));
    JUBIK_TRY(set_smem(k_adj_to_spec_ord_list<T, P>, ord_smem_bytes<T, P>()));
    if constexpr (sizeof(T) == 4 && P == 192) JUBIK_TRY(set_smem(k_fwd_run<T, P>, smem));
    attr_set[dev] = true;
  }
  return JUBIK_OK;
}

// Launch with programmatic stream serialisation when pdl: the kernel may be
// scheduled while the previous kernel of the stream drains (see pdl_wait).
template <typename T, int P, typename KernelT, typename... ArgsT>
int launch_pdl_smem(KernelT kern, int64_t grid, size_t smem, bool pdl, cudaStream_t s,
                    ArgsT... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(Tr<T, P>::NT);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cuda_status(cudaLaunchKernelEx(&cfg, kern, args...), "fused kernel launch");
}

template <typename T, int P, typename KernelT, typename... ArgsT>
int launch_pdl(KernelT kern, int64_t grid, bool pdl, cudaStream_t s, ArgsT... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(Tr<T, P>::NT);
  cfg.dynamicSmemBytes = Tr<T, P>::SMEM;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cuda_status(cudaLaunchKernelEx(&cfg, kern, args...), "fused kernel launch");
}

// Geometries whose patch outputs share whole block rows of 64 field rows (see
// k_fwd_run): P = 192 from 64-row strides and a 32-pixel margin, a field of
// whole strides (no clamped start), and runs of run_len (2 or 4) patch rows.
inline bool run_geometry(const Geom& g, int run_len) {
  return (run_len == 2 || run_len == 4) && g.P == 192 && g.dx == 64 && g.margin == 32 &&
         g.nx == g.n * 64 && g.ny == g.n * 64 && g.n % run_len == 0 && g.M >= 2;
}

// Run length of the module-shared forward when the plan leaves it to the
// library: the one whose busiest CTA does the least work.  A CTA of the
// 152-CTA loop processes ceil(items / G) items of run_len units each, and a
// unit inside a run costs about 0.87 (runs of 4) or 0.93 (runs of 2) of one
// reduced on its own (fewer block-row reductions; measured forward times at
// 768^2 and 1024^2 x 7 modules x 3 energies, where every choice gives the
// busiest CTA the same number of units).
inline int auto_run_len(const Geom& g) {
  const int64_t G = sm_count(), U = g.units();
  int best = 1;
  double best_cost = (double)((U + G - 1) / G);
  const int cand[2] = {2, 4};
  const double f[2] = {0.93, 0.87};
  for (int i = 0; i < 2; ++i) {
    if (!run_geometry(g, cand[i])) continue;
    const int64_t items = U / cand[i];
    const double cost = (double)((items + G - 1) / G) * cand[i] * f[i];
    if (cost < best_cost) {
      best_cost = cost;
      best = cand[i];
    }
  }
  return best;
}

// Grid of the ordered adjoint over g's units (its CTAs' unit ranges and spill
// slots depend on it).
template <typename T, int P>
int64_t ord_grid(const Geom& g) {
  return loop_grid<T, P>(k_adj_to_spec_ord<T, P>, g.units(), ord_smem_bytes<T, P>());
}

template <typename T, int P>
int launch_one(const Geom& g, const FusedLaunch& f, int which, cudaStream_t s) {
  JUBIK_TRY((ensure_smem_attrs<T, P>()));
  const Args a = make_args(g, f, which, sizeof(T));
  const int64_t units = g.units();
  const int64_t patches = (int64_t)g.E * g.n * g.n;
  if (units <= 0) return JUBIK_OK;
  if (units > 0x7fffffffLL) {
    set_error("too many patch units for one launch");
    return JUBIK_ERR_UNSUPPORTED;
  }
  if ((which != FUSED_FWD_UNITS && which != FUSED_ADJ_UNITS) && !f.spec) {
    set_error("module-shared kernels need the spectrum workspace");
    return JUBIK_ERR_STATE;
  }
  // every one-problem launch accumulates its output exactly in two words
  auto need = [&](bool ok, const char* what) {
    if (!ok) set_error("fused stage %d: %s missing", which, what);
    return ok;
  };
  switch (which) {
    case FUSED_FWD_UNITS:
    case FUSED_ADJ_UNITS:
      if (!need(f.out_lo && f.bnd_in && f.bnd_n > 0, "low-word plane or input bound"))
        return JUBIK_ERR_STATE;
      return which == FUSED_FWD_UNITS
                 ? launch_pdl<T, P>(k_fused<T, P, false>, units, f.pdl, s, a)
                 : launch_pdl<T, P>(k_fused<T, P, true>, units, f.pdl, s, a);
    case FUSED_FWD_SKY:
      if (!need(f.out_lo && f.bnd_out, "low-word plane or bound record")) return JUBIK_ERR_STATE;
      return launch_pdl<T, P>(k_sky_spec<T, P, OneProblem>, patches, f.pdl, s, OneProblem{a});
    case FUSED_FWD_FROM_SPEC:
      if (!need(f.out_lo && f.bnd_in && f.bnd_n == patches, "low-word plane or input bound"))
        return JUBIK_ERR_STATE;
      if constexpr (sizeof(T) == 4 && P == 192) {
        const int r = f.fwd_run > 0 ? f.fwd_run : auto_run_len(g);
        if (run_geometry(g, r)) {
          const int64_t items = units / r;
          Args ar = a;
          ar.run_len = r;
          set_div_consts(ar, units);
          return launch_pdl<T, P>(k_fwd_run<T, P>, loop_grid<T, P>(k_fwd_run<T, P>, items),
                                  f.pdl, s, ar, (int)items);
        }
      }
      return launch_pdl<T, P>(k_fwd_from_spec<T, P, OneProblem>,
                              loop_grid<T, P>(k_fwd_from_spec<T, P, OneProblem>, units), f.pdl,
                              s, OneProblem{a}, (int)units);
    case FUSED_ADJ_TO_SPEC: {
      // contiguous unit ranges, as many CTAs as fit at once (and as the spill holds)
      const int64_t grid = ord_grid<T, P>(g);
      if (!need(f.spill && f.loop_grid == grid, "spill slots")) return JUBIK_ERR_STATE;
      Args al = a;
      const int64_t zbytes = (int64_t)g.E * g.pixels() * (int64_t)sizeof(T);
      al.zchunk = ((zbytes + grid - 1) / grid + 15) & ~(int64_t)15;
      return launch_pdl_smem<T, P>(k_adj_to_spec_ord<T, P>, grid, ord_smem_bytes<T, P>(), f.pdl,
                                   s, al, (int)units);
    }
    case FUSED_ADJ_FROM_SPEC:
      if (!need(f.out_lo && f.bnd_in && f.bnd_n > 0 && f.spill &&
                    f.loop_grid == ord_grid<T, P>(g),
                "low-word plane, spill slots or input bound"))
        return JUBIK_ERR_STATE;
      return launch_pdl<T, P>(k_adj_from_spec<T, P, OneProblem>, patches, f.pdl, s,
                              OneProblem{a});
    default:
      set_error("unknown fused stage %d", which);
      return JUBIK_ERR_INVALID_ARGUMENT;
  }
}

template <typename T, int P>
int launch_group(const void* list, const int* starts, int nprob, int64_t blocks, bool adj,
                 bool pdl, cudaStream_t s) {
  JUBIK_TRY((ensure_smem_attrs<T, P>()));
  if (blocks <= 0) return JUBIK_OK;
  if (blocks > 0x7fffffffLL) {
    set_error("too many patch units for one launch");
    return JUBIK_ERR_UNSUPPORTED;
  }
  const Args* l = (const Args*)list;
  return adj ? launch_pdl<T, P>(k_fused_group<T, P, true>, blocks, pdl, s, l, starts, nprob)
             : launch_pdl<T, P>(k_fused_group<T, P, false>, blocks, pdl, s, l, starts, nprob);
}

// One module-shared stage over a list of problems of one FFT side: starts
// (device) index the (energy, patch) items for FUSED_FWD_SKY / FUSED_ADJ_FROM_SPEC
// and the units for FUSED_FWD_FROM_SPEC / FUSED_ADJ_TO_SPEC; count is the total.
template <typename T, int P>
int launch_group_shared(const void* list, const int* starts, int nprob, int64_t count,
                        int which, bool pdl, cudaStream_t s) {
  JUBIK_TRY((ensure_smem_attrs<T, P>()));
  if (count <= 0) return JUBIK_OK;
  if (count > 0x7fffffffLL) {
    set_error("too many patch units for one launch");
    return JUBIK_ERR_UNSUPPORTED;
  }
  const ProblemList src{(const Args*)list, starts, nprob};
  switch (which) {
    case FUSED_FWD_SKY: return launch_pdl<T, P>(k_sky_spec<T, P, ProblemList>, count, pdl, s, src);
    case FUSED_FWD_FROM_SPEC:
      return launch_pdl<T, P>(k_fwd_from_spec<T, P, ProblemList>,
                              loop_grid<T, P>(k_fwd_from_spec<T, P, ProblemList>, count), pdl, s,
                              src, (int)count);
    case FUSED_ADJ_TO_SPEC:  // starts: each problem's CTA range; count: all CTAs
      return launch_pdl_smem<T, P>(k_adj_to_spec_ord_list<T, P>, count, ord_smem_bytes<T, P>(),
                                   pdl, s, (const Args*)list, starts, nprob);
    case FUSED_ADJ_FROM_SPEC:
      return launch_pdl<T, P>(k_adj_from_spec<T, P, ProblemList>, count, pdl, s, src);
    default:
      set_error("unknown module-shared stage %d", which);
      return JUBIK_ERR_INVALID_ARGUMENT;
  }
}

template <typename T>
int dispatch_group_shared(int P, const void* list, const int* starts, int nprob, int64_t count,
                          int which, bool pdl, cudaStream_t s) {
  switch (P) {
    case 32: return launch_group_shared<T, 32>(list, starts, nprob, count, which, pdl, s);
    case 64: return launch_group_shared<T, 64>(list, starts, nprob, count, which, pdl, s);
    case 96: return launch_group_shared<T, 96>(list, starts, nprob, count, which, pdl, s);
    case 128: return launch_group_shared<T, 128>(list, starts, nprob, count, which, pdl, s);
    case 160:
      if constexpr (sizeof(T) == 4)
        return launch_group_shared<T, 160>(list, starts, nprob, count, which, pdl, s);
      break;
    case 192:
      if constexpr (sizeof(T) == 4)
        return launch_group_shared<T, 192>(list, starts, nprob, count, which, pdl, s);
      break;
    default: break;
  }
  set_error("fused path does not cover P=%d for this dtype", P);
  return JUBIK_ERR_UNSUPPORTED;
}

template <typename T>
int dispatch_group(int P, const void* list, const int* starts, int nprob, int64_t blocks,
                   bool adj, bool pdl, cudaStream_t s) {
  switch (P) {
    case 32: return launch_group<T, 32>(list, starts, nprob, blocks, adj, pdl, s);
    case 64: return launch_group<T, 64>(list, starts, nprob, blocks, adj, pdl, s);
    case 96: return launch_group<T, 96>(list, starts, nprob, blocks, adj, pdl, s);
    case 128: return launch_group<T, 128>(list, starts, nprob, blocks, adj, pdl, s);
    case 160:
      if constexpr (sizeof(T) == 4) return launch_group<T, 160>(list, starts, nprob, blocks, adj,
                                                                pdl, s);
      break;
    case 192:
      if constexpr (sizeof(T) == 4) return launch_group<T, 192>(list, starts, nprob, blocks, adj,
                                                                pdl, s);
      break;
    default: break;
  }
  set_error("fused path does not cover P=%d for this dtype", P);
  return JUBIK_ERR_UNSUPPORTED;
}

template <typename T>
int dispatch(const Geom& g, const FusedLaunch& f, int which, cudaStream_t s) {
  switch (g.P) {
    case 32: return launch_one<T, 32>(g, f, which, s);
    case 64: return launch_one<T, 64>(g, f, which, s);
    case 96: return launch_one<T, 96>(g, f, which, s);
    case 128: return launch_one<T, 128>(g, f, which, s);
    case 160:
      if constexpr (sizeof(T) == 4) return launch_one<T, 160>(g, f, which, s);
      break;
    case 192:
      if constexpr (sizeof(T) == 4) return launch_one<T, 192>(g, f, which, s);
      break;
    default: break;
  }
  set_error("fused path does not cover P=%d for this dtype", g.P);
  return JUBIK_ERR_UNSUPPORTED;
}

}  // namespace

// Streaming multiprocessors of the current device (cached per device).
int sm_count() {
  constexpr int kMaxDev = 64;
  static std::atomic<int> n[kMaxDev];  // 0 = not looked up yet
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDev) return 1;
  int v = n[dev].load(std::memory_order_relaxed);
  if (v <= 0) {
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v < 1) {
      cudaGetLastError();
      v = 1;
    }
    n[dev].store(v, std::memory_order_relaxed);
  }
  return v;
}

bool fused_supported(int P, int dtype) {
  switch (P) {
    case 32: case 64: case 96: case 128: return true;
    case 160: case 192: return dtype == JUBIK_F32;
    default: return false;
  }
}

size_t fused_spec_bytes(const Geom& g, int dtype) {
  const size_t c = dtype == JUBIK_F32 ? 8 : 16;
  return c * (size_t)g.E * g.n * g.n * g.P * (g.P / 2);
}

template <typename T>
int ensure_attrs_dispatch(int P) {
  switch (P) {
    case 32: return ensure_smem_attrs<T, 32>();
    case 64: return ensure_smem_attrs<T, 64>();
    case 96: return ensure_smem_attrs<T, 96>();
    case 128: return ensure_smem_attrs<T, 128>();
    case 160:
      if constexpr (sizeof(T) == 4) return ensure_smem_attrs<T, 160>();
      break;
    case 192:
      if constexpr (sizeof(T) == 4) return ensure_smem_attrs<T, 192>();
      break;
    default: break;
  }
  return JUBIK_ERR_UNSUPPORTED;
}

template <typename T>
int64_t ord_grid_dispatch(const Geom& g) {
  switch (g.P) {
    case 32: return ord_grid<T, 32>(g);
    case 64: return ord_grid<T, 64>(g);
    case 96: return ord_grid<T, 96>(g);
    case 128: return ord_grid<T, 128>(g);
    case 160:
      if constexpr (sizeof(T) == 4) return ord_grid<T, 160>(g);
      break;
    case 192:
      if constexpr (sizeof(T) == 4) return ord_grid<T, 192>(g);
      break;
    default: break;
  }
  return 0;
}

size_t fused_smem_bytes(int P, int dtype) {
  const size_t c = dtype == JUBIK_F32 ? 8 : 16;
  const size_t H = P / 2, TP = P + 1, CH = H < 32 ? H : 32;
  return c * (H * TP + CH * TP);
}

int64_t fused_adj_grid(const Geom& g, int dtype) {
  if (!fused_supported(g.P, dtype)) return 0;
  if ((dtype == JUBIK_F32 ? ensure_attrs_dispatch<float>(g.P) : ensure_attrs_dispatch<double>(g.P)))
    return 0;
  return dtype == JUBIK_F32 ? ord_grid_dispatch<float>(g) : ord_grid_dispatch<double>(g);
}

// Run length the module-shared forward of geometry g uses for a request
// (0: the library's choice): 2 or 4 for the run-ordered kernel, 1 for one
// unit at a time.  Returns -1 for a request the geometry cannot take.
int fused_fwd_run_len(const Geom& g, int dtype, int requested) {
  const bool fits = dtype == JUBIK_F32 && g.P == 192;
  if (requested == 0) return fits ? auto_run_len(g) : 1;
  if (requested == 1) return 1;
  return fits && run_geometry(g, requested) ? requested : -1;
}

// CTAs of the ordered adjoint over a list of problems at FFT side P that the
// GPU holds at once (0 where the fused path does not cover P).
template <typename T>
int64_t ord_list_capacity(int P) {
  constexpr int64_t kMany = int64_t(1) << 30;  // more than any GPU holds
  switch (P) {
    case 32: return loop_grid<T, 32>(k_adj_to_spec_ord_list<T, 32>, kMany, ord_smem_bytes<T, 32>());
    case 64: return loop_grid<T, 64>(k_adj_to_spec_ord_list<T, 64>, kMany, ord_smem_bytes<T, 64>());
    case 96: return loop_grid<T, 96>(k_adj_to_spec_ord_list<T, 96>, kMany, ord_smem_bytes<T, 96>());
    case 128:
      return loop_grid<T, 128>(k_adj_to_spec_ord_list<T, 128>, kMany, ord_smem_bytes<T, 128>());
    case 160:
      if constexpr (sizeof(T) == 4)
        return loop_grid<T, 160>(k_adj_to_spec_ord_list<T, 160>, kMany, ord_smem_bytes<T, 160>());
      break;
    case 192:
      if constexpr (sizeof(T) == 4)
        return loop_grid<T, 192>(k_adj_to_spec_ord_list<T, 192>, kMany, ord_smem_bytes<T, 192>());
      break;
    default: break;
  }
  return 0;
}

int64_t fused_ord_capacity(int P, int dtype) {
  if (!fused_supported(P, dtype)) return 0;
  if ((dtype == JUBIK_F32 ? ensure_attrs_dispatch<float>(P) : ensure_attrs_dispatch<double>(P)))
    return 0;
  return dtype == JUBIK_F32 ? ord_list_capacity<float>(P) : ord_list_capacity<double>(P);
}

int fused_run(const Geom& g, int dtype, const FusedLaunch& a, int which, cudaStream_t s) {
  return dtype == JUBIK_F32 ? dispatch<float>(g, a, which, s) : dispatch<double>(g, a, which, s);
}

size_t fused_args_size() { return sizeof(Args); }

void fused_args_fill(const Geom& g, int dtype, const FusedLaunch& f, int which, void* dst) {
  const Args a = make_args(g, f, which, dtype == JUBIK_F32 ? sizeof(float) : sizeof(double));
  memcpy(dst, &a, sizeof(Args));
}

int fused_group_shared_run(int P, int dtype, const void* list, const int* starts, int nprob,
                           int64_t count, int which, bool pdl, cudaStream_t s) {
  return dtype == JUBIK_F32
             ? dispatch_group_shared<float>(P, list, starts, nprob, count, which, pdl, s)
             : dispatch_group_shared<double>(P, list, starts, nprob, count, which, pdl, s);
}

int fused_group_run(int P, int dtype, const void* list, const int* starts, int nprob,
                    int64_t blocks, bool adj, bool pdl, cudaStream_t s) {
  return dtype == JUBIK_F32
             ? dispatch_group<float>(P, list, starts, nprob, blocks, adj, pdl, s)
             : dispatch_group<double>(P, list, starts, nprob, blocks, adj, pdl, s);
}

}  // namespace jubik
