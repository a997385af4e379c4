// Shared device helpers for the GB300 J-UBIK response kernels.
//
// Complex values are stored as float2 / double2 (re, im).  Forward transforms
// use exp(-2*pi*i*n*k/N), matching numpy/JAX ``fftn`` as called at
// jubik/convolve.py:165-174.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <utility>
#include <type_traits>

namespace jubik {

template <typename T> struct cvec;
template <> struct cvec<float> { using type = float2; };
template <> struct cvec<double> { using type = double2; };
template <typename T> using cx = typename cvec<T>::type;

template <typename T>
__host__ __device__ __forceinline__ cx<T> mkc(T a, T b) {
  cx<T> r;
  r.x = a;
  r.y = b;
  return r;
}
template <typename T>
__device__ __forceinline__ cx<T> cadd(cx<T> a, cx<T> b) { return mkc<T>(a.x + b.x, a.y + b.y); }
template <typename T>
__device__ __forceinline__ cx<T> csub(cx<T> a, cx<T> b) { return mkc<T>(a.x - b.x, a.y - b.y); }
template <typename T>
__device__ __forceinline__ cx<T> cmul(cx<T> a, cx<T> b) {
  return mkc<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a * conj(b)
template <typename T>
__device__ __forceinline__ cx<T> cmulc(cx<T> a, cx<T> b) {
  return mkc<T>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
template <typename T>
__device__ __forceinline__ cx<T> cconj(cx<T> a) { return mkc<T>(a.x, -a.y); }
template <typename T>
__device__ __forceinline__ cx<T> cneg(cx<T> a) { return mkc<T>(-a.x, -a.y); }
// multiply by +i and by -i
template <typename T>
__device__ __forceinline__ cx<T> cmul_i(cx<T> a) { return mkc<T>(-a.y, a.x); }
template <typename T>
__device__ __forceinline__ cx<T> cmul_mi(cx<T> a) { return mkc<T>(a.y, -a.x); }
template <typename T>
__device__ __forceinline__ cx<T> cscale(cx<T> a, T s) { return mkc<T>(a.x * s, a.y * s); }

// Compile-time loop: f(std::integral_constant<int, i>) for i in [0, N).
template <typename F, int... Is>
__device__ __forceinline__ void sfor_impl(F&& f, std::integer_sequence<int, Is...>) {
  (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, typename F>
__device__ __forceinline__ void sfor(F&& f) {
  sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// cos(2*pi*j/48) for j in [0, 12]: exact decimal expansions of the
// mathematical constants (every codelet size divides 48).
__host__ __device__ constexpr double cos48_q(int j) {
  return j == 0    ? 1.0
         : j == 1  ? 0.9914448613738104111445575
         : j == 2  ? 0.9659258262890682867497432
         : j == 3  ? 0.9238795325112867561281832
         : j == 4  ? 0.8660254037844386467637232
         : j == 5  ? 0.7933533402912351645797770
         : j == 6  ? 0.7071067811865475244008444
         : j == 7  ? 0.6087614290087206394160975
         : j == 8  ? 0.5
         : j == 9  ? 0.3826834323650897717284600
         : j == 10 ? 0.2588190451025207623488988
         : j == 11 ? 0.1305261922200515915484062
                   : 0.0;
}
__host__ __device__ constexpr double cos48(int j) {
  j = ((j % 48) + 48) % 48;
  if (j <= 12) return cos48_q(j);
  if (j <= 24) return -cos48_q(24 - j);
  if (j <= 36) return -cos48_q(j - 24);
  return cos48_q(48 - j);
}
__host__ __device__ constexpr double sin48(int j) { return cos48(j - 12); }

// cos(2*pi*j/160) for j in [0, 40]: for the codelet sizes that divide 160
// (5, 10, 20, 32), not 48.
__host__ __device__ constexpr double cos160_q(int j) {
  return j == 0    ? 1.0
         : j == 1  ? 0.9992290362407229347371263
         : j == 2  ? 0.9969173337331279761977734
         : j == 3  ? 0.9930684569549262956374372
         : j == 4  ? 0.9876883405951377261900402
         : j == 5  ? 0.9807852804032304491261822
         : j == 6  ? 0.9723699203976766018336458
         : j == 7  ? 0.9624552364536472876302664
         : j == 8  ? 0.9510565162951535721164393
         : j == 9  ? 0.9381913359224841344523397
         : j == 10 ? 0.9238795325112867561281832
         : j == 11 ? 0.9081431738250812992580858
         : j == 12 ? 0.8910065241883678623597096
         : j == 13 ? 0.8724960070727971145251611
         : j == 14 ? 0.8526401643540922215193835
         : j == 15 ? 0.8314696123025452370787884
         : j == 16 ? 0.8090169943749474241022934
         : j == 17 ? 0.7853169308807449274703403
         : j == 18 ? 0.7604059656000309381745944
         : j == 19 ? 0.7343225094356855356361262
         : j == 20 ? 0.7071067811865475244008444
         : j == 21 ? 0.6788007455329417413938556
         : j == 22 ? 0.6494480483301836557263208
         : j == 23 ? 0.6190939493098339869415609
         : j == 24 ? 0.587785252292473129168706
         : j == 25 ? 0.5555702330196022247428308
         : j == 26 ? 0.5224985647159488649878979
         : j == 27 ? 0.4886212414969549474201909
         : j == 28 ? 0.4539904997395467915604084
         : j == 29 ? 0.4186597375374280866755652
         : j == 30 ? 0.38268343236508977172846
         : j == 31 ? 0.346117057077492976468215
         : j == 32 ? 0.3090169943749474241022934
         : j == 33 ? 0.2714404498650742533437874
         : j == 34 ? 0.2334453638559054117677444
         : j == 35 ? 0.1950903220161282678482849
         : j == 36 ? 0.1564344650402308690101053
         : j == 37 ? 0.1175373974578376441055683
         : j == 38 ? 0.07845909572784494503296025
         : j == 39 ? 0.03925981575906860902080336
                   : 0.0;
}
__host__ __device__ constexpr double cos160(int j) {
  j = ((j % 160) + 160) % 160;
  if (j <= 40) return cos160_q(j);
  if (j <= 80) return -cos160_q(80 - j);
  if (j <= 120) return -cos160_q(j - 80);
  return cos160_q(160 - j);
}
__host__ __device__ constexpr double sin160(int j) { return cos160(j - 40); }

// v * w_N^E with w_N = exp(-2 pi i / N) (forward) or its conjugate (INV).
// N must divide 48 or 160.  Exponents that are multiples of N/4 become sign flips.
template <int N, int E, bool INV, typename T>
__device__ __forceinline__ cx<T> twc(cx<T> v) {
  constexpr int e = ((E % N) + N) % N;
  if constexpr (e == 0) {
    return v;
  } else if constexpr (2 * e == N) {
    return cneg<T>(v);
  } else if constexpr (4 * e == N) {
    return INV ? cmul_i<T>(v) : cmul_mi<T>(v);
  } else if constexpr (4 * e == 3 * N) {
    return INV ? cmul_mi<T>(v) : cmul_i<T>(v);
  } else if constexpr (48 % N == 0) {
    constexpr int j = e * (48 / N);
    constexpr T c = (T)cos48(j);
    constexpr T s = INV ? (T)sin48(j) : (T)(-sin48(j));
    return mkc<T>(v.x * c - v.y * s, v.x * s + v.y * c);
  } else {
    static_assert(160 % N == 0, "twiddle table: N must divide 48 or 160");
    constexpr int j = e * (160 / N);
    constexpr T c = (T)cos160(j);
    constexpr T s = INV ? (T)sin160(j) : (T)(-sin160(j));
    return mkc<T>(v.x * c - v.y * s, v.x * s + v.y * c);
  }
}

}  // namespace jubik
