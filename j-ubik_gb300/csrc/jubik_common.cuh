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

// v * w_N^E with w_N = exp(-2 pi i / N) (forward) or its conjugate (INV).
// N must divide 48.  Exponents that are multiples of N/4 become sign flips.
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
  } else {
    constexpr int j = e * (48 / N);
    constexpr T c = (T)cos48(j);
    constexpr T s = INV ? (T)sin48(j) : (T)(-sin48(j));
    return mkc<T>(v.x * c - v.y * s, v.x * s + v.y * c);
  }
}

}  // namespace jubik
