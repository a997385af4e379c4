// Register-resident small DFTs (sizes 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12,
// 16, 20, 24, 32) in natural order, fully unrolled at compile time.  Composite sizes use one level of
// Cooley-Tukey, N = N1 * N2 with n = N2*n1 + n2 and k = k1 + N1*k2:
//   X[k1 + N1 k2] = sum_n2 w_N2^(n2 k2) w_N^(n2 k1) sum_n1 x[N2 n1 + n2] w_N1^(n1 k1)
#pragma once

#include "jubik_common.cuh"

namespace jubik {

template <int N, bool INV, typename T> struct Dft;

template <bool INV, typename T> struct Dft<1, INV, T> {
  __device__ __forceinline__ static void run(cx<T>*) {}
};

template <bool INV, typename T> struct Dft<2, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) {
    cx<T> a = v[0];
    v[0] = cadd<T>(a, v[1]);
    v[1] = csub<T>(a, v[1]);
  }
};

template <bool INV, typename T> struct Dft<3, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) {
    constexpr T s3 = (T)0.8660254037844386467637232;  // sin(2 pi / 3)
    cx<T> t1 = cadd<T>(v[1], v[2]);
    cx<T> t2 = mkc<T>(v[0].x - (T)0.5 * t1.x, v[0].y - (T)0.5 * t1.y);
    cx<T> t3 = mkc<T>(s3 * (v[1].x - v[2].x), s3 * (v[1].y - v[2].y));
    v[0] = cadd<T>(v[0], t1);
    if (INV) {
      v[1] = cadd<T>(t2, cmul_i<T>(t3));
      v[2] = csub<T>(t2, cmul_i<T>(t3));
    } else {
      v[1] = csub<T>(t2, cmul_i<T>(t3));
      v[2] = cadd<T>(t2, cmul_i<T>(t3));
    }
  }
};

template <bool INV, typename T> struct Dft<4, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) {
    cx<T> t0 = cadd<T>(v[0], v[2]);
    cx<T> t1 = csub<T>(v[0], v[2]);
    cx<T> t2 = cadd<T>(v[1], v[3]);
    cx<T> t3 = csub<T>(v[1], v[3]);
    v[0] = cadd<T>(t0, t2);
    v[2] = csub<T>(t0, t2);
    if (INV) {
      v[1] = cadd<T>(t1, cmul_i<T>(t3));
      v[3] = csub<T>(t1, cmul_i<T>(t3));
    } else {
      v[1] = csub<T>(t1, cmul_i<T>(t3));
      v[3] = cadd<T>(t1, cmul_i<T>(t3));
    }
  }
};

// 5 points: with t1 = x1 + x4, t2 = x2 + x3, t3 = x1 - x4, t4 = x2 - x3,
//   X1,4 = x0 + c1 t1 + c2 t2 -/+ i (s1 t3 + s2 t4)
//   X2,3 = x0 + c2 t1 + c1 t2 -/+ i (s2 t3 - s1 t4)
// (c_k = cos(2 pi k / 5), s_k = sin(2 pi k / 5); the inverse flips the i terms).
template <bool INV, typename T> struct Dft<5, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) {
    constexpr T c1 = (T)0.3090169943749474241022934;   // cos(2 pi / 5)
    constexpr T c2 = (T)-0.8090169943749474241022934;  // cos(4 pi / 5)
    constexpr T s1 = (T)0.9510565162951535721164393;   // sin(2 pi / 5)
    constexpr T s2 = (T)0.5877852522924731291687060;   // sin(4 pi / 5)
    const cx<T> t1 = cadd<T>(v[1], v[4]), t2 = cadd<T>(v[2], v[3]);
    const cx<T> t3 = csub<T>(v[1], v[4]), t4 = csub<T>(v[2], v[3]);
    const cx<T> a1 = mkc<T>(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
    const cx<T> a2 = mkc<T>(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
    const cx<T> b1 = mkc<T>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y);
    const cx<T> b2 = mkc<T>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y);
    v[0] = cadd<T>(v[0], cadd<T>(t1, t2));
    if (INV) {
      v[1] = cadd<T>(a1, cmul_i<T>(b1));
      v[4] = csub<T>(a1, cmul_i<T>(b1));
      v[2] = cadd<T>(a2, cmul_i<T>(b2));
      v[3] = csub<T>(a2, cmul_i<T>(b2));
    } else {
      v[1] = csub<T>(a1, cmul_i<T>(b1));
      v[4] = cadd<T>(a1, cmul_i<T>(b1));
      v[2] = csub<T>(a2, cmul_i<T>(b2));
      v[3] = cadd<T>(a2, cmul_i<T>(b2));
    }
  }
};

// Odd N (7, 9, 11), direct: with t_q = x_q + x_{N-q}, u_q = x_q - x_{N-q},
//   X_k, X_{N-k} = x_0 + sum_q cos(2 pi q k / N) t_q -/+ i sum_q sin(2 pi q k / N) u_q,
// q, k = 1 .. (N - 1) / 2 (the inverse flips the i terms).  odd_cos / odd_sin
// hold cos and sin of 2 pi m / N for m = 0 .. (N - 1) / 2 to 25 digits (m = 0
// occurs for composite N: q k = 9 for N = 9).
__host__ __device__ constexpr double odd_cos(int N, int m) {
  if (m == 0) return 1.0;
  switch (N * 16 + m) {
    case 7 * 16 + 1: return 0.6234898018587335305250049;
    case 7 * 16 + 2: return -0.2225209339563144042889026;
    case 7 * 16 + 3: return -0.9009688679024191262361023;
    case 9 * 16 + 1: return 0.7660444431189780352023926;
    case 9 * 16 + 2: return 0.1736481776669303488517166;
    case 9 * 16 + 3: return -0.5;
    case 9 * 16 + 4: return -0.9396926207859083840541093;
    case 11 * 16 + 1: return 0.8412535328311811688618117;
    case 11 * 16 + 2: return 0.4154150130018864255292741;
    case 11 * 16 + 3: return -0.1423148382732851404437927;
    case 11 * 16 + 4: return -0.6548607339452850640569251;
    case 11 * 16 + 5: return -0.9594929736144973898903681;
    default: return 0.0;
  }
}
__host__ __device__ constexpr double odd_sin(int N, int m) {
  switch (N * 16 + m) {
    case 7 * 16 + 1: return 0.7818314824680298087084445;
    case 7 * 16 + 2: return 0.9749279121818236070181317;
    case 7 * 16 + 3: return 0.4338837391175581204757683;
    case 9 * 16 + 1: return 0.6427876096865393263226434;
    case 9 * 16 + 2: return 0.9848077530122080593667430;
    case 9 * 16 + 3: return 0.8660254037844386467637232;
    case 9 * 16 + 4: return 0.3420201433256687330440996;
    case 11 * 16 + 1: return 0.5406408174555975821076360;
    case 11 * 16 + 2: return 0.9096319953545183714117154;
    case 11 * 16 + 3: return 0.9898214418809327323760920;
    case 11 * 16 + 4: return 0.7557495743542582837740358;
    case 11 * 16 + 5: return 0.2817325568414296977114179;
    default: return 0.0;
  }
}

template <int N, bool INV, typename T>
__device__ __forceinline__ void dft_odd(cx<T>* v) {
  constexpr int H = (N - 1) / 2;
  cx<T> t[H], u[H];
  const cx<T> x0 = v[0];
  cx<T> sum = x0;
  sfor<H>([&](auto qc) {
    constexpr int q = decltype(qc)::value;
    t[q] = cadd<T>(v[q + 1], v[N - 1 - q]);
    u[q] = csub<T>(v[q + 1], v[N - 1 - q]);
    sum = cadd<T>(sum, t[q]);
  });
  sfor<H>([&](auto kc) {
    constexpr int k = decltype(kc)::value + 1;
    cx<T> a = x0, b = mkc<T>((T)0, (T)0);
    sfor<H>([&](auto qc) {
      constexpr int q = decltype(qc)::value + 1;
      constexpr int m = (q * k) % N;
      constexpr T c = (T)odd_cos(N, m <= H ? m : N - m);
      constexpr T sn = (T)(m <= H ? odd_sin(N, m) : -odd_sin(N, N - m));
      a = mkc<T>(a.x + c * t[q - 1].x, a.y + c * t[q - 1].y);
      b = mkc<T>(b.x + sn * u[q - 1].x, b.y + sn * u[q - 1].y);
    });
    if (INV) {
      v[k] = cadd<T>(a, cmul_i<T>(b));
      v[N - k] = csub<T>(a, cmul_i<T>(b));
    } else {
      v[k] = csub<T>(a, cmul_i<T>(b));
      v[N - k] = cadd<T>(a, cmul_i<T>(b));
    }
  });
  v[0] = sum;
}
template <bool INV, typename T> struct Dft<7, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_odd<7, INV, T>(v); }
};
template <bool INV, typename T> struct Dft<9, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_odd<9, INV, T>(v); }
};
template <bool INV, typename T> struct Dft<11, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_odd<11, INV, T>(v); }
};

template <int N1, int N2, bool INV, typename T>
__device__ __forceinline__ void dft_ct(cx<T>* v) {
  constexpr int N = N1 * N2;
  cx<T> y[N];
  sfor<N2>([&](auto n2c) {
    constexpr int n2 = decltype(n2c)::value;
    cx<T> t[N1];
    sfor<N1>([&](auto n1c) { t[decltype(n1c)::value] = v[N2 * decltype(n1c)::value + n2]; });
    Dft<N1, INV, T>::run(t);
    sfor<N1>([&](auto k1c) {
      constexpr int k1 = decltype(k1c)::value;
      y[k1 * N2 + n2] = twc<N, n2 * k1, INV, T>(t[k1]);
    });
  });
  sfor<N1>([&](auto k1c) {
    constexpr int k1 = decltype(k1c)::value;
    cx<T> t[N2];
    sfor<N2>([&](auto n2c) { t[decltype(n2c)::value] = y[k1 * N2 + decltype(n2c)::value]; });
    Dft<N2, INV, T>::run(t);
    sfor<N2>([&](auto k2c) { v[k1 + N1 * decltype(k2c)::value] = t[decltype(k2c)::value]; });
  });
}

template <bool INV, typename T> struct Dft<6, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_ct<3, 2, INV, T>(v); }
};
template <bool INV, typename T> struct Dft<8, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_ct<4, 2, INV, T>(v); }
};
template <bool INV, typename T> struct Dft<12, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_ct<3, 4, INV, T>(v); }
};
template <bool INV, typename T> struct Dft<16, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_ct<4, 4, INV, T>(v); }
};
template <bool INV, typename T> struct Dft<10, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_ct<5, 2, INV, T>(v); }
};
template <bool INV, typename T> struct Dft<20, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_ct<4, 5, INV, T>(v); }
};
template <bool INV, typename T> struct Dft<24, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_ct<3, 8, INV, T>(v); }
};
template <bool INV, typename T> struct Dft<32, INV, T> {
  __device__ __forceinline__ static void run(cx<T>* v) { dft_ct<4, 8, INV, T>(v); }
};

}  // namespace jubik
