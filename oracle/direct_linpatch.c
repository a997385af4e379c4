/*
 * Independent CPU restatement of jubik/convolve.py:66-145 (TEST INFRASTRUCTURE).
 *
 * Only tests/ and the smoke check call this; it is part of the oracle, not
 * the product.  It recomputes linpatch_convolve by DIRECT circular convolution
 * (no FFT) so that it shares no code path with the numpy oracle:
 *
 *   for patch k (row start (k % n)*dx, column start (k // n)*dx, clamped as
 *   jax.lax.dynamic_slice clamps, convolve.py:55-63), energy e:
 *     p[y][x]  = w[y-m] w[x-m] x_e[r0 - h + y - m][c0 - h + x - m]   (zero outside)
 *     h[u][v]  = kernel[k][e][a][b] / sum(kernel[k][e])  at u = (a - dx) mod P,
 *                v = (b - dx) mod P                          (convolve.py:104-131)
 *     q        = p (*) h, circular on P x P                   (convolve.py:148-176)
 *     out_e[r0 - h + y - m][c0 - h + x - m] += q[y][x]         (convolve.py:135-144)
 *
 * with w the bilinear weights of convolve.py:18-25, h = dx // 2, P = 2dx + 2m.
 */
#include <stdlib.h>
#include <string.h>

static void bilinear(int K, double* b) {
  int hh = K / 2;
  for (int i = 0; i < hh; ++i) {
    double a = (hh == 1) ? 0.0 : (double)i * (1.0 / (double)(hh - 1));
    if (i == hh - 1 && hh > 1) a = 1.0;
    b[i] = a;
    b[K - 1 - i] = a;
  }
}

/* x: (E, nx, ny); kernel: (n*n, E, 2dx, 2dx) pre-cut; out: (E, nx, ny).
 * Returns 0, or -1 for an invalid geometry. */
int oracle_linpatch_direct(const double* x, int E, int nx, int ny, int n, int margin,
                           const double* kernel, double* out) {
  const int dx = nx / n, dy = ny / n;
  if (n < 1 || dx < 1 || dx != dy || margin < 1) return -1;
  const int K = 2 * dx, P = K + 2 * margin, hx = dx / 2;
  const int rmax = nx + 2 * hx - K, cmax = ny + 2 * hx - K;
  if (rmax < 0 || cmax < 0) return -1;
  double* w = (double*)malloc(sizeof(double) * K);
  double* p = (double*)malloc(sizeof(double) * P * P);
  double* hk = (double*)malloc(sizeof(double) * P * P);
  if (!w || !p || !hk) {
    free(w);
    free(p);
    free(hk);
    return -1;
  }
  bilinear(K, w);
  memset(out, 0, sizeof(double) * (size_t)E * nx * ny);
  for (int k = 0; k < n * n; ++k) {
    int r0 = (k % n) * dx;
    if (r0 > rmax) r0 = rmax;
    int c0 = (k / n) * dx;
    if (c0 > cmax) c0 = cmax;
    const int rb = r0 - hx - margin, cb = c0 - hx - margin;
    for (int e = 0; e < E; ++e) {
      const double* ke = kernel + ((size_t)k * E + e) * K * K;
      double sum = 0.0;
      for (int i = 0; i < K * K; ++i) sum += ke[i];
      memset(hk, 0, sizeof(double) * P * P);
      for (int a = 0; a < K; ++a)
        for (int b = 0; b < K; ++b) {
          int u = ((a - dx) % P + P) % P, v = ((b - dx) % P + P) % P;
          hk[u * P + v] = ke[a * K + b] / sum;
        }
      for (int y = 0; y < P; ++y)
        for (int xx = 0; xx < P; ++xx) {
          int ya = y - margin, xa = xx - margin, row = rb + y, col = cb + xx;
          double v = 0.0;
          if (ya >= 0 && ya < K && xa >= 0 && xa < K && row >= 0 && row < nx && col >= 0 &&
              col < ny)
            v = (w[ya] * w[xa]) * x[((size_t)e * nx + row) * ny + col];
          p[y * P + xx] = v;
        }
      for (int y = 0; y < P; ++y) {
        const int row = rb + y;
        if (row < 0 || row >= nx) continue;
        for (int xx = 0; xx < P; ++xx) {
          const int col = cb + xx;
          if (col < 0 || col >= ny) continue;
          double acc = 0.0;
          for (int u = 0; u < P; ++u) {
            const int sy = ((y - u) % P + P) % P;
            for (int v = 0; v < P; ++v) {
              const double hv = hk[u * P + v];
              if (hv != 0.0) acc += hv * p[sy * P + ((xx - v) % P + P) % P];
            }
          }
          out[((size_t)e * nx + row) * ny + col] += acc;
        }
      }
    }
  }
  free(w);
  free(p);
  free(hk);
  return 0;
}
