/*
 * cufft_shim.c -- the two cuFFT calls of the reference (src/fft_dir.f90:12 cufftExecD2Z,
 * src/fft_inv.f90:12 cufftExecZ2D) for the transliterated reference (oracle/_ref).
 * TEST INFRASTRUCTURE ONLY.
 *
 * cuFFT is a closed third-party library (linked with -cudalib=cufft, Makefile:7; version not
 * pinned, nvhpc/23.11 in src/jobscript:18). This file implements the transforms from the
 * definitions cuFFT documents for a 2D plan of nx x ny (nx the slow dimension):
 *   D2Z  X[k1][k2] = sum_{n1,n2} x[n1][n2] exp(-2 pi i (k1 n1/nx + k2 n2/ny)), k2 <= ny/2,
 *   Z2D  the same sum with +i over the Hermitian half, unnormalised,
 * in place, each real row padded to 2 (ny/2+1) doubles. For Z2D the imaginary parts of the
 * k2 = 0 and k2 = ny/2 values after the k1-transform are ignored (a Hermitian input has none)
 * and the two padding doubles of each row are set to zero; cuFFT leaves them unspecified and the
 * reference never reads them.
 *
 * Algorithms: a radix-2 Stockham autosort FFT (no bit reversal) for the columns and for the
 * half-length complex transform of the rows, whose real values are packed in pairs
 * z[m] = x[2m] + i x[2m+1] and split with the twiddles exp(-2 pi i k/ny). Twiddles are cos/sin of
 * 2 pi k / L. OpenMP over rows and column blocks; every output value is computed by one thread in
 * a fixed order, so results do not depend on the thread count.
 */
#include <complex.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "f2c_rt.h"

#define SHIM_PLANS 16
#define SHIM_D2Z 1
#define SHIM_Z2D 2

typedef struct {
  int L;
  double _Complex* w; /* exp(-2 pi i k / L), k < L */
} tw_table;

typedef struct {
  int used, nx, ny, type;
  tw_table tc, th, tr; /* columns (nx), half rows (ny/2), rows (ny) */
} shim_plan;

static shim_plan g_plans[SHIM_PLANS];

static int tw_init(tw_table* t, int L) {
  t->L = L;
  t->w = (double _Complex*)malloc(sizeof(double _Complex) * (size_t)(L > 0 ? L : 1));
  if (!t->w) return 1;
  const double pi = 3.14159265358979323846;
  for (int k = 0; k < L; ++k) {
    const double a = 2.0 * pi * (double)k / (double)L;
    t->w[k] = cos(a) - I * sin(a);
  }
  return 0;
}

/* Stockham radix-2: a (length L, power of two) transformed in place; sign -1 forward, +1
 * inverse; tmp holds L values. */
static void fft_stockham(double _Complex* a, double _Complex* tmp, const tw_table* t, int sign) {
  const int L = t->L;
  double _Complex* x = a;
  double _Complex* y = tmp;
  for (int half = L / 2, s = 1; half >= 1; half /= 2, s *= 2) {
    /* stage: L/2s blocks of stride s */
    for (int p = 0; p < half; ++p) {
      double _Complex w = t->w[p * s];
      if (sign > 0) w = conj(w);
      for (int q = 0; q < s; ++q) {
        const double _Complex u = x[q + s * p];
        const double _Complex v = x[q + s * (p + half)];
        y[q + s * (2 * p)] = u + v;
        y[q + s * (2 * p + 1)] = (u - v) * w;
      }
    }
    double _Complex* sw = x;
    x = y;
    y = sw;
  }
  if (x != a) memcpy(a, x, sizeof(double _Complex) * (size_t)L);
}

int f2c_cufft_plan2d(int* plan, int nx, int ny, int type) {
  if (nx < 2 || ny < 4 || (nx & (nx - 1)) || (ny & (ny - 1))) return 1;
  for (int p = 0; p < SHIM_PLANS; ++p) {
    if (!g_plans[p].used) {
      shim_plan* s = &g_plans[p];
      s->used = 1;
      s->nx = nx;
      s->ny = ny;
      s->type = type;
      if (tw_init(&s->tc, nx) || tw_init(&s->th, ny / 2) || tw_init(&s->tr, ny)) return 1;
      *plan = p + 1;
      return 0;
    }
  }
  return 1;
}

int f2c_cufft_destroy(int plan) {
  if (plan < 1 || plan > SHIM_PLANS || !g_plans[plan - 1].used) return 1;
  shim_plan* s = &g_plans[plan - 1];
  free(s->tc.w);
  free(s->th.w);
  free(s->tr.w);
  memset(s, 0, sizeof *s);
  return 0;
}

static void columns(const shim_plan* s, double _Complex* z, int sign) {
  const int nx = s->nx, nh = s->ny / 2 + 1;
#pragma omp parallel
  {
    double _Complex* col = (double _Complex*)malloc(sizeof(double _Complex) * 2 * (size_t)nx);
#pragma omp for schedule(static)
    for (int c = 0; c < nh; ++c) {
      for (int r = 0; r < nx; ++r) col[r] = z[(size_t)r * nh + c];
      fft_stockham(col, col + nx, &s->tc, sign);
      for (int r = 0; r < nx; ++r) z[(size_t)r * nh + c] = col[r];
    }
    free(col);
  }
}

int cufftexecd2z(int plan, void* idata, void* odata) {
  if (plan < 1 || plan > SHIM_PLANS || idata != odata) return 1;
  const shim_plan* s = &g_plans[plan - 1];
  const int nx = s->nx, ny = s->ny, m = ny / 2, nh = m + 1;
  double* x = (double*)idata;
  double _Complex* z = (double _Complex*)idata;
#pragma omp parallel
  {
    double _Complex* h = (double _Complex*)malloc(sizeof(double _Complex) * 2 * (size_t)m);
#pragma omp for schedule(static)
    for (int r = 0; r < nx; ++r) {
      double* row = x + (size_t)r * (ny + 2);
      for (int k = 0; k < m; ++k) h[k] = row[2 * k] + I * row[2 * k + 1];
      fft_stockham(h, h + m, &s->th, -1);
      /* X[k] = (H[k] + conj H[m-k]) / 2 - i W^k (H[k] - conj H[m-k]) / 2 */
      double _Complex* out = z + (size_t)r * nh;
      const double _Complex h0 = h[0];
      out[0] = creal(h0) + cimag(h0);
      out[m] = creal(h0) - cimag(h0);
      for (int k = 1; k <= m / 2; ++k) {
        const double _Complex a = h[k], b = conj(h[m - k]);
        const double _Complex e = 0.5 * (a + b), o = -0.5 * I * (a - b);
        const double _Complex a2 = h[m - k], b2 = conj(h[k]);
        const double _Complex e2 = 0.5 * (a2 + b2), o2 = -0.5 * I * (a2 - b2);
        out[k] = e + s->tr.w[k] * o;
        out[m - k] = e2 + s->tr.w[m - k] * o2;
      }
    }
    free(h);
  }
  columns(s, z, -1);
  return 0;
}

int cufftexecz2d(int plan, void* idata, void* odata) {
  if (plan < 1 || plan > SHIM_PLANS || idata != odata) return 1;
  const shim_plan* s = &g_plans[plan - 1];
  const int nx = s->nx, ny = s->ny, m = ny / 2, nh = m + 1;
  double _Complex* z = (double _Complex*)idata;
  double* x = (double*)idata;
  columns(s, z, +1);
#pragma omp parallel
  {
    double _Complex* h = (double _Complex*)malloc(sizeof(double _Complex) * 2 * (size_t)m);
#pragma omp for schedule(static)
    for (int r = 0; r < nx; ++r) {
      const double _Complex* in = z + (size_t)r * nh;
      /* H[k] = (X[k] + conj X[m-k]) + i conj(W^k)... inverse of the split above, with the
       * imaginary parts of X[0] and X[m] ignored */
      for (int k = 0; k < m; ++k) {
        double _Complex a = in[k], b = conj(in[m - k]);
        if (k == 0) {
          a = creal(in[0]);
          b = creal(in[m]);
        }
        const double _Complex e = a + b;
        const double _Complex o = (a - b) * conj(s->tr.w[k]);
        h[k] = e + I * o;
      }
      fft_stockham(h, h + m, &s->th, +1);
      double* row = x + (size_t)r * (ny + 2);
      for (int k = 0; k < m; ++k) {
        row[2 * k] = creal(h[k]);
        row[2 * k + 1] = cimag(h[k]);
      }
      row[ny] = 0.0;
      row[ny + 1] = 0.0;
    }
    free(h);
  }
  return 0;
}
