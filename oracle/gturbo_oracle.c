/*
 * gturbo_oracle.c -- CPU FP64 ORACLE for the Gturbo time-stepping hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the reference that the CUDA path is
 * compared against (tests, the smoke check and the CPU-baseline leg of the
 * benchmark). It is never linked into, called by or shipped with the product
 * library.
 *
 * It restates the reference's Fortran routines line by line, on the same
 * memory layout (complex(8) z(N/2+1,N) == real(8) z(N+2,N)), in the same loop
 * and operation order, with the same LCG and real(4) rann:
 *   defk          src/defk.f90:12-73
 *   iniforcing    src/iniforcing.f90:11-68
 *   nlt           src/nlt.f90:17-63
 *   fft_dir       src/fft_dir.f90:11-21   (D2Z in place, then /NY then /NX)
 *   fft_inv       src/fft_inv.f90:11-13   (Z2D in place, unnormalised)
 *   produ         src/produ.f90:11-23
 *   trunc         src/trunc.f90:10-25
 *   step / step4  src/rkstep.f90:11-73, 91-128
 *   forcing, rann src/forcing.f90:16-51
 *   spectrum / fluxes / glob  src/diagnostics.f90:19-166
 *
 * The reference's FFTs are cuFFT library calls (closed, not vendored, version
 * not pinned: nvhpc/23.11 in src/jobscript:18). They are restated here from
 * the DFT definitions cuFFT documents for D2Z/Z2D:
 *   forward X[k] = sum_n x[n] exp(-2 pi i k n / N), inverse with +i, both
 *   unnormalised; 2D = rows (x, contiguous) then columns (y) for D2Z and the
 *   reverse for Z2D.
 * The row transforms use the half-length packing (N real values as N/2
 * complex), the column transforms a radix-2 complex FFT with twiddles taken
 * directly from cos/sin. For Z2D the imaginary parts of the kx=0 and kx=N/2
 * values are ignored (Hermitian input), the convention of numpy's irfft2.
 *
 * PINNED to the reference's own statements: the reference cannot be compiled
 * (nvfortran + OpenACC + cuFFT; no Fortran compiler exists here or on the GPU
 * host) and ships no test vectors, so its Fortran library sources are
 * transliterated mechanically into C (oracle/f2c_ref.py -> oracle/_ref, the
 * cuFFT calls answered by a shim following cuFFT's documented definitions).
 * This oracle matches it bit for bit on every routine without a transform
 * (tables, mode list, LCG, trunc, produ, forcing, diagnostics) and to rounding
 * on the rest; the golden vectors of tests/golden/ are computed by it. It is
 * also checked against an independent numpy restatement, analytic known
 * answers and the closed form of the LCG.
 *
 * Threads: OpenMP over rows / column blocks (deterministic: every output value
 * is computed by exactly one thread in a fixed order). Reductions
 * (diagnostics, forcing) are serial, in the reference's loop order.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/gturbo.h"

typedef struct {
  int L;
  double* tw;  /* L/2 complex: exp(-2 pi i k / L) */
  int* rev;    /* bit reversal of [0, L) */
} cfft_plan;

typedef struct or_ctx {
  gt_params p;
  int N, NY, NH, NBIN, split, rko, truncate;  /* N = NX (row length), NY rows */
  double dkx, dky, dt2, dt3, dt6, sdt, fkxsmax, fkysmax, rtrunc2;
  double *fkx, *fky, *fkxs, *fkys;
  int* jc;
  double *emk, *emkx, *emky;
  int nf;
  int ikxf[GT_NFORC], ikyf[GT_NFORC];
  double ff[GT_NFORC][2];
  double inpz, inpe;
  cfft_plan col;   /* length N   */
  cfft_plan half;  /* length N/2 */
  double* wrow;    /* N/2+1 complex: exp(-2 pi i k / N) */
  int nthreads;
} or_ctx;

/* ------------------------------------------------------------------------ */
/* FFT building blocks                                                      */
/* ------------------------------------------------------------------------ */

static int ilog2(int L) { int m = 0; while ((1 << m) < L) m++; return m; }

static int plan_init(cfft_plan* p, int L) {
  p->L = L;
  p->tw = (double*)malloc(sizeof(double) * (L > 1 ? L : 2));
  p->rev = (int*)malloc(sizeof(int) * L);
  if (!p->tw || !p->rev) return -1;
  const double twopi = 2.0 * 3.14159265358979323846;
  for (int k = 0; k < L / 2; k++) {
    double a = twopi * (double)k / (double)L;
    p->tw[2 * k] = cos(a);
    p->tw[2 * k + 1] = -sin(a);
  }
  int m = ilog2(L);
  for (int i = 0; i < L; i++) {
    int r = 0;
    for (int b = 0; b < m; b++)
      if (i & (1 << b)) r |= 1 << (m - 1 - b);
    p->rev[i] = r;
  }
  return 0;
}

static void plan_free(cfft_plan* p) { free(p->tw); free(p->rev); }

/* In-place complex FFT of length L on interleaved doubles. sign = -1 forward
 * (exp(-i...)), +1 inverse (exp(+i...)); unnormalised. */
static void cfft(const cfft_plan* p, double* a, int sign) {
  const int L = p->L;
  for (int i = 0; i < L; i++) {
    int j = p->rev[i];
    if (i < j) {
      double tr = a[2 * i], ti = a[2 * i + 1];
      a[2 * i] = a[2 * j]; a[2 * i + 1] = a[2 * j + 1];
      a[2 * j] = tr; a[2 * j + 1] = ti;
    }
  }
  for (int len = 2; len <= L; len <<= 1) {
    int half = len >> 1, step = L / len;
    for (int s = 0; s < L; s += len) {
      for (int k = 0; k < half; k++) {
        double wr = p->tw[2 * k * step];
        double wi = p->tw[2 * k * step + 1];
        if (sign > 0) wi = -wi;
        double* x0 = a + 2 * (s + k);
        double* x1 = a + 2 * (s + k + half);
        double tr = wr * x1[0] - wi * x1[1];
        double ti = wr * x1[1] + wi * x1[0];
        x1[0] = x0[0] - tr; x1[1] = x0[1] - ti;
        x0[0] = x0[0] + tr; x0[1] = x0[1] + ti;
      }
    }
  }
}

/* Row R2C, in place on N+2 doubles (x in r[0..N-1] -> X[0..N/2]). */
static void rfft_row(const or_ctx* c, double* r) {
  const int N = c->N, M = N / 2;
  cfft(&c->half, r, -1);
  double z0r = r[0], z0i = r[1];
  for (int k = 1; k <= M / 2; k++) {
    int q = M - k;
    double ar = r[2 * k], ai = r[2 * k + 1];
    double br = r[2 * q], bi = r[2 * q + 1];
    /* X[k] = 1/2 (Z[k] + conj Z[q]) - i/2 W^k (Z[k] - conj Z[q]) */
    double sr = ar + br, si = ai - bi;  /* Z[k] + conj Z[q] */
    double dr = ar - br, di = ai + bi;  /* Z[k] - conj Z[q] */
    double wr = c->wrow[2 * k], wi = c->wrow[2 * k + 1];
    double tr = wr * dr - wi * di, ti = wr * di + wi * dr;  /* W^k d */
    double xkr = 0.5 * (sr + ti), xki = 0.5 * (si - tr);
    /* X[q] = 1/2 (Z[q] + conj Z[k]) - i/2 W^q (Z[q] - conj Z[k]) */
    double s2r = br + ar, s2i = bi - ai;
    double d2r = br - ar, d2i = bi + ai;
    double w2r = c->wrow[2 * q], w2i = c->wrow[2 * q + 1];
    double t2r = w2r * d2r - w2i * d2i, t2i = w2r * d2i + w2i * d2r;
    double xqr = 0.5 * (s2r + t2i), xqi = 0.5 * (s2i - t2r);
    r[2 * k] = xkr; r[2 * k + 1] = xki;
    r[2 * q] = xqr; r[2 * q + 1] = xqi;
  }
  r[0] = z0r + z0i; r[1] = 0.0;
  r[N] = z0r - z0i; r[N + 1] = 0.0;
}

/* Row C2R, in place on N+2 doubles (X[0..N/2] -> x[0..N-1]); padding zeroed. */
static void irfft_row(const or_ctx* c, double* r) {
  const int N = c->N, M = N / 2;
  double x0 = r[0], xm = r[N];  /* imaginary parts of X[0], X[M] ignored */
  for (int k = 1; k <= M / 2; k++) {
    int q = M - k;
    double ar = r[2 * k], ai = r[2 * k + 1];   /* X[k] */
    double br = r[2 * q], bi = r[2 * q + 1];   /* X[q] */
    /* Z[k] = (X[k] + conj X[q]) + i W^-k (X[k] - conj X[q]) */
    double sr = ar + br, si = ai - bi;
    double dr = ar - br, di = ai + bi;
    double wr = c->wrow[2 * k], wi = -c->wrow[2 * k + 1];
    double tr = wr * dr - wi * di, ti = wr * di + wi * dr;
    double zkr = sr - ti, zki = si + tr;
    /* Z[q] = (X[q] + conj X[k]) + i W^-q (X[q] - conj X[k]) */
    double s2r = br + ar, s2i = bi - ai;
    double d2r = br - ar, d2i = bi + ai;
    double w2r = c->wrow[2 * q], w2i = -c->wrow[2 * q + 1];
    double t2r = w2r * d2r - w2i * d2i, t2i = w2r * d2i + w2i * d2r;
    double zqr = s2r - t2i, zqi = s2i + t2r;
    r[2 * k] = zkr; r[2 * k + 1] = zki;
    r[2 * q] = zqr; r[2 * q + 1] = zqi;
  }
  /* k = 0: Z[0] = (X0 + XM) + i (X0 - XM) with X0, XM real */
  r[0] = x0 + xm;
  r[1] = x0 - xm;
  cfft(&c->half, r, +1);
  r[N] = 0.0; r[N + 1] = 0.0;
}

#define COLB 8

/* Complex FFT along y of every column kx of the spectral field, in place. */
static void col_fft(const or_ctx* c, double* z, int sign) {
  const int N = c->NY, NH = c->NH;  /* column length NY */
  const int nblk = (NH + COLB - 1) / COLB;
#pragma omp parallel
  {
    double* buf = (double*)malloc(sizeof(double) * 2 * (size_t)N * COLB);
#pragma omp for schedule(static)
    for (int b = 0; b < nblk; b++) {
      int i0 = b * COLB, nb = NH - i0 < COLB ? NH - i0 : COLB;
      for (int j = 0; j < N; j++)
        for (int t = 0; t < nb; t++) {
          const double* src = z + 2 * ((size_t)j * NH + i0 + t);
          buf[2 * ((size_t)t * N + j)] = src[0];
          buf[2 * ((size_t)t * N + j) + 1] = src[1];
        }
      for (int t = 0; t < nb; t++) cfft(&c->col, buf + 2 * (size_t)t * N, sign);
      for (int j = 0; j < N; j++)
        for (int t = 0; t < nb; t++) {
          double* dst = z + 2 * ((size_t)j * NH + i0 + t);
          dst[0] = buf[2 * ((size_t)t * N + j)];
          dst[1] = buf[2 * ((size_t)t * N + j) + 1];
        }
    }
    free(buf);
  }
}

/* ------------------------------------------------------------------------ */
/* Public oracle API                                                        */
/* ------------------------------------------------------------------------ */

void or_destroy(or_ctx* c);

/* defk (src/defk.f90:12-73) + the derived scalars of inieuler
 * (src/inieuler.f90:22-36, 78-81) + iniforcing (src/iniforcing.f90:11-68).
 * Returns NULL on error; *err = GT_ERR_ARG / GT_ERR_NFORC / GT_ERR_NOMEM. */
or_ctx* or_create(const gt_params* p, int* err) {
  *err = GT_ERR_ARG;
  int N = p->n;
  const int NY = p->ny > 0 ? p->ny : N;
  if (N < 16 || N > 16384 || (N & (N - 1))) return NULL;
  if (NY < 16 || NY > 16384 || (NY & (NY - 1))) return NULL;
  or_ctx* c = (or_ctx*)calloc(1, sizeof(or_ctx));
  if (!c) { *err = GT_ERR_NOMEM; return NULL; }
  c->p = *p;
  c->N = N; c->NY = NY; c->NH = N / 2 + 1; c->NBIN = N / 2;
  const int NH = c->NH;
#ifdef _OPENMP
  c->nthreads = omp_get_max_threads();
#else
  c->nthreads = 1;
#endif
  /* inieuler.f90:22-36 */
  int split = 0;
  if (p->alpnu < 1.0005 && p->alpnu > 0.9995 && p->alpmu < 0.0005 && p->alpmu > -0.0005) split = 1;
  if (p->rko == 4) split = 0;
  if (p->split == 0 || p->split == 1) split = p->split;
  c->split = split;
  c->rko = (p->rko == 4) ? 4 : 2;
  c->truncate = p->truncate;
  /* inieuler.f90:78-81 */
  c->sdt = sqrt(p->dt);
  c->dt2 = p->dt / 2.0;
  c->dt3 = p->dt / 3.0;
  c->dt6 = p->dt / 6.0;

  c->fkx = (double*)malloc(sizeof(double) * NH);
  c->fkxs = (double*)malloc(sizeof(double) * NH);
  c->fky = (double*)malloc(sizeof(double) * NY);
  c->fkys = (double*)malloc(sizeof(double) * NY);
  c->jc = (int*)malloc(sizeof(int) * NY);
  c->emk = (double*)malloc(sizeof(double) * (size_t)NH * NY);
  c->emkx = (double*)malloc(sizeof(double) * NH);
  c->emky = (double*)malloc(sizeof(double) * NY);
  c->wrow = (double*)malloc(sizeof(double) * 2 * (N / 2 + 1));
  if (!c->fkx || !c->fkxs || !c->fky || !c->fkys || !c->jc || !c->emk || !c->emkx ||
      !c->emky || !c->wrow || plan_init(&c->col, NY) || plan_init(&c->half, N / 2)) {
    or_destroy(c);
    *err = GT_ERR_NOMEM;
    return NULL;
  }
  /* defk.f90:12-15 conjugate index (0-based) */
  c->jc[0] = 0;
  for (int j = 1; j < NY; j++) c->jc[j] = NY - j;
  /* defk.f90:18-36 */
  c->dkx = 2.0 * 3.14159265358979323846 / p->xlx;
  c->dky = 2.0 * 3.14159265358979323846 / p->xly;
  for (int i = 0; i < NH; i++) c->fkx[i] = (double)i * c->dkx;
  for (int j = 0; j <= NY / 2; j++) c->fky[j] = (double)j * c->dky;
  for (int j = NY / 2 + 1; j < NY; j++) c->fky[j] = (double)(j - NY) * c->dky;
  for (int i = 0; i < NH; i++) c->fkxs[i] = c->fkx[i] * c->fkx[i];
  for (int j = 0; j < NY; j++) c->fkys[j] = c->fky[j] * c->fky[j];
  /* defk.f90:43-50 */
  for (int j = 0; j < NY; j++)
    for (int i = 0; i < NH; i++) {
      if (i == 0 && j == 0) { c->emk[0] = 0.0; continue; }
      double fk2 = c->fkxs[i] + c->fkys[j];
      double scra = p->nu * pow(fk2, p->alpnu) + p->mu * pow(fk2, p->alpmu);
      c->emk[(size_t)j * NH + i] = exp(-0.5 * p->dt * scra);
    }
  /* defk.f90:58-68 */
  for (int j = 0; j < NY; j++) {
    double fk2 = c->fkys[j];
    double scra = p->nu * pow(fk2, p->alpnu) + p->mu;
    c->emky[j] = exp(-0.5 * p->dt * scra);
  }
  for (int i = 0; i < NH; i++) {
    double fk2 = c->fkxs[i];
    double scra = p->nu * pow(fk2, p->alpnu);
    c->emkx[i] = exp(-0.5 * p->dt * scra);
  }
  /* defk.f90:71-73 */
  c->fkxsmax = c->fkxs[N / 2];
  c->fkysmax = c->fkys[NY / 2];
  c->rtrunc2 = p->rtrunc * p->rtrunc;
  /* twiddles of the row post-processing */
  for (int k = 0; k <= N / 2; k++) {
    double a = 2.0 * 3.14159265358979323846 * (double)k / (double)N;
    c->wrow[2 * k] = cos(a);
    c->wrow[2 * k + 1] = -sin(a);
  }

  /* iniforcing.f90:11-68, same mode order */
  c->nf = 0; c->inpe = 0.0; c->inpz = 0.0;
  const double famp = p->famp, k1f2 = p->k1f * p->k1f, k2f2 = p->k2f * p->k2f;
  for (int pass = 0; pass < 3; pass++) {
    int ilo, ihi;
    if (pass == 0) { ilo = 0; ihi = 0; }
    else if (pass == 1) { ilo = 1; ihi = N / 2 - 1; }
    else { ilo = N / 2; ihi = N / 2; }
    for (int i = ilo; i <= ihi; i++) {
      int jlo = (pass == 0) ? 1 : 0;
      int jhi = (pass == 1) ? NY - 1 : NY / 2;
      for (int j = jlo; j <= jhi; j++) {
        double k2 = c->fkxs[i] + c->fkys[j];
        double k2n = c->fkxs[i] / c->fkxsmax + c->fkys[j] / c->fkysmax;
        if (k2n <= c->rtrunc2 && k2 <= k2f2 && k2 > k1f2) {
          if (c->nf >= GT_NFORC) { or_destroy(c); *err = GT_ERR_NFORC; return NULL; }
          c->ikxf[c->nf] = i;
          c->ikyf[c->nf] = j;
          c->ff[c->nf][0] = 1.0;
          c->ff[c->nf][1] = 1.0;
          c->nf++;
          c->inpz = c->inpz + famp * famp;
          c->inpe = c->inpe + famp * famp / pow(k2, p->alpv / 2.0);
        }
      }
    }
  }
  *err = GT_OK;
  return c;
}

void or_destroy(or_ctx* c) {
  if (!c) return;
  free(c->fkx); free(c->fky); free(c->fkxs); free(c->fkys); free(c->jc);
  free(c->emk); free(c->emkx); free(c->emky); free(c->wrow);
  plan_free(&c->col); plan_free(&c->half);
  free(c);
}

void or_info(const or_ctx* c, gt_info* info) {
  memset(info, 0, sizeof(*info));
  info->n = c->N; info->nh = c->NH; info->nbin = c->NBIN;
  info->rko = c->rko; info->split = c->split; info->truncate = c->truncate;
  info->nf = c->nf;
  info->ny = c->NY;
  info->field_doubles = (int64_t)(c->N + 2) * c->NY;
  info->dkx = c->dkx; info->dky = c->dky;
  info->inpz = c->inpz; info->inpe = c->inpe;
  info->fkxsmax = c->fkxsmax; info->fkysmax = c->fkysmax; info->rtrunc2 = c->rtrunc2;
}

int or_forcing_modes(const or_ctx* c, int32_t* ikxf, int32_t* ikyf) {
  for (int k = 0; k < c->nf; k++) { ikxf[k] = c->ikxf[k]; ikyf[k] = c->ikyf[k]; }
  return c->nf;
}

void or_tables(const or_ctx* c, double* emk, double* fkx, double* fky) {
  if (emk) memcpy(emk, c->emk, sizeof(double) * (size_t)c->NH * c->NY);
  if (fkx) memcpy(fkx, c->fkx, sizeof(double) * c->NH);
  if (fky) memcpy(fky, c->fky, sizeof(double) * c->NY);
}

/* fft_dir (src/fft_dir.f90:11-21): D2Z in place, then z(:,j)=z(:,j)/NY/NX. */
void or_fft_dir(const or_ctx* c, double* z) {
  const int N = c->N, NY = c->NY, NS = N + 2;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < NY; j++) rfft_row(c, z + (size_t)j * NS);
  col_fft(c, z, -1);
#pragma omp parallel for schedule(static)
  for (int j = 0; j < NY; j++) {
    double* r = z + (size_t)j * NS;
    for (int i = 0; i < NS; i++) r[i] = r[i] / (double)NY / (double)N;
  }
}

/* fft_inv (src/fft_inv.f90:11-13): Z2D in place, unnormalised. */
void or_fft_inv(const or_ctx* c, double* z) {
  const int N = c->N, NY = c->NY, NS = N + 2;
  col_fft(c, z, +1);
#pragma omp parallel for schedule(static)
  for (int j = 0; j < NY; j++) irfft_row(c, z + (size_t)j * NS);
}

/* trunc (src/trunc.f90:10-25) */
void or_trunc(const or_ctx* c, double* z) {
  const int NY = c->NY, NH = c->NH;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < NY; j++) {
    double k1 = c->fkys[j] / c->fkysmax;
    for (int i = 0; i < NH; i++) {
      double k2 = k1 + c->fkxs[i] / c->fkxsmax;
      if (k2 > c->rtrunc2) {
        z[2 * ((size_t)j * NH + i)] = 0.0;
        z[2 * ((size_t)j * NH + i) + 1] = 0.0;
      }
    }
  }
  z[0] = 0.0; z[1] = 0.0;
}

/* produ (src/produ.f90:11-23) */
void or_produ(const or_ctx* c, const double* z, double* u, double* v) {
  const int N = c->N, NY = c->NY, NS = N + 2;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < NY; j++) {
    for (int i = 0; i < NS; i++) {
      size_t o = (size_t)j * NS + i;
      if (i < N) {
        u[o] = z[o] * u[o];
        v[o] = z[o] * v[o];
      } else {
        u[o] = 0.0;
        v[o] = 0.0;
      }
    }
  }
}

/* nlt (src/nlt.f90:17-63) */
void or_nlt(const or_ctx* c, double* z, double* u, double* v) {
  const int N = c->N, NY = c->NY, NH = c->NH;
  const size_t ns = (size_t)(N + 2) * NY;
  memset(u, 0, sizeof(double) * ns);
  memset(v, 0, sizeof(double) * ns);
  const double ea = c->p.alpv / 2.0;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < NY; j++) {
    for (int i = 0; i < NH; i++) {
      if (i == 0 && j == 0) continue;
      double k2 = c->fkxs[i] + c->fkys[j];
      double ka = pow(k2, ea);
      double kx = c->fkx[i] / ka;
      double ky = c->fky[j] / ka;
      size_t o = 2 * ((size_t)j * NH + i);
      u[o] = -ky * z[o + 1];
      u[o + 1] = +ky * z[o];
      v[o] = +kx * z[o + 1];
      v[o + 1] = -kx * z[o];
    }
  }
  or_fft_inv(c, z);
  or_fft_inv(c, v);
  or_fft_inv(c, u);
  or_produ(c, z, u, v);
  or_fft_dir(c, u);
  or_fft_dir(c, v);
#pragma omp parallel for schedule(static)
  for (int j = 0; j < NY; j++) {
    for (int i = 0; i < NH; i++) {
      size_t o = 2 * ((size_t)j * NH + i);
      z[o] = +c->fkx[i] * u[o + 1] + c->fky[j] * v[o + 1];
      z[o + 1] = -c->fkx[i] * u[o] - c->fky[j] * v[o];
    }
  }
  if (c->truncate == 1) or_trunc(c, z);
}

static inline double emk_at(const or_ctx* c, int i, int j) {
  return c->split ? c->emkx[i] * c->emky[j] : c->emk[(size_t)j * c->NH + i];
}

/* step (src/rkstep.f90:2-76) */
void or_step(const or_ctx* c, double* z, double* znl, double* u, double* v) {
  const int N = c->N, NY = c->NY, NH = c->NH;
  const size_t ns = (size_t)(N + 2) * NY;
  memcpy(znl, z, sizeof(double) * ns);
  or_nlt(c, znl, u, v);
#pragma omp parallel for schedule(static)
  for (int j = 0; j < NY; j++)
    for (int i = 0; i < NH; i++) {
      size_t o = 2 * ((size_t)j * NH + i);
      double e = emk_at(c, i, j);
      znl[o] = e * (z[o] + c->dt2 * znl[o]);
      znl[o + 1] = e * (z[o + 1] + c->dt2 * znl[o + 1]);
    }
  znl[0] = 0.0; znl[1] = 0.0;
  or_nlt(c, znl, u, v);
  const double dt = c->p.dt;
#pragma omp parallel for schedule(static)
  for (int j = 0; j < NY; j++)
    for (int i = 0; i < NH; i++) {
      size_t o = 2 * ((size_t)j * NH + i);
      double e = emk_at(c, i, j);
      z[o] = e * (e * z[o] + dt * znl[o]);
      z[o + 1] = e * (e * z[o + 1] + dt * znl[o + 1]);
    }
  z[0] = 0.0; z[1] = 0.0;
}

/* step4 (src/rkstep.f90:82-131) */
void or_step4(const or_ctx* c, double* z, double* znl, double* znew, double* u, double* v) {
  const int N = c->N, NY = c->NY, NH = c->NH;
  const size_t ns = (size_t)(N + 2) * NY;
  const size_t nc = (size_t)NY * NH;
  const double dt = c->p.dt, dt2 = c->dt2, dt3 = c->dt3, dt6 = c->dt6;
  memcpy(znl, z, sizeof(double) * ns);
  or_nlt(c, znl, u, v);
#pragma omp parallel for schedule(static)
  for (size_t m = 0; m < nc; m++) {
    double e = c->emk[m];
    znew[2 * m] = e * e * (z[2 * m] + dt6 * znl[2 * m]);
    znew[2 * m + 1] = e * e * (z[2 * m + 1] + dt6 * znl[2 * m + 1]);
    znl[2 * m] = e * (z[2 * m] + dt2 * znl[2 * m]);
    znl[2 * m + 1] = e * (z[2 * m + 1] + dt2 * znl[2 * m + 1]);
  }
  or_nlt(c, znl, u, v);
#pragma omp parallel for schedule(static)
  for (size_t m = 0; m < nc; m++) {
    double e = c->emk[m];
    znew[2 * m] = znew[2 * m] + dt3 * e * znl[2 * m];
    znew[2 * m + 1] = znew[2 * m + 1] + dt3 * e * znl[2 * m + 1];
    znl[2 * m] = e * z[2 * m] + dt2 * znl[2 * m];
    znl[2 * m + 1] = e * z[2 * m + 1] + dt2 * znl[2 * m + 1];
  }
  or_nlt(c, znl, u, v);
#pragma omp parallel for schedule(static)
  for (size_t m = 0; m < nc; m++) {
    double e = c->emk[m];
    znew[2 * m] = znew[2 * m] + dt3 * e * znl[2 * m];
    znew[2 * m + 1] = znew[2 * m + 1] + dt3 * e * znl[2 * m + 1];
    znl[2 * m] = e * (e * z[2 * m] + dt * znl[2 * m]);
    znl[2 * m + 1] = e * (e * z[2 * m + 1] + dt * znl[2 * m + 1]);
  }
  or_nlt(c, znl, u, v);
#pragma omp parallel for schedule(static)
  for (size_t m = 0; m < nc; m++) {
    z[2 * m] = znew[2 * m] + dt6 * znl[2 * m];
    z[2 * m + 1] = znew[2 * m + 1] + dt6 * znl[2 * m + 1];
  }
  z[0] = 0.0; z[1] = 0.0;
}

/* rann (src/forcing.f90:40-51): irand = iand(69069*irand+1, 7FFFFFFF) in
 * 32-bit wrap-around arithmetic; the double quotient is stored as real(4). */
float or_rann(int32_t* irand) {
  uint32_t x = (uint32_t)(*irand);
  x = (69069u * x + 1u) & 0x7FFFFFFFu;
  *irand = (int32_t)x;
  return (float)((double)x / (double)0x7FFFFFFF);
}

/* forcing (src/forcing.f90:16-33), serial in k as the reference's
 * `parallel loop seq`. */
void or_forcing(const or_ctx* c, double* z, int32_t* seed) {
  const double pi2 = 2.0 * 3.14159265358979;
  const int NH = c->NH;
  const double sf = c->sdt * c->p.famp;
  for (int k = 0; k < c->nf; k++) {
    int i = c->ikxf[k], j = c->ikyf[k];
    double te = pi2 * (double)or_rann(seed);
    double cc = cos(te), cs = sin(te);
    size_t o = 2 * ((size_t)j * NH + i);
    z[o] = z[o] + sf * c->ff[k][0] * cc;
    z[o + 1] = z[o + 1] + sf * c->ff[k][1] * cs;
    if (i == 0 || i == NH - 1) {
      size_t oc = 2 * ((size_t)c->jc[j] * NH + i);
      z[oc] = z[oc] + sf * c->ff[k][0] * cc;
      z[oc + 1] = z[oc + 1] - sf * c->ff[k][1] * cs;
    }
  }
}

/* spectrum + fluxes + glob (src/diagnostics.f90:19-45, 75-109, 138-163).
 * Serial, in the reference's (j outer, i inner) order. Outputs (NULL = skip):
 * sp, sz, fle, flz: NBIN doubles; glob: {ee, zz, disz_nu, disz_mu, dise_nu, dise_mu}. */
void or_diag(const or_ctx* c, const double* z, const double* znl, double* sp, double* sz,
             double* fle, double* flz, double* glob) {
  const int NY = c->NY, NH = c->NH, NBIN = c->NBIN;
  const double dk = c->dkx, alpv = c->p.alpv;
  const double nu = c->p.nu, mu = c->p.mu, alpnu = c->p.alpnu, alpmu = c->p.alpmu;
  double* spb = (double*)calloc(NBIN, sizeof(double));
  double* szb = (double*)calloc(NBIN, sizeof(double));
  double* flem = (double*)calloc(NBIN, sizeof(double));
  double* flzm = (double*)calloc(NBIN, sizeof(double));
  double ee = 0, zz = 0, dnu = 0, dmu = 0, enu = 0, emu = 0;
  for (int j = 0; j < NY; j++) {
    for (int i = 0; i < NH; i++) {
      if (i == 0 && j == 0) continue;
      size_t o = 2 * ((size_t)j * NH + i);
      double zr = z[o], zi = z[o + 1];
      double k2 = c->fkxs[i] + c->fkys[j];
      double k = sqrt(k2);
      double ka = pow(k2, alpv / 2.0);
      int ib = (int)(k / dk) + 1;
      double a2 = hypot(zr, zi);
      a2 = a2 * a2;
      /* spectrum: fac 1/2 on the kx=0 and Nyquist columns */
      double fac = (i == 0 || i == NH - 1) ? 0.5 : 1.0;
      if (ib < NBIN) {
        spb[ib - 1] = spb[ib - 1] + fac * a2 / ka;
        szb[ib - 1] = szb[ib - 1] + fac * a2;
      }
      /* glob */
      ee = ee + fac * a2 / ka;
      zz = zz + fac * a2;
      dnu = dnu + 2.0 * fac * nu * pow(k2, alpnu) * a2;
      dmu = dmu + 2.0 * fac * mu * pow(k2, alpmu) * a2;
      enu = enu + 2.0 * fac * nu * pow(k2, alpnu - alpv / 2.0) * a2;
      emu = emu + 2.0 * fac * mu * pow(k2, alpmu - alpv / 2.0) * a2;
      /* fluxes: fac 2 interior, 1 on the edge columns */
      if (znl) {
        double ff = (i == 0 || i == NH - 1) ? 1.0 : 2.0;
        double fz = zr * znl[o] + zi * znl[o + 1];
        double fe = fz / ka;
        if (ib < NBIN) {
          flzm[ib - 1] = flzm[ib - 1] + ff * fz;
          flem[ib - 1] = flem[ib - 1] + ff * fe;
        }
      }
    }
  }
  if (sp) for (int b = 0; b < NBIN; b++) sp[b] = spb[b] / dk;
  if (sz) for (int b = 0; b < NBIN; b++) sz[b] = szb[b] / dk;
  if (znl && (fle || flz)) {
    for (int b = 0; b < NBIN; b++) {
      double se = 0, sq = 0;
      for (int b2 = b; b2 < NBIN; b2++) { se += flem[b2]; sq += flzm[b2]; }
      if (fle) fle[b] = se;
      if (flz) flz[b] = sq;
    }
  }
  if (glob) {
    glob[0] = ee; glob[1] = zz; glob[2] = dnu; glob[3] = dmu; glob[4] = enu; glob[5] = emu;
  }
  free(spb); free(szb); free(flem); free(flzm);
}

/* One iteration of the main loop body (src/main.f90:97-137) without I/O:
 * step/step4, then (when diag != 0) znl=z; nlt(znl) and the diagnostics,
 * then forcing. Diagnostic outputs as in or_diag (NULL = skip). */
void or_main_step(const or_ctx* c, double* z, double* znl, double* znew, double* u, double* v,
                  int32_t* seed, int diag, double* sp, double* sz, double* fle, double* flz,
                  double* glob) {
  if (c->rko == 4) or_step4(c, z, znl, znew, u, v);
  else or_step(c, z, znl, u, v);
  if (diag) {
    memcpy(znl, z, sizeof(double) * (size_t)(c->N + 2) * c->NY);
    or_nlt(c, znl, u, v);
    or_diag(c, z, znl, sp, sz, fle, flz, glob);
  }
  or_forcing(c, z, seed);
}

int or_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void or_set_num_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* ------------------------------------------------------------------------ */
/* Counter-based forcing (no counterpart in the reference): Philox4x64-10    */
/* (Salmon et al., SC'11), the generator numpy calls Philox.                 */
/* ------------------------------------------------------------------------ */

void or_philox4x64_10(const uint64_t ctr_in[4], const uint64_t key[2], uint64_t out[4]) {
  uint64_t x0 = ctr_in[0], x1 = ctr_in[1], x2 = ctr_in[2], x3 = ctr_in[3];
  uint64_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; r++) {
    if (r > 0) {
      k0 += 0x9E3779B97F4A7C15ull;
      k1 += 0xBB67AE8584CAA73Bull;
    }
    unsigned __int128 p0 = (unsigned __int128)0xD2E7470EE14C6C93ull * x0;
    unsigned __int128 p1 = (unsigned __int128)0xCA5A826395121157ull * x2;
    uint64_t hi0 = (uint64_t)(p0 >> 64), lo0 = (uint64_t)p0;
    uint64_t hi1 = (uint64_t)(p1 >> 64), lo1 = (uint64_t)p1;
    uint64_t y0 = hi1 ^ x1 ^ k0, y1 = lo1, y2 = hi0 ^ x3 ^ k1, y3 = lo0;
    x0 = y0; x1 = y1; x2 = y2; x3 = y3;
  }
  out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

/* The forcing kick with phase 2 pi u, u = top 53 bits of Philox((step, k, 0, 0), (key, 0))[0]. */
void or_forcing_philox(const or_ctx* c, double* z, uint64_t key, uint64_t step) {
  const int NH = c->NH;
  const double sf = c->sdt * c->p.famp;
  const uint64_t kk[2] = {key, 0};
  for (int k = 0; k < c->nf; k++) {
    uint64_t ctr[4] = {step, (uint64_t)k, 0, 0}, o[4];
    or_philox4x64_10(ctr, kk, o);
    double u = (double)(o[0] >> 11) * (1.0 / 9007199254740992.0);
    double te = 2.0 * 3.14159265358979323846 * u;
    double cc = cos(te), cs = sin(te);
    int i = c->ikxf[k], j = c->ikyf[k];
    size_t o2 = 2 * ((size_t)j * NH + i);
    z[o2] = z[o2] + sf * c->ff[k][0] * cc;
    z[o2 + 1] = z[o2 + 1] + sf * c->ff[k][1] * cs;
    if (i == 0 || i == NH - 1) {
      size_t oc = 2 * ((size_t)c->jc[j] * NH + i);
      z[oc] = z[oc] + sf * c->ff[k][0] * cc;
      z[oc + 1] = z[oc + 1] - sf * c->ff[k][1] * cs;
    }
  }
}
