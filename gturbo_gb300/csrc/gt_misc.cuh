// gt_misc.cuh -- non-templated kernels of the Gturbo hot path: trunc, produ, the stochastic
// forcing, the diagnostics and the table set-up. Included by the host translation unit only.
#pragma once

#include "gt_kernels.cuh"

namespace gt {

// trunc (trunc.f90:10-25): zero outside the ellipse, then the mean mode.
__global__ void k_trunc(double2* z, int n, int nh, const int* __restrict__ kcut) {
  const size_t total = (size_t)n * nh;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < total;
       o += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(o / nh), i = (int)(o % nh);
    if (min(j, n - j) > __ldg(&kcut[i]) || o == 0) z[o] = czero();
  }
}

// produ (produ.f90:11-23) on an n x ny field (rows of n + 2 doubles)
__global__ void k_produ(const double* __restrict__ z, double* u, double* v, int n, int ny) {
  const int ns = n + 2;
  const size_t total = (size_t)ns * ny;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < total;
       o += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(o % ns);
    if (i < n) {
      const double zz = z[o];
      u[o] = zz * u[o];
      v[o] = zz * v[o];
    } else {
      u[o] = 0.0;
      v[o] = 0.0;
    }
  }
}

// forcing (forcing.f90:16-33). Mode k uses the LCG state after k+1 draws from seed0:
// x_{k+1} = (A[k] x0 + B[k]) mod 2^31 with A, B the jump-ahead coefficients of the map
// x -> 69069 x + 1 (computed on the host), so the phases equal the serial rann sequence.
// Distinct modes never touch the same value except a self-conjugate mode, which one thread
// handles in the reference's order.
__global__ void k_forcing(double2* z, int nh, int nf, const int* __restrict__ ikx,
                          const int* __restrict__ iky, const int* __restrict__ jc,
                          const uint32_t* __restrict__ lcga, const uint32_t* __restrict__ lcgb,
                          const double2* __restrict__ ff, uint32_t seed0, double sf) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nf) return;
  const int i = ikx[k], j = iky[k];
  const double2 inc = forcing_increment(k, lcga, lcgb, ff, seed0, sf);
  double2* p = z + (size_t)j * nh + i;
  *p = add_kick(*p, inc, false);
  if (i == 0 || i == nh - 1) {
    double2* pc = z + (size_t)jc[j] * nh + i;
    *pc = add_kick(*pc, inc, true);
  }
}

// This step's kick increments of the nf forced modes, for the fused final-stage store.
__global__ void k_kick_values(double2* kick, int nf, const uint32_t* __restrict__ lcga,
                              const uint32_t* __restrict__ lcgb, const double2* __restrict__ ff,
                              uint32_t seed0, double sf) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < nf) kick[k] = forcing_increment(k, lcga, lcgb, ff, seed0, sf);
}

// ---------------------------------------------------------------------------------------
// Diagnostics (diagnostics.f90): deterministic, atomics-free.
// Shell sums: block g sums every bin over the rows of group g, rows and modes in ascending
// order; a second kernel adds the groups in order. Global sums: per-row block reductions in a
// fixed tree order, then the rows in a fixed tree order.
// ---------------------------------------------------------------------------------------
// Rows per group of the shell sums: N/256 (at least 1), so every size has up to 256 groups.
__host__ __device__ constexpr int diag_row_group(int n) { return n >= 256 ? n / 256 : 1; }
__host__ __device__ constexpr int diag_groups(int n) { return n / diag_row_group(n); }
constexpr int kDiagThreads = 256;

struct DiagArgs {
  const double2* z;
  const double2* znl;   // may be null: no fluxes
  const double* fkxs;
  const double* fkys;
  const double* kainv;  // 1/|k|^alpha table [n][nh] or null (then pow per mode)
  int n, nh, nbin;       // n: rows (NY); nh = NX/2+1 columns; nbin = NX/2
  int unit_k;           // 1: dkx = dky = 1 (box 2 pi), integer wavenumbers -> integer bins
  double dk, alpv;
  double nu, mu, alpnu, alpmu;
  int inu, imu;         // alpnu, alpmu as small non-negative integers (-1: not one)
  double* part;         // [ngroups][nbin][4]: sp, sz, flem, flzm
  double* rowsum;       // [n][6]
};

// smallest s >= 0 with s*s >= x (x < 2^52)
__device__ __forceinline__ int isqrt_ceil(long long x) {
  if (x <= 0) return 0;
  long long s = (long long)sqrtf((float)x);
  while (s * s < x) ++s;
  while (s > 0 && (s - 1) * (s - 1) >= x) --s;
  return (int)s;
}

__device__ __forceinline__ int diag_bin(const DiagArgs& D, int i, int j) {
  const double k = sqrt(__ldg(&D.fkxs[i]) + __ldg(&D.fkys[j]));
  return (int)(k / D.dk);  // 0-based: reference ib - 1
}

// The modes [lo, hi) of row j in bin b. The bin index is non-decreasing in i along a row.
__device__ __forceinline__ void diag_segment(const DiagArgs& D, int b, int j, double fkys, int& lo, int& hi) {
  if (D.unit_k) {
    // integer wavenumbers: int(sqrt(k2)) = floor(sqrt(i^2 + ky^2)) exactly (k2 < 2^52), so
    // b^2 <= i^2 + ky^2 < (b+1)^2 gives the segment in integer arithmetic
    const long long ky = min(j, D.n - j);
    lo = min(isqrt_ceil((long long)b * b - ky * ky), D.nh);
    hi = min(isqrt_ceil((long long)(b + 1) * (b + 1) - ky * ky), D.nh);
  } else {
    // the analytic estimate of the first i with bin >= b, corrected with the exact bin function
    const double kb = (double)b * D.dk;
    const double rem = kb * kb - fkys;
    lo = rem > 0.0 ? (int)ceil(sqrt(rem) / D.dk) : 0;
    lo = min(max(lo, 0), D.nh);
    while (lo > 0 && diag_bin(D, lo - 1, j) >= b) --lo;
    while (lo < D.nh && diag_bin(D, lo, j) < b) ++lo;
    hi = lo;
    while (hi < D.nh && diag_bin(D, hi, j) == b) ++hi;
  }
}

// Shell sums of one group of rows (diagnostics.f90:30-44, 90-104). For each row of the group the
// block first stages every mode's contributions (sp, sz, flem, flzm terms) in shared memory,
// one mode per thread with coalesced loads; then the thread of bin b adds its bin's segment of
// that row in ascending i. Per (bin, group) the order is rows ascending, modes ascending.
// MB bins per thread (nbin <= 256 MB); dynamic shared memory nh * 32 bytes.
template <int MB>
__global__ void __launch_bounds__(kDiagThreads) k_diag_bins(DiagArgs D) {
  extern __shared__ double4 contrib[];
  const int g = blockIdx.x, t = threadIdx.x;
  const int rg = diag_row_group(D.n);
  double acc[MB][4];
#pragma unroll
  for (int m = 0; m < MB; ++m) acc[m][0] = acc[m][1] = acc[m][2] = acc[m][3] = 0.0;
  for (int j = g * rg; j < (g + 1) * rg; ++j) {
    const double fkys = __ldg(&D.fkys[j]);
    for (int i = t; i < D.nh; i += kDiagThreads) {
      double4 c = make_double4(0.0, 0.0, 0.0, 0.0);
      if (i != 0 || j != 0) {
        const size_t o = (size_t)j * D.nh + i;
        const double2 q = D.z[o];
        // 1/|k|^alpha from the table when the handle has one (else a pow per mode)
        const double ikv = D.kainv ? __ldg(&D.kainv[o]) : 1.0 / pow(__ldg(&D.fkxs[i]) + fkys, D.alpv / 2.0);
        const double a2 = q.x * q.x + q.y * q.y;
        const double fac = (i == 0 || i == D.nh - 1) ? 0.5 : 1.0;
        c.x = fac * a2 * ikv;
        c.y = fac * a2;
        if (D.znl) {
          const double2 w = D.znl[o];
          const double ff = (i == 0 || i == D.nh - 1) ? 1.0 : 2.0;
          const double f = q.x * w.x + q.y * w.y;
          c.z = ff * (f * ikv);
          c.w = ff * f;
        }
      }
      contrib[i] = c;
    }
    __syncthreads();
#pragma unroll
    for (int m = 0; m < MB; ++m) {
      const int b = t + m * kDiagThreads;
      if (b < D.nbin - 1) {
        int lo, hi;
        diag_segment(D, b, j, fkys, lo, hi);
        for (int i = lo; i < hi; ++i) {
          const double4 c = contrib[i];
          acc[m][0] += c.x;
          acc[m][1] += c.y;
          acc[m][2] += c.z;
          acc[m][3] += c.w;
        }
      }
    }
    __syncthreads();  // the next row reuses contrib
  }
#pragma unroll
  for (int m = 0; m < MB; ++m) {
    const int b = t + m * kDiagThreads;
    if (b < D.nbin) {
      double* p = D.part + ((size_t)g * D.nbin + b) * 4;
      p[0] = acc[m][0]; p[1] = acc[m][1]; p[2] = acc[m][2]; p[3] = acc[m][3];
    }
  }
}

// A small non-negative integer exponent as an int (-1: not one), for ipow_sq.
inline int diag_int_exponent(double a) {
  return (a >= 0.0 && a <= 64.0 && a == (double)(int)a) ? (int)a : -1;
}

// Dynamic shared memory of k_diag_bins (nh columns) and k_diag_suffix (nbin bins).
inline size_t diag_bins_smem(int nh) { return (size_t)nh * sizeof(double4); }
inline size_t diag_suffix_smem(int nbin) { return (size_t)nbin * sizeof(double2); }

// out[b*4 + q] = sum over groups (in order); then spectra / dk and flux suffix sums.
__global__ void k_diag_bins_final(DiagArgs D, double* out /* [nbin][4] */) {
  const int ngroups = diag_groups(D.n);
  const int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b < D.nbin) {
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int g = 0; g < ngroups; ++g)
      for (int q = 0; q < 4; ++q) s[q] += D.part[((size_t)g * D.nbin + b) * 4 + q];
    out[b * 4 + 0] = s[0] / D.dk;
    out[b * 4 + 1] = s[1] / D.dk;
    out[b * 4 + 2] = s[2];
    out[b * 4 + 3] = s[3];
  }
}

// One block of kDiagThreads threads; dynamic shared memory nbin * 16 bytes (the flux columns
// of bins, staged once so that every suffix sum reads shared memory).
__global__ void __launch_bounds__(kDiagThreads) k_diag_suffix(const double* bins, double* fl, int nbin) {
  extern __shared__ double2 flx[];
  for (int b = threadIdx.x; b < nbin; b += kDiagThreads) flx[b] = make_double2(bins[b * 4 + 2], bins[b * 4 + 3]);
  __syncthreads();
  for (int b = threadIdx.x; b < nbin; b += kDiagThreads) {
    double se = 0.0, sq = 0.0;
    for (int b2 = b; b2 < nbin; ++b2) {  // sum(flem(i:NBIN)), diagnostics.f90:106-107
      se += flx[b2].x;
      sq += flx[b2].y;
    }
    fl[b * 2 + 0] = se;
    fl[b * 2 + 1] = sq;
  }
}

// The shell-sum kernel for D.n (bins per thread from nbin = n/2).
inline void diag_launch_bins(const DiagArgs& D, cudaStream_t s) {
  const int ng = diag_groups(D.n);
  const size_t smem = diag_bins_smem(D.nh);
  const int mb = (D.nbin + kDiagThreads - 1) / kDiagThreads;
  if (mb <= 1) k_diag_bins<1><<<ng, kDiagThreads, smem, s>>>(D);
  else if (mb <= 2) k_diag_bins<2><<<ng, kDiagThreads, smem, s>>>(D);
  else if (mb <= 4) k_diag_bins<4><<<ng, kDiagThreads, smem, s>>>(D);
  else if (mb <= 8) k_diag_bins<8><<<ng, kDiagThreads, smem, s>>>(D);
  else k_diag_bins<16><<<ng, kDiagThreads, smem, s>>>(D);
}

// Raises the shared-memory limit of the shell-sum kernels for the largest grids (n = 8192).
inline cudaError_t diag_prepare() {
  cudaError_t e = cudaSuccess;
  const cudaFuncAttribute attr = cudaFuncAttributeMaxDynamicSharedMemorySize;
  if ((e = cudaFuncSetAttribute(k_diag_bins<8>, attr, (int)diag_bins_smem(4096 / 2 + 1)))) return e;
  if ((e = cudaFuncSetAttribute(k_diag_bins<16>, attr, (int)diag_bins_smem(8192 / 2 + 1)))) return e;
  return cudaFuncSetAttribute(k_diag_suffix, attr, (int)diag_suffix_smem(8192 / 2));
}

// x^n for a small non-negative integer n by repeated squaring
__device__ __forceinline__ double ipow_sq(double x, int n) {
  double r = 1.0;
  while (n > 0) {
    if (n & 1) r *= x;
    x *= x;
    n >>= 1;
  }
  return r;
}

// glob (diagnostics.f90:147-163): per-row sums with a fixed-order block reduction.
__global__ void k_diag_glob_rows(DiagArgs D) {
  const int j = blockIdx.x;
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const double fkys = __ldg(&D.fkys[j]);
  for (int i = threadIdx.x; i < D.nh; i += blockDim.x) {
    if (i == 0 && j == 0) continue;
    const size_t o = (size_t)j * D.nh + i;
    const double2 q = D.z[o];
    const double k2 = __ldg(&D.fkxs[i]) + fkys;
    const double ikv = D.kainv ? __ldg(&D.kainv[o]) : 1.0 / pow(k2, D.alpv / 2.0);
    const double a2 = q.x * q.x + q.y * q.y;
    const double fac = (i == 0 || i == D.nh - 1) ? 0.5 : 1.0;
    // k2^alpnu, k2^alpmu: by repeated squaring for small integer exponents (the usual
    // hyperviscosity and drag), else from one log (pow costs ~2x log + exp in FP64); the
    // alpha-shifted powers of diagnostics.f90:160-161 are these divided by ka
    double knu, kmu;
    if (D.inu >= 0 && D.imu >= 0) {
      knu = ipow_sq(k2, D.inu);
      kmu = ipow_sq(k2, D.imu);
    } else {
      const double lk = log(k2);
      knu = exp(D.alpnu * lk);
      kmu = D.alpmu == 0.0 ? 1.0 : exp(D.alpmu * lk);
    }
    const double fa = fac * a2;
    const double fai = fa * ikv;
    acc[0] += fai;
    acc[1] += fa;
    acc[2] += 2.0 * D.nu * knu * fa;
    acc[3] += 2.0 * D.mu * kmu * fa;
    acc[4] += 2.0 * D.nu * knu * fai;
    acc[5] += 2.0 * D.mu * kmu * fai;
  }
  __shared__ double red[6][256];
  for (int q = 0; q < 6; ++q) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 6; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 6) D.rowsum[(size_t)j * 6 + threadIdx.x] = red[threadIdx.x][0];
}

// Six warps (192 threads), warp q sums column q of the row sums: lane l adds rows l, l+32, ...
// in order, then the lanes combine in a fixed shuffle tree.
__global__ void k_diag_glob_final(DiagArgs D, double* glob) {
  const int q = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (q >= 6) return;
  double s = 0.0;
  for (int j = lane; j < D.n; j += 32) s += D.rowsum[(size_t)j * 6 + q];
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  if (lane == 0) glob[q] = s;
}

// ---------------------------------------------------------------------------------------
// Table set-up (defk.f90:43-50 and nlt.f90:26-27 on the device).
// ---------------------------------------------------------------------------------------
__global__ void k_init_tables(double* emk, double* kainv, const double* __restrict__ fkxs,
                              const double* __restrict__ fkys, int n, int nh, double nu,
                              double alpnu, double mu, double alpmu, double alpv, double dt) {
  const size_t total = (size_t)n * nh;
  for (size_t o = blockIdx.x * (size_t)blockDim.x + threadIdx.x; o < total;
       o += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(o / nh), i = (int)(o % nh);
    if (o == 0) {
      emk[0] = 0.0;
      kainv[0] = 0.0;
      continue;
    }
    const double fk2 = fkxs[i] + fkys[j];
    const double scra = nu * pow(fk2, alpnu) + mu * pow(fk2, alpmu);
    emk[o] = exp(-0.5 * dt * scra);
    kainv[o] = 1.0 / pow(fk2, alpv / 2.0);
  }
}

}  // namespace gt
