// gt_kernels.cuh -- device kernels of the Gturbo hot path (templated on the grid size N).
//
// Field layout (identical to the reference): spectral complex(8) z(N/2+1, N) == double2
// z[N][NH] (NH = N/2+1, kx fastest); physical real(8) z(N+2, N) == double z[N][N+2].
//
// The nonlinear term nlt (src/nlt.f90) is three fused passes instead of the reference's
// 5 cuFFT calls and 8 elementwise kernels:
//   A  column pass, inverse y-FFT of q, u = i ky/|k|^a q and v = -i kx/|k|^a q
//      (the multiplies of nlt.f90:22-36 fused into the load);
//   B  row pass: C2R of q and of u+iv, the physical product (produ.f90:11-23), R2C of
//      (u+iv)q, and the split into the two product spectra;
//   C  column pass: forward y-FFT of both products, N = -i(kx A + ky B)/N^2 (nlt.f90:54-61,
//      fft_dir.f90:17-21), the 2/3 mask (trunc.f90:10-25) and the Runge-Kutta stage update
//      of rkstep.f90 fused into the store.
// With truncate=1 the columns kx > kxlim hold no retained mode: pass C writes N=0 there
// without transforming, and pass A stores zeros without transforming for any such column
// block whose input is entirely zero. A device flag tells pass B whether any column beyond
// kxlim carried data (an untruncated input); only then does pass B read those columns.
// Up to 2048^2 the column passes A and C also exist split by field (one field of one column per
// CTA, the *_field_tile functions), which evens out the SMs' share of the 2/3-rule columns.
#pragma once

#include <cooperative_groups.h>

#include "gt_fft.cuh"

namespace gt {

// Runge-Kutta epilogues of pass C (rkstep.f90). nh = the nonlinear term just computed.
enum Epi : int {
  EPI_NLT = 0,   // out = N                                              (nlt)
  EPI_RK2A = 1,  // znl = e (z + dt/2 N), znl(1,1)=0                     (rkstep.f90:31-43)
  EPI_RK2B = 2,  // z   = e (e z + dt N), z(1,1)=0                       (rkstep.f90:61-73)
  EPI_RK4A = 3,  // znew = e e (z + dt/6 N); znl = e (z + dt/2 N)        (rkstep.f90:95-102)
  EPI_RK4B = 4,  // znew += dt/3 e N; znl = e z + dt/2 N                 (rkstep.f90:104-111)
  EPI_RK4C = 5,  // znew += dt/3 e N; znl = e (e z + dt N)               (rkstep.f90:113-120)
  EPI_RK4D = 6,  // z = znew + dt/6 N, z(1,1)=0                          (rkstep.f90:122-128)
};

struct EpiArgs {
  int mode;
  int split;            // 1: e = emkx(i)*emky(j) (rkstep.f90:21-27, 51-57)
  double2* out;         // N (EPI_NLT) / znl / z
  double2* znew;
  const double2* z;     // state read by the stage update
  const double* emk;    // [N][NH]
  const double* emkx;   // [NH]
  const double* emky;   // [N]
  double dt, dt2, dt3, dt6;
  // The forcing kick of forcing.f90:16-33 added to the final stage's store (EPI_RK2B, EPI_RK4D)
  // when fmap is set. fmap[i * fh + jj] over the window i < fwi, |ky| < fwj (jj = j for j < fwj,
  // j - (N - fh) for the rows of negative ky) holds -1 or the mode index k, with bit 30 set
  // where (i, j) is the conjugate partner of mode k on the kx = 0 or Nyquist column.
  const int* fmap;
  int fwi, fwj, fh;
  const double2* kick;   // this step's per-mode increments (forcing_increment)
  int ny;                // rows of the field (NY): the row index wrap of the forced window
};

// The kick of forced mode k: phase te = 2 pi rann of the (k+1)-th LCG draw from seed0
// (x -> 69069 x + 1 mod 2^31, rann rounded to real(4) as in the reference); the value gains
// sf ff (cos te, sin te), its conjugate partner sf ff (cos te, -sin te). forcing_increment and
// add_kick are the one definition that the forcing kernel and the fused final-stage store share,
// so both give the same bits.
__device__ __forceinline__ double2 forcing_increment(int k, const uint32_t* lcga, const uint32_t* lcgb,
                                                     const double2* ff, uint32_t seed0, double sf) {
  const double pi2 = 2.0 * 3.14159265358979;  // forcing.f90:10
  const uint32_t x = (__ldg(&lcga[k]) * seed0 + __ldg(&lcgb[k])) & 0x7FFFFFFFu;
  const float rr = (float)((double)x / 2147483647.0);
  const double te = pi2 * (double)rr;
  double sn, cs;
  sincos(te, &sn, &cs);
  const double2 f = __ldg(&ff[k]);
  return make_double2((sf * f.x) * cs, (sf * f.y) * sn);
}
__device__ __forceinline__ double2 add_kick(double2 a, double2 inc, bool conj) {
  return make_double2(a.x + inc.x, conj ? a.y - inc.y : a.y + inc.y);
}

// The fused kick at (i, j) of an NY x NH field, if (i, j) is forced.
__device__ __forceinline__ double2 fused_kick(const EpiArgs& E, int i, int j, int NH, double2 r) {
  if (i >= E.fwi) return r;
  const int N = E.ny;
  int jj;
  if (j < E.fwj) jj = j;
  else if (j >= N - (E.fh - E.fwj)) jj = j - (N - E.fh);
  else return r;
  const int e = __ldg(&E.fmap[i * E.fh + jj]);
  if (e < 0) return r;
  return add_kick(r, E.kick[e & 0x3FFFFFFF], (e >> 30) & 1);
}

// KICK: the fused forcing kick is compiled in (the final stage's pass C only; the intermediate
// stages' kernels stay free of its registers).
template <bool KICK = false>
__device__ __forceinline__ void epilogue(const EpiArgs& E, int i, int j, int NH, double2 nh) {
  const size_t o = (size_t)j * NH + i;
  if (E.mode == EPI_NLT) {
    E.out[o] = nh;
    return;
  }
  const double e = E.split ? __ldg(&E.emkx[i]) * __ldg(&E.emky[j]) : __ldg(&E.emk[o]);
  const bool origin = (i == 0 && j == 0);
  switch (E.mode) {
    case EPI_RK2A: {
      const double2 z = E.z[o];
      const double2 r = make_double2(e * (z.x + E.dt2 * nh.x), e * (z.y + E.dt2 * nh.y));
      E.out[o] = origin ? make_double2(0.0, 0.0) : r;
      break;
    }
    case EPI_RK2B: {
      const double2 z = E.z[o];
      double2 r = make_double2(e * (e * z.x + E.dt * nh.x), e * (e * z.y + E.dt * nh.y));
      if (origin) r = make_double2(0.0, 0.0);
      if (KICK && E.fmap) r = fused_kick(E, i, j, NH, r);
      E.out[o] = r;
      break;
    }
    case EPI_RK4A: {
      const double2 z = E.z[o];
      const double ee = e * e;
      E.znew[o] = make_double2(ee * (z.x + E.dt6 * nh.x), ee * (z.y + E.dt6 * nh.y));
      E.out[o] = make_double2(e * (z.x + E.dt2 * nh.x), e * (z.y + E.dt2 * nh.y));
      break;
    }
    case EPI_RK4B: {
      const double2 z = E.z[o];
      const double2 w = E.znew[o];
      const double d3 = E.dt3 * e;
      E.znew[o] = make_double2(w.x + d3 * nh.x, w.y + d3 * nh.y);
      E.out[o] = make_double2(e * z.x + E.dt2 * nh.x, e * z.y + E.dt2 * nh.y);
      break;
    }
    case EPI_RK4C: {
      const double2 z = E.z[o];
      const double2 w = E.znew[o];
      const double d3 = E.dt3 * e;
      E.znew[o] = make_double2(w.x + d3 * nh.x, w.y + d3 * nh.y);
      E.out[o] = make_double2(e * (e * z.x + E.dt * nh.x), e * (e * z.y + E.dt * nh.y));
      break;
    }
    case EPI_RK4D: {
      const double2 w = E.znew[o];
      double2 r = make_double2(w.x + E.dt6 * nh.x, w.y + E.dt6 * nh.y);
      if (origin) r = make_double2(0.0, 0.0);
      if (KICK && E.fmap) r = fused_kick(E, i, j, NH, r);
      E.out[o] = r;
      break;
    }
    default:
      break;
  }
}

// Launch shapes. Column kernels: COLS columns per CTA (interleaved in shared memory so that a
// warp's loads cover COLS*16 contiguous bytes of each row), T = N/16 threads per column.
// Row kernels: ROWS rows per CTA, T threads per row.
template <int N>
struct Shape {
  static constexpr int NH = N / 2 + 1;
  static constexpr int T = N / 16;
  // One column per CTA from N=1024 up: the 2/3 rule leaves ~N/3 active columns, and small
  // CTAs let the block scheduler spread them evenly over the 152 SMs (the FP64 pipe is
  // shared by the resident CTAs, so an SM's time is its number of columns).
  static constexpr int COLS = (N >= 1024) ? 1 : (128 / T > 16 ? 16 : 128 / T);
  static constexpr int COL_THREADS = COLS * T;
  static constexpr int COL_CTAS = (NH + COLS - 1) / COLS;
  static constexpr size_t COL_SMEM = (size_t)padded(N) * COLS * sizeof(double2);
  static constexpr int ROWS = (T >= 128) ? 1 : (128 / T > N ? N : 128 / T);
  static constexpr int ROW_THREADS = ROWS * T;
  static constexpr int ROW_CTAS = N / ROWS;
  static constexpr size_t ROW_SMEM = (size_t)(padded(N) + padded(N / 2)) * ROWS * sizeof(double2);
};

__device__ __forceinline__ double2 czero() { return make_double2(0.0, 0.0); }

// Entry of a pass kernel that may be launched with programmatic dependent launch (its launch
// overlaps the completion of the previous kernel on the stream). It waits for that kernel to
// complete and its writes to be visible; after an ordinary launch the wait returns at once. No
// kernel signals griddepcontrol.launch_dependents early: the next launch goes ahead as this
// kernel's CTAs exit. (An early signal at kernel entry, which let the next pass's CTAs take SMs
// and wait there during this pass's tail, made 8192^2 steps 7 % slower.)
__device__ __forceinline__ void pdl_enter() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// 1 unless both parts are +-0 (integer test of the bit patterns)
__device__ __forceinline__ int nonzero2(double2 a) {
  return ((__double_as_longlong(a.x) | __double_as_longlong(a.y)) << 1) != 0;
}

// Zero-band test of a column pass A: the rows j in [3N/8, 5N/8) of a truncated field are zero in
// every column (|ky| <= N/3), so the first radix pass of the column's inverse transforms can leave
// them out. Tested on the loaded values, because a caller may pass an untruncated field.
template <int R>
__device__ __forceinline__ bool column_zband(const double2 (&v)[R]) {
  if constexpr (R < 8) {
    return false;  // no zero band for radix 4
  } else {
    int bz = 0;
#pragma unroll
    for (int s = 0; s < R; ++s)
      if (in_zband(R, s)) bz |= nonzero2(v[s]);
    return !__syncthreads_or(bz);
  }
}

// Minimum resident CTAs per SM requested from ptxas (register budget) for N >= 1024: up to
// GT_*_MINB, but never so many that a thread gets fewer than GT_*_REGS registers. The CTA grows
// with N (N/16 threads per row or column): 3 column / 2 row CTAs at 2048^2 (168 / 255
// registers), 2 at 4096^2 (128 registers: a few spills, but faster on GB300 than one CTA with
// 254), 1 at 8192^2 (the register file allows 128 at 512 threads). Requesting the 2048^2
// counts at 4096^2 and 8192^2 capped the kernels at 40-85 registers, and they spilled heavily.
#ifndef GT_ROW_MINB
#define GT_ROW_MINB 2
#endif
#ifndef GT_COL_MINB
#define GT_COL_MINB 3
#endif
#ifndef GT_ROW_REGS
#define GT_ROW_REGS 128
#endif
#ifndef GT_COL_REGS
#define GT_COL_REGS 128
#endif
constexpr int min_blocks(int cap, int threads, int regs) {
  const int fit = 65536 / (threads * regs);
  return fit < 1 ? 1 : (fit < cap ? fit : cap);
}
template <int N>
struct MinBlocks {
  static constexpr int ROW = N >= 1024 ? min_blocks(GT_ROW_MINB, Shape<N>::ROW_THREADS, GT_ROW_REGS) : 1;
  static constexpr int COL = N >= 1024 ? min_blocks(GT_COL_MINB, Shape<N>::COL_THREADS, GT_COL_REGS) : 1;
};

// ---------------------------------------------------------------------------------------
// The three passes as tile functions. A tile is one CTA's work: C adjacent columns (passes
// A and C) or ROWS rows (pass B) of one field. The single-field kernels run tile = blockIdx.x;
// the ensemble kernels read (member, tile) from a work list, so members of different sizes
// share one launch (256-thread CTAs with 8 values per thread from N = 128 to 2048).
// ---------------------------------------------------------------------------------------

// One nonlinear-term evaluation of one field.
struct NltArgs {
  int n;                 // grid size (dispatch key of the ensemble kernels)
  const double2* zin;    // pass A input (may alias q)
  double2* q;            // transformed q (pass A out, pass B in)
  double2* u;            // pass A out / pass B in-out / pass C in
  double2* v;
  const double* kainv;   // 1/|k|^alpha [N][NH]
  const double* fkx;
  const double* fky;
  const int* kcut;       // largest kept |ky| per column
  const double2* tw;     // twiddle buffer of the column transforms (length NY)
  const double2* twr;    // twiddle buffer of the row transforms (length NX; = tw when square)
  int nh;                // columns NX/2+1 (the row stride of every field)
  double cscale;         // 0.5 / (NX NY): pass C's normalisation of the packed product transforms
  int kxlim, kin, kout, truncate;
  int* flag;             // untruncated-input flag of this field
  EpiArgs epi;
  // Optional (null: not written): pass B stores the physical fields of this evaluation, row y
  // at phys_uv[y*N + x] = u + i v and phys_q[y*N/2 + m] = q[2m] + i q[2m+1]. The adjoint's
  // backward sweep keeps them from the recomputed forward stages instead of transforming again.
  double2* phys_uv;
  double2* phys_q;
  // Per-column counters (NH ints, zero between launches) of the field-split pass C in its
  // counter form: the second of a column's two CTAs runs its epilogue.
  int* colcnt;
};

// Columns of the field (NX/2+1) and pass C's normalisation 0.5/(NX NY): compile-time constants of
// a square grid (RT = false), the values in the arguments for a non-square one (RT = true), whose
// column kernels are separate instantiations so that the square grids' kernels keep their
// constant strides (and their register counts).
template <int N, bool RT>
__device__ __forceinline__ int col_count(const NltArgs& a) { return RT ? a.nh : N / 2 + 1; }
template <int N, bool RT>
__device__ __forceinline__ double col_scale(const NltArgs& a) {
  return RT ? a.cscale : 0.5 / ((double)N * (double)N);
}

// Pass A: inverse y-transforms of u, v and q (in that order: zin may alias q, as the
// reference destroys z, so q is re-read from zin before the q column is overwritten).
template <int N, int C, int R = 16, bool RT = false>
__device__ __forceinline__ void colinv_tile(const NltArgs& a, int tile) {
  constexpr int T = N / R;
  const int NH = col_count<N, RT>(a);
  extern __shared__ double2 smem[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  const int i = tile * C + c;
  const bool valid = i < NH;
  const int ic = valid ? i : NH - 1;
  double2* sm = smem + c;
  const double2* zin = a.zin;
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = valid ? zin[(size_t)(t + s * T) * NH + ic] : czero();
  // A column beyond the 2/3 ellipse (i > kxlim) carries data only if the caller passed an
  // untruncated field: then raise the flag so that pass B reads every column. A tile made
  // only of such columns needs no transform when all of them are zero: it stores zeros, which
  // pass B reads if another tile raised the flag.
  int nz = 0;
  if (valid && i > a.kxlim) {
#pragma unroll
    for (int s = 0; s < R; ++s) nz |= (v[s].x != 0.0) | (v[s].y != 0.0);
  }
  const bool skip = (tile * C > a.kxlim) ? !__syncthreads_or(nz) : false;
  if (skip) {
    if (valid) {
#pragma unroll
      for (int s = 0; s < R; ++s) {
        const size_t o = (size_t)(t + s * T) * NH + i;
        a.u[o] = czero();
        a.v[o] = czero();
        a.q[o] = czero();
      }
    }
    return;
  }
  if (nz) atomicExch(a.flag, 1);
  const bool zb = column_zband<R>(v);
  const double kx = __ldg(&a.fkx[ic]);
  // u = i ky/|k|^a q  (nlt.f90:29-32)
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int j = t + s * T;
    const double m = __ldg(&a.fky[j]) * __ldg(&a.kainv[(size_t)j * NH + ic]);
    v[s] = make_double2(-m * v[s].y, m * v[s].x);
  }
  fft_regs<N, R, true, C>(v, sm, t, a.tw, 0, zb);
  if (valid) {
#pragma unroll
    for (int s = 0; s < R; ++s) a.u[(size_t)(t + s * T) * NH + i] = v[s];
  }
  // v = -i kx/|k|^a q  (nlt.f90:33-34)
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int j = t + s * T;
    const double2 q = valid ? zin[(size_t)j * NH + ic] : czero();
    const double m = kx * __ldg(&a.kainv[(size_t)j * NH + ic]);
    v[s] = make_double2(m * q.y, -m * q.x);
  }
  __syncthreads();
  fft_regs<N, R, true, C>(v, sm, t, a.tw, 0, zb);
  if (valid) {
#pragma unroll
    for (int s = 0; s < R; ++s) a.v[(size_t)(t + s * T) * NH + i] = v[s];
  }
  // q (nlt.f90:41)
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = valid ? zin[(size_t)(t + s * T) * NH + ic] : czero();
  __syncthreads();
  fft_regs<N, R, true, C>(v, sm, t, a.tw, 0, zb);
  if (valid) {
#pragma unroll
    for (int s = 0; s < R; ++s) a.q[(size_t)(t + s * T) * NH + i] = v[s];
  }
}

// Pass B: per row y, C2R of q (half-length packing) and of u+iv (one complex transform of
// length N), p = (u+iv) q, R2C of p, then A = P[k] + conj P[N-k] = 2 FFT(uq)[k] and
// B = -i (P[k] - conj P[N-k]) = 2 FFT(vq)[k] written over U and V for k <= kout.
// Inputs beyond column kin are taken as zero unless the flag says pass A wrote them.
template <int N, int ROWS, int R = 16>
__device__ __forceinline__ void row_tile(const NltArgs& a, int tile) {
  constexpr int T = N / R, NH = N / 2 + 1, M = N / 2;
  extern __shared__ double2 smem[];
  const int r = threadIdx.x / T, t = threadIdx.x % T;
  const int y = tile * ROWS + r;
  double2* cs = smem + (size_t)r * (padded(N) + padded(M));
  double2* zs = cs + padded(N);
  const int kl = (*a.flag) ? M : a.kin;
  const double2* qrow = a.q + (size_t)y * NH;
  const double2* urow = a.u + (size_t)y * NH;
  const double2* vrow = a.v + (size_t)y * NH;
  // C[k] = U[k] + i V[k], C[N-k] = conj U[k] + i conj V[k]; Im of U, V at k=0, N/2 dropped.
  // Beyond kl the inputs are zero: the branches (uniform within all but one warp) store zeros
  // without the FP64 additions.
#pragma unroll
  for (int s = 0; s <= R / 2; ++s) {
    const int k = t + s * T;
    if (k <= M) {
      if (k > kl) {
        cs[padix(k)] = czero();
        cs[padix(N - k)] = czero();
      } else {
        const double2 U = urow[k];
        const double2 V = vrow[k];
        if (k == 0 || k == M) {
          cs[padix(k)] = make_double2(U.x, V.x);
        } else {
          cs[padix(k)] = make_double2(U.x - V.y, U.y + V.x);
          cs[padix(N - k)] = make_double2(U.x + V.y, V.x - U.y);
        }
      }
    }
  }
  // Z[k] = (Q[k] + conj Q[M-k]) + i W^-k (Q[k] - conj Q[M-k]), k < M; Im Q[0], Q[M] dropped.
  // Where only one of Q[k], Q[M-k] lies within kl, the sum and difference need no additions.
#pragma unroll
  for (int s = 0; s < R / 2; ++s) {
    const int k = t + s * T;
    const bool hp = k <= kl, hb = M - k <= kl;
    double2 p = hp ? qrow[k] : czero();
    double2 b = hb ? qrow[M - k] : czero();
    if (k == 0) { p.y = 0.0; b.y = 0.0; }
    double2 sm_, d;
    if (hp && hb) {
      sm_ = make_double2(p.x + b.x, p.y - b.y);
      d = make_double2(p.x - b.x, p.y + b.y);
    } else if (hp) {
      sm_ = p;
      d = p;
    } else {
      sm_ = make_double2(b.x, -b.y);
      d = make_double2(-b.x, b.y);
    }
    zs[padix(k)] = pack_c2r(sm_, d, __ldg(&a.twr[k]));
  }
  __syncthreads();
  // q: inverse length-M transform, R/2 values per thread; result back to zs
  {
    double2 h[R / 2];
#pragma unroll
    for (int s = 0; s < R / 2; ++s) h[s] = zs[padix(t + s * T)];
    __syncthreads();
    fft_regs<M, R / 2, true, 1>(h, zs, t, a.twr, 1);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R / 2; ++s) zs[padix(t + s * T)] = h[s];
    if (a.phys_q) {
#pragma unroll
      for (int s = 0; s < R / 2; ++s) a.phys_q[(size_t)y * M + t + s * T] = h[s];
    }
  }
  // u + i v: inverse length-N transform; C[k] = 0 for kl < k < N - kl
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = cs[padix(t + s * T)];
  __syncthreads();
  fft_regs<N, R, true, 1>(v, cs, t, a.twr, 0, 8 * kl < 3 * N);
  __syncthreads();
  if (a.phys_uv) {
#pragma unroll
    for (int s = 0; s < R; ++s) a.phys_uv[(size_t)y * N + t + s * T] = v[s];
  }
  // p = (u + i v) q  (produ.f90:18-19); q[2m] = Re z[m], q[2m+1] = Im z[m]
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int x = t + s * T;
    const double2 zq = zs[padix(x >> 1)];
    const double q = (x & 1) ? zq.y : zq.x;
    v[s] = make_double2(v[s].x * q, v[s].y * q);
  }
  fft_regs<N, R, false, 1>(v, cs, t, a.twr, 0);
  __syncthreads();
#pragma unroll
  for (int s = 0; s < R; ++s) cs[padix(t + s * T)] = v[s];
  __syncthreads();
  double2* urw = a.u + (size_t)y * NH;
  double2* vrw = a.v + (size_t)y * NH;
#pragma unroll
  for (int s = 0; s <= R / 2; ++s) {
    const int k = t + s * T;
    if (k <= a.kout) {
      const double2 P = cs[padix(k)];
      const double2 Q = cs[padix((N - k) & (N - 1))];
      urw[k] = make_double2(P.x + Q.x, P.y - Q.y);
      vrw[k] = make_double2(P.y + Q.y, Q.x - P.x);
    }
  }
}

// Pass C: forward y-transforms of A and B, N = -i (kx A + ky B) / (2 N^2), the 2/3 mask
// (row j of column i is kept iff min(j, N-j) <= kcut[i]) and the stage epilogue.
template <int N, int C, int R = 16, bool KICK = false, bool RT = false>
__device__ __forceinline__ void colfwd_tile(const NltArgs& a, int tile) {
  constexpr int T = N / R;
  const int NH = col_count<N, RT>(a);
  extern __shared__ double2 smem[];
  if (tile == 0 && threadIdx.x == 0) *a.flag = 0;  // pass B of this nlt is complete
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  const int i = tile * C + c;
  const bool valid = i < NH;
  const int ic = valid ? i : NH - 1;
  if (tile * C > a.kxlim) {
    // no retained mode in this tile: N = 0
    if (valid) {
#pragma unroll
      for (int s = 0; s < R; ++s) epilogue<KICK>(a.epi, i, t + s * T, NH, czero());
    }
  } else {
    double2* sm = smem + c;
    double2* af = a.u;
    const double2* bf = a.v;
    const double scale = col_scale<N, RT>(a);
    const double kxs = __ldg(&a.fkx[ic]) * scale;
    double2 v[R];
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = valid ? af[(size_t)(t + s * T) * NH + ic] : czero();
    fft_regs<N, R, false, C>(v, sm, t, a.tw, 0);
    // keep kx*FA in place of A (the same thread re-reads it below)
    if (valid) {
#pragma unroll
      for (int s = 0; s < R; ++s)
        af[(size_t)(t + s * T) * NH + i] = make_double2(kxs * v[s].x, kxs * v[s].y);
    }
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = valid ? bf[(size_t)(t + s * T) * NH + ic] : czero();
    __syncthreads();
    fft_regs<N, R, false, C>(v, sm, t, a.tw, 0);
    if (valid) {
      const int kc = a.truncate ? __ldg(&a.kcut[i]) : N;
#pragma unroll
      for (int s = 0; s < R; ++s) {
        const int j = t + s * T;
        const double kys = __ldg(&a.fky[j]) * scale;
        const double2 fa = af[(size_t)j * NH + i];
        // N = -i (kx A + ky B): re = kx Im A + ky Im B, im = -(kx Re A + ky Re B)
        double2 nh = make_double2(fma(kys, v[s].y, fa.y), -fma(kys, v[s].x, fa.x));
        const int aj = min(j, N - j);
        if (aj > kc || (i == 0 && j == 0 && a.truncate)) nh = czero();
        epilogue<KICK>(a.epi, i, j, NH, nh);
      }
    }
  }
}

// Pass C of one Runge-Kutta stage followed by pass A of the next one on the same columns: the
// stage value written by the epilogue is re-read by the thread that wrote it. The two
// evaluations use different untruncated-input flags (next.flag != cur.flag): pass C clears
// cur.flag while pass A may raise next.flag.
template <int N, int C, int R = 16, bool RT = false>
__device__ __forceinline__ void colfwd_colinv_tile(const NltArgs& cur, const NltArgs& next, int tile) {
  colfwd_tile<N, C, R, false, RT>(cur, tile);
  __syncthreads();
  colinv_tile<N, C, R, RT>(next, tile);
}

// ---- grouped column tiles ------------------------------------------------------------------
// One column per CTA, worked on by kColGroups thread groups of T = N/R threads. The independent
// transforms of the column (u, v, q in pass A; A and B in pass C) run at the same time, one per
// group, instead of one after another: for grids whose column passes leave most SMs idle, this
// shortens the dependent chain of a CTA. Every group executes the same transform code, so every
// thread meets the same sequence of block barriers; a group with nothing to transform (pass C)
// transforms zeros.
constexpr int kColGroups = 3;

// Pass A, group g transforming field g (0: u, 1: v, 2: q). zin may alias q: every group loads
// its column before the barrier that precedes the stores.
template <int N, int R>
__device__ __forceinline__ void colinv_grp_tile(const NltArgs& a, int tile) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int i = tile;  // one column per CTA, i < NH
  double2* sm = smem + (size_t)g * padded(N);
  const double2* zin = a.zin;
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = zin[(size_t)(t + s * T) * NH + i];
  // a column beyond the 2/3 ellipse carries data only for an untruncated input; an all-zero
  // one stores zeros without a transform (see colinv_tile)
  int nz = 0;
  if (i > a.kxlim) {
#pragma unroll
    for (int s = 0; s < R; ++s) nz |= (v[s].x != 0.0) | (v[s].y != 0.0);
  }
  const bool skip = (i > a.kxlim) ? !__syncthreads_or(nz) : false;
  if (skip) {
    double2* dst = g == 0 ? a.u : g == 1 ? a.v : a.q;
#pragma unroll
    for (int s = 0; s < R; ++s) dst[(size_t)(t + s * T) * NH + i] = czero();
    return;
  }
  if (nz) atomicExch(a.flag, 1);
  const bool zb = column_zband<R>(v);
  if (g == 0) {  // u = i ky/|k|^a q  (nlt.f90:29-32)
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const int j = t + s * T;
      const double m = __ldg(&a.fky[j]) * __ldg(&a.kainv[(size_t)j * NH + i]);
      v[s] = make_double2(-m * v[s].y, m * v[s].x);
    }
  } else if (g == 1) {  // v = -i kx/|k|^a q  (nlt.f90:33-34)
    const double kx = __ldg(&a.fkx[i]);
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const int j = t + s * T;
      const double m = kx * __ldg(&a.kainv[(size_t)j * NH + i]);
      v[s] = make_double2(m * v[s].y, -m * v[s].x);
    }
  }
  fft_regs<N, R, true, 1>(v, sm, t, a.tw, 0, zb);
  __syncthreads();  // every load of zin is done before q (which may alias it) is written
  double2* dst = g == 0 ? a.u : g == 1 ? a.v : a.q;
#pragma unroll
  for (int s = 0; s < R; ++s) dst[(size_t)(t + s * T) * NH + i] = v[s];
}

// Pass C: group 0 transforms A, group 1 transforms B, group 2 zeros; group 0 hands kx*FA to
// group 1 through its exchange buffer (free once fft_regs has returned), and group 1 forms N
// and runs the epilogue.
template <int N, int R, bool KICK = false>
__device__ __forceinline__ void colfwd_grp_tile(const NltArgs& a, int tile) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  if (tile == 0 && threadIdx.x == 0) *a.flag = 0;  // pass B of this nlt is complete
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int i = tile;
  if (i > a.kxlim) {
    // no retained mode in this column: N = 0
    if (g == 0) {
#pragma unroll
      for (int s = 0; s < R; ++s) epilogue<KICK>(a.epi, i, t + s * T, NH, czero());
    }
  } else {
    double2* sm = smem + (size_t)g * padded(N);
    const double scale = 0.5 / ((double)N * (double)N);
    const double2* src = g == 0 ? a.u : a.v;
    double2 v[R];
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = g < 2 ? src[(size_t)(t + s * T) * NH + i] : czero();
    fft_regs<N, R, false, 1>(v, sm, t, a.tw, 0);
    if (g == 0) {
      const double kxs = __ldg(&a.fkx[i]) * scale;
#pragma unroll
      for (int s = 0; s < R; ++s) sm[padix(t + s * T)] = make_double2(kxs * v[s].x, kxs * v[s].y);
    }
    __syncthreads();
    if (g == 1) {
      const double2* fa = smem;  // group 0's buffer
      const int kc = a.truncate ? __ldg(&a.kcut[i]) : N;
#pragma unroll
      for (int s = 0; s < R; ++s) {
        const int j = t + s * T;
        const double kys = __ldg(&a.fky[j]) * scale;
        const double2 f = fa[padix(j)];
        // N = -i (kx A + ky B): re = kx Im A + ky Im B, im = -(kx Re A + ky Re B)
        double2 nh = make_double2(fma(kys, v[s].y, f.y), -fma(kys, v[s].x, f.x));
        const int aj = min(j, N - j);
        if (aj > kc || (i == 0 && j == 0 && a.truncate)) nh = czero();
        epilogue<KICK>(a.epi, i, j, NH, nh);
      }
    }
  }
}

// Pass B with two thread groups of T = N/R threads on one row, each with an exchange buffer
// of its own: group 0 transforms u + i v while group 1 transforms q, extended to a Hermitian
// spectrum of length N (its inverse transform is real q), so that both groups run the same
// transform from the same call site and every thread meets the same barrier instructions.
// Group 0 then forms the product and runs the forward transform; group 1 runs the same call on
// its own buffer and discards the result.
template <int N, int R>
__device__ __forceinline__ void row_grp_tile(const NltArgs& a, int tile) {
  constexpr int T = N / R, NH = N / 2 + 1, M = N / 2;
  extern __shared__ double2 smem[];
  const int g = threadIdx.x / T, t = threadIdx.x % T;
  const int y = tile;  // one row per CTA
  double2* cs = smem;               // group 0: u + i v, then the product
  double2* qs = smem + padded(N);   // group 1: q
  double2* buf = g == 0 ? cs : qs;
  const int kl = (*a.flag) ? M : a.kin;
  const double2* urow = a.u + (size_t)y * NH;
  const double2* qrow = a.q + (size_t)y * NH;
  const double2* vrow = a.v + (size_t)y * NH;
  // group 0: C[k] = U[k] + i V[k], C[N-k] = conj U[k] + i conj V[k];
  // group 1: C[k] = Q[k], C[N-k] = conj Q[k]; Im of the k=0 and N/2 values dropped
#pragma unroll
  for (int s = 0; s <= R / 2; ++s) {
    const int k = t + s * T;
    if (k <= M) {
      const double2 U = (k <= kl) ? (g == 0 ? urow[k] : qrow[k]) : czero();
      const double2 V = (g == 0 && k <= kl) ? vrow[k] : czero();
      if (k == 0 || k == M) {
        buf[padix(k)] = make_double2(U.x, V.x);
      } else {
        buf[padix(k)] = make_double2(U.x - V.y, U.y + V.x);
        buf[padix(N - k)] = make_double2(U.x + V.y, V.x - U.y);
      }
    }
  }
  __syncthreads();
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = buf[padix(t + s * T)];
  __syncthreads();
  fft_regs<N, R, true, 1>(v, buf, t, a.twr, 0, 8 * kl < 3 * N);  // both groups
  // group 0 holds u + i v, group 1 holds q (real part) at x = t + s*T
  __syncthreads();
  if (g == 1) {
#pragma unroll
    for (int s = 0; s < R; ++s) qs[padix(t + s * T)] = v[s];
  }
  if (g == 0 && a.phys_uv) {
#pragma unroll
    for (int s = 0; s < R; ++s) a.phys_uv[(size_t)y * N + t + s * T] = v[s];
  }
  __syncthreads();
  if (g == 1 && a.phys_q) {  // packed as q[2m] + i q[2m+1]
#pragma unroll
    for (int s = 0; s < R / 2; ++s) {
      const int m = t + s * T;
      a.phys_q[(size_t)y * M + m] = make_double2(qs[padix(2 * m)].x, qs[padix(2 * m + 1)].x);
    }
  }
  if (g == 0) {  // p = (u + i v) q  (produ.f90:18-19)
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const double q = qs[padix(t + s * T)].x;
      v[s] = make_double2(v[s].x * q, v[s].y * q);
    }
  }
  __syncthreads();  // every read of qs is done before group 1 reuses it as exchange buffer
  fft_regs<N, R, false, 1>(v, buf, t, a.twr, 0);  // both groups; group 1's result is unused
  __syncthreads();
  if (g == 0) {
#pragma unroll
    for (int s = 0; s < R; ++s) cs[padix(t + s * T)] = v[s];
  }
  __syncthreads();
  // A = P[k] + conj P[N-k], B = -i (P[k] - conj P[N-k]) for k <= kout, by both groups
  double2* urw = a.u + (size_t)y * NH;
  double2* vrw = a.v + (size_t)y * NH;
  for (int k = threadIdx.x; k <= a.kout; k += 2 * T) {
    const double2 P = cs[padix(k)];
    const double2 Q = cs[padix((N - k) & (N - 1))];
    urw[k] = make_double2(P.x + Q.x, P.y - Q.y);
    vrw[k] = make_double2(P.y + Q.y, Q.x - P.x);
  }
}

// Pass C of one stage and pass A of the next on the same column (see colfwd_colinv_tile).
template <int N, int R>
__device__ __forceinline__ void colfwd_colinv_grp_tile(const NltArgs& cur, const NltArgs& next, int tile) {
  colfwd_grp_tile<N, R>(cur, tile);
  __syncthreads();
  colinv_grp_tile<N, R>(next, tile);
}

// ---- field-split column tiles --------------------------------------------------------------
// One field of one column per CTA (C = 1, T = N/R threads), so that a column pass has 3 (pass A)
// or 2 (pass C) work units per column instead of one: 683 active columns at 2048^2 are 4.5 per
// SM, and the last SMs to finish would otherwise idle for up to a whole column.

// Pass A, field g of column i: unit = 3 i + g (g = 0: u, 1: v, 2: q). q must not alias zin: the
// caller passes a q buffer of its own (the three units of a column run in different CTAs).
template <int N, int R, bool RT = false>
__device__ __forceinline__ void colinv_field_tile(const NltArgs& a, int unit) {
  constexpr int T = N / R;
  const int NH = col_count<N, RT>(a);
  extern __shared__ double2 smem[];
  const int i = unit / 3, g = unit % 3, t = threadIdx.x;
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = a.zin[(size_t)(t + s * T) * NH + i];
  // beyond the 2/3 ellipse: zeros without a transform for an all-zero column, else raise the
  // untruncated-input flag (see colinv_tile)
  int nz = 0;
  if (i > a.kxlim) {
#pragma unroll
    for (int s = 0; s < R; ++s) nz |= nonzero2(v[s]);
  }
  const bool skip = (i > a.kxlim) ? !__syncthreads_or(nz) : false;
  double2* dst = g == 0 ? a.u : g == 1 ? a.v : a.q;
  if (skip) {
#pragma unroll
    for (int s = 0; s < R; ++s) dst[(size_t)(t + s * T) * NH + i] = czero();
    return;
  }
  if (nz) atomicExch(a.flag, 1);
  const bool zb = column_zband<R>(v);
  if (g == 0) {  // u = i ky/|k|^a q  (nlt.f90:29-32)
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const int j = t + s * T;
      const double m = __ldg(&a.fky[j]) * __ldg(&a.kainv[(size_t)j * NH + i]);
      v[s] = make_double2(-m * v[s].y, m * v[s].x);
    }
  } else if (g == 1) {  // v = -i kx/|k|^a q  (nlt.f90:33-34)
    const double kx = __ldg(&a.fkx[i]);
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const int j = t + s * T;
      const double m = kx * __ldg(&a.kainv[(size_t)j * NH + i]);
      v[s] = make_double2(m * v[s].y, -m * v[s].x);
    }
  }
  fft_regs<N, R, true, 1>(v, smem, t, a.tw, 0, zb);
#pragma unroll
  for (int s = 0; s < R; ++s) dst[(size_t)(t + s * T) * NH + i] = v[s];
}

// Units of the field-split pass C: two per column up to kxlim, then one per column beyond it
// (N = 0 there: the epilogue only).
__host__ __device__ inline int colfwd_split_units(int nh, int kxlim) { return 2 * (kxlim + 1) + (nh - 1 - kxlim); }

// Pass C's value at (i, j) of the split forms from the column transforms fa = scale kx A (scaled
// by the caller) and fb = B, A = F(u q), B = F(v q) (ky's factor carries the scale for B):
// N = -i (kx A + ky B), re = kx Im A + ky Im B, im = -(kx Re A + ky Re B); zero outside the 2/3
// cut (kc) and at the mean; then the stage epilogue.
template <int N, bool KICK, bool RT = false>
__device__ __forceinline__ void colfwd_store(const NltArgs& a, int i, int j, int kc, double scale, double2 fa,
                                             double2 fb) {
  const double kys = __ldg(&a.fky[j]) * scale;
  double2 nh = make_double2(fma(kys, fb.y, fa.y), -fma(kys, fb.x, fa.x));
  const int aj = min(j, N - j);
  if (aj > kc || (i == 0 && j == 0 && a.truncate)) nh = czero();
  epilogue<KICK>(a.epi, i, j, col_count<N, RT>(a), nh);
}

// Pass C, unit 2 i + g (g = 0: A, 1: B) of column i <= kxlim: the forward transform of the
// field, written back in place (kx*FA for A). The second of the column's two CTAs to finish
// (a per-column counter, no waiting) reads the other field and runs the epilogue. Its
// loads of the other CTA's column go through L2 (__ldcg) after that CTA's __threadfence.
template <int N, int R, bool KICK, bool RT = false>
__device__ __forceinline__ void colfwd_field_tile(const NltArgs& a, int unit) {
  constexpr int T = N / R;
  const int NH = col_count<N, RT>(a);
  extern __shared__ double2 smem[];
  __shared__ int last;
  const int t = threadIdx.x;
  if (unit == 0 && t == 0) *a.flag = 0;  // pass B of this nlt is complete
  const int nact = 2 * (a.kxlim + 1);
  if (unit >= nact) {
    const int i = a.kxlim + 1 + (unit - nact);
#pragma unroll
    for (int s = 0; s < R; ++s) epilogue<KICK>(a.epi, i, t + s * T, NH, czero());
    return;
  }
  const int i = unit >> 1, g = unit & 1;
  const double scale = col_scale<N, RT>(a);
  double2* own = g == 0 ? a.u : a.v;
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = own[(size_t)(t + s * T) * NH + i];
  fft_regs<N, R, false, 1>(v, smem, t, a.tw, 0);
  if (g == 0) {
    const double kxs = __ldg(&a.fkx[i]) * scale;
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = make_double2(kxs * v[s].x, kxs * v[s].y);
  }
#pragma unroll
  for (int s = 0; s < R; ++s) own[(size_t)(t + s * T) * NH + i] = v[s];
  __threadfence();
  __syncthreads();
  if (t == 0) last = atomicAdd(&a.colcnt[i], 1) == 1;
  __syncthreads();
  if (!last) return;
  if (t == 0) a.colcnt[i] = 0;  // ready for the next launch
  const double2* other = g == 0 ? a.v : a.u;
  const int kc = a.truncate ? __ldg(&a.kcut[i]) : N;
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int j = t + s * T;
    const double2 o = __ldcg(&other[(size_t)j * NH + i]);
    colfwd_store<N, KICK, RT>(a, i, j, kc, scale, g == 0 ? v[s] : o, g == 0 ? o : v[s]);
  }
}

// Pass C split by field, the column's two CTAs forming one 2-CTA cluster (unit = 2 i + g, g = 0
// transforms A = F(u q), g = 1 B = F(v q)). Each CTA leaves the half of its transformed column
// that the other CTA needs in its own shared memory; after a cluster barrier each CTA runs the
// epilogue for its half of the rows (g = 0: j < N/2), reading the other field from the partner's
// shared memory. No global round trip and no per-column counter; the epilogue work is shared.
// A second cluster barrier keeps each CTA's shared memory alive until the partner has read it.
// Columns beyond the 2/3 cut: each CTA stores the zero-input epilogue of its half.
template <int N, int R, bool KICK, bool RT = false>
__device__ __forceinline__ void colfwd_cluster_tile(const NltArgs& a, int unit) {
  constexpr int T = N / R, H = R / 2;
  const int NH = col_count<N, RT>(a);
  extern __shared__ double2 smem[];
  const int t = threadIdx.x;
  const int i = unit >> 1, g = unit & 1;
  if (unit == 0 && t == 0) *a.flag = 0;  // pass B of this nlt is complete
  if (i > a.kxlim) {  // both CTAs of the cluster take this branch: no barrier is pending
#pragma unroll
    for (int s = 0; s < H; ++s) epilogue<KICK>(a.epi, i, t + (g * H + s) * T, NH, czero());
    return;
  }
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const double scale = col_scale<N, RT>(a);
  const double2* own = g == 0 ? a.u : a.v;
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = own[(size_t)(t + s * T) * NH + i];
  fft_regs<N, R, false, 1>(v, smem, t, a.tw, 0);
  if (g == 0) {
    const double kxs = __ldg(&a.fkx[i]) * scale;
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = make_double2(kxs * v[s].x, kxs * v[s].y);
  }
  // fft_regs ends with a barrier after its last shared-memory read: the buffer is free
#pragma unroll
  for (int s = 0; s < H; ++s) {
    const int j = t + ((1 - g) * H + s) * T;
    smem[j] = v[(1 - g) * H + s];
  }
  cluster.sync();
  const double2* peer = cluster.map_shared_rank(smem, (unsigned)(g ^ 1));
  const int kc = a.truncate ? __ldg(&a.kcut[i]) : N;
#pragma unroll
  for (int s = 0; s < H; ++s) {
    const int j = t + (g * H + s) * T;
    const double2 o = peer[j];
    colfwd_store<N, KICK, RT>(a, i, j, kc, scale, g == 0 ? v[g * H + s] : o, g == 0 ? o : v[g * H + s]);
  }
  cluster.sync();
}

// ---- single-field kernels ---------------------------------------------------------------
template <int N>
__global__ void __launch_bounds__(Shape<N>::COL_THREADS, MinBlocks<N>::COL)
k_nlt_colinv(NltArgs a) {
  pdl_enter();
  colinv_tile<N, Shape<N>::COLS>(a, blockIdx.x);
}

template <int N>
__global__ void __launch_bounds__(Shape<N>::ROW_THREADS, MinBlocks<N>::ROW)
k_nlt_row(NltArgs a) {
  pdl_enter();
  row_tile<N, Shape<N>::ROWS>(a, blockIdx.x);
}

template <int N>
__global__ void __launch_bounds__(Shape<N>::COL_THREADS, MinBlocks<N>::COL)
k_nlt_colfwd(NltArgs a) {
  pdl_enter();
  colfwd_tile<N, Shape<N>::COLS, 16, true>(a, blockIdx.x);
}

template <int N>
__global__ void __launch_bounds__(Shape<N>::COL_THREADS, MinBlocks<N>::COL)
k_nlt_colfwd_inv(NltArgs cur, NltArgs next) {
  pdl_enter();
  colfwd_colinv_tile<N, Shape<N>::COLS>(cur, next, blockIdx.x);
}

// ---- launch variants of the nonlinear-term passes (picked per handle by gt_autotune) ------
// V = 0: R = 16 values per thread, Shape<N>'s tiles (best from ~1024^2 up);
// V = 1: R = 8,  one column / row per CTA;
// V = 2: R = 4,  one column / row per CTA (small grids: 4x the threads of V = 0, for the
//        latency-bound regime where a pass leaves most SMs idle);
// V = 3: R = 4,  grouped tiles: a column's transforms side by side in 3 thread groups, a row's
//        u + i v and q transforms side by side in 2;
// V = 4: R = 8,  grouped tiles;
// V = 5: 2 values per thread: the column passes one column per CTA with twice the threads of
//        V = 2 (grids whose column passes have fewer warps than the SMs have sub-partitions),
//        the row pass grouped like V = 3 (its q transform at full length, so no half-length
//        transform needs R >= 4).
// The row pass and the column passes take their variants separately (GtOp::row_variant).
template <int N, int V>
struct Var {
  static constexpr bool GROUPED = V == 3 || V == 4;           // grouped column tiles
  static constexpr bool ROW_GROUPED = V == 3 || V == 4 || V == 5;
  static constexpr int R = V == 0 ? 16 : (V == 1 || V == 4) ? 8 : 4;
  static constexpr int CR = V == 5 ? 2 : R;  // values per thread of the column passes
  static constexpr int RR = V == 5 ? 2 : R;  // values per thread of the row pass
  static constexpr int T = N / R;
  static constexpr int NH = N / 2 + 1;
  static constexpr int COLS = V == 0 ? Shape<N>::COLS : 1;
  static constexpr int ROWS = V == 0 ? Shape<N>::ROWS : 1;
  static constexpr int COL_THREADS = GROUPED ? kColGroups * T : COLS * (N / CR);
  static constexpr int ROW_THREADS = ROW_GROUPED ? 2 * (N / RR) : ROWS * T;
  static constexpr int COL_CTAS = (NH + COLS - 1) / COLS;
  static constexpr int ROW_CTAS = N / ROWS;
  static constexpr size_t COL_SMEM = (size_t)padded(N) * (GROUPED ? kColGroups : COLS) * sizeof(double2);
  // grouped rows: two length-N exchange buffers (u + i v and q)
  static constexpr size_t ROW_SMEM = ROW_GROUPED ? (size_t)2 * padded(N) * sizeof(double2)
                                             : (size_t)(padded(N) + padded(N / 2)) * ROWS * sizeof(double2);
  static constexpr bool OK = V == 0 || (V == 1 && N <= 8192) || (V >= 2 && V <= 4 && N <= 1024) ||
                              (V == 5 && N >= 32 && N <= 512);
};

// RT = true: the column count at run time (non-square grids; ungrouped variants only)
template <int N, int V, bool RT = false>
__global__ void __launch_bounds__(Var<N, V>::COL_THREADS) k_nltv_colinv(NltArgs a) {
  pdl_enter();
  if constexpr (Var<N, V>::OK && Var<N, V>::GROUPED) colinv_grp_tile<N, Var<N, V>::R>(a, blockIdx.x);
  else if constexpr (Var<N, V>::OK) colinv_tile<N, Var<N, V>::COLS, Var<N, V>::CR, RT>(a, blockIdx.x);
}
// Without a CTA count ptxas keeps the 8-value row kernels at 76-80 registers (3 CTAs per SM);
// an explicit count of 1 lets them grow to 164. GT_VROW_MINB sets a count for the 8-value rows
// from 1024 up.
#ifdef GT_VROW_MINB
#define GT_VROW_BOUNDS(N, V) __launch_bounds__(Var<N, V>::ROW_THREADS, (V == 1 && N >= 1024) ? GT_VROW_MINB : 1)
#else
#define GT_VROW_BOUNDS(N, V) __launch_bounds__(Var<N, V>::ROW_THREADS)
#endif
template <int N, int V>
__global__ void GT_VROW_BOUNDS(N, V) k_nltv_row(NltArgs a) {
  pdl_enter();
  if constexpr (Var<N, V>::OK && Var<N, V>::ROW_GROUPED) row_grp_tile<N, Var<N, V>::RR>(a, blockIdx.x);
  else if constexpr (Var<N, V>::OK) row_tile<N, Var<N, V>::ROWS, Var<N, V>::R>(a, blockIdx.x);
}
template <int N, int V, bool RT = false>
__global__ void __launch_bounds__(Var<N, V>::COL_THREADS) k_nltv_colfwd(NltArgs a) {
  pdl_enter();
  if constexpr (Var<N, V>::OK && Var<N, V>::GROUPED) colfwd_grp_tile<N, Var<N, V>::R, true>(a, blockIdx.x);
  else if constexpr (Var<N, V>::OK) colfwd_tile<N, Var<N, V>::COLS, Var<N, V>::CR, true, RT>(a, blockIdx.x);
}
template <int N, int V, bool RT = false>
__global__ void __launch_bounds__(Var<N, V>::COL_THREADS) k_nltv_colfwd_inv(NltArgs cur, NltArgs next) {
  pdl_enter();
  if constexpr (Var<N, V>::OK && Var<N, V>::GROUPED)
    colfwd_colinv_grp_tile<N, Var<N, V>::R>(cur, next, blockIdx.x);
  else if constexpr (Var<N, V>::OK)
    colfwd_colinv_tile<N, Var<N, V>::COLS, Var<N, V>::CR, RT>(cur, next, blockIdx.x);
}

// Field-split column kernels (variants with one column per CTA and no thread groups).
// At least GT_SPLIT_MINB CTAs per SM (at most GT_SPLIT_REGS registers per thread) for the 8- and
// 4-value variants: 3 and 80, as the fused kernels of those variants reach without a bound.
#ifndef GT_SPLIT_MINB
#define GT_SPLIT_MINB 3
#endif
#ifndef GT_SPLIT_REGS
#define GT_SPLIT_REGS 80
#endif
template <int N, int V>
struct SplitVar {
  static constexpr bool OK = Var<N, V>::OK && !Var<N, V>::GROUPED && Var<N, V>::COLS == 1;
  static constexpr int THREADS = N / Var<N, V>::CR;
  static constexpr int MINB = V == 0 ? MinBlocks<N>::COL : min_blocks(GT_SPLIT_MINB, THREADS, GT_SPLIT_REGS);
  static constexpr size_t SMEM = (size_t)padded(N) * sizeof(double2);
};
template <int N, int V, bool RT = false>
__global__ void __launch_bounds__(SplitVar<N, V>::THREADS, SplitVar<N, V>::MINB) k_nlt_colinv_fs(NltArgs a) {
  pdl_enter();
  if constexpr (SplitVar<N, V>::OK) colinv_field_tile<N, Var<N, V>::CR, RT>(a, blockIdx.x);
}
// KICK: the final stage with the fused forcing kick
template <int N, int V, bool KICK, bool RT = false>
__global__ void __launch_bounds__(SplitVar<N, V>::THREADS, SplitVar<N, V>::MINB) k_nlt_colfwd_fs(NltArgs a) {
  pdl_enter();
  if constexpr (SplitVar<N, V>::OK) colfwd_field_tile<N, Var<N, V>::CR, KICK, RT>(a, blockIdx.x);
}
// the same pass with the column's two CTAs as one cluster (grid 2 NH)
template <int N, int V, bool KICK, bool RT = false>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(SplitVar<N, V>::THREADS, SplitVar<N, V>::MINB)
    k_nlt_colfwd_cl(NltArgs a) {
  pdl_enter();
  if constexpr (SplitVar<N, V>::OK) colfwd_cluster_tile<N, Var<N, V>::CR, KICK, RT>(a, blockIdx.x);
}

// ---- ensemble kernels: one launch per pass for every member ------------------------------
// CTA b works on tile tiles[b] = (member, tile) of the member's field; members may differ in
// size (N = 128 ... 2048), alpha, dt and tables. Every CTA holds 2048 values of one member (C * N =
// 2048 column values, ROWS * N = 2048 row values) with the same shared memory; the tile family
// (gt_ens.cu: R = 16, 8 or 4 values per thread, 2048 / R threads) is picked per ensemble. The
// default family is 256-thread CTAs with 8 values per thread and at least 3 CTAs per SM (at most
// 85 registers per thread).
constexpr int kEnsThreads = 256;
constexpr int kEnsMinBlocks = 3;
constexpr size_t kEnsColSmem = (size_t)padded(2048) * sizeof(double2);
constexpr size_t kEnsRowSmem = (size_t)(padded(2048) + padded(1024)) * sizeof(double2);

struct EnsTile {
  int member;
  int tile;
};

// Tiles per field of each ensemble pass (C = ROWS = 2048/N columns or rows per CTA).
__host__ __device__ constexpr int ens_col_tiles(int n) { return (n / 2 + 1 + (2048 / n) - 1) / (2048 / n); }
__host__ __device__ constexpr int ens_row_tiles(int n) { return n / (2048 / n); }

// ---------------------------------------------------------------------------------------
// Standalone transforms (fft_inv.f90, fft_dir.f90) and elementwise routines.
// ---------------------------------------------------------------------------------------

// y-transform of every column; forward results are multiplied by `scale`.
template <int N, bool INV, bool RT = false>
__global__ void __launch_bounds__(Shape<N>::COL_THREADS)
k_col_fft(double2* z, const double2* __restrict__ tw, double scale, int nh) {
  using S = Shape<N>;
  constexpr int T = S::T, C = S::COLS;
  const int NH = RT ? nh : S::NH;
  extern __shared__ double2 smem[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  const int i = blockIdx.x * C + c;
  const bool valid = i < NH;
  const int ic = valid ? i : NH - 1;
  double2 v[16];
#pragma unroll
  for (int s = 0; s < 16; ++s) v[s] = valid ? z[(size_t)(t + s * T) * NH + ic] : czero();
  fft_regs<N, 16, INV, C>(v, smem + c, t, tw, 0);
  if (valid) {
#pragma unroll
    for (int s = 0; s < 16; ++s)
      z[(size_t)(t + s * T) * NH + i] = INV ? v[s] : make_double2(v[s].x * scale, v[s].y * scale);
  }
}

// Row C2R in place (NH complex -> N real + 2 zero pads), half-length packing.
template <int N>
__global__ void __launch_bounds__(Shape<N>::ROW_THREADS)
k_row_c2r(double* z, const double2* __restrict__ tw) {
  using S = Shape<N>;
  constexpr int T = S::T, NH = S::NH, M = N / 2;
  extern __shared__ double2 smem[];
  const int r = threadIdx.x / T, t = threadIdx.x % T;
  const int y = blockIdx.x * S::ROWS + r;
  double2* zs = smem + (size_t)r * padded(M);
  double2* row = reinterpret_cast<double2*>(z) + (size_t)y * NH;
  double2 h[8];
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const int k = t + s * T;
    double2 a = row[k], b = row[M - k];
    if (k == 0) { a.y = 0.0; b.y = 0.0; }
    const double2 sm_ = make_double2(a.x + b.x, a.y - b.y);
    const double2 d = make_double2(a.x - b.x, a.y + b.y);
    h[s] = pack_c2r(sm_, d, __ldg(&tw[k]));
  }
  fft_regs<M, 8, true, 1>(h, zs, t, tw, 1);
  __syncthreads();  // every thread has read its row values before the row is overwritten
#pragma unroll
  for (int s = 0; s < 8; ++s) row[t + s * T] = h[s];
  if (t == 0) row[M] = czero();
}

// Row C2R of a column-transformed field written as real(4) (N floats per row, no padding): the
// physical field of a dump (src/write.f90:29-51) without a float64 round trip through HBM.
template <int N>
__global__ void __launch_bounds__(Shape<N>::ROW_THREADS)
k_row_c2r_f32(const double* __restrict__ z, float* __restrict__ out, const double2* __restrict__ tw) {
  using S = Shape<N>;
  constexpr int T = S::T, NH = S::NH, M = N / 2;
  extern __shared__ double2 smem[];
  const int r = threadIdx.x / T, t = threadIdx.x % T;
  const int y = blockIdx.x * S::ROWS + r;
  double2* zs = smem + (size_t)r * padded(M);
  const double2* row = reinterpret_cast<const double2*>(z) + (size_t)y * NH;
  double2 h[8];
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const int k = t + s * T;
    double2 a = row[k], b = row[M - k];
    if (k == 0) { a.y = 0.0; b.y = 0.0; }
    const double2 sm_ = make_double2(a.x + b.x, a.y - b.y);
    const double2 d = make_double2(a.x - b.x, a.y + b.y);
    h[s] = pack_c2r(sm_, d, __ldg(&tw[k]));
  }
  fft_regs<M, 8, true, 1>(h, zs, t, tw, 1);
  float2* orow = reinterpret_cast<float2*>(out) + (size_t)y * M;
#pragma unroll
  for (int s = 0; s < 8; ++s) orow[t + s * T] = make_float2((float)h[s].x, (float)h[s].y);
}

// Row R2C of a real(4) record (src/read.f90:3-27 widens it to real(8) with zero padding; the
// row transform of fft_dir follows): in[y*N + x] float -> z row y, NH complex values.
template <int N>
__global__ void __launch_bounds__(Shape<N>::ROW_THREADS)
k_row_r2c_f32(const float* __restrict__ in, double* __restrict__ z, const double2* __restrict__ tw) {
  using S = Shape<N>;
  constexpr int T = S::T, NH = S::NH, M = N / 2;
  extern __shared__ double2 smem[];
  const int r = threadIdx.x / T, t = threadIdx.x % T;
  const int y = blockIdx.x * S::ROWS + r;
  double2* zs = smem + (size_t)r * padded(M);
  const float2* irow = reinterpret_cast<const float2*>(in) + (size_t)y * M;
  double2* row = reinterpret_cast<double2*>(z) + (size_t)y * NH;
  double2 h[8];
#pragma unroll
  for (int s = 0; s < 8; ++s) {  // z[m] = x[2m] + i x[2m+1], widened exactly
    const float2 w = irow[t + s * T];
    h[s] = make_double2((double)w.x, (double)w.y);
  }
  fft_regs<M, 8, false, 1>(h, zs, t, tw, 1);
  __syncthreads();
#pragma unroll
  for (int s = 0; s < 8; ++s) zs[padix(t + s * T)] = h[s];
  __syncthreads();
#pragma unroll
  for (int s = 0; s <= 8; ++s) {
    const int k = t + s * T;
    if (k <= M) {
      const double2 a = zs[padix(k & (M - 1))];
      const double2 b = zs[padix((M - k) & (M - 1))];
      const double2 sm_ = make_double2(a.x + b.x, a.y - b.y);
      const double2 d = make_double2(a.x - b.x, a.y + b.y);
      const double2 tt = twmul<false>(d, __ldg(&tw[k]));
      row[k] = make_double2(0.5 * (sm_.x + tt.y), 0.5 * (sm_.y - tt.x));
    }
  }
}

// Row R2C in place (N real -> NH complex), half-length packing.
template <int N>
__global__ void __launch_bounds__(Shape<N>::ROW_THREADS)
k_row_r2c(double* z, const double2* __restrict__ tw) {
  using S = Shape<N>;
  constexpr int T = S::T, NH = S::NH, M = N / 2;
  extern __shared__ double2 smem[];
  const int r = threadIdx.x / T, t = threadIdx.x % T;
  const int y = blockIdx.x * S::ROWS + r;
  double2* zs = smem + (size_t)r * padded(M);
  double2* row = reinterpret_cast<double2*>(z) + (size_t)y * NH;
  double2 h[8];
#pragma unroll
  for (int s = 0; s < 8; ++s) h[s] = row[t + s * T];  // z[m] = x[2m] + i x[2m+1]
  fft_regs<M, 8, false, 1>(h, zs, t, tw, 1);
  __syncthreads();
#pragma unroll
  for (int s = 0; s < 8; ++s) zs[padix(t + s * T)] = h[s];
  __syncthreads();
  // X[k] = 1/2 (Z[k] + conj Z[M-k]) - i/2 W^k (Z[k] - conj Z[M-k]), k in [0, M]
#pragma unroll
  for (int s = 0; s <= 8; ++s) {
    const int k = t + s * T;
    if (k <= M) {
      const double2 a = zs[padix(k & (M - 1))];
      const double2 b = zs[padix((M - k) & (M - 1))];
      const double2 sm_ = make_double2(a.x + b.x, a.y - b.y);
      const double2 d = make_double2(a.x - b.x, a.y + b.y);
      const double2 tt = twmul<false>(d, __ldg(&tw[k]));
      row[k] = make_double2(0.5 * (sm_.x + tt.y), 0.5 * (sm_.y - tt.x));
    }
  }
}

}  // namespace gt
