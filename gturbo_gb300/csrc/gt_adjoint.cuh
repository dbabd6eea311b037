// gt_adjoint.cuh -- tangent-linear and discrete adjoint of the nonlinear term and of the Lawson
// RK2 and RK4 steps (no counterpart in the reference). Same three-pass structure and FFT engine as
// the forward passes; N <= 4096 (the row passes keep 3 length-N rows in shared memory).
//
// Notation: F(q) = T o R[-i kx (u q) - i ky (v q)] with q, u, v = C2R(q^), C2R(Mu q^), C2R(Mv q^),
// Mu = i ky/|k|^a, Mv = -i kx/|k|^a, R = D2Z/N^2 (normalised forward) and T the 2/3 mask.
// The state space is the stored half-spectrum with the real inner product
// <a, b> = sum Re(conj(a) b); there C2R^T = c o D2Z (c = 2 on interior columns, 1 on the kx=0
// and Nyquist columns) and R^T = C2R(w o .)/N^2 (w = 1/2 interior, 1 on those two columns), so
//   dF(q; dq)   = T o R[-i kx (du q + u dq) - i ky (dv q + v dq)]
//   dF(q)^T l   = c o D2Z[u a + v b] + conj(Mu) c o D2Z[q a] + conj(Mv) c o D2Z[q b],
//                 a, b = C2R(w o i kx T l)/N^2, C2R(w o i ky T l)/N^2.
#pragma once

#include "gt_kernels.cuh"

namespace gt {

// ---------------------------------------------------------------------------------------
// Tangent-linear: the forward nonlinear term and its derivative in one pass sequence.
// ---------------------------------------------------------------------------------------
enum TlmMode : int {
  TLM_STAGE_A = 0,  // w = P0 e (z + dt/2 N),      dw = P0 e (dz + dt/2 dN)
  TLM_STAGE_B = 1,  // z = P0 e (e z + dt N),       dz = P0 e (e dz + dt dN)   (in place)
  TLM_PLAIN = 2,    // N and dN left in u and du (the RK4 stages update elementwise)
};

struct TlmArgs {
  int n;
  const double2* x;   // stage input (state)
  const double2* dx;  // stage input (tangent)
  double2 *q, *u, *v, *dq, *du, *dv;  // scratch; A, B, dA, dB leave in u, v, du, dv
  const double* kainv;
  const double* fkx;
  const double* fky;
  const int* kcut;
  const double2* tw;
  int truncate;
  int mode;
  double2* z;         // step-start state (read; written by stage B)
  double2* dz;        // step-start tangent (read; written by stage B)
  double2* w;         // stage A outputs
  double2* dw;
  const double* emk;
  const double* emkx;
  const double* emky;
  int split;
  double dt, dt2;
  int* colcnt;        // per-column counters of the field-split tangent pass C (NH ints, zero)
};

__device__ __forceinline__ double stage_e(const double* emk, const double* emkx, const double* emky,
                                          int split, int i, int j, int NH) {
  return split ? __ldg(&emkx[i]) * __ldg(&emky[j]) : __ldg(&emk[(size_t)j * NH + i]);
}

template <int N, int C, int R = 16>
__device__ __forceinline__ void tlm_colinv_tile(const TlmArgs& a, int tile) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  const int i = tile * C + c;
  const bool valid = i < NH;
  const int ic = valid ? i : NH - 1;
  double2* sm = smem + c;
  const double kx = __ldg(&a.fkx[ic]);
  double2 v[R];
  for (int f = 0; f < 6; ++f) {
    const double2* src = f < 3 ? a.x : a.dx;
    double2* dst = f == 0 ? a.q : f == 1 ? a.u : f == 2 ? a.v : f == 3 ? a.dq : f == 4 ? a.du : a.dv;
    const int kind = f % 3;  // 0: q, 1: Mu q, 2: Mv q
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const int j = t + s * T;
      const size_t o = (size_t)j * NH + ic;
      const double2 q = valid ? src[o] : czero();
      if (kind == 0) {
        v[s] = q;
      } else if (kind == 1) {
        const double m = __ldg(&a.fky[j]) * __ldg(&a.kainv[o]);
        v[s] = make_double2(-m * q.y, m * q.x);
      } else {
        const double m = kx * __ldg(&a.kainv[o]);
        v[s] = make_double2(m * q.y, -m * q.x);
      }
    }
    __syncthreads();
    fft_regs<N, R, true, C>(v, sm, t, a.tw, 0);
    if (valid) {
#pragma unroll
      for (int s = 0; s < R; ++s) dst[(size_t)(t + s * T) * NH + i] = v[s];
    }
  }
}

// X + iY as one complex spectrum of length N from two half spectra (Im at k=0, N/2 dropped)
template <int N, int R = 16>
__device__ __forceinline__ void pair_spectrum(double2* cs, const double2* xrow, const double2* yrow, int t,
                                              int kl = N / 2) {
  constexpr int T = N / R, M = N / 2;
#pragma unroll
  for (int s = 0; s <= R / 2; ++s) {
    const int k = t + s * T;
    if (k <= M) {
      const double2 X = (k <= kl) ? xrow[k] : czero();
      const double2 Y = (k <= kl) ? yrow[k] : czero();
      if (k == 0 || k == M) {
        cs[padix(k)] = make_double2(X.x, Y.x);
      } else {
        cs[padix(k)] = make_double2(X.x - Y.y, X.y + Y.x);
        cs[padix(N - k)] = make_double2(X.x + Y.y, Y.x - X.y);
      }
    }
  }
}

// split P (length N, in smem) into 2 FFT(Re p)[k] -> xrow, 2 FFT(Im p)[k] -> yrow, k <= N/2
template <int N, int R = 16>
__device__ __forceinline__ void split_spectrum(const double2* cs, double2* xrow, double2* yrow, int t) {
  constexpr int T = N / R, M = N / 2;
#pragma unroll
  for (int s = 0; s <= R / 2; ++s) {
    const int k = t + s * T;
    if (k <= M) {
      const double2 P = cs[padix(k)];
      const double2 Q = cs[padix((N - k) & (N - 1))];
      xrow[k] = make_double2(P.x + Q.x, P.y - Q.y);
      yrow[k] = make_double2(P.y + Q.y, Q.x - P.x);
    }
  }
}

template <int N, int ROWS, int R = 16>
__device__ __forceinline__ void tlm_row_tile(const TlmArgs& a, int tile) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  const int r = threadIdx.x / T, t = threadIdx.x % T;
  const int y = tile * ROWS + r;
  double2* c1 = smem + (size_t)r * 3 * padded(N);
  double2* c2 = c1 + padded(N);
  double2* c3 = c2 + padded(N);
  const size_t ro = (size_t)y * NH;
  pair_spectrum<N, R>(c1, a.u + ro, a.v + ro, t);    // u + i v
  pair_spectrum<N, R>(c2, a.du + ro, a.dv + ro, t);  // du + i dv
  pair_spectrum<N, R>(c3, a.q + ro, a.dq + ro, t);   // q + i dq
  __syncthreads();
  double2 v[R];
  double2* bufs[3] = {c1, c2, c3};
  for (int b = 0; b < 3; ++b) {
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = bufs[b][padix(t + s * T)];
    __syncthreads();
    fft_regs<N, R, true, 1>(v, bufs[b], t, a.tw, 0);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R; ++s) bufs[b][padix(t + s * T)] = v[s];
  }
  __syncthreads();
  // products: p = (u + i v) q, dp = (du + i dv) q + (u + i v) dq
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int x = padix(t + s * T);
    const double2 uv = c1[x], duv = c2[x], qq = c3[x];
    c1[x] = make_double2(uv.x * qq.x, uv.y * qq.x);
    c2[x] = make_double2(fma(duv.x, qq.x, uv.x * qq.y), fma(duv.y, qq.x, uv.y * qq.y));
  }
  __syncthreads();
  for (int b = 0; b < 2; ++b) {
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = bufs[b][padix(t + s * T)];
    __syncthreads();
    fft_regs<N, R, false, 1>(v, bufs[b], t, a.tw, 0);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R; ++s) bufs[b][padix(t + s * T)] = v[s];
  }
  __syncthreads();
  split_spectrum<N, R>(c1, a.u + ro, a.v + ro, t);
  split_spectrum<N, R>(c2, a.du + ro, a.dv + ro, t);
}

template <int N, int C, int R = 16>
__device__ __forceinline__ void tlm_colfwd_tile(const TlmArgs& a, int tile) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  const int i = tile * C + c;
  const bool valid = i < NH;
  const int ic = valid ? i : NH - 1;
  double2* sm = smem + c;
  const double scale = 0.5 / ((double)N * (double)N);
  const double kxs = __ldg(&a.fkx[ic]) * scale;
  const int kc = a.truncate ? (valid ? __ldg(&a.kcut[i]) : -1) : N;
  double2 v[R];
  for (int pr = 0; pr < 2; ++pr) {
    double2* af = pr == 0 ? a.u : a.du;
    const double2* bf = pr == 0 ? a.v : a.dv;
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = valid ? af[(size_t)(t + s * T) * NH + ic] : czero();
    __syncthreads();
    fft_regs<N, R, false, C>(v, sm, t, a.tw, 0);
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
#pragma unroll
      for (int s = 0; s < R; ++s) {
        const int j = t + s * T;
        const size_t o = (size_t)j * NH + i;
        const double kys = __ldg(&a.fky[j]) * scale;
        const double2 fa = af[o];
        double2 nh = make_double2(fma(kys, v[s].y, fa.y), -fma(kys, v[s].x, fa.x));
        if (min(j, N - j) > kc || (i == 0 && j == 0 && a.truncate)) nh = czero();
        af[o] = nh;  // N (pr = 0) or dN (pr = 1) in place of A / dA
      }
    }
  }
  if (!valid || a.mode == TLM_PLAIN) return;
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int j = t + s * T;
    const size_t o = (size_t)j * NH + i;
    const double e = stage_e(a.emk, a.emkx, a.emky, a.split, i, j, NH);
    const bool origin = (i == 0 && j == 0);
    const double2 nh = a.u[o], dn = a.du[o];
    const double2 z = a.z[o], dz = a.dz[o];
    if (a.mode == TLM_STAGE_A) {
      a.w[o] = origin ? czero() : make_double2(e * (z.x + a.dt2 * nh.x), e * (z.y + a.dt2 * nh.y));
      a.dw[o] = origin ? czero() : make_double2(e * (dz.x + a.dt2 * dn.x), e * (dz.y + a.dt2 * dn.y));
    } else {
      a.z[o] = origin ? czero() : make_double2(e * (e * z.x + a.dt * nh.x), e * (e * z.y + a.dt * nh.y));
      a.dz[o] = origin ? czero() : make_double2(e * (e * dz.x + a.dt * dn.x), e * (e * dz.y + a.dt * dn.y));
    }
  }
}

// ---------------------------------------------------------------------------------------
// Adjoint of the RK2 step, in two halves (each one transposed nonlinear term):
//   ADJ_STAGE_B: input lin = l' (gradient after the step), linearisation point x = w:
//       lw  = dF(w)^T (dt e P0 l')
//       lam = e e P0 l' + e P0 lw          rho = dt/2 e P0 lw
//   ADJ_STAGE_A: input lin = rho, linearisation point x = z:
//       lam += dF(z)^T rho
// The RK4 adjoint combines plain transposed terms with elementwise updates:
//   ADJ_PLAIN:   lam = dF(x)^T lin
// ---------------------------------------------------------------------------------------
enum AdjMode : int {
  ADJ_STAGE_B = 0,
  ADJ_STAGE_A = 1,
  ADJ_PLAIN = 2,
};

struct AdjArgs {
  int n;
  int kxlim;           // last column with a retained mode (N/2 without dealiasing)
  const double2* x;    // linearisation point
  const double2* lin;  // adjoint input (l' or rho)
  // Optional: the physical u + i v and packed q at x, as pass B of the forward evaluation at x
  // stored them (NltArgs::phys_uv / phys_q). Given them, pass A transforms only the adjoint
  // inputs a, b (whose columns beyond kxlim are zero after the 2/3 mask) and pass B skips the
  // three inverse transforms of x.
  const double2* phys_uv;
  const double2* phys_q;
  double2 *q, *u, *v, *a, *b;  // scratch; S1, S2, S3 leave in q, u, v
  const double* kainv;
  const double* fkx;
  const double* fky;
  const int* kcut;
  const double2* tw;
  int truncate;
  int mode;
  double2* lam;        // output / accumulator
  double2* rho;        // ADJ_STAGE_B second output
  const double* emk;
  const double* emkx;
  const double* emky;
  int split;
  double dt, dt2;
  int* colcnt;         // per-column counters of the field-split transposed pass C (NH ints, zero)
};

template <int N, int C, int R = 16>
__device__ __forceinline__ void adj_colinv_tile(const AdjArgs& a, int tile) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  const int i = tile * C + c;
  const bool valid = i < NH;
  const int ic = valid ? i : NH - 1;
  double2* sm = smem + c;
  const double kx = __ldg(&a.fkx[ic]);
  const int kc = a.truncate ? __ldg(&a.kcut[ic]) : N;
  const double wcol = (ic == 0 || ic == NH - 1) ? 1.0 : 0.5;
  double2 v[R];
  const bool phys = a.phys_uv != nullptr;
  if (phys && tile * C > a.kxlim) return;  // a, b are zero there; pass B reads them as zero
  for (int f = phys ? 3 : 0; f < 5; ++f) {
    double2* dst = f == 0 ? a.q : f == 1 ? a.u : f == 2 ? a.v : f == 3 ? a.a : a.b;
#pragma unroll
    for (int s = 0; s < R; ++s) {
      const int j = t + s * T;
      const size_t o = (size_t)j * NH + ic;
      if (f < 3) {
        const double2 q = valid ? a.x[o] : czero();
        if (f == 0) {
          v[s] = q;
        } else if (f == 1) {
          const double m = __ldg(&a.fky[j]) * __ldg(&a.kainv[o]);
          v[s] = make_double2(-m * q.y, m * q.x);
        } else {
          const double m = kx * __ldg(&a.kainv[o]);
          v[s] = make_double2(m * q.y, -m * q.x);
        }
      } else {
        double2 l = valid ? a.lin[o] : czero();
        if (a.mode == ADJ_STAGE_B) {
          const double e = stage_e(a.emk, a.emkx, a.emky, a.split, ic, j, NH) * a.dt;
          l = (ic == 0 && j == 0) ? czero() : make_double2(e * l.x, e * l.y);
        }
        if (min(j, N - j) > kc || (ic == 0 && j == 0 && a.truncate)) l = czero();
        // w o (i k) l
        const double k = (f == 3 ? kx : __ldg(&a.fky[j])) * wcol;
        v[s] = make_double2(-k * l.y, k * l.x);
      }
    }
    __syncthreads();
    fft_regs<N, R, true, C>(v, sm, t, a.tw, 0);
    if (valid) {
#pragma unroll
      for (int s = 0; s < R; ++s) dst[(size_t)(t + s * T) * NH + i] = v[s];
    }
  }
}

template <int N, int ROWS, int R = 16>
__device__ __forceinline__ void adj_row_tile(const AdjArgs& a, int tile) {
  constexpr int T = N / R, NH = N / 2 + 1, M = N / 2;
  extern __shared__ double2 smem[];
  const int r = threadIdx.x / T, t = threadIdx.x % T;
  const int y = tile * ROWS + r;
  double2* c1 = smem + (size_t)r * (2 * padded(N) + padded(M));
  double2* c2 = c1 + padded(N);
  double2* zs = c2 + padded(N);
  const size_t ro = (size_t)y * NH;
  double2 v[R];
  double2* bufs[2] = {c1, c2};
  if (a.phys_uv) {
    // u + i v and the packed q at x, stored by the forward evaluation's pass B; a + i b
    // (zero beyond column kxlim) is the only row to transform
    const double2* uvrow = a.phys_uv + (size_t)y * N;
    const double2* pqrow = a.phys_q + (size_t)y * M;
#pragma unroll
    for (int s = 0; s < R; ++s) c1[padix(t + s * T)] = uvrow[t + s * T];
#pragma unroll
    for (int s = 0; s < R / 2; ++s) zs[padix(t + s * T)] = pqrow[t + s * T];
    pair_spectrum<N, R>(c2, a.a + ro, a.b + ro, t, a.kxlim);  // a + i b
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = c2[padix(t + s * T)];
    __syncthreads();
    fft_regs<N, R, true, 1>(v, c2, t, a.tw, 0);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R; ++s) c2[padix(t + s * T)] = v[s];
  } else {
    pair_spectrum<N, R>(c1, a.u + ro, a.v + ro, t);  // u + i v
    pair_spectrum<N, R>(c2, a.a + ro, a.b + ro, t);  // a + i b
    const double2* qrow = a.q + ro;
#pragma unroll
    for (int s = 0; s < R / 2; ++s) {  // half-length C2R packing of q
      const int k = t + s * T;
      double2 p = qrow[k], b = qrow[M - k];
      if (k == 0) { p.y = 0.0; b.y = 0.0; }
      const double2 sm_ = make_double2(p.x + b.x, p.y - b.y);
      const double2 d = make_double2(p.x - b.x, p.y + b.y);
      zs[padix(k)] = pack_c2r(sm_, d, __ldg(&a.tw[k]));
    }
    __syncthreads();
    {
      double2 h[R / 2];
#pragma unroll
      for (int s = 0; s < R / 2; ++s) h[s] = zs[padix(t + s * T)];
      __syncthreads();
      fft_regs<M, R / 2, true, 1>(h, zs, t, a.tw, 1);
      __syncthreads();
#pragma unroll
      for (int s = 0; s < R / 2; ++s) zs[padix(t + s * T)] = h[s];
    }
    for (int b = 0; b < 2; ++b) {
#pragma unroll
      for (int s = 0; s < R; ++s) v[s] = bufs[b][padix(t + s * T)];
      __syncthreads();
      fft_regs<N, R, true, 1>(v, bufs[b], t, a.tw, 0);
      __syncthreads();
#pragma unroll
      for (int s = 0; s < R; ++s) bufs[b][padix(t + s * T)] = v[s];
    }
  }
  __syncthreads();
  // s1 = u a + v b (into zs, as packed pairs), s2 + i s3 = q (a + i b) (into c2); a, b / N^2
  const double inv = 1.0 / ((double)N * (double)N);
  double s1v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int x = t + s * T;
    const double2 uv = c1[padix(x)];
    const double2 ab = c2[padix(x)];
    const double2 zq = zs[padix(x >> 1)];
    const double q = (x & 1) ? zq.y : zq.x;
    const double ax = ab.x * inv, bx = ab.y * inv;
    s1v[s] = fma(uv.x, ax, uv.y * bx);
    c2[padix(x)] = make_double2(q * ax, q * bx);
  }
  __syncthreads();
  // repack s1 as z[m] = s1[2m] + i s1[2m+1] in zs (x even -> .x, odd -> .y)
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int x = t + s * T;
    double* zd = reinterpret_cast<double*>(zs + padix(x >> 1));
    zd[x & 1] = s1v[s];
  }
  __syncthreads();
  // forward transforms: s2 + i s3 (length N), s1 (half length)
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = c2[padix(t + s * T)];
  __syncthreads();
  fft_regs<N, R, false, 1>(v, c2, t, a.tw, 0);
  __syncthreads();
#pragma unroll
  for (int s = 0; s < R; ++s) c2[padix(t + s * T)] = v[s];
  {
    double2 h[R / 2];
#pragma unroll
    for (int s = 0; s < R / 2; ++s) h[s] = zs[padix(t + s * T)];
    __syncthreads();
    fft_regs<M, R / 2, false, 1>(h, zs, t, a.tw, 1);
    __syncthreads();
#pragma unroll
    for (int s = 0; s < R / 2; ++s) zs[padix(t + s * T)] = h[s];
  }
  __syncthreads();
  split_spectrum<N, R>(c2, a.u + ro, a.v + ro, t);  // 2 FFT(s2), 2 FFT(s3)
  // 2 FFT(s1)[k] = (Z[k] + conj Z[M-k]) - i W^k (Z[k] - conj Z[M-k]), k in [0, M]
  double2* s1row = a.q + ro;
#pragma unroll
  for (int s = 0; s <= R / 2; ++s) {
    const int k = t + s * T;
    if (k <= M) {
      const double2 p = zs[padix(k & (M - 1))];
      const double2 b = zs[padix((M - k) & (M - 1))];
      const double2 sm_ = make_double2(p.x + b.x, p.y - b.y);
      const double2 d = make_double2(p.x - b.x, p.y + b.y);
      const double2 tt = twmul<false>(d, __ldg(&a.tw[k]));
      s1row[k] = make_double2(sm_.x + tt.y, sm_.y - tt.x);
    }
  }
}

template <int N, int C, int R = 16>
__device__ __forceinline__ void adj_colfwd_tile(const AdjArgs& a, int tile) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  const int c = threadIdx.x % C, t = threadIdx.x / C;
  const int i = tile * C + c;
  const bool valid = i < NH;
  const int ic = valid ? i : NH - 1;
  double2* sm = smem + c;
  const double kx = __ldg(&a.fkx[ic]);
  // c o (.)/2: the row pass delivered 2 FFT(s); c = 1 on kx=0 and Nyquist, 2 inside
  const double cw = (ic == 0 || ic == NH - 1) ? 0.5 : 1.0;
  double2 v[R];
  for (int f = 0; f < 3; ++f) {
    const double2* src = f == 0 ? a.q : f == 1 ? a.u : a.v;
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = valid ? src[(size_t)(t + s * T) * NH + ic] : czero();
    __syncthreads();
    fft_regs<N, R, false, C>(v, sm, t, a.tw, 0);
    if (valid) {
#pragma unroll
      for (int s = 0; s < R; ++s) {
        const int j = t + s * T;
        const size_t o = (size_t)j * NH + i;
        double2 acc;
        if (f == 0) {
          acc = make_double2(cw * v[s].x, cw * v[s].y);
        } else {
          // conj(Mu) = -i ky/|k|^a, conj(Mv) = +i kx/|k|^a
          const double m = (f == 1 ? -__ldg(&a.fky[j]) : kx) * __ldg(&a.kainv[o]) * cw;
          const double2 prev = a.q[o];
          acc = make_double2(fma(-m, v[s].y, prev.x), fma(m, v[s].x, prev.y));
        }
        a.q[o] = acc;
      }
    }
  }
  if (!valid) return;
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int j = t + s * T;
    const size_t o = (size_t)j * NH + i;
    const double2 g = a.q[o];
    if (a.mode == ADJ_STAGE_B) {
      const double e = stage_e(a.emk, a.emkx, a.emky, a.split, i, j, NH);
      const bool origin = (i == 0 && j == 0);
      const double2 l = a.lin[o];
      a.lam[o] = origin ? czero() : make_double2(e * (e * l.x + g.x), e * (e * l.y + g.y));
      a.rho[o] = origin ? czero() : make_double2(a.dt2 * e * g.x, a.dt2 * e * g.y);
    } else if (a.mode == ADJ_PLAIN) {
      a.lam[o] = g;
    } else {
      const double2 l = a.lam[o];
      a.lam[o] = make_double2(l.x + g.x, l.y + g.y);
    }
  }
}

// ---- field-split tangent-linear column tiles (one field of one column per CTA, C = 1) ------------

// Tangent pass A, field f of column i (unit 6 i + f): q, Mu q, Mv q of x (f = 0, 1, 2) and of dx.
template <int N, int R>
__device__ __forceinline__ void tlm_colinv_field_tile(const TlmArgs& a, int unit) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  const int i = unit / 6, f = unit % 6, t = threadIdx.x;
  const double kx = __ldg(&a.fkx[i]);
  const double2* src = f < 3 ? a.x : a.dx;
  double2* dst = f == 0 ? a.q : f == 1 ? a.u : f == 2 ? a.v : f == 3 ? a.dq : f == 4 ? a.du : a.dv;
  const int kind = f % 3;  // 0: q, 1: Mu q, 2: Mv q
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int j = t + s * T;
    const size_t o = (size_t)j * NH + i;
    const double2 q = src[o];
    if (kind == 0) {
      v[s] = q;
    } else if (kind == 1) {
      const double m = __ldg(&a.fky[j]) * __ldg(&a.kainv[o]);
      v[s] = make_double2(-m * q.y, m * q.x);
    } else {
      const double m = kx * __ldg(&a.kainv[o]);
      v[s] = make_double2(m * q.y, -m * q.x);
    }
  }
  fft_regs<N, R, true, 1>(v, smem, t, a.tw, 0);
#pragma unroll
  for (int s = 0; s < R; ++s) dst[(size_t)(t + s * T) * NH + i] = v[s];
}

// Tangent pass C, field f of column i (unit 4 i + f; f = 0, 1, 2, 3: A, B, dA, dB): the forward
// transform written back in place (kx-scaled for A and dA). The fourth of the column's CTAs to
// finish (a per-column counter, no waiting) forms N and dN as tlm_colfwd_tile does and runs the
// stage update.
template <int N, int R>
__device__ __forceinline__ void tlm_colfwd_field_tile(const TlmArgs& a, int unit) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  __shared__ int last;
  const int i = unit / 4, f = unit % 4, t = threadIdx.x;
  const double scale = 0.5 / ((double)N * (double)N);
  double2* own = f == 0 ? a.u : f == 1 ? a.v : f == 2 ? a.du : a.dv;
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = own[(size_t)(t + s * T) * NH + i];
  fft_regs<N, R, false, 1>(v, smem, t, a.tw, 0);
  if ((f & 1) == 0) {
    const double kxs = __ldg(&a.fkx[i]) * scale;
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = make_double2(kxs * v[s].x, kxs * v[s].y);
  }
#pragma unroll
  for (int s = 0; s < R; ++s) own[(size_t)(t + s * T) * NH + i] = v[s];
  __threadfence();
  __syncthreads();
  if (t == 0) last = atomicAdd(&a.colcnt[i], 1) == 3;
  __syncthreads();
  if (!last) return;
  if (t == 0) a.colcnt[i] = 0;  // ready for the next launch
  const int kc = a.truncate ? __ldg(&a.kcut[i]) : N;
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int j = t + s * T;
    const size_t o = (size_t)j * NH + i;
    const double2 fa = f == 0 ? v[s] : __ldcg(&a.u[o]);
    const double2 fb = f == 1 ? v[s] : __ldcg(&a.v[o]);
    const double2 dfa = f == 2 ? v[s] : __ldcg(&a.du[o]);
    const double2 dfb = f == 3 ? v[s] : __ldcg(&a.dv[o]);
    const double kys = __ldg(&a.fky[j]) * scale;
    double2 nh = make_double2(fma(kys, fb.y, fa.y), -fma(kys, fb.x, fa.x));
    double2 dn = make_double2(fma(kys, dfb.y, dfa.y), -fma(kys, dfb.x, dfa.x));
    if (min(j, N - j) > kc || (i == 0 && j == 0 && a.truncate)) {
      nh = czero();
      dn = czero();
    }
    a.u[o] = nh;   // N and dN in place of A and dA (TLM_PLAIN reads them there)
    a.du[o] = dn;
    if (a.mode == TLM_PLAIN) continue;
    const double e = stage_e(a.emk, a.emkx, a.emky, a.split, i, j, NH);
    const bool origin = (i == 0 && j == 0);
    const double2 z = a.z[o], dz = a.dz[o];
    if (a.mode == TLM_STAGE_A) {
      a.w[o] = origin ? czero() : make_double2(e * (z.x + a.dt2 * nh.x), e * (z.y + a.dt2 * nh.y));
      a.dw[o] = origin ? czero() : make_double2(e * (dz.x + a.dt2 * dn.x), e * (dz.y + a.dt2 * dn.y));
    } else {
      a.z[o] = origin ? czero() : make_double2(e * (e * z.x + a.dt * nh.x), e * (e * z.y + a.dt * nh.y));
      a.dz[o] = origin ? czero() : make_double2(e * (e * dz.x + a.dt * dn.x), e * (e * dz.y + a.dt * dn.y));
    }
  }
}

// Tangent pass C with the column's four CTAs (A, B, dA, dB) as one 4-CTA cluster. Each CTA keeps
// its transformed field (kx-scaled for A and dA) in its own shared memory for the rows the others
// combine; after a cluster barrier CTA f forms N and dN for the rows j = t + s T with s = f, f + 4,
// ..., reading the other three fields from the partners' shared memory, and runs the stage update
// there (the per-value arithmetic of tlm_colfwd_field_tile). A second barrier keeps the shared
// memory alive until the partners have read it. The transformed B and dB are not written back:
// nothing reads them after this pass.
template <int N, int R>
__device__ __forceinline__ void tlm_colfwd_cluster_tile(const TlmArgs& a, int unit) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  const int i = unit / 4, f = unit % 4, t = threadIdx.x;
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const double scale = 0.5 / ((double)N * (double)N);
  const double2* own = f == 0 ? a.u : f == 1 ? a.v : f == 2 ? a.du : a.dv;
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = own[(size_t)(t + s * T) * NH + i];
  fft_regs<N, R, false, 1>(v, smem, t, a.tw, 0);
  if ((f & 1) == 0) {
    const double kxs = __ldg(&a.fkx[i]) * scale;
#pragma unroll
    for (int s = 0; s < R; ++s) v[s] = make_double2(kxs * v[s].x, kxs * v[s].y);
  }
  // fft_regs ends with a barrier after its last shared-memory read: the buffer is free
#pragma unroll
  for (int s = 0; s < R; ++s)
    if (s % 4 != f) smem[t + s * T] = v[s];
  cluster.sync();
  const double2* pa = cluster.map_shared_rank(smem, 0u);
  const double2* pb = cluster.map_shared_rank(smem, 1u);
  const double2* pda = cluster.map_shared_rank(smem, 2u);
  const double2* pdb = cluster.map_shared_rank(smem, 3u);
  const int kc = a.truncate ? __ldg(&a.kcut[i]) : N;
#pragma unroll
  for (int s = 0; s < R; ++s) {
    if (s % 4 != f) continue;
    const int j = t + s * T;
    const size_t o = (size_t)j * NH + i;
    const double2 fa = f == 0 ? v[s] : pa[j];
    const double2 fb = f == 1 ? v[s] : pb[j];
    const double2 dfa = f == 2 ? v[s] : pda[j];
    const double2 dfb = f == 3 ? v[s] : pdb[j];
    const double kys = __ldg(&a.fky[j]) * scale;
    double2 nh = make_double2(fma(kys, fb.y, fa.y), -fma(kys, fb.x, fa.x));
    double2 dn = make_double2(fma(kys, dfb.y, dfa.y), -fma(kys, dfb.x, dfa.x));
    if (min(j, N - j) > kc || (i == 0 && j == 0 && a.truncate)) {
      nh = czero();
      dn = czero();
    }
    a.u[o] = nh;   // N and dN in place of A and dA (TLM_PLAIN reads them there)
    a.du[o] = dn;
    if (a.mode == TLM_PLAIN) continue;
    const double e = stage_e(a.emk, a.emkx, a.emky, a.split, i, j, NH);
    const bool origin = (i == 0 && j == 0);
    const double2 z = a.z[o], dz = a.dz[o];
    if (a.mode == TLM_STAGE_A) {
      a.w[o] = origin ? czero() : make_double2(e * (z.x + a.dt2 * nh.x), e * (z.y + a.dt2 * nh.y));
      a.dw[o] = origin ? czero() : make_double2(e * (dz.x + a.dt2 * dn.x), e * (dz.y + a.dt2 * dn.y));
    } else {
      a.z[o] = origin ? czero() : make_double2(e * (e * z.x + a.dt * nh.x), e * (e * z.y + a.dt * nh.y));
      a.dz[o] = origin ? czero() : make_double2(e * (e * dz.x + a.dt * dn.x), e * (e * dz.y + a.dt * dn.y));
    }
  }
  cluster.sync();
}

// ---- field-split transposed column tiles (one field of one column per CTA, C = 1) ---------------

// Fields of the transposed pass A: q, u, v from x (f = 0, 1, 2) and a, b from lin (3, 4); with
// the physical fields of x only a and b, on the columns up to kxlim.
__host__ __device__ inline int adj_colinv_split_units(int nh, int kxlim, bool phys) {
  return phys ? 2 * (kxlim + 1) : 5 * nh;
}

template <int N, int R>
__device__ __forceinline__ void adj_colinv_field_tile(const AdjArgs& a, int unit) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  const bool phys = a.phys_uv != nullptr;
  const int nfield = phys ? 2 : 5;
  const int i = unit / nfield, f = (phys ? 3 : 0) + unit % nfield, t = threadIdx.x;
  const double kx = __ldg(&a.fkx[i]);
  const int kc = a.truncate ? __ldg(&a.kcut[i]) : N;
  const double wcol = (i == 0 || i == NH - 1) ? 1.0 : 0.5;
  double2* dst = f == 0 ? a.q : f == 1 ? a.u : f == 2 ? a.v : f == 3 ? a.a : a.b;
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int j = t + s * T;
    const size_t o = (size_t)j * NH + i;
    if (f < 3) {
      const double2 q = a.x[o];
      if (f == 0) {
        v[s] = q;
      } else if (f == 1) {
        const double m = __ldg(&a.fky[j]) * __ldg(&a.kainv[o]);
        v[s] = make_double2(-m * q.y, m * q.x);
      } else {
        const double m = kx * __ldg(&a.kainv[o]);
        v[s] = make_double2(m * q.y, -m * q.x);
      }
    } else {
      double2 l = a.lin[o];
      if (a.mode == ADJ_STAGE_B) {
        const double e = stage_e(a.emk, a.emkx, a.emky, a.split, i, j, NH) * a.dt;
        l = (i == 0 && j == 0) ? czero() : make_double2(e * l.x, e * l.y);
      }
      if (min(j, N - j) > kc || (i == 0 && j == 0 && a.truncate)) l = czero();
      // w o (i k) l
      const double k = (f == 3 ? kx : __ldg(&a.fky[j])) * wcol;
      v[s] = make_double2(-k * l.y, k * l.x);
    }
  }
  fft_regs<N, R, true, 1>(v, smem, t, a.tw, 0);
#pragma unroll
  for (int s = 0; s < R; ++s) dst[(size_t)(t + s * T) * NH + i] = v[s];
}

// The transposed pass C's value at (i, j) of the split forms from the transformed fields fq, fu,
// fv, in the order q, u, v of adj_colfwd_tile: g = c (fq + conj(Mu) fu + conj(Mv) fv) with
// conj(Mu) = -i ky/|k|^a, conj(Mv) = +i kx/|k|^a and c = cw (the row pass delivered 2 FFT(s);
// 1/2 on kx = 0 and Nyquist), stored to q, then the stage update of a.mode.
template <int N>
__device__ __forceinline__ void adj_colfwd_store(const AdjArgs& a, int i, int j, double kx, double cw, double2 fq,
                                                 double2 fu, double2 fv) {
  constexpr int NH = N / 2 + 1;
  const size_t o = (size_t)j * NH + i;
  double2 g = make_double2(cw * fq.x, cw * fq.y);
  const double mu = -__ldg(&a.fky[j]) * __ldg(&a.kainv[o]) * cw;
  g = make_double2(fma(-mu, fu.y, g.x), fma(mu, fu.x, g.y));
  const double mv = kx * __ldg(&a.kainv[o]) * cw;
  g = make_double2(fma(-mv, fv.y, g.x), fma(mv, fv.x, g.y));
  a.q[o] = g;
  if (a.mode == ADJ_STAGE_B) {
    const double e = stage_e(a.emk, a.emkx, a.emky, a.split, i, j, NH);
    const bool origin = (i == 0 && j == 0);
    const double2 l = a.lin[o];
    a.lam[o] = origin ? czero() : make_double2(e * (e * l.x + g.x), e * (e * l.y + g.y));
    a.rho[o] = origin ? czero() : make_double2(a.dt2 * e * g.x, a.dt2 * e * g.y);
  } else if (a.mode == ADJ_PLAIN) {
    a.lam[o] = g;
  } else {
    const double2 l = a.lam[o];
    a.lam[o] = make_double2(l.x + g.x, l.y + g.y);
  }
}

// Transposed pass C, field f of column i (unit 3 i + f; f = 0, 1, 2: q, u, v): the forward
// transform written back in place; the third of the column's CTAs to finish (a per-column
// counter, no waiting) reads the other two through L2, forms the accumulated gradient in the
// order q, u, v of adj_colfwd_tile and runs the stage update.
template <int N, int R>
__device__ __forceinline__ void adj_colfwd_field_tile(const AdjArgs& a, int unit) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  __shared__ int last;
  const int i = unit / 3, f = unit % 3, t = threadIdx.x;
  double2* own = f == 0 ? a.q : f == 1 ? a.u : a.v;
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = own[(size_t)(t + s * T) * NH + i];
  fft_regs<N, R, false, 1>(v, smem, t, a.tw, 0);
#pragma unroll
  for (int s = 0; s < R; ++s) own[(size_t)(t + s * T) * NH + i] = v[s];
  __threadfence();
  __syncthreads();
  if (t == 0) last = atomicAdd(&a.colcnt[i], 1) == 2;
  __syncthreads();
  if (!last) return;
  if (t == 0) a.colcnt[i] = 0;  // ready for the next launch
  const double kx = __ldg(&a.fkx[i]);
  // c o (.)/2: the row pass delivered 2 FFT(s); c = 1 on kx=0 and Nyquist, 2 inside
  const double cw = (i == 0 || i == NH - 1) ? 0.5 : 1.0;
#pragma unroll
  for (int s = 0; s < R; ++s) {
    const int j = t + s * T;
    const size_t o = (size_t)j * NH + i;
    const double2 fq = f == 0 ? v[s] : __ldcg(&a.q[o]);
    const double2 fu = f == 1 ? v[s] : __ldcg(&a.u[o]);
    const double2 fv = f == 2 ? v[s] : __ldcg(&a.v[o]);
    adj_colfwd_store<N>(a, i, j, kx, cw, fq, fu, fv);
  }
}

// The same pass with the column's three CTAs (q, u, v) as one 3-CTA cluster. Each CTA leaves its
// transformed field in its own shared memory for the rows the others combine; after a cluster
// barrier CTA f combines the rows j = t + s T with s = f, f + 3, ..., reading the other two
// fields from the partners' shared memory, and runs the update there (the same per-value
// arithmetic as above). A second barrier keeps the shared memory alive until the partners have
// read it. The transformed u and v are not written back: nothing reads them after this pass.
template <int N, int R>
__device__ __forceinline__ void adj_colfwd_cluster_tile(const AdjArgs& a, int unit) {
  constexpr int T = N / R, NH = N / 2 + 1;
  extern __shared__ double2 smem[];
  const int i = unit / 3, f = unit % 3, t = threadIdx.x;
  namespace cg = cooperative_groups;
  cg::cluster_group cluster = cg::this_cluster();
  const double2* own = f == 0 ? a.q : f == 1 ? a.u : a.v;
  double2 v[R];
#pragma unroll
  for (int s = 0; s < R; ++s) v[s] = own[(size_t)(t + s * T) * NH + i];
  fft_regs<N, R, false, 1>(v, smem, t, a.tw, 0);
  // fft_regs ends with a barrier after its last shared-memory read: the buffer is free
#pragma unroll
  for (int s = 0; s < R; ++s)
    if (s % 3 != f) smem[t + s * T] = v[s];
  cluster.sync();
  const double2* pq = cluster.map_shared_rank(smem, 0u);
  const double2* pu = cluster.map_shared_rank(smem, 1u);
  const double2* pv = cluster.map_shared_rank(smem, 2u);
  const double kx = __ldg(&a.fkx[i]);
  const double cw = (i == 0 || i == NH - 1) ? 0.5 : 1.0;
#pragma unroll
  for (int s = 0; s < R; ++s) {
    if (s % 3 != f) continue;
    const int j = t + s * T;
    adj_colfwd_store<N>(a, i, j, kx, cw, f == 0 ? v[s] : pq[j], f == 1 ? v[s] : pu[j], f == 2 ? v[s] : pv[j]);
  }
  cluster.sync();
}

// ---- kernels ------------------------------------------------------------------------------
template <int N>
struct AdjShape {
  static constexpr size_t TLM_ROW_SMEM = (size_t)3 * padded(N) * Shape<N>::ROWS * sizeof(double2);
  static constexpr size_t ADJ_ROW_SMEM =
      (size_t)(2 * padded(N) + padded(N / 2)) * Shape<N>::ROWS * sizeof(double2);
  static constexpr bool OK = (N <= 4096);
};

template <int N>
__global__ void __launch_bounds__(Shape<N>::COL_THREADS) k_tlm_colinv(TlmArgs a) {
  pdl_enter();
  if constexpr (AdjShape<N>::OK) tlm_colinv_tile<N, Shape<N>::COLS>(a, blockIdx.x);
}
template <int N>
__global__ void __launch_bounds__(Shape<N>::ROW_THREADS) k_tlm_row(TlmArgs a) {
  pdl_enter();
  if constexpr (AdjShape<N>::OK) tlm_row_tile<N, Shape<N>::ROWS>(a, blockIdx.x);
}
template <int N>
__global__ void __launch_bounds__(Shape<N>::COL_THREADS) k_tlm_colfwd(TlmArgs a) {
  pdl_enter();
  if constexpr (AdjShape<N>::OK) tlm_colfwd_tile<N, Shape<N>::COLS>(a, blockIdx.x);
}
template <int N>
__global__ void __launch_bounds__(Shape<N>::COL_THREADS) k_adj_colinv(AdjArgs a) {
  pdl_enter();
  if constexpr (AdjShape<N>::OK) adj_colinv_tile<N, Shape<N>::COLS>(a, blockIdx.x);
}
template <int N>
__global__ void __launch_bounds__(Shape<N>::ROW_THREADS) k_adj_row(AdjArgs a) {
  pdl_enter();
  if constexpr (AdjShape<N>::OK) adj_row_tile<N, Shape<N>::ROWS>(a, blockIdx.x);
}
template <int N>
__global__ void __launch_bounds__(Shape<N>::COL_THREADS) k_adj_colfwd(AdjArgs a) {
  pdl_enter();
  if constexpr (AdjShape<N>::OK) adj_colfwd_tile<N, Shape<N>::COLS>(a, blockIdx.x);
}

// The tangent-linear and adjoint passes in launch variant V of the nonlinear-term passes
// (Var<N, V>: 8 or 4 values per thread, one column / row per block).
template <int N, int V>
struct AdjVar {
  using W = Var<N, V>;
  static constexpr size_t TLM_ROW_SMEM = (size_t)3 * padded(N) * W::ROWS * sizeof(double2);
  static constexpr size_t ADJ_ROW_SMEM = (size_t)(2 * padded(N) + padded(N / 2)) * W::ROWS * sizeof(double2);
  static constexpr bool OK = W::OK && !W::GROUPED && V != 5 && AdjShape<N>::OK;  // 5: the tiles of 2
};

template <int N, int V>
__global__ void __launch_bounds__(Var<N, V>::COL_THREADS) k_tlmv_colinv(TlmArgs a) {
  pdl_enter();
  if constexpr (AdjVar<N, V>::OK) tlm_colinv_tile<N, Var<N, V>::COLS, Var<N, V>::R>(a, blockIdx.x);
}
template <int N, int V>
__global__ void __launch_bounds__(Var<N, V>::ROW_THREADS) k_tlmv_row(TlmArgs a) {
  pdl_enter();
  if constexpr (AdjVar<N, V>::OK) tlm_row_tile<N, Var<N, V>::ROWS, Var<N, V>::R>(a, blockIdx.x);
}
template <int N, int V>
__global__ void __launch_bounds__(Var<N, V>::COL_THREADS) k_tlmv_colfwd(TlmArgs a) {
  pdl_enter();
  if constexpr (AdjVar<N, V>::OK) tlm_colfwd_tile<N, Var<N, V>::COLS, Var<N, V>::R>(a, blockIdx.x);
}
template <int N, int V>
__global__ void __launch_bounds__(Var<N, V>::COL_THREADS) k_adjv_colinv(AdjArgs a) {
  pdl_enter();
  if constexpr (AdjVar<N, V>::OK) adj_colinv_tile<N, Var<N, V>::COLS, Var<N, V>::R>(a, blockIdx.x);
}
template <int N, int V>
__global__ void __launch_bounds__(Var<N, V>::ROW_THREADS) k_adjv_row(AdjArgs a) {
  pdl_enter();
  if constexpr (AdjVar<N, V>::OK) adj_row_tile<N, Var<N, V>::ROWS, Var<N, V>::R>(a, blockIdx.x);
}
template <int N, int V>
__global__ void __launch_bounds__(Var<N, V>::COL_THREADS) k_adjv_colfwd(AdjArgs a) {
  pdl_enter();
  if constexpr (AdjVar<N, V>::OK) adj_colfwd_tile<N, Var<N, V>::COLS, Var<N, V>::R>(a, blockIdx.x);
}

// the field-split transposed column passes (variants with one column per CTA, no groups)
template <int N, int V>
struct AdjSplitVar {
  static constexpr bool OK = SplitVar<N, V>::OK && V != 5 && AdjShape<N>::OK;
};
template <int N, int V>
__global__ void __launch_bounds__(SplitVar<N, V>::THREADS, SplitVar<N, V>::MINB) k_tlm_colinv_fs(TlmArgs a) {
  pdl_enter();
  if constexpr (AdjSplitVar<N, V>::OK) tlm_colinv_field_tile<N, Var<N, V>::R>(a, blockIdx.x);
}
template <int N, int V>
__global__ void __launch_bounds__(SplitVar<N, V>::THREADS, SplitVar<N, V>::MINB) k_tlm_colfwd_fs(TlmArgs a) {
  pdl_enter();
  if constexpr (AdjSplitVar<N, V>::OK) tlm_colfwd_field_tile<N, Var<N, V>::R>(a, blockIdx.x);
}
template <int N, int V>
__global__ void __launch_bounds__(SplitVar<N, V>::THREADS, SplitVar<N, V>::MINB) k_adj_colinv_fs(AdjArgs a) {
  pdl_enter();
  if constexpr (AdjSplitVar<N, V>::OK) adj_colinv_field_tile<N, Var<N, V>::R>(a, blockIdx.x);
}
// the tangent pass C with the column's four CTAs as one cluster (grid 4 NH)
template <int N, int V>
__global__ void __cluster_dims__(4, 1, 1) __launch_bounds__(SplitVar<N, V>::THREADS, SplitVar<N, V>::MINB)
    k_tlm_colfwd_cl(TlmArgs a) {
  pdl_enter();
  if constexpr (AdjSplitVar<N, V>::OK) tlm_colfwd_cluster_tile<N, Var<N, V>::R>(a, blockIdx.x);
}
template <int N, int V>
__global__ void __launch_bounds__(SplitVar<N, V>::THREADS, SplitVar<N, V>::MINB) k_adj_colfwd_fs(AdjArgs a) {
  pdl_enter();
  if constexpr (AdjSplitVar<N, V>::OK) adj_colfwd_field_tile<N, Var<N, V>::R>(a, blockIdx.x);
}
template <int N, int V>
__global__ void __cluster_dims__(3, 1, 1) __launch_bounds__(SplitVar<N, V>::THREADS, SplitVar<N, V>::MINB)
    k_adj_colfwd_cl(AdjArgs a) {
  pdl_enter();
  if constexpr (AdjSplitVar<N, V>::OK) adj_colfwd_cluster_tile<N, Var<N, V>::R>(a, blockIdx.x);
}

}  // namespace gt
