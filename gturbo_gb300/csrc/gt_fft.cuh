// gt_fft.cuh -- FP64 Stockham FFT engine for sm_103a.
//
// GB300 executes FP64 at ~1/58 of its FP32 rate (about 600 G DFMA/s over the chip), so every
// transform here is bound by the number of FP64 instructions, not by HBM. The engine is built
// around that:
//   * each thread holds R complex values in registers (x[t + s*T], T = L/R threads per
//     transform) and applies one radix-RP butterfly (RP <= R) per pass, so a length-2048
//     transform is three passes (16, 16, 8) with two shared-memory exchanges;
//   * the first pass reads straight from global memory and the last pass leaves its outputs
//     in registers in the same x[t + s*T] pattern, so the callers load from and store to HBM
//     without an extra shared-memory round trip and fuse their own pre/post arithmetic;
//   * twiddles come from a precomputed table (no FP64 sin/cos), butterflies are written so
//     that nvcc contracts the multiplies into FMAs;
//   * shared memory is padded one slot in 16 (padix) so the stride-R stores of the early
//     passes hit distinct banks.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gt {

#define GT_HD_INL __host__ __device__ __forceinline__

__device__ __forceinline__ int padix(int o) { return o + (o >> 4); }
__host__ __device__ constexpr int padded(int n) { return n + (n >> 4); }

GT_HD_INL double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
GT_HD_INL double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// a * (-i) for the forward transform, a * (+i) for the inverse
template <bool INV>
GT_HD_INL double2 mul_w4(double2 a) {
  return INV ? make_double2(-a.y, a.x) : make_double2(a.y, -a.x);
}

// a * w for the forward transform, a * conj(w) for the inverse (w = exp(-2 pi i k / L))
template <bool INV>
GT_HD_INL double2 twmul(double2 a, double2 w) {
  if (INV) return make_double2(fma(a.x, w.x, a.y * w.y), fma(a.y, w.x, -(a.x * w.y)));
  return make_double2(fma(a.x, w.x, -(a.y * w.y)), fma(a.y, w.x, a.x * w.y));
}

// s + i conj(w) d: the term of the half-length C2R packing, Z[k] = S[k] + i W^-k D[k], as four
// FMAs (the twiddle product is accumulated into s instead of being formed and then added).
GT_HD_INL double2 pack_c2r(double2 s, double2 d, double2 w) {
  return make_double2(fma(d.x, w.y, fma(-d.y, w.x, s.x)), fma(d.x, w.x, fma(d.y, w.y, s.y)));
}

// The W8^1 and W8^3 twiddles are c * P(a) with c = 1/sqrt(2) and P made of additions only.
// The butterflies below keep P unscaled and fold c into the following additions as FMAs
// (e +- c P), which removes the two multiplies per twiddle.
constexpr double kC8 = 0.70710678118654752440;  // cos(pi/4)

// W8^1: forward (1-i)/sqrt2, inverse (1+i)/sqrt2
template <bool INV>
GT_HD_INL double2 w8_1_unscaled(double2 a) {
  return INV ? make_double2(a.x - a.y, a.x + a.y) : make_double2(a.x + a.y, a.y - a.x);
}
// W8^3: forward -(1+i)/sqrt2, inverse (-1+i)/sqrt2
template <bool INV>
GT_HD_INL double2 w8_3_unscaled(double2 a) {
  return INV ? make_double2(-(a.x + a.y), a.x - a.y) : make_double2(a.y - a.x, -(a.x + a.y));
}
// e + s c P and e - s c P (s = +-1 folded into c)
GT_HD_INL double2 fma_c(double c, double2 p, double2 e) { return make_double2(fma(c, p.x, e.x), fma(c, p.y, e.y)); }

template <bool INV>
GT_HD_INL void dft2(double2& a0, double2& a1) {
  double2 t = a0;
  a0 = cadd(t, a1);
  a1 = csub(t, a1);
}

template <bool INV>
GT_HD_INL void dft4(double2& a0, double2& a1, double2& a2, double2& a3) {
  double2 t0 = cadd(a0, a2), t1 = csub(a0, a2);
  double2 t2 = cadd(a1, a3), t3 = mul_w4<INV>(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

// Radix-8 as 2 x radix-4: even/odd DFT4s, W8^k twiddles, radix-2 combine. Natural order.
template <bool INV>
GT_HD_INL void dft8(double2* a) {
  double2 e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  double2 o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  dft4<INV>(e0, e1, e2, e3);
  dft4<INV>(o0, o1, o2, o3);
  const double2 p1 = w8_1_unscaled<INV>(o1);
  const double2 p3 = w8_3_unscaled<INV>(o3);
  o2 = mul_w4<INV>(o2);
  a[0] = cadd(e0, o0); a[4] = csub(e0, o0);
  a[1] = fma_c(kC8, p1, e1); a[5] = fma_c(-kC8, p1, e1);
  a[2] = cadd(e2, o2); a[6] = csub(e2, o2);
  a[3] = fma_c(kC8, p3, e3); a[7] = fma_c(-kC8, p3, e3);
}

// Radix-16 as 4 x radix-4 with W16^(n1*k2) twiddles (b[n1][k2] = a[n1 + 4 k2] after the first
// stage, X[k2 + 4 k1] from the second). Natural order in and out.
template <bool INV>
GT_HD_INL void dft16(double2* a) {
  const double c16 = 0.92387953251128675613;  // cos(pi/8)
  const double s16 = 0.38268343236508977173;  // sin(pi/8)
#pragma unroll
  for (int n1 = 0; n1 < 4; ++n1) dft4<INV>(a[n1], a[n1 + 4], a[n1 + 8], a[n1 + 12]);
  double2 X[16];
  // k2 = 0: no twiddles
  {
    double2 y0 = a[0], y1 = a[1], y2 = a[2], y3 = a[3];
    dft4<INV>(y0, y1, y2, y3);
    X[0] = y0; X[4] = y1; X[8] = y2; X[12] = y3;
  }
  // k2 = 1: (b0, W16^1 b1, W16^2 b2, W16^3 b3); W16^2 = W8^1 folded into t0, t1
  {
    const double2 b1 = twmul<INV>(a[5], make_double2(c16, -s16));
    const double2 p2 = w8_1_unscaled<INV>(a[6]);
    const double2 b3 = twmul<INV>(a[7], make_double2(s16, -c16));
    const double2 t0 = fma_c(kC8, p2, a[4]), t1 = fma_c(-kC8, p2, a[4]);
    const double2 t2 = cadd(b1, b3), t3 = mul_w4<INV>(csub(b1, b3));
    X[1] = cadd(t0, t2); X[9] = csub(t0, t2); X[5] = cadd(t1, t3); X[13] = csub(t1, t3);
  }
  // k2 = 2: (b0, W8^1 b1, W4 b2, W8^3 b3); both W8 factors share c: c (P1 +- P3)
  {
    const double2 p1 = w8_1_unscaled<INV>(a[9]);
    const double2 b2 = mul_w4<INV>(a[10]);
    const double2 p3 = w8_3_unscaled<INV>(a[11]);
    const double2 t0 = cadd(a[8], b2), t1 = csub(a[8], b2);
    const double2 sp = cadd(p1, p3), dm = mul_w4<INV>(csub(p1, p3));
    X[2] = fma_c(kC8, sp, t0); X[10] = fma_c(-kC8, sp, t0);
    X[6] = fma_c(kC8, dm, t1); X[14] = fma_c(-kC8, dm, t1);
  }
  // k2 = 3: (b0, W16^3 b1, W16^6 b2, W16^9 b3); W16^6 = W8^3 folded into t0, t1
  {
    const double2 b1 = twmul<INV>(a[13], make_double2(s16, -c16));
    const double2 p2 = w8_3_unscaled<INV>(a[14]);
    const double2 b3 = twmul<INV>(a[15], make_double2(-c16, s16));
    const double2 t0 = fma_c(kC8, p2, a[12]), t1 = fma_c(-kC8, p2, a[12]);
    const double2 t2 = cadd(b1, b3), t3 = mul_w4<INV>(csub(b1, b3));
    X[3] = cadd(t0, t2); X[11] = csub(t0, t2); X[7] = cadd(t1, t3); X[15] = csub(t1, t3);
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = X[k];
}

template <int RP, bool INV>
GT_HD_INL void dft(double2* a) {
  if constexpr (RP == 2) dft2<INV>(a[0], a[1]);
  else if constexpr (RP == 4) dft4<INV>(a[0], a[1], a[2], a[3]);
  else if constexpr (RP == 8) dft8<INV>(a);
  else if constexpr (RP == 16) dft16<INV>(a);
  else static_assert(RP == 1, "unsupported radix");
}

// One Stockham pass (radix RP = min(R, L/Ns)) and, recursively, the rest of the transform.
//   v   : the thread's R values, v[s] = x[t + s*T]; on return X[t + s*T] (natural order)
//   sm  : exchange buffer; element o lives at sm[padix(o) * SS]
//   tw  : table exp(-2 pi i k / (L << twshift)), k in [0, L << twshift)
template <int L, int R, int Ns, bool INV, int SS>
struct StockhamPass {
  static constexpr int RP = (L / Ns >= R) ? R : (L / Ns);
  static constexpr bool LAST = (Ns * RP == L);
  static constexpr int T = L / R;
  static constexpr int NB = R / RP;

  __device__ __forceinline__ static void run(double2 (&v)[R], double2* sm, int t,
                                             const double2* __restrict__ tw, int twshift) {
#pragma unroll
    for (int m = 0; m < NB; ++m) {
      const int b = t + m * T;
      const int k = b & (Ns - 1);
      double2 a[RP];
#pragma unroll
      for (int r = 0; r < RP; ++r) a[r] = v[m + r * NB];
      if constexpr (Ns > 1) {
#pragma unroll
        for (int r = 1; r < RP; ++r) {
          const double2 w = __ldg(&tw[(r * k * (L / (Ns * RP))) << twshift]);
          a[r] = twmul<INV>(a[r], w);
        }
      }
      dft<RP, INV>(a);
      if constexpr (LAST) {
#pragma unroll
        for (int r = 0; r < RP; ++r) v[m + r * NB] = a[r];
      } else {
        const int base = (b - k) * RP + k;
#pragma unroll
        for (int r = 0; r < RP; ++r) sm[padix(base + r * Ns) * SS] = a[r];
      }
    }
    if constexpr (!LAST) {
      __syncthreads();
#pragma unroll
      for (int s = 0; s < R; ++s) v[s] = sm[padix(t + s * T) * SS];
      __syncthreads();
      StockhamPass<L, R, Ns * RP, INV, SS>::run(v, sm, t, tw, twshift);
    }
  }
};

// Full transform of length L held as R values per thread (see StockhamPass). Every thread of
// the block must call it, from the same call site (it contains __syncthreads when L > R).
template <int L, int R, bool INV, int SS>
__device__ __forceinline__ void fft_regs(double2 (&v)[R], double2* sm, int t,
                                         const double2* __restrict__ tw, int twshift) {
  static_assert((L & (L - 1)) == 0 && L >= R, "L must be a power of two >= R");
  StockhamPass<L, R, 1, INV, SS>::run(v, sm, t, tw, twshift);
}

}  // namespace gt
