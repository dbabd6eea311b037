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

__device__ __forceinline__ int padix(int o) { return o + (o >> 4); }
__host__ __device__ constexpr int padded(int n) { return n + (n >> 4); }

__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// a * (-i) for the forward transform, a * (+i) for the inverse
template <bool INV>
__device__ __forceinline__ double2 mul_w4(double2 a) {
  return INV ? make_double2(-a.y, a.x) : make_double2(a.y, -a.x);
}

// a * w for the forward transform, a * conj(w) for the inverse (w = exp(-2 pi i k / L))
template <bool INV>
__device__ __forceinline__ double2 twmul(double2 a, double2 w) {
  if (INV) return make_double2(fma(a.x, w.x, a.y * w.y), fma(a.y, w.x, -(a.x * w.y)));
  return make_double2(fma(a.x, w.x, -(a.y * w.y)), fma(a.y, w.x, a.x * w.y));
}

// a * c * (1 -+ i): the W8^1 twiddle (forward: (1-i)/sqrt2, inverse (1+i)/sqrt2)
template <bool INV>
__device__ __forceinline__ double2 mul_w8_1(double2 a) {
  const double c = 0.70710678118654752440;
  return INV ? make_double2(c * (a.x - a.y), c * (a.x + a.y))
             : make_double2(c * (a.x + a.y), c * (a.y - a.x));
}
// W8^3 (forward: -(1+i)/sqrt2, inverse: (-1+i)/sqrt2)
template <bool INV>
__device__ __forceinline__ double2 mul_w8_3(double2 a) {
  const double c = 0.70710678118654752440;
  return INV ? make_double2(-c * (a.x + a.y), c * (a.x - a.y))
             : make_double2(c * (a.y - a.x), -c * (a.x + a.y));
}

template <bool INV>
__device__ __forceinline__ void dft2(double2& a0, double2& a1) {
  double2 t = a0;
  a0 = cadd(t, a1);
  a1 = csub(t, a1);
}

template <bool INV>
__device__ __forceinline__ void dft4(double2& a0, double2& a1, double2& a2, double2& a3) {
  double2 t0 = cadd(a0, a2), t1 = csub(a0, a2);
  double2 t2 = cadd(a1, a3), t3 = mul_w4<INV>(csub(a1, a3));
  a0 = cadd(t0, t2);
  a2 = csub(t0, t2);
  a1 = cadd(t1, t3);
  a3 = csub(t1, t3);
}

// Radix-8 as 2 x radix-4: even/odd DFT4s, W8^k twiddles, radix-2 combine. Natural order.
template <bool INV>
__device__ __forceinline__ void dft8(double2* a) {
  double2 e0 = a[0], e1 = a[2], e2 = a[4], e3 = a[6];
  double2 o0 = a[1], o1 = a[3], o2 = a[5], o3 = a[7];
  dft4<INV>(e0, e1, e2, e3);
  dft4<INV>(o0, o1, o2, o3);
  o1 = mul_w8_1<INV>(o1);
  o2 = mul_w4<INV>(o2);
  o3 = mul_w8_3<INV>(o3);
  a[0] = cadd(e0, o0); a[4] = csub(e0, o0);
  a[1] = cadd(e1, o1); a[5] = csub(e1, o1);
  a[2] = cadd(e2, o2); a[6] = csub(e2, o2);
  a[3] = cadd(e3, o3); a[7] = csub(e3, o3);
}

// Radix-16 as 4 x radix-4 with W16^(n1*k2) twiddles. Natural order in and out.
template <bool INV>
__device__ __forceinline__ void dft16(double2* a) {
  const double c8 = 0.92387953251128675613;  // cos(pi/8)
  const double s8 = 0.38268343236508977173;  // sin(pi/8)
#pragma unroll
  for (int n1 = 0; n1 < 4; ++n1) dft4<INV>(a[n1], a[n1 + 4], a[n1 + 8], a[n1 + 12]);
  // b[n1][k2] sits in a[n1 + 4*k2]; twiddle by W16^(n1*k2)
  // n1 = 1: k2 = 1,2,3 -> W16^1, W16^2, W16^3
  a[5] = twmul<INV>(a[5], make_double2(c8, -s8));
  a[9] = mul_w8_1<INV>(a[9]);
  a[13] = twmul<INV>(a[13], make_double2(s8, -c8));
  // n1 = 2: W16^2, W16^4, W16^6
  a[6] = mul_w8_1<INV>(a[6]);
  a[10] = mul_w4<INV>(a[10]);
  a[14] = mul_w8_3<INV>(a[14]);
  // n1 = 3: W16^3, W16^6, W16^9
  a[7] = twmul<INV>(a[7], make_double2(s8, -c8));
  a[11] = mul_w8_3<INV>(a[11]);
  a[15] = twmul<INV>(a[15], make_double2(-c8, s8));
#pragma unroll
  for (int k2 = 0; k2 < 4; ++k2) dft4<INV>(a[4 * k2], a[4 * k2 + 1], a[4 * k2 + 2], a[4 * k2 + 3]);
  // X[k2 + 4*k1] sits in a[4*k2 + k1]: transpose the 4x4 block
  double2 t;
  t = a[1]; a[1] = a[4]; a[4] = t;
  t = a[2]; a[2] = a[8]; a[8] = t;
  t = a[3]; a[3] = a[12]; a[12] = t;
  t = a[6]; a[6] = a[9]; a[9] = t;
  t = a[7]; a[7] = a[13]; a[13] = t;
  t = a[11]; a[11] = a[14]; a[14] = t;
}

template <int RP, bool INV>
__device__ __forceinline__ void dft(double2* a) {
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
// the block must call it (it contains __syncthreads when L > R).
template <int L, int R, bool INV, int SS>
__device__ __forceinline__ void fft_regs(double2 (&v)[R], double2* sm, int t,
                                         const double2* __restrict__ tw, int twshift) {
  static_assert((L & (L - 1)) == 0 && L >= R, "L must be a power of two >= R");
  StockhamPass<L, R, 1, INV, SS>::run(v, sm, t, tw, twshift);
}

}  // namespace gt
