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
//     that nvcc contracts the multiplies into FMAs, and the upper half of each twiddled
//     butterfly's inputs uses the Linzer-Feig form c (1 + i t) of its twiddle, whose c folds into
//     the first additions (a radix-16 pass: 188 instead of 212 FP64 instructions per thread);
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

// a (1 + i t): the twiddle c (1 + i t) without its real factor c, as two FMAs (Linzer and Feig,
// "Modified FFTs for fused multiply-add architectures", Math. Comp. 60 (1993)). The factor c is
// folded into the additions that follow (e +- c y), so a twiddle costs two FMAs instead of four
// operations.
GT_HD_INL double2 mul_1pit(double2 a, double t) { return make_double2(fma(-t, a.y, a.x), fma(t, a.x, a.y)); }

// W16^1 = c16 (1 - i t16) and W16^3 = c16 (t16 - i), t16 = tan(pi/8); conjugates for the inverse.
constexpr double kC16 = 0.92387953251128675613;  // cos(pi/8)
constexpr double kT16 = 0.41421356237309504880;  // tan(pi/8) = sqrt(2) - 1
// a (1 - i t16) forward, a (1 + i t16) inverse
template <bool INV>
GT_HD_INL double2 w16_1_unscaled(double2 a) { return mul_1pit(a, INV ? kT16 : -kT16); }
// a (t16 - i) forward, a (t16 + i) inverse
template <bool INV>
GT_HD_INL double2 w16_3_unscaled(double2 a) {
  return INV ? make_double2(fma(kT16, a.x, -a.y), fma(kT16, a.y, a.x))
             : make_double2(fma(kT16, a.x, a.y), fma(kT16, a.y, -a.x));
}

// ---- butterflies from first-level pairs -------------------------------------------------------
// Every radix-RP butterfly starts with the sums and differences of the input pairs
// (r, r + RP/2): s_r = a_r + a_{r+RP/2}, d_r = a_r - a_{r+RP/2}, r < RP/2. dft_pairs finishes the
// transform from them, in natural order. The plain butterfly (dft) forms the pairs with
// additions; the twiddled one of the Stockham passes (dft_tw) forms them with FMAs from the
// Linzer-Feig form of the upper twiddle.

// Radix 16 as 4 x radix-4 with W16^(n1*k2) twiddles (b[n1][k2] = a[n1 + 4 k2] after the first
// stage, X[k2 + 4 k1] from the second). SCALED: b[n1][k2] carries the factor c_n1 (c_0 = 1) of
// the first stage, and sc = {c1, c2, mu = c3/c1, c2 cos(pi/4), c1 cos(pi/8), c1 cos(pi/4)} folds
// it into the FMAs of the second stage (no extra instruction).
template <bool INV, bool SCALED = false>
GT_HD_INL void dft16_stage2(double2* a, const double* sc = nullptr) {
  // multipliers of the W8 fold on b2 (k2 = 1, 3), of c16 (k2 = 1, 3) and of the W8 fold on b1, b3
  // (k2 = 2)
  double c1 = 1.0, c2 = 1.0, mu = 1.0, f8b2 = kC8, f16 = kC16, f8b1 = kC8;
  if constexpr (SCALED) {
    c1 = sc[0]; c2 = sc[1]; mu = sc[2]; f8b2 = sc[3]; f16 = sc[4]; f8b1 = sc[5];
  }
  double2 X[16];
  // k2 = 0: no twiddles
  {
    double2 t0, t1, t2, t3;
    if constexpr (SCALED) {
      t0 = fma_c(c2, a[2], a[0]); t1 = fma_c(-c2, a[2], a[0]);
      t2 = fma_c(mu, a[3], a[1]); t3 = mul_w4<INV>(fma_c(-mu, a[3], a[1]));
      X[0] = fma_c(c1, t2, t0); X[8] = fma_c(-c1, t2, t0); X[4] = fma_c(c1, t3, t1); X[12] = fma_c(-c1, t3, t1);
    } else {
      t0 = cadd(a[0], a[2]); t1 = csub(a[0], a[2]);
      t2 = cadd(a[1], a[3]); t3 = mul_w4<INV>(csub(a[1], a[3]));
      X[0] = cadd(t0, t2); X[8] = csub(t0, t2); X[4] = cadd(t1, t3); X[12] = csub(t1, t3);
    }
  }
  // k2 = 1: (b0, W16^1 b1, W16^2 b2, W16^3 b3). W16^1 b1 + W16^3 b3 = c16 (u1 + u3) with u1, u3 the
  // unscaled products; c16 and the c of W16^2 = W8^1 are folded into the output FMAs.
  {
    const double2 u1 = w16_1_unscaled<INV>(a[5]), u3 = w16_3_unscaled<INV>(a[7]);
    const double2 p2 = w8_1_unscaled<INV>(a[6]);
    const double2 t0 = fma_c(f8b2, p2, a[4]), t1 = fma_c(-f8b2, p2, a[4]);
    double2 sp, dm;
    if constexpr (SCALED) {
      sp = fma_c(mu, u3, u1); dm = mul_w4<INV>(fma_c(-mu, u3, u1));
    } else {
      sp = cadd(u1, u3); dm = mul_w4<INV>(csub(u1, u3));
    }
    X[1] = fma_c(f16, sp, t0); X[9] = fma_c(-f16, sp, t0);
    X[5] = fma_c(f16, dm, t1); X[13] = fma_c(-f16, dm, t1);
  }
  // k2 = 2: (b0, W8^1 b1, W4 b2, W8^3 b3); both W8 factors share c: c (P1 +- P3)
  {
    const double2 p1 = w8_1_unscaled<INV>(a[9]);
    const double2 b2 = mul_w4<INV>(a[10]);
    const double2 p3 = w8_3_unscaled<INV>(a[11]);
    double2 t0, t1, sp, dm;
    if constexpr (SCALED) {
      t0 = fma_c(c2, b2, a[8]); t1 = fma_c(-c2, b2, a[8]);
      sp = fma_c(mu, p3, p1); dm = mul_w4<INV>(fma_c(-mu, p3, p1));
    } else {
      t0 = cadd(a[8], b2); t1 = csub(a[8], b2);
      sp = cadd(p1, p3); dm = mul_w4<INV>(csub(p1, p3));
    }
    X[2] = fma_c(f8b1, sp, t0); X[10] = fma_c(-f8b1, sp, t0);
    X[6] = fma_c(f8b1, dm, t1); X[14] = fma_c(-f8b1, dm, t1);
  }
  // k2 = 3: (b0, W16^3 b1, W16^6 b2, W16^9 b3) with W16^9 = -W16^1: c16 (u3 - u1)
  {
    const double2 u3 = w16_3_unscaled<INV>(a[13]), u1 = w16_1_unscaled<INV>(a[15]);
    const double2 p2 = w8_3_unscaled<INV>(a[14]);
    const double2 t0 = fma_c(f8b2, p2, a[12]), t1 = fma_c(-f8b2, p2, a[12]);
    double2 sp, dm;
    if constexpr (SCALED) {
      sp = fma_c(-mu, u1, u3); dm = mul_w4<INV>(fma_c(mu, u1, u3));
    } else {
      sp = csub(u3, u1); dm = mul_w4<INV>(cadd(u3, u1));
    }
    X[3] = fma_c(f16, sp, t0); X[11] = fma_c(-f16, sp, t0);
    X[7] = fma_c(f16, dm, t1); X[15] = fma_c(-f16, dm, t1);
  }
#pragma unroll
  for (int k = 0; k < 16; ++k) a[k] = X[k];
}

template <int RP, bool INV>
GT_HD_INL void dft_pairs(const double2* s, const double2* d, double2* a) {
  if constexpr (RP == 2) {
    a[0] = s[0];
    a[1] = d[0];
  } else if constexpr (RP == 4) {
    const double2 t3 = mul_w4<INV>(d[1]);
    a[0] = cadd(s[0], s[1]); a[2] = csub(s[0], s[1]);
    a[1] = cadd(d[0], t3); a[3] = csub(d[0], t3);
  } else if constexpr (RP == 8) {
    // radix 8 as 2 x radix-4 (even and odd inputs), W8^k twiddles, radix-2 combine
    const double2 we = mul_w4<INV>(d[2]), wo = mul_w4<INV>(d[3]);
    const double2 e0 = cadd(s[0], s[2]), e2 = csub(s[0], s[2]), e1 = cadd(d[0], we), e3 = csub(d[0], we);
    const double2 o0 = cadd(s[1], s[3]), o1 = cadd(d[1], wo), o3 = csub(d[1], wo);
    const double2 o2 = mul_w4<INV>(csub(s[1], s[3]));
    const double2 p1 = w8_1_unscaled<INV>(o1);
    const double2 p3 = w8_3_unscaled<INV>(o3);
    a[0] = cadd(e0, o0); a[4] = csub(e0, o0);
    a[1] = fma_c(kC8, p1, e1); a[5] = fma_c(-kC8, p1, e1);
    a[2] = cadd(e2, o2); a[6] = csub(e2, o2);
    a[3] = fma_c(kC8, p3, e3); a[7] = fma_c(-kC8, p3, e3);
  } else if constexpr (RP == 16) {
    // first stage: the radix-4 of inputs (n1, n1+4, n1+8, n1+12) from pairs n1 and n1+4
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) {
      const double2 t3 = mul_w4<INV>(d[n1 + 4]);
      a[n1] = cadd(s[n1], s[n1 + 4]);
      a[n1 + 8] = csub(s[n1], s[n1 + 4]);
      a[n1 + 4] = cadd(d[n1], t3);
      a[n1 + 12] = csub(d[n1], t3);
    }
    dft16_stage2<INV>(a);
  } else {
    static_assert(RP == 2, "unsupported radix");
  }
}

// The zero band of a first radix pass: inputs a[r] = x[t + r T] (T = L/RP) with r T in
// [3L/8, 5L/8). A spectrum cut below 3L/8 on both sides of L/2 (the 2/3 rule keeps |k| <= L/3) is
// zero there for every t: r in [6, 10) for RP = 16, [3, 5) for RP = 8, none below.
__host__ __device__ constexpr bool in_zband(int rp, int r) { return 8 * r >= 3 * rp && 8 * (r + 1) <= 5 * rp; }

// Plain radix-RP DFT of a[0..RP), natural order in and out. ZB: the zero-band inputs are known
// to be zero, and their additions are left out (16 of the 144 FP64 instructions of radix 16).
template <int RP, bool INV, bool ZB = false>
GT_HD_INL void dft(double2* a) {
  constexpr int H = RP / 2;
  double2 s[H], d[H];
#pragma unroll
  for (int r = 0; r < H; ++r) {
    if (ZB && in_zband(RP, r + H)) {
      s[r] = a[r];
      d[r] = a[r];
    } else if (ZB && in_zband(RP, r)) {
      s[r] = a[r + H];
      d[r] = make_double2(-a[r + H].x, -a[r + H].y);
    } else {
      s[r] = cadd(a[r], a[r + H]);
      d[r] = csub(a[r], a[r + H]);
    }
  }
  dft_pairs<RP, INV>(s, d, a);
}

// Radix-RP DFT of the twiddled inputs a_r w_r (a_r conj(w_r) for the inverse), w_0 = 1:
//   wl[r], 0 < r < RP/2 : w_r
//   lh[r], r < RP/2     : w_{r+RP/2} in Linzer-Feig form (c, t), w = c (1 + i t)
// The lower twiddle is an ordinary product; the upper one is mul_1pit with its c folded into the
// pair's sum and difference, a_r w_r +- c y.
template <int RP, bool INV>
GT_HD_INL void dft_tw(double2* a, const double2* wl, const double2* lh) {
  constexpr int H = RP / 2;
  double2 s[H], d[H];
#pragma unroll
  for (int r = 0; r < H; ++r) {
    const double2 lo = (r == 0) ? a[0] : twmul<INV>(a[r], wl[r]);
    const double2 y = mul_1pit(a[r + H], INV ? -lh[r].y : lh[r].y);
    s[r] = fma_c(lh[r].x, y, lo);
    d[r] = fma_c(-lh[r].x, y, lo);
  }
  dft_pairs<RP, INV>(s, d, a);
}

// ---- twiddled butterflies with carried scales (Linzer and Feig, every level) -------------------
// The pass tables hold, for each base angle m of a radix-RP pass (twiddles w_r = W^(r m),
// W = exp(-2 pi i / n), written w_r = c_r (1 + i t_r) as in the Linzer-Feig half of the twiddle
// table, c_0 = 1, t_0 = 0), an entry of lf_entry_doubles(RP) doubles:
//   e[r - 1]        t_r                 r = 1 .. RP-1
//   e[RP - 1 + r]   rho_r = c_{r+H}/c_r  r < H = RP/2
//   then RP = 16: sig_g = c_{g+4}/c_g (g < 4), c1, c2, c3/c1, c2 cos(pi/4), c1 cos(pi/8), c1 cos(pi/4)
//        RP = 8:  c2, c1, c3/c1, c1 cos(pi/4)
//        RP = 4:  c1
// Every twiddle is y_r = a_r (1 + i t_r), two FMAs. The sum and difference of pair (r, r+H) are
// y_r +- rho_r y_{r+H} and carry the factor c_r; the ratios and products above let every later
// addition absorb those factors as an FMA multiplier. Per thread and butterfly this takes radix 16
// from 188 to 174 FP64 instructions, radix 8 from 72 to 66 and radix 4 from 24 to 22.
__host__ __device__ constexpr int lf_entry_doubles(int rp) { return rp == 16 ? 34 : rp == 8 ? 16 : rp == 4 ? 6 : 0; }
// A pass of radix RP that follows passes of total radix Ns (span P = Ns RP) takes the entries of
// the base angles m = k n / P, i.e. the twiddles W_P^(r k), for k = b mod Ns. Each such pass has a
// table of its own in the twiddle buffer of a length-n table, for Ns = 2, 4, ..., n / RP, stored
// field by field: the double2 q of entry k sits at lf_pass_table(RP, n, Ns) + q Ns + k. The
// threads of a warp hold consecutive k, so each of their loads reads one contiguous run (2–4
// L1 lines) instead of one line per thread. The entries depend on P alone, so the tables of a
// length-n buffer also serve the transforms of length n/2 that read it with twshift = 1.
// Number of double2 of the radix-rp tables (all Ns) of a length-n buffer.
__host__ __device__ constexpr int lf_section_size(int rp, int n) {
  return n / rp >= 2 ? (lf_entry_doubles(rp) / 2) * (2 * (n / rp) - 2) : 0;
}
// Offset (in double2) of the radix-rp tables: after the n twiddles and their n Linzer-Feig forms.
__host__ __device__ constexpr int lf_section_offset(int rp, int n) {
  return 2 * n + (rp <= 8 ? lf_section_size(16, n) : 0) + (rp <= 4 ? lf_section_size(8, n) : 0);
}
// Offset (in double2) of the radix-rp table of the pass that follows total radix ns (ns >= 2).
__host__ __device__ constexpr int lf_pass_table(int rp, int n, int ns) {
  return lf_section_offset(rp, n) + (lf_entry_doubles(rp) / 2) * (ns - 2);
}
// Number of double2 in the whole twiddle buffer of a length-n table.
__host__ __device__ constexpr int twiddle_buffer_size(int n) {
  return lf_section_offset(4, n) + lf_section_size(4, n);
}

// The pass-table entry of base angle m (host side): lf[j] = (c_j, t_j), j < n, the Linzer-Feig
// half of the twiddle table. Ratios are formed in long double from the stored c.
template <int RP>
inline void make_lf_entry(const double2* lf, int n, int m, double* e) {
  constexpr int H = RP / 2;
  long double c[RP];
  for (int r = 0; r < RP; ++r) {
    const double2 ct = lf[(int)(((long long)r * m) % n)];
    c[r] = ct.x;
    if (r > 0) e[r - 1] = ct.y;
  }
  for (int r = 0; r < H; ++r) e[RP - 1 + r] = (double)(c[r + H] / c[r]);
  double* x = e + RP - 1 + H;
  if constexpr (RP == 16) {
    for (int g = 0; g < 4; ++g) x[g] = (double)(c[g + 4] / c[g]);
    x[4] = (double)c[1];
    x[5] = (double)c[2];
    x[6] = (double)(c[3] / c[1]);
    x[7] = (double)(c[2] * (long double)kC8);
    x[8] = (double)(c[1] * (long double)kC16);
    x[9] = (double)(c[1] * (long double)kC8);
    x[10] = 0.0;  // padding
  } else if constexpr (RP == 8) {
    x[0] = (double)c[2];
    x[1] = (double)c[1];
    x[2] = (double)(c[3] / c[1]);
    x[3] = (double)(c[1] * (long double)kC8);
    x[4] = 0.0;  // padding
  } else if constexpr (RP == 4) {
    x[0] = (double)c[1];
  }
}

template <int RP, bool INV>
GT_HD_INL void dft_lf(double2* a, const double* e) {
  static_assert(RP == 4 || RP == 8 || RP == 16, "carried-scale butterflies exist for radix 4, 8, 16");
  constexpr int H = RP / 2;
  double2 s[H], d[H];
#pragma unroll
  for (int r = 0; r < H; ++r) {
    const double2 lo = (r == 0) ? a[0] : mul_1pit(a[r], INV ? -e[r - 1] : e[r - 1]);
    const double2 hi = mul_1pit(a[r + H], INV ? -e[r + H - 1] : e[r + H - 1]);
    const double rho = e[RP - 1 + r];
    s[r] = fma_c(rho, hi, lo);
    d[r] = fma_c(-rho, hi, lo);
  }
  const double* x = e + RP - 1 + H;
  if constexpr (RP == 4) {
    const double c1 = x[0];
    const double2 t3 = mul_w4<INV>(d[1]);
    a[0] = fma_c(c1, s[1], s[0]); a[2] = fma_c(-c1, s[1], s[0]);
    a[1] = fma_c(c1, t3, d[0]); a[3] = fma_c(-c1, t3, d[0]);
  } else if constexpr (RP == 8) {
    const double c2 = x[0], c1 = x[1], mu = x[2], c1k = x[3];
    const double2 we = mul_w4<INV>(d[2]), wo = mul_w4<INV>(d[3]);
    const double2 e0 = fma_c(c2, s[2], s[0]), e2 = fma_c(-c2, s[2], s[0]);
    const double2 e1 = fma_c(c2, we, d[0]), e3 = fma_c(-c2, we, d[0]);
    const double2 o0 = fma_c(mu, s[3], s[1]), o2 = mul_w4<INV>(fma_c(-mu, s[3], s[1]));
    const double2 o1 = fma_c(mu, wo, d[1]), o3 = fma_c(-mu, wo, d[1]);
    const double2 p1 = w8_1_unscaled<INV>(o1), p3 = w8_3_unscaled<INV>(o3);
    a[0] = fma_c(c1, o0, e0); a[4] = fma_c(-c1, o0, e0);
    a[2] = fma_c(c1, o2, e2); a[6] = fma_c(-c1, o2, e2);
    a[1] = fma_c(c1k, p1, e1); a[5] = fma_c(-c1k, p1, e1);
    a[3] = fma_c(c1k, p3, e3); a[7] = fma_c(-c1k, p3, e3);
  } else {
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) {
      const double sig = x[n1];
      const double2 t3 = mul_w4<INV>(d[n1 + 4]);
      a[n1] = fma_c(sig, s[n1 + 4], s[n1]);
      a[n1 + 8] = fma_c(-sig, s[n1 + 4], s[n1]);
      a[n1 + 4] = fma_c(sig, t3, d[n1]);
      a[n1 + 12] = fma_c(-sig, t3, d[n1]);
    }
    dft16_stage2<INV, true>(a, x + 4);
  }
}

// One Stockham pass (radix RP = min(R, L/Ns)) and, recursively, the rest of the transform.
//   v   : the thread's R values, v[s] = x[t + s*T]; on return X[t + s*T] (natural order)
//   sm  : exchange buffer; element o lives at sm[padix(o) * SS]
//   tw  : twiddle buffer of a length-n table, n = L << twshift: tw[k] = exp(-2 pi i k / n) and
//         tw[n + k] = (c, t) with tw[k] = c (1 + i t), k < n, then the pass tables of dft_lf
//         (lf_pass_table; twiddle_buffer_size(n) double2 in all)
template <int L, int R, int Ns, bool INV, int SS>
struct StockhamPass {
  static constexpr int RP = (L / Ns >= R) ? R : (L / Ns);
  static constexpr bool LAST = (Ns * RP == L);
  static constexpr int T = L / R;
  static constexpr int NB = R / RP;

  __device__ __forceinline__ static void run(double2 (&v)[R], double2* sm, int t,
                                             const double2* __restrict__ tw, int twshift,
                                             bool zband) {
#pragma unroll
    for (int m = 0; m < NB; ++m) {
      const int b = t + m * T;
      const int k = b & (Ns - 1);
      double2 a[RP];
#pragma unroll
      for (int r = 0; r < RP; ++r) a[r] = v[m + r * NB];
      if constexpr (Ns > 1 && RP == 2) {
        const double2 lh = __ldg(&tw[(L << twshift) + ((k * (L / (Ns * 2))) << twshift)]);
        dft_tw<2, INV>(a, nullptr, &lh);
      } else if constexpr (Ns > 1) {
        constexpr int E = lf_entry_doubles(RP);
        const double2* __restrict__ ent = tw + lf_pass_table(RP, L << twshift, Ns) + k;
        double e[E];
#pragma unroll
        for (int q = 0; q < E / 2; ++q) {
          const double2 p = __ldg(&ent[q * Ns]);
          e[2 * q] = p.x;
          e[2 * q + 1] = p.y;
        }
        dft_lf<RP, INV>(a, e);
      } else if (NB == 1 && zband) {
        dft<RP, INV, true>(a);
      } else {
        dft<RP, INV>(a);
      }
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
      StockhamPass<L, R, Ns * RP, INV, SS>::run(v, sm, t, tw, twshift, false);
    }
  }
};

// Full transform of length L held as R values per thread (see StockhamPass). Every thread of
// the block must call it, from the same call site (it contains __syncthreads when L > R).
// zband (uniform over the block): the inputs x[j], j in [3L/8, 5L/8), are zero (see in_zband).
template <int L, int R, bool INV, int SS>
__device__ __forceinline__ void fft_regs(double2 (&v)[R], double2* sm, int t,
                                         const double2* __restrict__ tw, int twshift,
                                         bool zband = false) {
  static_assert((L & (L - 1)) == 0 && L >= R, "L must be a power of two >= R");
  StockhamPass<L, R, 1, INV, SS>::run(v, sm, t, tw, twshift, zband);
}

}  // namespace gt
