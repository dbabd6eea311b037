// Host check of the register butterflies of gt_fft.cuh against a naive DFT (built and run by
// tests/test_fft_kernels.py; test infrastructure only).
#include <cmath>
#include <cstdio>
#include <random>
#include <vector>

#include "../../gturbo_gb300/csrc/gt_fft.cuh"

template <int R, bool INV>
static double check(std::mt19937_64& rng) {
  std::normal_distribution<double> nd;
  double worst = 0.0;
  for (int trial = 0; trial < 50; ++trial) {
    double2 a[R], x[R];
    for (int k = 0; k < R; ++k) x[k] = a[k] = make_double2(nd(rng), nd(rng));
    gt::dft<R, INV>(a);
    const double sgn = INV ? 1.0 : -1.0;
    for (int k = 0; k < R; ++k) {
      long double re = 0, im = 0;
      for (int n = 0; n < R; ++n) {
        const long double ang = sgn * 2.0L * 3.14159265358979323846264338327950288L * (long double)((k * n) % R) / R;
        re += x[n].x * cosl(ang) - x[n].y * sinl(ang);
        im += x[n].x * sinl(ang) + x[n].y * cosl(ang);
      }
      const double err = std::hypot((double)(a[k].x - re), (double)(a[k].y - im));
      worst = std::fmax(worst, err);
    }
  }
  return worst;
}

// The twiddled butterfly of the Stockham passes, dft_tw, against a naive DFT of the twiddled
// inputs a_r w^r (conjugated for the inverse), for twiddles w = exp(-2 pi i k / n) built the way
// the solver's table is (including the angles pi/2 and 3pi/2, whose cosine is 0).
template <int R, bool INV>
static double check_twiddled(std::mt19937_64& rng) {
  std::normal_distribution<double> nd;
  const int n = 64 * R;
  double worst = 0.0;
  for (int k = 0; k < 64; ++k) {
    double2 a[R], x[R], wl[R / 2], lh[R / 2];
    for (int r = 0; r < R; ++r) x[r] = a[r] = make_double2(nd(rng), nd(rng));
    auto tw = [&](int m, double2& w, double2& lf) {
      m %= n;
      const long double ang = -2.0L * 3.14159265358979323846264338327950288L * (long double)m / n;
      double c = (m == n / 4 || m == 3 * n / 4) ? 0.0 : (double)cosl(ang);
      double s = (m == 0 || m == n / 2) ? 0.0 : (double)sinl(ang);
      w = make_double2(c, s);
      const double cl = c != 0.0 ? c : std::ldexp(1.0, -60);
      lf = make_double2(cl, s / cl);
    };
    double2 dummy;
    for (int r = 0; r < R / 2; ++r) {
      tw(r * k, wl[r], dummy);
      tw((r + R / 2) * k, dummy, lh[r]);
    }
    gt::dft_tw<R, INV>(a, wl, lh);
    const long double sg = INV ? 1.0L : -1.0L, pi2 = 2.0L * 3.14159265358979323846264338327950288L;
    for (int q = 0; q < R; ++q) {
      long double re = 0, im = 0;
      for (int r = 0; r < R; ++r) {
        // twiddle w^r = exp(sg i 2 pi r k / n), then the DFT kernel exp(sg i 2 pi q r / R)
        const long double ang = sg * pi2 * ((long double)(r * k % n) / n + (long double)((q * r) % R) / R);
        re += x[r].x * cosl(ang) - x[r].y * sinl(ang);
        im += x[r].x * sinl(ang) + x[r].y * cosl(ang);
      }
      worst = std::fmax(worst, std::hypot((double)(a[q].x - re), (double)(a[q].y - im)));
    }
  }
  return worst;
}

// The carried-scale butterflies dft_lf against a naive DFT of the twiddled inputs a_r w^(r m),
// with the pass-table entries made by the solver's own make_lf_entry from a Linzer-Feig table
// (c, t) built like the solver's, over every base angle m of a length-n table.
template <int R, bool INV>
static double check_lf(std::mt19937_64& rng, int n) {
  std::normal_distribution<double> nd;
  const long double pi2 = 2.0L * 3.14159265358979323846264338327950288L;
  std::vector<double2> lf(n);
  for (int k = 0; k < n; ++k) {
    const long double ang = -pi2 * (long double)k / n;
    const double c = (k == n / 4 || k == 3 * n / 4) ? 0.0 : (double)cosl(ang);
    const double sn = (k == 0 || k == n / 2) ? 0.0 : (double)sinl(ang);
    const double cl = c != 0.0 ? c : std::ldexp(1.0, -60);
    lf[k] = make_double2(cl, sn / cl);
  }
  double worst = 0.0;
  for (int m = 0; m < n / R; ++m) {
    double e[gt::lf_entry_doubles(R)];
    gt::make_lf_entry<R>(lf.data(), n, m, e);
    double2 a[R], x[R];
    for (int r = 0; r < R; ++r) x[r] = a[r] = make_double2(nd(rng), nd(rng));
    gt::dft_lf<R, INV>(a, e);
    const long double sg = INV ? 1.0L : -1.0L;
    for (int q = 0; q < R; ++q) {
      long double re = 0, im = 0;
      for (int r = 0; r < R; ++r) {
        const long double ang = sg * pi2 * ((long double)((long long)r * m % n) / n + (long double)((q * r) % R) / R);
        re += x[r].x * cosl(ang) - x[r].y * sinl(ang);
        im += x[r].x * sinl(ang) + x[r].y * cosl(ang);
      }
      worst = std::fmax(worst, std::hypot((double)(a[q].x - re), (double)(a[q].y - im)));
    }
  }
  return worst;
}

// twmul (a w forward, a conj(w) inverse) and pack_c2r (s + i conj(w) d) against long double
static double check_products(std::mt19937_64& rng) {
  std::normal_distribution<double> nd;
  double worst = 0.0;
  for (int trial = 0; trial < 1000; ++trial) {
    const double2 a = make_double2(nd(rng), nd(rng)), sv = make_double2(nd(rng), nd(rng));
    const double th = 6.283185307179586 * (trial + 0.5) / 1000.0;
    const double2 w = make_double2(std::cos(th), -std::sin(th));
    const long double ax = a.x, ay = a.y, wx = w.x, wy = w.y;
    const double2 f = gt::twmul<false>(a, w), b = gt::twmul<true>(a, w), p = gt::pack_c2r(sv, a, w);
    // conj(w) a = (wx ax + wy ay, wx ay - wy ax); i conj(w) a = (-(wx ay - wy ax), wx ax + wy ay)
    const long double e[6] = {f.x - (ax * wx - ay * wy), f.y - (ax * wy + ay * wx),
                              b.x - (wx * ax + wy * ay), b.y - (wx * ay - wy * ax),
                              p.x - (sv.x - (wx * ay - wy * ax)), p.y - (sv.y + (wx * ax + wy * ay))};
    for (long double d : e) worst = std::fmax(worst, (double)fabsl(d));
  }
  return worst;
}

int main() {
  std::mt19937_64 rng(7);
  const double e[8] = {check<2, false>(rng), check<2, true>(rng), check<4, false>(rng), check<4, true>(rng),
                       check<8, false>(rng), check<8, true>(rng), check<16, false>(rng), check<16, true>(rng)};
  const char* names[8] = {"2f", "2i", "4f", "4i", "8f", "8i", "16f", "16i"};
  int bad = 0;
  for (int k = 0; k < 8; ++k) {
    std::printf("radix %s max err %.3e\n", names[k], e[k]);
    if (!(e[k] < 1e-14)) bad = 1;
  }
  const double et[8] = {check_twiddled<2, false>(rng), check_twiddled<2, true>(rng),
                        check_twiddled<4, false>(rng), check_twiddled<4, true>(rng),
                        check_twiddled<8, false>(rng), check_twiddled<8, true>(rng),
                        check_twiddled<16, false>(rng), check_twiddled<16, true>(rng)};
  for (int k = 0; k < 8; ++k) {
    std::printf("twiddled radix %s max err %.3e\n", names[k], et[k]);
    if (!(et[k] < 1e-14)) bad = 1;
  }
  // every base angle of the tables of n = 64 .. 8192 (radix 16, 8, 4; forward and inverse)
  double el = 0.0;
  for (int n = 64; n <= 8192; n *= 2) {
    const double v[6] = {check_lf<16, false>(rng, n), check_lf<16, true>(rng, n), check_lf<8, false>(rng, n),
                         check_lf<8, true>(rng, n), check_lf<4, false>(rng, n), check_lf<4, true>(rng, n)};
    for (double x : v) el = std::fmax(el, x);
  }
  std::printf("carried-scale radix 16/8/4 max err %.3e\n", el);
  if (!(el < 1e-14)) bad = 1;
  const double ep = check_products(rng);
  std::printf("twmul / pack_c2r max err %.3e\n", ep);
  if (!(ep < 1e-14)) bad = 1;
  return bad;
}
