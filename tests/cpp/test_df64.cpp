// Host check of the double-float arithmetic of the FP64 hopping term
// (grid_gb300/csrc/gb_df64.cuh, compiled here by g++): the integer split and widening,
// sums and Dot2 products against long double, on random values over 80 binades.
#include "gb_df64.cuh"

#include <cmath>
#include <cstdio>
#include <random>

using gb::dfloat;
using gb::DfDot;

static int failures = 0;
static void expect(bool ok, const char* what, double got, double bound) {
  if (!ok && failures++ < 10) std::printf("FAIL %s: %.3e > %.3e\n", what, got, bound);
}

int main() {
  std::mt19937_64 rng(20251204);
  std::normal_distribution<double> nd(0.0, 1.0);
  auto draw = [&]() { return nd(rng) * std::ldexp(1.0, int(rng() % 80) - 40); };
  const double u48 = std::ldexp(1.0, -48);
  double w_split = 0, w_round = 0, w_sum = 0, w_dot = 0;

  // split: hi is the double rounded to a float, hi + lo within 2^-48 of it; widening is exact
  for (int i = 0; i < 1000000; i++) {
    const double d = draw();
    const dfloat s = gb::df::split(d);
    const long double err = std::fabs((long double)s.hi + (long double)s.lo - (long double)d) / std::fabs(d);
    w_split = std::fmax(w_split, double(err));
    expect(err <= u48, "split", double(err), u48);
    expect(std::fabs(double(s.hi) - d) <= std::ldexp(std::fabs(d), -24), "split hi", std::fabs(double(s.hi) - d), 0);
    expect(gb::df::widen(s.hi) == double(s.hi) && gb::df::widen(s.lo) == double(s.lo), "widen", 0, 0);
    const double back = gb::df::to_double(s);
    w_round = std::fmax(w_round, std::fabs(back - d) / std::fabs(d));
    expect(std::fabs(back - d) <= u48 * std::fabs(d), "round trip", std::fabs(back - d) / std::fabs(d), u48);
  }
  {
    const dfloat z = gb::df::split(0.0), m = gb::df::split(-0.0);
    expect(z.hi == 0.f && z.lo == 0.f && m.hi == 0.f && m.lo == 0.f && std::signbit(m.hi), "zero", 0, 0);
    expect(gb::df::to_double(z) == 0.0, "zero back", 0, 0);
    const dfloat t = gb::df::split(1e-30);  // below 2^-74: hi alone, lo dropped
    expect(std::fabs(double(t.hi) - 1e-30) <= 1e-30 * std::ldexp(1.0, -24) && t.lo == 0.f, "tiny", 0, 0);
    const dfloat u = gb::df::split(-1e-40);  // below 2^-126: a signed zero
    expect(u.hi == 0.f && std::signbit(u.hi) && u.lo == 0.f, "below float range", 0, 0);
    const double inf = HUGE_VAL;
    expect(std::isinf(gb::df::split(inf).hi) && std::isinf(gb::df::split(1e300).hi), "overflow", 0, 0);
    expect(std::isnan(gb::df::split(std::nan("")).hi), "nan", 0, 0);
    expect(std::isnan(gb::df::widen(std::nanf(""))) && std::isinf(gb::df::widen(HUGE_VALF)), "widen special", 0, 0);
    expect(gb::df::widen(-0.f) == 0.0 && std::signbit(gb::df::widen(-0.f)), "widen zero", 0, 0);
    for (double d : {std::ldexp(1.0, -74), std::ldexp(1.0, -73) * 1.3, std::ldexp(1.0, 126) * 1.7, -std::ldexp(1.0, -60)}) {
      const dfloat s = gb::df::split(d);
      expect(std::fabs((long double)s.hi + s.lo - d) <= std::ldexp(std::fabs(d), -48), "range ends", d, 0);
    }
  }

  // sums as the Dhop chains them: one projection a +- b, then eight accumulations
  for (int i = 0; i < 200000; i++) {
    double v[16];
    long double exact = 0, mag = 0;
    dfloat acc(0);
    for (int k = 0; k < 8; k++) {
      v[2 * k] = nd(rng);
      v[2 * k + 1] = nd(rng);
      const dfloat h = gb::df::split(v[2 * k]) - gb::df::split(v[2 * k + 1]);
      acc = k == 0 ? h : acc + h;
      exact += (long double)v[2 * k] - (long double)v[2 * k + 1];
      mag += std::fabs((long double)v[2 * k]) + std::fabs((long double)v[2 * k + 1]);
    }
    const double err = double(std::fabs((long double)gb::df::to_double(acc) - exact) / mag);
    w_sum = std::fmax(w_sum, err);
    expect(err <= 6 * u48, "sum chain", err, 6 * u48);
  }

  // the SU(3) row: six real products of mixed sign, as su3_mul forms them
  for (int i = 0; i < 200000; i++) {
    double a[6], b[6];
    long double exact = 0, mag = 0;
    DfDot dot;
    for (int k = 0; k < 6; k++) {
      a[k] = nd(rng);
      b[k] = nd(rng);
      const dfloat x = gb::df::split(a[k]), y = gb::df::split(b[k]);
      if (k == 0) dot.first(x, y); else dot.mac(x, y);
      exact += (long double)a[k] * (long double)b[k];
      mag += std::fabs((long double)a[k] * (long double)b[k]);
    }
    const double err = double(std::fabs((long double)gb::df::to_double(dot.result()) - exact) / mag);
    w_dot = std::fmax(w_dot, err);
    expect(err <= 8 * u48, "dot", err, 8 * u48);
  }

  // a hopping-term site as the kernel forms it: eight legs of (two-spinor = f_a -+ f_b,
  // projected in double, then split) x (3x3 complex link in double-float), accumulated in
  // double-float; relative L2 error over many sites against long double
  long double e2 = 0, n2 = 0;
  for (int site = 0; site < 20000; site++) {
    long double xr[6] = {}, xi[6] = {};
    dfloat ar[6], ai[6];
    for (int leg = 0; leg < 8; leg++) {
      double U[18], f[24];
      for (double& x : U) x = 0.5 * nd(rng);
      for (double& x : f) x = nd(rng);
      dfloat hr[6], hi[6];
      long double lr[6], li[6];
      for (int k = 0; k < 6; k++) {
        hr[k] = gb::df::split(f[4 * k] - f[4 * k + 1]);
        hi[k] = gb::df::split(f[4 * k + 2] + f[4 * k + 3]);
        lr[k] = (long double)f[4 * k] - f[4 * k + 1];
        li[k] = (long double)f[4 * k + 2] + f[4 * k + 3];
      }
      for (int sp = 0; sp < 2; sp++)
        for (int a = 0; a < 3; a++) {
          DfDot re, im;
          long double er = 0, ei = 0;
          for (int b = 0; b < 3; b++) {
            const dfloat ur = gb::df::split(U[(a * 3 + b) * 2]), ui = gb::df::split(U[(a * 3 + b) * 2 + 1]);
            const dfloat vr = hr[sp * 3 + b], vi = hi[sp * 3 + b];
            if (b == 0) { re.first(ur, vr); im.first(ur, vi); } else { re.mac(ur, vr); im.mac(ur, vi); }
            re.mac(-ui, vi);
            im.mac(ui, vr);
            er += (long double)U[(a * 3 + b) * 2] * lr[sp * 3 + b] - (long double)U[(a * 3 + b) * 2 + 1] * li[sp * 3 + b];
            ei += (long double)U[(a * 3 + b) * 2] * li[sp * 3 + b] + (long double)U[(a * 3 + b) * 2 + 1] * lr[sp * 3 + b];
          }
          const int o = sp * 3 + a;
          ar[o] = leg == 0 ? re.result() : ar[o] + re.result();
          ai[o] = leg == 0 ? im.result() : ai[o] + im.result();
          xr[o] += er;
          xi[o] += ei;
        }
    }
    for (int o = 0; o < 6; o++) {
      const long double dr = (long double)gb::df::to_double(ar[o]) - xr[o];
      const long double di = (long double)gb::df::to_double(ai[o]) - xi[o];
      e2 += dr * dr + di * di;
      n2 += xr[o] * xr[o] + xi[o] * xi[o];
    }
  }
  const double site_l2 = double(std::sqrt(e2 / n2));
  expect(site_l2 <= 1e-14, "site relative L2", site_l2, 1e-14);
  std::printf("hopping-term sites: relative L2 error %.2e\n", site_l2);
  std::printf("worst relative errors / 2^-48: split %.2f, round trip %.2f, sum chain %.2f, dot %.2f\n",
              w_split / u48, w_round / u48, w_sum / u48, w_dot / u48);
  if (failures) {
    std::printf("FAILED (%d)\n", failures);
    return 1;
  }
  std::printf("PASSED\n");
  return 0;
}
