// gb_approx.cpp -- coefficients of the Cayley-form operators with non-Moebius omega_s:
// Zolotarev's optimal rational approximation to sgn(x) on epsilon <= |x| <= 1
// (Grid/algorithms/approx/Zolotarev.cc:296-417, used by MobiusZolotarevFermion.h and
// ShamirZolotarevFermion.h through CayleyFermion5D::SetCoefficientsZolotarev).
//
// With k' = sqrt(1 - epsilon^2), K' = K(k') and the Jacobi functions of modulus k':
//   xi = 1 / dn(K'/n),  c_m = -(cn/sn)^2 at 2K'(m+1)/n,  c'_m = -(cn/sn)^2 at 2K'(m+1/2)/n
//   M = prod (1 - c_m) / (1 - c'_m),  1/lambda = xi prod (1 - c_m xi^2) / (1 - c'_m xi^2) / M
//   Delta = (1/lambda - 1) / (1/lambda + 1)   (the maximum of |R(x) - sgn(x)|)
// and the Cayley form R(x) = (1 - T(x)) / (1 + T(x)), T(x) = prod_j (x - g_j) / (x + g_j)
// (Chiu's domain-wall formulation) has
//   g_j = epsilon / dn(s + 2K'j/n, k'),  s = M F(phi, sqrt(1 - l^2)),  l = lambda,
//   sin^2 phi = (1 + 3l) / (1 + l)^3 (type 0) or (3 + l) / (4(1 + l)) (type 1).
// Elliptic functions are our own: Carlson's symmetric integral R_F by duplication
// (DLMF 19.36.1) for K and F, and the AGM / descending Landen recursion (DLMF 22.20.1,
// Abramowitz-Stegun 16.4) for sn, cn, dn.
#include <cmath>
#include <vector>

#include "gbdwf.h"
#include "gb_internal.h"

namespace {

// Carlson's R_F(x, y, z), x, y, z >= 0, at most one zero
double carlson_rf(double x, double y, double z) {
  for (int it = 0; it < 200; it++) {
    const double sx = std::sqrt(x), sy = std::sqrt(y), sz = std::sqrt(z);
    const double lam = sx * (sy + sz) + sy * sz;
    x = 0.25 * (x + lam);
    y = 0.25 * (y + lam);
    z = 0.25 * (z + lam);
    const double mu = (x + y + z) / 3.0;
    const double dx = 1.0 - x / mu, dy = 1.0 - y / mu, dz = 1.0 - z / mu;
    if (std::fmax(std::fabs(dx), std::fmax(std::fabs(dy), std::fabs(dz))) < 1e-4) {
      const double e2 = dx * dy - dz * dz, e3 = dx * dy * dz;
      return (1.0 - e2 / 10.0 + e3 / 14.0 + e2 * e2 / 24.0 - 3.0 * e2 * e3 / 44.0) / std::sqrt(mu);
    }
  }
  return (1.0) / std::sqrt((x + y + z) / 3.0);
}

// K(k) and F(phi, k), 0 <= phi <= pi/2
double ellip_k(double k) { return carlson_rf(0.0, 1.0 - k * k, 1.0); }
double ellip_f(double phi, double k) {
  const double s = std::sin(phi), c = std::cos(phi);
  return s * carlson_rf(c * c, 1.0 - k * k * s * s, 1.0);
}

// sn, cn, dn (u, k) by the AGM and the descending recursion of the amplitude
void sncndn(double u, double k, double& sn, double& cn, double& dn) {
  const int kmax = 40;
  double a[kmax + 1], c[kmax + 1];
  a[0] = 1.0;
  double b = std::sqrt(1.0 - k * k);
  c[0] = k;
  int n = 0;
  while (n < kmax && std::fabs(c[n]) > 1e-17 * a[n]) {
    a[n + 1] = 0.5 * (a[n] + b);
    c[n + 1] = 0.5 * (a[n] - b);
    b = std::sqrt(a[n] * b);
    n++;
  }
  double phi = std::ldexp(a[n] * u, n);
  double phi_prev = phi;
  for (int j = n; j > 0; j--) {
    phi_prev = phi;
    phi = 0.5 * (phi + std::asin(c[j] / a[j] * std::sin(phi)));
  }
  sn = std::sin(phi);
  cn = std::cos(phi);
  dn = n > 0 ? cn / std::cos(phi_prev - phi) : 1.0;
}

}  // namespace

extern "C" {

int gb_zolotarev(double epsilon, int n, int type, double* gamma, double* delta) {
  using gb::set_error;
  if (!gamma) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (!(epsilon > 0.0 && epsilon < 1.0) || n < 1 || (type != 0 && type != 1)) {
    set_error("zolotarev: need 0 < epsilon < 1, n >= 1, type 0 or 1");
    return GB_ERR_BAD_ARG;
  }
  const double ksq = epsilon * epsilon;
  const double kp = std::sqrt(1.0 - ksq);
  const double Kp = ellip_k(kp);
  const double z0 = 2.0 * Kp / double(n);
  double sn, cn, dn;
  sncndn(0.5 * z0, kp, sn, cn, dn);
  const double xi = 1.0 / dn, xisq = xi * xi;
  double M = 1.0, invlambda = xi;
  for (int m = 0; m < n / 2; m++) {
    sncndn(z0 * (m + 1.0), kp, sn, cn, dn);
    const double c = -(cn / sn) * (cn / sn);
    sncndn(z0 * (m + 0.5), kp, sn, cn, dn);
    const double cp = -(cn / sn) * (cn / sn);
    M *= (1.0 - c) / (1.0 - cp);
    invlambda *= (1.0 - c * xisq) / (1.0 - cp * xisq);
  }
  invlambda /= M;
  const double l = 1.0 / invlambda, opl = 1.0 + l;
  const double s2 = type == 1 ? (3.0 + l) / (4.0 * opl) : (1.0 + 3.0 * l) / (opl * opl * opl);
  const double phi = std::asin(std::sqrt(std::fmin(1.0, s2)));
  const double s = M * ellip_f(phi, std::sqrt(1.0 - l * l));
  for (int m = 0; m < n; m++) {
    sncndn(s + 2.0 * Kp * m / double(n), kp, sn, cn, dn);
    gamma[m] = epsilon / dn;
  }
  if (delta) *delta = (invlambda - 1.0) / (invlambda + 1.0);
  return GB_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Approx::computeZmobiusGamma (Grid/algorithms/approx/ZMobius.cc:73-183): the ZMobius
// omega_s of Ls_out slices that best approximate (in the minimax sense on 0 <= x <=
// lambda) the Moebius sign function of Ls_in slices with b + c = bpc_in,
//   eps_in(x) = (f(x) - f(-x)) / (f(x) + f(-x)),  f(x) = (1 / bpc_in + x)^Ls_in,
// by R(x) = N(x) / D(x), N odd of degree Ls_out - 1, D even and monic of degree Ls_out.
// Then f_out = D + N = prod_s (x + omega_s): the omegas are minus its roots, sorted by
// (real, imaginary) part and placed largest-first alternately from the two ends of the
// fifth dimension, and gamma_s = bpc_out * omega_s.
// Our method: the rational Remez exchange in long double (the levelled equations
// N(x_k) - eps(x_k) D(x_k) = (-1)^k E D(x_k), linearised in E by the previous D, then a
// new alternating set of error extrema on a fine grid), and Aberth's simultaneous
// iteration for the roots.
// ---------------------------------------------------------------------------------------
#include <algorithm>
#include <complex>

namespace {

using LD = long double;

LD eps_mobius(LD x, LD omega, int Ls) {
  const LD r = std::pow((omega - x) / (omega + x), LD(Ls));
  return (1 - r) / (1 + r);
}

// Gaussian elimination with partial pivoting; false when singular
bool solve_dense(std::vector<LD>& A, std::vector<LD>& b, int n) {
  for (int c = 0; c < n; c++) {
    int piv = c;
    for (int r = c + 1; r < n; r++)
      if (std::fabs(A[size_t(r) * n + c]) > std::fabs(A[size_t(piv) * n + c])) piv = r;
    if (A[size_t(piv) * n + c] == 0) return false;
    if (piv != c) {
      for (int k = 0; k < n; k++) std::swap(A[size_t(c) * n + k], A[size_t(piv) * n + k]);
      std::swap(b[c], b[piv]);
    }
    for (int r = c + 1; r < n; r++) {
      const LD f = A[size_t(r) * n + c] / A[size_t(c) * n + c];
      if (f == 0) continue;
      for (int k = c; k < n; k++) A[size_t(r) * n + k] -= f * A[size_t(c) * n + k];
      b[r] -= f * b[c];
    }
  }
  for (int r = n - 1; r >= 0; r--) {
    LD s = b[r];
    for (int k = r + 1; k < n; k++) s -= A[size_t(r) * n + k] * b[k];
    b[r] = s / A[size_t(r) * n + r];
  }
  return true;
}

struct Rational {  // N(x) = sum a[j] x^(2j+1), D(x) = x^L + sum d[j] x^(2j)
  int L;
  std::vector<LD> a, d;
  LD num(LD x) const {
    LD s = 0, p = x, x2 = x * x;
    for (LD c : a) { s += c * p; p *= x2; }
    return s;
  }
  LD den(LD x) const {
    LD s = 0, p = 1, x2 = x * x;
    for (LD c : d) { s += c * p; p *= x2; }
    return s + p;  // p = x^L after L/2 steps
  }
  LD eval(LD x) const { return num(x) / den(x); }
};

}  // namespace

extern "C" int gb_zmobius_gamma(int Ls_out, double bpc_out, int Ls_in, double bpc_in, double lambda_bound,
                                double* gamma, double* max_error) {
  using gb::set_error;
  if (!gamma) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (Ls_out < 2 || (Ls_out & 1) || Ls_out > 32 || Ls_in < 1 || !(bpc_in > 0) || !(bpc_out > 0) || !(lambda_bound > 0)) {
    set_error("computeZmobiusGamma: need even 2 <= Ls_out <= 32, Ls_in >= 1, b+c > 0, lambda > 0");
    return GB_ERR_BAD_ARG;
  }
  const int L = Ls_out, h = L / 2, n = L + 1;  // unknowns: a[h], d[h], E
  const LD omega = LD(1) / LD(bpc_in), lam = LD(lambda_bound);
  auto target = [&](LD x) { return eps_mobius(x, omega, Ls_in); };
  // error grid: dense near 0, where the sign function turns over
  const int G = 20000;
  std::vector<LD> xs(G);
  for (int i = 0; i < G; i++) {
    const LD t = LD(i + 1) / LD(G);
    xs[i] = lam * (LD(0.5) * t * t + LD(0.5) * t);
  }
  std::vector<LD> pts(n);
  for (int k = 0; k < n; k++) {
    const LD t = std::sin(LD(M_PI) * LD(k + 1) / LD(2 * n));
    pts[k] = lam * t * t;
  }
  Rational R{L, std::vector<LD>(h, 0), std::vector<LD>(h, 0)};
  LD E = 0, maxerr = 0;
  bool ok = false;
  for (int iter = 0; iter < 200; iter++) {
    // the levelled equations, E linearised by the previous denominator
    for (int inner = 0; inner < 50; inner++) {
      std::vector<LD> A(size_t(n) * n, 0), b(n, 0);
      for (int k = 0; k < n; k++) {
        const LD x = pts[k], x2 = x * x, ek = target(x), sk = (k & 1) ? -1 : 1;
        const LD dold = inner == 0 && iter == 0 ? std::pow(x, LD(L)) + 1 : R.den(x);
        LD p = x;
        for (int j = 0; j < h; j++) { A[size_t(k) * n + j] = p; p *= x2; }
        p = 1;
        for (int j = 0; j < h; j++) { A[size_t(k) * n + h + j] = -ek * p; p *= x2; }
        A[size_t(k) * n + L] = -sk * dold;
        b[k] = ek * std::pow(x, LD(L));
      }
      if (!solve_dense(A, b, n)) { set_error("computeZmobiusGamma: singular Remez system"); return GB_ERR_UNSUPPORTED; }
      for (int j = 0; j < h; j++) { R.a[j] = b[j]; R.d[j] = b[h + j]; }
      const LD Enew = b[L];
      const bool settled = std::fabs(Enew - E) <= LD(1e-12) * std::fabs(Enew);
      E = Enew;
      if (settled) break;
    }
    // the extrema of the error, one per run of constant sign, the largest L+1 kept in order
    std::vector<int> ext;
    std::vector<LD> err(G);
    for (int i = 0; i < G; i++) err[i] = R.eval(xs[i]) - target(xs[i]);
    int best = 0;
    for (int i = 1; i <= G; i++) {
      if (i == G || (err[i] > 0) != (err[best] > 0)) {
        ext.push_back(best);
        if (i < G) best = i;
      } else if (std::fabs(err[i]) > std::fabs(err[best])) {
        best = i;
      }
    }
    while (int(ext.size()) > n) {  // drop the smaller end, keeping the alternation
      if (std::fabs(err[ext.front()]) < std::fabs(err[ext.back()])) ext.erase(ext.begin());
      else ext.pop_back();
    }
    maxerr = 0;
    for (int i = 0; i < G; i++) maxerr = std::max(maxerr, std::fabs(err[i]));
    if (int(ext.size()) < n) { set_error("computeZmobiusGamma: fewer than %d alternation points", n); return GB_ERR_UNSUPPORTED; }
    LD mn = std::fabs(err[ext[0]]);
    for (int k = 0; k < n; k++) { pts[k] = xs[ext[k]]; mn = std::min(mn, std::fabs(err[ext[k]])); }
    if (maxerr - mn <= LD(1e-6) * maxerr) { ok = true; break; }
  }
  if (!ok) { set_error("computeZmobiusGamma: the Remez exchange did not settle"); return GB_ERR_NOT_CONVERGED; }
  // roots of c(x) = D(x) + N(x) (monic, degree L) by Aberth's iteration
  std::vector<LD> c(L + 1, 0);  // c[i] = coefficient of x^i
  for (int j = 0; j < h; j++) { c[2 * j] = R.d[j]; c[2 * j + 1] = R.a[j]; }
  c[L] = 1;
  using CX = std::complex<LD>;
  auto peval = [&](CX z, CX& dp) {
    CX p = c[L];
    dp = 0;
    for (int i = L - 1; i >= 0; i--) { dp = dp * z + p; p = p * z + c[i]; }
    return p;
  };
  LD radius = 0;
  for (int i = 0; i < L; i++) radius = std::max(radius, std::pow(std::fabs(c[i]), LD(1) / LD(L - i)));
  std::vector<CX> z(L);
  for (int i = 0; i < L; i++) z[i] = std::polar(radius, LD(2 * M_PI) * (LD(i) + LD(0.25)) / LD(L));
  for (int it = 0; it < 500; it++) {
    LD move = 0;
    for (int i = 0; i < L; i++) {
      CX dp;
      const CX p = peval(z[i], dp);
      if (p == CX(0)) continue;
      const CX w = p / dp;
      CX s = 0;
      for (int j = 0; j < L; j++)
        if (j != i) s += LD(1) / (z[i] - z[j]);
      const CX step = w / (LD(1) - w * s);
      z[i] -= step;
      move = std::max(move, std::abs(step) / std::max(LD(1e-300), std::abs(z[i])));
    }
    if (move < LD(1e-17)) break;
  }
  std::vector<CX> om(L);
  for (int i = 0; i < L; i++) om[i] = -z[i];
  std::sort(om.begin(), om.end(), [](const CX& a, const CX& b) {
    return a.real() < b.real() || (a.real() == b.real() && a.imag() < b.imag());
  });
  // largest first, alternately from the two ends (ZMobius.cc:130-141)
  std::vector<CX> placed(L);
  int lo = 0, hi = L - 1, ss = 0;
  for (int from = L - 1; from >= 0; from--, ss++) placed[(ss % 2 == 0) ? lo++ : hi--] = om[from];
  for (int s = 0; s < L; s++) {
    gamma[2 * s] = double(placed[s].real() * LD(bpc_out));
    gamma[2 * s + 1] = double(placed[s].imag() * LD(bpc_out));
  }
  if (max_error) *max_error = double(maxerr);
  return GB_OK;
}
