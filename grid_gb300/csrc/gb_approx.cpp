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
