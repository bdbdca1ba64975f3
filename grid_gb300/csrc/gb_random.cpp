// gb_random.cpp -- seeded synthetic inputs, the role of Grid's GridParallelRNG +
// SU3::HotConfiguration (Grid/qcd/utils/GaugeGroup.h:331-347) for the workloads here.
//
// Every random number is a pure function of (seed, element counter): a SplitMix64
// finaliser of the counter feeds a Box-Muller pair, so the fields do not depend on the
// number of host threads.  Gauge links: A with N(0,1) real and imaginary parts,
// H = (A + A^dagger)/2 - tr/3, U = exp(i eps H) (scaling and squaring with a Taylor
// core), then reunitarised (Gram-Schmidt rows 0,1; row 2 = conj(row0 x row1)), so
// det U = 1 to rounding.
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "gb_internal.h"

namespace {

using cd = std::complex<double>;

inline uint64_t mix64(uint64_t z) {
  z += 0x9e3779b97f4a7c15ull;
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
inline double uniform01(uint64_t seed, uint64_t ctr) {  // (0, 1]
  const uint64_t h = mix64(mix64(seed) ^ ctr);
  return (double((h >> 11) + 1)) * (1.0 / 9007199254740992.0);
}
// standard normal number `ctr`
inline double normal(uint64_t seed, uint64_t ctr) {
  const double u1 = uniform01(seed, 2 * ctr), u2 = uniform01(seed, 2 * ctr + 1);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

template <class F> void parallel_for(int64_t n, F&& f) {
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 1;
  if (nt > 64) nt = 64;
  if (n < 4096) nt = 1;
  std::vector<std::thread> th;
  const int64_t chunk = (n + nt - 1) / nt;
  for (unsigned t = 0; t < nt; t++) {
    const int64_t a = int64_t(t) * chunk, b = std::min<int64_t>(n, a + chunk);
    if (a >= b) break;
    th.emplace_back([a, b, &f]() { for (int64_t i = a; i < b; i++) f(i); });
  }
  for (auto& x : th) x.join();
}

struct M3 {
  cd m[3][3];
};
M3 mul(const M3& a, const M3& b) {
  M3 c;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      cd s = 0;
      for (int k = 0; k < 3; k++) s += a.m[i][k] * b.m[k][j];
      c.m[i][j] = s;
    }
  return c;
}
// exp(X) by scaling and squaring, 18-term Taylor core on ||X/2^k|| <= 1/2
M3 expm(const M3& X) {
  double nrm = 0;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) nrm += std::norm(X.m[i][j]);
  nrm = std::sqrt(nrm);
  int k = 0;
  while (nrm > 0.5) { nrm *= 0.5; k++; }
  const double sc = std::ldexp(1.0, -k);
  M3 Y, term, E;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      Y.m[i][j] = X.m[i][j] * sc;
      term.m[i][j] = (i == j) ? 1.0 : 0.0;
      E.m[i][j] = term.m[i][j];
    }
  for (int n = 1; n <= 18; n++) {
    term = mul(term, Y);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        term.m[i][j] /= double(n);
        E.m[i][j] += term.m[i][j];
      }
  }
  for (int s = 0; s < k; s++) E = mul(E, E);
  return E;
}
void reunitarise(M3& U) {
  // row 0
  double n0 = 0;
  for (int j = 0; j < 3; j++) n0 += std::norm(U.m[0][j]);
  n0 = 1.0 / std::sqrt(n0);
  for (int j = 0; j < 3; j++) U.m[0][j] *= n0;
  // row 1 orthogonal to row 0
  cd dot = 0;
  for (int j = 0; j < 3; j++) dot += std::conj(U.m[0][j]) * U.m[1][j];
  for (int j = 0; j < 3; j++) U.m[1][j] -= dot * U.m[0][j];
  double n1 = 0;
  for (int j = 0; j < 3; j++) n1 += std::norm(U.m[1][j]);
  n1 = 1.0 / std::sqrt(n1);
  for (int j = 0; j < 3; j++) U.m[1][j] *= n1;
  // row 2 = conj(row0 x row1)
  U.m[2][0] = std::conj(U.m[0][1] * U.m[1][2] - U.m[0][2] * U.m[1][1]);
  U.m[2][1] = std::conj(U.m[0][2] * U.m[1][0] - U.m[0][0] * U.m[1][2]);
  U.m[2][2] = std::conj(U.m[0][0] * U.m[1][1] - U.m[0][1] * U.m[1][0]);
}

}  // namespace

extern "C" {

int gb_random_gauge(const int dims[4], double eps, uint64_t seed, double* U) {
  if (!dims || !U) { gb::set_error("null argument"); return GB_ERR_BAD_ARG; }
  int64_t vol = 1;
  for (int k = 0; k < 4; k++) vol *= dims[k];
  cd* out = reinterpret_cast<cd*>(U);
  parallel_for(vol * 4, [&](int64_t link) {
    const uint64_t base = uint64_t(link) * 18;
    M3 A, X;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        const uint64_t c = base + uint64_t(i * 3 + j) * 2;
        A.m[i][j] = cd(normal(seed, c), normal(seed, c + 1));
      }
    // H = (A + A^dag)/2 - tr/3 ; X = i eps H
    cd tr = 0;
    M3 H;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) H.m[i][j] = 0.5 * (A.m[i][j] + std::conj(A.m[j][i]));
    for (int i = 0; i < 3; i++) tr += H.m[i][i];
    for (int i = 0; i < 3; i++) H.m[i][i] -= tr / 3.0;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) X.m[i][j] = cd(0, eps) * H.m[i][j];
    M3 E = expm(X);
    reunitarise(E);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) out[size_t(link) * 9 + i * 3 + j] = E.m[i][j];
  });
  return GB_OK;
}

int gb_unit_gauge(const int dims[4], double* U) {
  if (!dims || !U) { gb::set_error("null argument"); return GB_ERR_BAD_ARG; }
  int64_t vol = 1;
  for (int k = 0; k < 4; k++) vol *= dims[k];
  std::memset(U, 0, size_t(vol) * 4 * 18 * sizeof(double));
  for (int64_t l = 0; l < vol * 4; l++)
    for (int i = 0; i < 3; i++) U[size_t(l) * 18 + (i * 3 + i) * 2] = 1.0;
  return GB_OK;
}

int gb_random_gaussian(size_t n_complex, uint64_t seed, double* out) {
  if (!out) { gb::set_error("null argument"); return GB_ERR_BAD_ARG; }
  parallel_for(int64_t(n_complex), [&](int64_t i) {
    out[2 * i] = normal(seed, uint64_t(2 * i));
    out[2 * i + 1] = normal(seed, uint64_t(2 * i + 1));
  });
  return GB_OK;
}

int gb_random_z2(size_t n_complex, uint64_t seed, double* out) {
  if (!out) { gb::set_error("null argument"); return GB_ERR_BAD_ARG; }
  const double h = 1.0 / std::sqrt(2.0);
  parallel_for(int64_t(n_complex), [&](int64_t i) {
    const uint64_t b = mix64(mix64(seed ^ 0x5a5a5a5aull) ^ uint64_t(i));
    out[2 * i] = (b & 1) ? h : -h;
    out[2 * i + 1] = (b & 2) ? h : -h;
  });
  return GB_OK;
}

}  // extern "C"
