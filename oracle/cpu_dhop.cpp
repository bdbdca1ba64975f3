// cpu_dhop.cpp -- TEST INFRASTRUCTURE ONLY: the CPU baseline of the benchmark's reference
// arm and its inputs, with no dependence on the CUDA library.
//
// 1. The seeded synthetic inputs, restated from the library's generator so that the
//    reference arm builds the same gauge field and sources bit for bit without loading
//    the product: SplitMix64 finaliser of an element counter -> Box-Muller normals;
//    U = reunitarise(exp(i eps H)), H the traceless Hermitian part of a complex Gaussian
//    matrix (the role of Grid's GridParallelRNG + SU3::HotConfiguration,
//    Grid/qcd/utils/GaugeGroup.h:331-347).
//
// 2. Grid's CPU hopping-term algorithm for one checkerboard in single precision: per
//    output site and leg, the half-spinor projection (spProj, TwoSpinor.h:75-330), the
//    SU(3) link times the two-spinor (multLink, WilsonImpl.h:66-110), the reconstruction
//    into the accumulator (accumRecon), as in WilsonKernels::GenericDhopSite
//    (WilsonKernelsImplementation.h:57-69,113-163); OpenMP over 4D sites, and the fifth
//    dimension innermost and contiguous so that every link is read once per 4D site and
//    the compiler vectorises over s (Grid's 5D kernels loop s inside the site for the
//    same reuse, WilsonFermion5DImplementation.h:415-451).  Fields are held in a
//    structure-of-arrays layout [x_cb][component][re|im][L5]; conversion from and to the
//    canonical layout is outside the timed call.
#include <omp.h>

#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

using cd = std::complex<double>;

// ---- the seeded generator ----
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
inline double normal(uint64_t seed, uint64_t ctr) {
  const double u1 = uniform01(seed, 2 * ctr), u2 = uniform01(seed, 2 * ctr + 1);
  return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
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
// exp(X): scaling and squaring with an 18-term Taylor core on ||X / 2^k|| <= 1/2
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
// Gram-Schmidt on rows 0, 1; row 2 = conj(row 0 x row 1)
void reunitarise(M3& U) {
  double n0 = 0;
  for (int j = 0; j < 3; j++) n0 += std::norm(U.m[0][j]);
  n0 = 1.0 / std::sqrt(n0);
  for (int j = 0; j < 3; j++) U.m[0][j] *= n0;
  cd dot = 0;
  for (int j = 0; j < 3; j++) dot += std::conj(U.m[0][j]) * U.m[1][j];
  for (int j = 0; j < 3; j++) U.m[1][j] -= dot * U.m[0][j];
  double n1 = 0;
  for (int j = 0; j < 3; j++) n1 += std::norm(U.m[1][j]);
  n1 = 1.0 / std::sqrt(n1);
  for (int j = 0; j < 3; j++) U.m[1][j] *= n1;
  U.m[2][0] = std::conj(U.m[0][1] * U.m[1][2] - U.m[0][2] * U.m[1][1]);
  U.m[2][1] = std::conj(U.m[0][2] * U.m[1][0] - U.m[0][0] * U.m[1][2]);
  U.m[2][2] = std::conj(U.m[0][0] * U.m[1][1] - U.m[0][1] * U.m[1][0]);
}

// ---- the half-spinor Dhop ----
struct Hs {
  int L[4];
  int L5;
  int64_t vol, half;
  // per output parity: doubled links [x_cb][leg][9] (-1/2 and boundary phases folded in,
  // Grid's DoubleStore) and neighbour x_cb of the other parity [x_cb][leg]
  std::vector<std::complex<float>> links[2];
  std::vector<int> nbr[2];
  // per parity: a checkerboard field [x_cb][12][2][L5]
  std::vector<float> field[2];
};

inline void coords(const Hs& h, int64_t site, int x[4]) {
  for (int k = 0; k < 4; k++) {
    x[k] = int(site % h.L[k]);
    site /= h.L[k];
  }
}
inline int64_t lex(const Hs& h, const int x[4]) {
  return x[0] + int64_t(h.L[0]) * (x[1] + int64_t(h.L[1]) * (x[2] + int64_t(h.L[2]) * x[3]));
}

// one leg of one output site over all L5 slots: acc += recon(U * proj(psi))
template <int MU, int S>
inline void hs_leg(const float* __restrict psi, const std::complex<float>* __restrict U, float* __restrict acc, int L5) {
  // psi / acc: [12][2][L5], component k = spin * 3 + colour
  auto P = [&](int k, int ri) { return psi + (k * 2 + ri) * L5; };
  auto A = [&](int k, int ri) { return acc + (k * 2 + ri) * L5; };
  float hbuf[6 * 2 * 64], ubuf[6 * 2 * 64];  // L5 <= 64
  auto H = [&](int k, int ri) { return hbuf + (k * 2 + ri) * L5; };
  auto Uo = [&](int k, int ri) { return ubuf + (k * 2 + ri) * L5; };
  const float s = float(S);
  // projection to the two-spinor h (spins 0, 1)
  for (int c = 0; c < 3; c++) {
    const float *f0r = P(c, 0), *f0i = P(c, 1), *f1r = P(3 + c, 0), *f1i = P(3 + c, 1);
    const float *f2r = P(6 + c, 0), *f2i = P(6 + c, 1), *f3r = P(9 + c, 0), *f3i = P(9 + c, 1);
    float *h0r = H(c, 0), *h0i = H(c, 1), *h1r = H(3 + c, 0), *h1i = H(3 + c, 1);
#pragma omp simd
    for (int i = 0; i < L5; i++) {
      if (MU == 0) {  // h0 = f0 + S i f3, h1 = f1 + S i f2
        h0r[i] = f0r[i] - s * f3i[i]; h0i[i] = f0i[i] + s * f3r[i];
        h1r[i] = f1r[i] - s * f2i[i]; h1i[i] = f1i[i] + s * f2r[i];
      } else if (MU == 1) {  // h0 = f0 - S f3, h1 = f1 + S f2
        h0r[i] = f0r[i] - s * f3r[i]; h0i[i] = f0i[i] - s * f3i[i];
        h1r[i] = f1r[i] + s * f2r[i]; h1i[i] = f1i[i] + s * f2i[i];
      } else if (MU == 2) {  // h0 = f0 + S i f2, h1 = f1 - S i f3
        h0r[i] = f0r[i] - s * f2i[i]; h0i[i] = f0i[i] + s * f2r[i];
        h1r[i] = f1r[i] + s * f3i[i]; h1i[i] = f1i[i] - s * f3r[i];
      } else {  // h0 = f0 + S f2, h1 = f1 + S f3
        h0r[i] = f0r[i] + s * f2r[i]; h0i[i] = f0i[i] + s * f2i[i];
        h1r[i] = f1r[i] + s * f3r[i]; h1i[i] = f1i[i] + s * f3i[i];
      }
    }
  }
  // u = U h for both spins of the two-spinor
  for (int sp = 0; sp < 2; sp++)
    for (int a = 0; a < 3; a++) {
      const float u0r = U[a * 3 + 0].real(), u0i = U[a * 3 + 0].imag();
      const float u1r = U[a * 3 + 1].real(), u1i = U[a * 3 + 1].imag();
      const float u2r = U[a * 3 + 2].real(), u2i = U[a * 3 + 2].imag();
      const float *x0r = H(sp * 3 + 0, 0), *x0i = H(sp * 3 + 0, 1), *x1r = H(sp * 3 + 1, 0), *x1i = H(sp * 3 + 1, 1);
      const float *x2r = H(sp * 3 + 2, 0), *x2i = H(sp * 3 + 2, 1);
      float *yr = Uo(sp * 3 + a, 0), *yi = Uo(sp * 3 + a, 1);
#pragma omp simd
      for (int i = 0; i < L5; i++) {
        yr[i] = u0r * x0r[i] - u0i * x0i[i] + u1r * x1r[i] - u1i * x1i[i] + u2r * x2r[i] - u2i * x2i[i];
        yi[i] = u0r * x0i[i] + u0i * x0r[i] + u1r * x1i[i] + u1i * x1r[i] + u2r * x2i[i] + u2i * x2r[i];
      }
    }
  // reconstruction into the accumulator
  for (int c = 0; c < 3; c++) {
    const float *u0r = Uo(c, 0), *u0i = Uo(c, 1), *u1r = Uo(3 + c, 0), *u1i = Uo(3 + c, 1);
    float *a0r = A(c, 0), *a0i = A(c, 1), *a1r = A(3 + c, 0), *a1i = A(3 + c, 1);
    float *a2r = A(6 + c, 0), *a2i = A(6 + c, 1), *a3r = A(9 + c, 0), *a3i = A(9 + c, 1);
#pragma omp simd
    for (int i = 0; i < L5; i++) {
      a0r[i] += u0r[i]; a0i[i] += u0i[i]; a1r[i] += u1r[i]; a1i[i] += u1i[i];
      if (MU == 0) {  // r2 += -S i u1, r3 += -S i u0
        a2r[i] += s * u1i[i]; a2i[i] -= s * u1r[i]; a3r[i] += s * u0i[i]; a3i[i] -= s * u0r[i];
      } else if (MU == 1) {  // r2 += S u1, r3 -= S u0
        a2r[i] += s * u1r[i]; a2i[i] += s * u1i[i]; a3r[i] -= s * u0r[i]; a3i[i] -= s * u0i[i];
      } else if (MU == 2) {  // r2 += -S i u0, r3 += S i u1
        a2r[i] += s * u0i[i]; a2i[i] -= s * u0r[i]; a3r[i] -= s * u1i[i]; a3i[i] += s * u1r[i];
      } else {  // r2 += S u0, r3 += S u1
        a2r[i] += s * u0r[i]; a2i[i] += s * u0i[i]; a3r[i] += s * u1r[i]; a3i[i] += s * u1i[i];
      }
    }
  }
}

template <int DAG> void hs_dhop(const Hs& h, int out_parity) {
  const std::vector<float>& in = h.field[1 - out_parity];
  std::vector<float>& out = const_cast<std::vector<float>&>(h.field[out_parity]);
  const std::complex<float>* links = h.links[out_parity].data();
  const int* nbr = h.nbr[out_parity].data();
  const int L5 = h.L5;
  const size_t per = size_t(24) * L5;
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < h.half; x++) {
    float* acc = &out[size_t(x) * per];
    std::memset(acc, 0, per * sizeof(float));
    const std::complex<float>* U = links + size_t(x) * 72;
    const int* nb = nbr + size_t(x) * 8;
    constexpr int F = DAG ? 1 : -1, B = -F;  // projector sign of forward / backward legs
    hs_leg<0, F>(&in[size_t(nb[0]) * per], U + 0 * 9, acc, L5);
    hs_leg<1, F>(&in[size_t(nb[1]) * per], U + 1 * 9, acc, L5);
    hs_leg<2, F>(&in[size_t(nb[2]) * per], U + 2 * 9, acc, L5);
    hs_leg<3, F>(&in[size_t(nb[3]) * per], U + 3 * 9, acc, L5);
    hs_leg<0, B>(&in[size_t(nb[4]) * per], U + 4 * 9, acc, L5);
    hs_leg<1, B>(&in[size_t(nb[5]) * per], U + 5 * 9, acc, L5);
    hs_leg<2, B>(&in[size_t(nb[6]) * per], U + 6 * 9, acc, L5);
    hs_leg<3, B>(&in[size_t(nb[7]) * per], U + 7 * 9, acc, L5);
  }
}

}  // namespace

extern "C" {

// canonical U[site][mu][3][3] complex double
void orc_random_gauge(const int* dims, double eps, uint64_t seed, double* U) {
  int64_t vol = 1;
  for (int k = 0; k < 4; k++) vol *= dims[k];
  cd* out = reinterpret_cast<cd*>(U);
#pragma omp parallel for schedule(static)
  for (int64_t link = 0; link < vol * 4; link++) {
    const uint64_t base = uint64_t(link) * 18;
    M3 A, X, H;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        const uint64_t c = base + uint64_t(i * 3 + j) * 2;
        A.m[i][j] = cd(normal(seed, c), normal(seed, c + 1));
      }
    cd tr = 0;
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
  }
}

// n complex numbers with N(0,1) real and imaginary parts
void orc_random_gaussian(int64_t n, uint64_t seed, double* out) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    out[2 * i] = normal(seed, uint64_t(2 * i));
    out[2 * i + 1] = normal(seed, uint64_t(2 * i + 1));
  }
}

// A half-spinor Dhop for the 4D lattice dims with L5 fifth-dimension slots (<= 64):
// canonical U[site][mu][3][3], boundary phases (re, im) x 4.
void* orc_hs_create(const int* dims, int L5, const double* U, const double* phases) {
  if (L5 < 1 || L5 > 64) return nullptr;
  Hs* h = new Hs;
  for (int k = 0; k < 4; k++) h->L[k] = dims[k];
  h->L5 = L5;
  h->vol = int64_t(dims[0]) * dims[1] * dims[2] * dims[3];
  h->half = h->vol / 2;
  const cd* Uc = reinterpret_cast<const cd*>(U);
  cd ph[4];
  for (int k = 0; k < 4; k++) ph[k] = cd(phases[2 * k], phases[2 * k + 1]);
  for (int p = 0; p < 2; p++) {
    h->links[p].assign(size_t(h->half) * 72, 0.f);
    h->nbr[p].assign(size_t(h->half) * 8, 0);
    h->field[p].assign(size_t(h->half) * 24 * L5, 0.f);
  }
  for (int64_t site = 0; site < h->vol; site++) {
    int x[4];
    coords(*h, site, x);
    const int p = (x[0] + x[1] + x[2] + x[3]) & 1;
    const int64_t xcb = site >> 1;
    for (int mu = 0; mu < 4; mu++) {
      int y[4] = {x[0], x[1], x[2], x[3]};
      y[mu] = (x[mu] + 1) % h->L[mu];
      h->nbr[p][size_t(xcb) * 8 + mu] = int(lex(*h, y) >> 1);
      y[mu] = (x[mu] - 1 + h->L[mu]) % h->L[mu];
      const int64_t back = lex(*h, y);
      h->nbr[p][size_t(xcb) * 8 + mu + 4] = int(back >> 1);
      const cd pf = (x[mu] == h->L[mu] - 1) ? ph[mu] : cd(1, 0);
      const cd pb = (x[mu] == 0) ? std::conj(ph[mu]) : cd(1, 0);
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
          h->links[p][(size_t(xcb) * 8 + mu) * 9 + a * 3 + b] =
              std::complex<float>(-0.5 * pf * Uc[(size_t(site) * 4 + mu) * 9 + a * 3 + b]);
          h->links[p][(size_t(xcb) * 8 + mu + 4) * 9 + a * 3 + b] =
              std::complex<float>(-0.5 * pb * std::conj(Uc[(size_t(back) * 4 + mu) * 9 + b * 3 + a]));
        }
    }
  }
  return h;
}
void orc_hs_free(void* p) { delete static_cast<Hs*>(p); }

// canonical checkerboard half (complex double [x_cb][L5][12]) <-> the handle's field of
// that parity (outside the timed call)
void orc_hs_set(void* p, int parity, const double* canon) {
  Hs* h = static_cast<Hs*>(p);
  const int L5 = h->L5;
  float* f = h->field[parity].data();
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < h->half; x++)
    for (int s = 0; s < L5; s++)
      for (int k = 0; k < 12; k++)
        for (int ri = 0; ri < 2; ri++)
          f[((size_t(x) * 12 + k) * 2 + ri) * L5 + s] = float(canon[((size_t(x) * L5 + s) * 12 + k) * 2 + ri]);
}
void orc_hs_get(void* p, int parity, double* canon) {
  const Hs* h = static_cast<const Hs*>(p);
  const int L5 = h->L5;
  const float* f = h->field[parity].data();
#pragma omp parallel for schedule(static)
  for (int64_t x = 0; x < h->half; x++)
    for (int s = 0; s < L5; s++)
      for (int k = 0; k < 12; k++)
        for (int ri = 0; ri < 2; ri++)
          canon[((size_t(x) * L5 + s) * 12 + k) * 2 + ri] = f[((size_t(x) * 12 + k) * 2 + ri) * L5 + s];
}
// Dhop onto the sites of out_parity from the handle's field of the other parity
void orc_hs_dhop(void* p, int out_parity, int dag) {
  const Hs* h = static_cast<const Hs*>(p);
  if (dag) hs_dhop<1>(*h, out_parity);
  else hs_dhop<0>(*h, out_parity);
}

}  // extern "C"
