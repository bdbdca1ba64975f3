// oracle.hpp -- CPU restatement of Grid's Wilson / Moebius domain-wall fermion hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA library is compared
// against; the product never links, loads or calls it.  Only tests/, the smoke check and
// the CPU-baseline leg of bench.py use it.
//
// Parity pinning: Grid cannot be compiled in this environment (it needs Eigen, OpenSSL,
// GMP/MPFR and autotools, none of which are present), and Grid ships no golden data files.
// The restatement is therefore pinned by the known-answer tests that Grid's own test
// programs hold for this path (see tests/test_oracle_pins.py):
//   * DoubleStore + site-loop Dhop equals the naive Cshift formula
//       (benchmarks/Benchmark_dwf.cc:145-158, 222-232; dagger :235-261)
//   * DhopEO (+) DhopOE == Dhop                 (benchmarks/Benchmark_dwf.cc:329-356)
//   * Meo+Moe+Mee+Moo == M, adjointness of Mooee/Meooe, MooeeInv.Mooee == 1,
//     MpcDagMpc Hermitian                       (tests/core/Test_mobius_even_odd.cc)
//   * free-field (U = 1) propagator against the momentum-space formula
//       (tests/core/Test_fft.cc:159,313; WilsonFermionImplementation.h:177-230)
//   * mixed-precision CG agrees with FP64 CG   (tests/Test_dwf_mixedcg_prec.cc:215)
//
// Conventions (all restated from the reference, file:line in the reference checkout):
//   gamma basis            Grid/qcd/spin/TwoSpinor.h:67-140
//   leg order / dagger     Grid/qcd/action/fermion/implementation/WilsonKernelsImplementation.h:113-163
//   DoubleStore + phases   Grid/qcd/action/fermion/WilsonImpl.h:127-171
//   -1/2 link scaling      Grid/qcd/action/fermion/implementation/WilsonFermionImplementation.h:82-107
//   diag_mass = 4 + m      Grid/qcd/action/fermion/implementation/WilsonFermionImplementation.h:69-72
//   5D parity, DW          Grid/qcd/action/fermion/WilsonFermion5D.h:37-61,
//                          Grid/qcd/action/fermion/implementation/WilsonFermion5DImplementation.h:447-451
//   Cayley coefficients    Grid/qcd/action/fermion/implementation/CayleyFermion5DImplementation.h:155-271,410-535
//   M5D / MooeeInv         Grid/qcd/action/fermion/implementation/CayleyFermion5Dcache.h:41-230
//   Schur operator         Grid/algorithms/LinearOperator.h:286-349
//   red-black solve        Grid/algorithms/iterative/SchurRedBlack.h:236-291,373-436
//   CG                     Grid/algorithms/iterative/ConjugateGradient.h:68-257
//   reliable-update CG     Grid/algorithms/iterative/ConjugateGradientReliableUpdate.h:77-269
//   multishift CG          Grid/algorithms/iterative/ConjugateGradientMultiShift.h:76-330
//   Dminus, 4D<->5D        Grid/qcd/action/fermion/implementation/CayleyFermion5DImplementation.h:57-153
//
// Canonical host layout (also the library's C-ABI layout):
//   4D site index  site = x + Lx*(y + Ly*(z + Lz*t))
//   gauge          U[site][mu][a][b]              complex<double>, mu = x,y,z,t
//   fermion        psi[site][s][spin][colour]     complex, s = 0..L5-1 innermost of the site
//   half field     psi[site>>1][s][spin][colour]  over the sites of one parity (Lx even)
//   parity         (x+y+z+t) & 1, Even = 0; the fifth coordinate takes no part.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>

namespace orc {

template <class R> using cplx = std::complex<R>;
template <class R> using Field = std::vector<cplx<R>>;

constexpr int Ns = 4, Nc = 3, Nsc = 12;

// ---------------------------------------------------------------------------------------
// Geometry
// ---------------------------------------------------------------------------------------
struct Geom {
  int L[4];
  int64_t vol;
  explicit Geom(const int* d) {
    vol = 1;
    for (int i = 0; i < 4; i++) { L[i] = d[i]; vol *= d[i]; }
  }
  void coords(int64_t site, int x[4]) const {
    for (int i = 0; i < 4; i++) { x[i] = int(site % L[i]); site /= L[i]; }
  }
  int64_t index(const int x[4]) const {
    return x[0] + int64_t(L[0]) * (x[1] + int64_t(L[1]) * (x[2] + int64_t(L[2]) * x[3]));
  }
  int parity(int64_t site) const {
    int x[4]; coords(site, x);
    return (x[0] + x[1] + x[2] + x[3]) & 1;
  }
  int64_t shift(int64_t site, int mu, int disp) const {
    int x[4]; coords(site, x);
    x[mu] = ((x[mu] + disp) % L[mu] + L[mu]) % L[mu];
    return index(x);
  }
};

// ---------------------------------------------------------------------------------------
// Gamma matrices in Grid's basis (TwoSpinor.h:67-140 comments; spProj*/spRecon* bodies)
// ---------------------------------------------------------------------------------------
inline const cplx<double>& gamma_el(int mu, int i, int j) {
  static const cplx<double> I(0, 1), O(0, 0), P(1, 0), M(-1, 0);
  static const cplx<double> G[5][4][4] = {
      {{O, O, O, I}, {O, O, I, O}, {O, -I, O, O}, {-I, O, O, O}},  // gamma_x
      {{O, O, O, M}, {O, O, P, O}, {O, P, O, O}, {M, O, O, O}},    // gamma_y
      {{O, O, I, O}, {O, O, O, -I}, {-I, O, O, O}, {O, I, O, O}},  // gamma_z
      {{O, O, P, O}, {O, O, O, P}, {P, O, O, O}, {O, P, O, O}},    // gamma_t
      {{P, O, O, O}, {O, P, O, O}, {O, O, M, O}, {O, O, O, M}},    // gamma_5
  };
  return G[mu][i][j];
}

// ---------------------------------------------------------------------------------------
// Field helpers
// ---------------------------------------------------------------------------------------
template <class R> inline double norm2(const Field<R>& a) {
  double s = 0;
#pragma omp parallel for reduction(+ : s)
  for (int64_t i = 0; i < int64_t(a.size()); i++) s += double(std::norm(a[i]));
  return s;
}
template <class R> inline cplx<double> inner(const Field<R>& a, const Field<R>& b) {
  double re = 0, im = 0;
#pragma omp parallel for reduction(+ : re, im)
  for (int64_t i = 0; i < int64_t(a.size()); i++) {
    cplx<double> z = std::conj(cplx<double>(a[i])) * cplx<double>(b[i]);
    re += z.real(); im += z.imag();
  }
  return {re, im};
}
// z = a*x + y
template <class R> inline void axpy(Field<R>& z, R a, const Field<R>& x, const Field<R>& y) {
#pragma omp parallel for
  for (int64_t i = 0; i < int64_t(z.size()); i++) z[i] = a * x[i] + y[i];
}
template <class R> inline void pick_cb(const Geom& g, int L5, int parity, const Field<R>& full, Field<R>& half) {
  half.assign(size_t(g.vol / 2) * L5 * Nsc, cplx<R>(0));
#pragma omp parallel for
  for (int64_t site = 0; site < g.vol; site++) {
    if (g.parity(site) != parity) continue;
    std::copy_n(&full[size_t(site) * L5 * Nsc], L5 * Nsc, &half[size_t(site >> 1) * L5 * Nsc]);
  }
}
template <class R> inline void set_cb(const Geom& g, int L5, int parity, const Field<R>& half, Field<R>& full) {
  full.resize(size_t(g.vol) * L5 * Nsc);
#pragma omp parallel for
  for (int64_t site = 0; site < g.vol; site++) {
    if (g.parity(site) != parity) continue;
    std::copy_n(&half[size_t(site >> 1) * L5 * Nsc], L5 * Nsc, &full[size_t(site) * L5 * Nsc]);
  }
}

// ---------------------------------------------------------------------------------------
// DoubleStore (WilsonImpl.h:127-171) with the -1/2 of ImportGauge folded in
//   Ud[x][mu]   = -1/2 * U_mu(x) * (phase_mu if x_mu == L_mu-1)
//   Ud[x][mu+4] = -1/2 * U_mu(x-mu)^dagger * (conj(phase_mu) if x_mu == 0)
// ---------------------------------------------------------------------------------------
template <class R>
void double_store(const Geom& g, const cplx<double>* U, const cplx<double>* phase, std::vector<cplx<R>>& Ud) {
  Ud.assign(size_t(g.vol) * 8 * 9, cplx<R>(0));
#pragma omp parallel for
  for (int64_t site = 0; site < g.vol; site++) {
    int x[4]; g.coords(site, x);
    for (int mu = 0; mu < 4; mu++) {
      cplx<double> pf = (x[mu] == g.L[mu] - 1) ? phase[mu] : cplx<double>(1, 0);
      cplx<double> pb = (x[mu] == 0) ? std::conj(phase[mu]) : cplx<double>(1, 0);
      int64_t back = g.shift(site, mu, -1);
      const cplx<double>* Uf = U + (size_t(site) * 4 + mu) * 9;
      const cplx<double>* Ub = U + (size_t(back) * 4 + mu) * 9;
      for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) {
          Ud[(size_t(site) * 8 + mu) * 9 + a * 3 + b] = cplx<R>(-0.5 * pf * Uf[a * 3 + b]);
          Ud[(size_t(site) * 8 + mu + 4) * 9 + a * 3 + b] = cplx<R>(-0.5 * pb * std::conj(Ub[b * 3 + a]));
        }
    }
  }
}

// ---------------------------------------------------------------------------------------
// Site-loop Dhop on full canonical fields (WilsonKernelsImplementation.h:113-163).
// Non-dagger: out(x) = sum_mu (1 - g_mu) Ud_mu(x) in(x+mu) + (1 + g_mu) Ud_{mu+4}(x) in(x-mu)
// Dagger swaps the projector signs.  The restatement applies U to all four spins and then
// the 4x4 projector (1 -/+ gamma_mu); the half-spinor trick is not used here.
// out_parity >= 0 restricts the output sites (DhopEO/DhopOE); other sites are untouched.
// ---------------------------------------------------------------------------------------
template <class R>
void dhop(const Geom& g, int L5, const std::vector<cplx<R>>& Ud, const Field<R>& in, Field<R>& out, int dag,
          int out_parity = -1) {
  out.resize(in.size());
#pragma omp parallel for schedule(static)
  for (int64_t site = 0; site < g.vol; site++) {
    if (out_parity >= 0 && g.parity(site) != out_parity) continue;
    for (int s = 0; s < L5; s++) {
      cplx<R> res[Nsc];
      for (auto& r : res) r = 0;
      for (int leg = 0; leg < 8; leg++) {
        int mu = leg & 3;
        int disp = leg < 4 ? +1 : -1;
        int64_t nb = g.shift(site, mu, disp);
        const cplx<R>* U = &Ud[(size_t(site) * 8 + leg) * 9];
        const cplx<R>* p = &in[(size_t(nb) * L5 + s) * Nsc];
        cplx<R> phi[Nsc];
        for (int sp = 0; sp < Ns; sp++)
          for (int a = 0; a < Nc; a++) {
            cplx<R> acc = 0;
            for (int b = 0; b < Nc; b++) acc += U[a * 3 + b] * p[sp * 3 + b];
            phi[sp * 3 + a] = acc;
          }
        // forward leg uses (1 - gamma), backward (1 + gamma); dagger swaps
        R sign = (disp > 0) ? R(-1) : R(1);
        if (dag) sign = -sign;
        for (int sp = 0; sp < Ns; sp++)
          for (int a = 0; a < Nc; a++) {
            cplx<R> gp = 0;
            for (int sq = 0; sq < Ns; sq++) gp += cplx<R>(gamma_el(mu, sp, sq)) * phi[sq * 3 + a];
            res[sp * 3 + a] += phi[sp * 3 + a] + sign * gp;
          }
      }
      std::copy_n(res, Nsc, &out[(size_t(site) * L5 + s) * Nsc]);
    }
  }
}

// Force term, DerivInternal + InsertForce5D (WilsonFermion5DImplementation.h:212-246,
// WilsonImpl.h:193-238) on full canonical fields, double precision:
//   mat[x][mu]_ab = sum_s sum_spin [(1 -+ g_mu) Ud_mu(x) B(x+mu, s)]_{spin,a} conj(A(x,s)_{spin,b})
// (minus: non-dagger) for the sites of out_parity (all sites when < 0); mat is
// [site][mu][3][3] and untouched elsewhere.
inline void dhop_deriv(const Geom& g, int L5, const std::vector<cplx<double>>& Ud, const Field<double>& A,
                       const Field<double>& B, std::vector<cplx<double>>& mat, int dag, int out_parity = -1) {
  mat.resize(size_t(g.vol) * 4 * 9);
#pragma omp parallel for schedule(static)
  for (int64_t site = 0; site < g.vol; site++) {
    if (out_parity >= 0 && g.parity(site) != out_parity) continue;
    for (int mu = 0; mu < 4; mu++) {
      const int64_t nb = g.shift(site, mu, +1);
      const cplx<double>* U = &Ud[(size_t(site) * 8 + mu) * 9];
      const double sign = dag ? 1.0 : -1.0;
      cplx<double> F[9] = {};
      for (int s = 0; s < L5; s++) {
        const cplx<double>* p = &B[(size_t(nb) * L5 + s) * Nsc];
        const cplx<double>* a = &A[(size_t(site) * L5 + s) * Nsc];
        cplx<double> phi[Nsc], bt[Nsc];
        for (int sp = 0; sp < Ns; sp++)
          for (int c = 0; c < Nc; c++) {
            cplx<double> acc = 0;
            for (int d = 0; d < Nc; d++) acc += U[c * 3 + d] * p[sp * 3 + d];
            phi[sp * 3 + c] = acc;
          }
        for (int sp = 0; sp < Ns; sp++)
          for (int c = 0; c < Nc; c++) {
            cplx<double> gp = 0;
            for (int sq = 0; sq < Ns; sq++) gp += gamma_el(mu, sp, sq) * phi[sq * 3 + c];
            bt[sp * 3 + c] = phi[sp * 3 + c] + sign * gp;
          }
        for (int ca = 0; ca < 3; ca++)
          for (int cb = 0; cb < 3; cb++)
            for (int sp = 0; sp < Ns; sp++) F[ca * 3 + cb] += bt[sp * 3 + ca] * std::conj(a[sp * 3 + cb]);
      }
      std::copy_n(F, 9, &mat[(size_t(site) * 4 + mu) * 9]);
    }
  }
}

// Naive Cshift-form Dhop (benchmarks/Benchmark_dwf.cc:145-158 non-dagger, :235-261 dagger),
// written from the undoubled links and the boundary phases, as an independent check of
// DoubleStore + the site loop.
template <class R>
void dhop_naive(const Geom& g, int L5, const cplx<double>* U, const cplx<double>* phase, const Field<R>& in,
                Field<R>& out, int dag) {
  size_t n = in.size();
  std::vector<cplx<double>> ref(n, 0), tmp(n), sh(n);
  auto link = [&](int64_t site, int mu, int a, int b) {
    int x[4]; g.coords(site, x);
    cplx<double> ph = (x[mu] == g.L[mu] - 1) ? phase[mu] : cplx<double>(1, 0);
    return ph * U[(size_t(site) * 4 + mu) * 9 + a * 3 + b];
  };
  double sgn = dag ? 1.0 : -1.0;  // non-dag: ref += tmp - G tmp (forward)
  for (int mu = 0; mu < 4; mu++) {
    // Cshift(src, mu, +1)(x) = src(x+mu)
    for (int64_t site = 0; site < g.vol; site++) {
      int64_t nb = g.shift(site, mu, +1);
      for (int k = 0; k < L5 * Nsc; k++) sh[size_t(site) * L5 * Nsc + k] = cplx<double>(in[size_t(nb) * L5 * Nsc + k]);
    }
    // tmp = U_mu * shifted
    for (int64_t site = 0; site < g.vol; site++)
      for (int s = 0; s < L5; s++)
        for (int sp = 0; sp < Ns; sp++)
          for (int a = 0; a < Nc; a++) {
            cplx<double> acc = 0;
            for (int b = 0; b < Nc; b++) acc += link(site, mu, a, b) * sh[(size_t(site) * L5 + s) * Nsc + sp * 3 + b];
            tmp[(size_t(site) * L5 + s) * Nsc + sp * 3 + a] = acc;
          }
    for (int64_t site = 0; site < g.vol; site++)
      for (int s = 0; s < L5; s++)
        for (int sp = 0; sp < Ns; sp++)
          for (int a = 0; a < Nc; a++) {
            size_t o = (size_t(site) * L5 + s) * Nsc;
            cplx<double> gt = 0;
            for (int sq = 0; sq < Ns; sq++) gt += gamma_el(mu, sp, sq) * tmp[o + sq * 3 + a];
            ref[o + sp * 3 + a] += tmp[o + sp * 3 + a] + sgn * gt;
          }
    // tmp = adj(U_mu) * src ; then Cshift(tmp, mu, -1)(x) = tmp(x-mu)
    for (int64_t site = 0; site < g.vol; site++)
      for (int s = 0; s < L5; s++)
        for (int sp = 0; sp < Ns; sp++)
          for (int a = 0; a < Nc; a++) {
            cplx<double> acc = 0;
            for (int b = 0; b < Nc; b++)
              acc += std::conj(link(site, mu, b, a)) * cplx<double>(in[(size_t(site) * L5 + s) * Nsc + sp * 3 + b]);
            tmp[(size_t(site) * L5 + s) * Nsc + sp * 3 + a] = acc;
          }
    for (int64_t site = 0; site < g.vol; site++) {
      int64_t nb = g.shift(site, mu, -1);
      for (int k = 0; k < L5 * Nsc; k++) sh[size_t(site) * L5 * Nsc + k] = tmp[size_t(nb) * L5 * Nsc + k];
    }
    for (int64_t site = 0; site < g.vol; site++)
      for (int s = 0; s < L5; s++)
        for (int sp = 0; sp < Ns; sp++)
          for (int a = 0; a < Nc; a++) {
            size_t o = (size_t(site) * L5 + s) * Nsc;
            cplx<double> gt = 0;
            for (int sq = 0; sq < Ns; sq++) gt += gamma_el(mu, sp, sq) * sh[o + sq * 3 + a];
            ref[o + sp * 3 + a] += sh[o + sp * 3 + a] - sgn * gt;
          }
  }
  out.resize(n);
  for (size_t i = 0; i < n; i++) out[i] = cplx<R>(-0.5 * ref[i]);
}

// ---------------------------------------------------------------------------------------
// Cayley / Moebius coefficients (CayleyFermion5DImplementation.h:410-535) with the
// Moebius tanh choice gamma_s = 1 (MobiusFermion.h:63-67; approx/Zolotarev.cc:471-473).
// ---------------------------------------------------------------------------------------
// coefficient conjugation: the identity for real Moebius coefficients
inline double cj(double x) { return x; }
inline cplx<double> cj(const cplx<double>& x) { return std::conj(x); }

// SetCoefficientsInternal (CayleyFermion5DImplementation.h:410-535) with omega_s = gamma_s:
// 1 for Moebius (real coefficients), complex for ZMobius (ZMobiusFermion.h)
template <class C> struct CayleyT {
  int Ls = 0;
  double mf = 0, M5 = 0, b = 0, c = 0;
  std::vector<C> omega, bs, cs, bee, cee, dee, lee, leem, uee, ueem;
  void setup(int Ls_, double mf_, double M5_, double b_, double c_, const std::vector<C>& omega_) {
    Ls = Ls_; mf = mf_; M5 = M5_; b = b_; c = c_;
    omega = omega_;
    bs.assign(Ls, C(0)); cs.assign(Ls, C(0)); bee.assign(Ls, C(0)); cee.assign(Ls, C(0));
    dee.assign(Ls, C(0)); lee.assign(Ls, C(0)); leem.assign(Ls, C(0)); uee.assign(Ls, C(0)); ueem.assign(Ls, C(0));
    for (int i = 0; i < Ls; i++) {
      bs[i] = 0.5 * ((b + c) / omega[i] + (b - c));
      cs[i] = 0.5 * ((b + c) / omega[i] - (b - c));
      bee[i] = bs[i] * (4.0 - M5) + 1.0;
      cee[i] = 1.0 - cs[i] * (4.0 - M5);
    }
    const std::vector<C>& aee = cee;
    for (int i = 0; i < Ls; i++) {
      dee[i] = bee[i];
      if (i < Ls - 1) {
        lee[i] = -cee[i + 1] / bee[i];
        leem[i] = mf * cee[Ls - 1] / bee[0];
        for (int j = 0; j < i; j++) leem[i] *= aee[j] / bee[j + 1];
        uee[i] = -aee[i] / bee[i];
        ueem[i] = C(mf);
        for (int j = 1; j <= i; j++) ueem[i] *= cee[j] / bee[j];
        ueem[i] *= aee[0] / bee[0];
      }
    }
    C delta_d = mf * cee[Ls - 1];
    for (int j = 0; j < Ls - 1; j++) delta_d *= cee[j] / bee[j];
    dee[Ls - 1] += delta_d;
  }
  void setup(int Ls_, double mf_, double M5_, double b_, double c_) {  // Moebius: omega_s = 1
    setup(Ls_, mf_, M5_, b_, c_, std::vector<C>(Ls_, C(1.0)));
  }
};
using Cayley = CayleyT<double>;

// M5D / M5Ddag (CayleyFermion5Dcache.h:41-115) on an n4 x Ls field (full or half):
//   non-dag: chi[s] = diag[s] phi[s] + upper[s] P- psi[s+1] + lower[s] P+ psi[s-1]
//   dag    : chi[s] = diag[s] phi[s] + upper[s] P+ psi[s+1] + lower[s] P- psi[s-1]
// with P+ = spins {0,1}, P- = spins {2,3} (gamma_5 = diag(1,1,-1,-1)).
template <class R, class C = double>
void m5d(int64_t n4, int Ls, const Field<R>& psi, const Field<R>& phi, Field<R>& chi, const std::vector<C>& lower,
         const std::vector<C>& diag, const std::vector<C>& upper, int dag) {
  Field<R> res(psi.size());
#pragma omp parallel for
  for (int64_t x = 0; x < n4; x++)
    for (int s = 0; s < Ls; s++) {
      int sp = (s + 1) % Ls, sm = (s - 1 + Ls) % Ls;
      size_t o = (size_t(x) * Ls + s) * Nsc, op = (size_t(x) * Ls + sp) * Nsc, om = (size_t(x) * Ls + sm) * Nsc;
      for (int k = 0; k < Nsc; k++) {
        bool upper_spin = k < 6;  // spins 0,1
        cplx<R> v = cplx<R>(diag[s]) * phi[o + k];
        if (!dag) v += upper_spin ? cplx<R>(lower[s]) * psi[om + k] : cplx<R>(upper[s]) * psi[op + k];
        else      v += upper_spin ? cplx<R>(upper[s]) * psi[op + k] : cplx<R>(lower[s]) * psi[om + k];
        res[o + k] = v;
      }
    }
  chi.swap(res);
}

// ---------------------------------------------------------------------------------------
// Operator interface shared by Wilson and Moebius restatements.  Half fields carry an
// explicit parity argument (the parity of the input field).
// ---------------------------------------------------------------------------------------
template <class R> struct Op {
  Geom g;
  int L5;
  std::vector<cplx<R>> Ud;
  Op(const int* dims, int L5_) : g(dims), L5(L5_) {}
  virtual ~Op() {}
  int64_t half_sites() const { return g.vol / 2; }
  size_t full_len() const { return size_t(g.vol) * L5 * Nsc; }
  size_t half_len() const { return size_t(g.vol / 2) * L5 * Nsc; }

  void import_gauge(const cplx<double>* U, const cplx<double>* phase) { double_store<R>(g, U, phase, Ud); }
  void Dhop(const Field<R>& in, Field<R>& out, int dag) { dhop<R>(g, L5, Ud, in, out, dag); }
  // in has parity in_parity; out has the other parity
  void DhopCB(const Field<R>& in, Field<R>& out, int in_parity, int dag) {
    Field<R> fin(full_len(), cplx<R>(0)), fout(full_len(), cplx<R>(0));
    set_cb<R>(g, L5, in_parity, in, fin);
    dhop<R>(g, L5, Ud, fin, fout, dag, 1 - in_parity);
    pick_cb<R>(g, L5, 1 - in_parity, fout, out);
  }
  virtual void M(const Field<R>& in, Field<R>& out) = 0;
  virtual void Mdag(const Field<R>& in, Field<R>& out) = 0;
  virtual void Meooe(const Field<R>& in, Field<R>& out, int in_parity) = 0;
  virtual void MeooeDag(const Field<R>& in, Field<R>& out, int in_parity) = 0;
  virtual void Mooee(const Field<R>& in, Field<R>& out) = 0;
  virtual void MooeeDag(const Field<R>& in, Field<R>& out) = 0;
  virtual void MooeeInv(const Field<R>& in, Field<R>& out) = 0;
  virtual void MooeeInvDag(const Field<R>& in, Field<R>& out) = 0;
  // SetMass (CayleyFermion5D.h:75-78: the Cayley coefficients are rebuilt)
  virtual void set_mass(double m) = 0;

  void MdagM(const Field<R>& in, Field<R>& out) {
    Field<R> t; M(in, t); Mdag(t, out);
  }
  // SchurDiagMooeeOperator (LinearOperator.h:325-349), on the odd checkerboard
  void Mpc(const Field<R>& in, Field<R>& out) {
    Field<R> tmp, t2;
    Meooe(in, tmp, 1);
    MooeeInv(tmp, t2);
    Meooe(t2, tmp, 0);
    Mooee(in, out);
    axpy<R>(out, R(-1), tmp, out);
  }
  void MpcDag(const Field<R>& in, Field<R>& out) {
    Field<R> tmp, t2;
    MeooeDag(in, tmp, 1);
    MooeeInvDag(tmp, t2);
    MeooeDag(t2, tmp, 0);
    MooeeDag(in, out);
    axpy<R>(out, R(-1), tmp, out);
  }
  void MpcDagMpc(const Field<R>& in, Field<R>& out) {
    Field<R> t; Mpc(in, t); MpcDag(t, out);
  }
};

// WilsonFermion (WilsonFermionImplementation.h:113-176).  L5 > 1 stacks independent
// right-hand sides in the fifth slot; the operator is diagonal in it.
template <class R> struct Wilson : Op<R> {
  double mass, diag_mass;
  Wilson(const int* dims, int L5, double m) : Op<R>(dims, L5), mass(m), diag_mass(4.0 + m) {}
  void set_mass(double m) override { mass = m; diag_mass = 4.0 + m; }
  void M(const Field<R>& in, Field<R>& out) override {
    this->Dhop(in, out, 0); axpy<R>(out, R(diag_mass), in, out);
  }
  void Mdag(const Field<R>& in, Field<R>& out) override {
    this->Dhop(in, out, 1); axpy<R>(out, R(diag_mass), in, out);
  }
  void Meooe(const Field<R>& in, Field<R>& out, int p) override { this->DhopCB(in, out, p, 0); }
  void MeooeDag(const Field<R>& in, Field<R>& out, int p) override { this->DhopCB(in, out, p, 1); }
  void Mooee(const Field<R>& in, Field<R>& out) override {
    out.resize(in.size());
    for (size_t i = 0; i < in.size(); i++) out[i] = R(diag_mass) * in[i];
  }
  void MooeeDag(const Field<R>& in, Field<R>& out) override { Mooee(in, out); }
  void MooeeInv(const Field<R>& in, Field<R>& out) override {
    out.resize(in.size());
    for (size_t i = 0; i < in.size(); i++) out[i] = R(1.0 / diag_mass) * in[i];
  }
  void MooeeInvDag(const Field<R>& in, Field<R>& out) override { MooeeInv(in, out); }
};

// MobiusFermion / CayleyFermion5D (CayleyFermion5DImplementation.h:155-344,
// CayleyFermion5Dcache.h:117-230).  L5 = Ls.
// the Cayley-form operators (Moebius, ZMobius) beyond the common interface
template <class R> struct CayleyBase : Op<R> {
  CayleyBase(const int* dims, int L5) : Op<R>(dims, L5) {}
  virtual void Meooe5D(const Field<R>& psi, Field<R>& Din) = 0;
  virtual void MeooeDag5D(const Field<R>& psi, Field<R>& Din) = 0;
  virtual void Dminus(const Field<R>& psi, Field<R>& chi, int dag) = 0;
  virtual void ImportUnphysical(const Field<R>& in4, Field<R>& out5) const = 0;
  virtual void ImportPhysicalSource(const Field<R>& in4, Field<R>& out5) = 0;
  virtual void ExportPhysical(const Field<R>& in5, Field<R>& out4, bool solution) const = 0;
  virtual void P(const Field<R>& psi, Field<R>& chi, int dag) const = 0;
};

template <class R, class C = double> struct Mobius : CayleyBase<R> {
  CayleyT<C> cf;
  int Ls;
  Mobius(const int* dims, int Ls_, double mf, double M5, double b, double c) : CayleyBase<R>(dims, Ls_), Ls(Ls_) {
    cf.setup(Ls_, mf, M5, b, c);
  }
  // ZMobius: complex omega_s = gamma_s
  Mobius(const int* dims, int Ls_, double mf, double M5, double b, double c, const std::vector<C>& gamma)
      : CayleyBase<R>(dims, Ls_), Ls(Ls_) {
    cf.setup(Ls_, mf, M5, b, c, gamma);
  }
  int64_t n4(const Field<R>& f) const { return int64_t(f.size() / (size_t(Ls) * Nsc)); }
  void set_mass(double m) override {
    const std::vector<C> om = cf.omega;
    cf.setup(Ls, m, cf.M5, cf.b, cf.c, om);
  }
  // P / Pdag (CayleyFermion5DImplementation.h:70-88): chi_s = P- psi_s + P+ psi_{s+1} (P)
  // or P+ psi_{s-1} (Pdag), s cyclic; P+ keeps spins 0,1 (components k < 6)
  void P(const Field<R>& psi, Field<R>& chi, int dag) const override {
    const int64_t n = n4(psi);
    chi.resize(psi.size());
    for (int64_t x = 0; x < n; x++)
      for (int s = 0; s < Ls; s++) {
        const int sp = dag ? (s + Ls - 1) % Ls : (s + 1) % Ls;
        for (int k = 0; k < Nsc; k++)
          chi[(size_t(x) * Ls + s) * Nsc + k] = psi[(size_t(x) * Ls + (k < 6 ? sp : s)) * Nsc + k];
      }
  }

  void DW(const Field<R>& in, Field<R>& out, int dag) {
    this->Dhop(in, out, dag); axpy<R>(out, R(4.0 - cf.M5), in, out);
  }
  // Dminus / DminusDag (CayleyFermion5DImplementation.h:131-153): chi_s = psi_s - cs[s] (DW psi)_s,
  // conj(cs[s]) and DW^dag for the dagger
  void Dminus(const Field<R>& psi, Field<R>& chi, int dag) override {
    Field<R> t;
    DW(psi, t, dag);
    chi.resize(psi.size());
    const int64_t n = n4(psi);
    for (int64_t x = 0; x < n; x++)
      for (int s = 0; s < Ls; s++)
        for (int k = 0; k < Nsc; k++) {
          const size_t i = (size_t(x) * Ls + s) * Nsc + k;
          chi[i] = psi[i] - cplx<R>(dag ? cj(cf.cs[s]) : cf.cs[s]) * t[i];
        }
  }
  // ImportUnphysicalFermion (:101-114): s = 0 takes P+ in4, s = Ls-1 takes P- in4, the
  // rest is zero.  P+ keeps spins 0,1 and P- spins 2,3 (gamma5 = diag(1,1,-1,-1)).
  void ImportUnphysical(const Field<R>& in4, Field<R>& out5) const override {
    const int64_t n = int64_t(in4.size() / Nsc);
    out5.assign(size_t(n) * Ls * Nsc, cplx<R>(0, 0));
    for (int64_t x = 0; x < n; x++)
      for (int k = 0; k < Nsc; k++) {
        const size_t s = k < 6 ? 0 : size_t(Ls - 1);
        out5[(size_t(x) * Ls + s) * Nsc + k] = in4[size_t(x) * Nsc + k];
      }
  }
  // ImportPhysicalFermionSource (:116-129) = Dminus of the unphysical import
  void ImportPhysicalSource(const Field<R>& in4, Field<R>& out5) override {
    Field<R> t;
    ImportUnphysical(in4, t);
    Dminus(t, out5, 0);
  }
  // ExportPhysicalFermionSolution (:57-68): P- psi(s=0) + P+ psi(s=Ls-1);
  // ExportPhysicalFermionSource (:89-100): P+ psi(s=0) + P- psi(s=Ls-1)
  void ExportPhysical(const Field<R>& in5, Field<R>& out4, bool solution) const override {
    const int64_t n = n4(in5);
    out4.resize(size_t(n) * Nsc);
    for (int64_t x = 0; x < n; x++)
      for (int k = 0; k < Nsc; k++) {
        const bool upper = k < 6;
        const size_t s = (upper == solution) ? size_t(Ls - 1) : 0;
        out4[size_t(x) * Nsc + k] = in5[(size_t(x) * Ls + s) * Nsc + k];
      }
  }
  void Meooe5D(const Field<R>& psi, Field<R>& Din) override {
    std::vector<C> diag = cf.bs, upper = cf.cs, lower = cf.cs;
    upper[Ls - 1] = -cf.mf * upper[Ls - 1];
    lower[0] = -cf.mf * lower[0];
    m5d<R>(n4(psi), Ls, psi, psi, Din, lower, diag, upper, 0);
  }
  void MeooeDag5D(const Field<R>& psi, Field<R>& Din) override {
    std::vector<C> diag = cf.bs, upper(Ls), lower(Ls);
    for (int s = 0; s < Ls; s++) {
      if (s == 0) { upper[s] = cf.cs[s + 1]; lower[s] = -cf.mf * cf.cs[Ls - 1]; }
      else if (s == Ls - 1) { upper[s] = -cf.mf * cf.cs[0]; lower[s] = cf.cs[s - 1]; }
      else { upper[s] = cf.cs[s + 1]; lower[s] = cf.cs[s - 1]; }
    }
    for (int s = 0; s < Ls; s++) { diag[s] = cj(diag[s]); upper[s] = cj(upper[s]); lower[s] = cj(lower[s]); }
    m5d<R>(n4(psi), Ls, psi, psi, Din, lower, diag, upper, 1);
  }
  void Mooee(const Field<R>& psi, Field<R>& chi) override {
    std::vector<C> diag = cf.bee, upper(Ls), lower(Ls);
    for (int i = 0; i < Ls; i++) { upper[i] = -cf.cee[i]; lower[i] = -cf.cee[i]; }
    upper[Ls - 1] = -cf.mf * upper[Ls - 1];
    lower[0] = -cf.mf * lower[0];
    m5d<R>(n4(psi), Ls, psi, psi, chi, lower, diag, upper, 0);
  }
  void MooeeDag(const Field<R>& psi, Field<R>& chi) override {
    std::vector<C> diag = cf.bee, upper(Ls), lower(Ls);
    for (int s = 0; s < Ls; s++) {
      if (s == 0) { upper[s] = -cf.cee[s + 1]; lower[s] = cf.mf * cf.cee[Ls - 1]; }
      else if (s == Ls - 1) { upper[s] = cf.mf * cf.cee[0]; lower[s] = -cf.cee[s - 1]; }
      else { upper[s] = -cf.cee[s + 1]; lower[s] = -cf.cee[s - 1]; }
    }
    for (int s = 0; s < Ls; s++) { diag[s] = cj(diag[s]); upper[s] = cj(upper[s]); lower[s] = cj(lower[s]); }
    m5d<R>(n4(psi), Ls, psi, psi, chi, lower, diag, upper, 1);
  }
  // LDU solve along s (CayleyFermion5Dcache.h:117-170), component by component.
  // MooeeInvDag conjugates the swapped factors (CayleyFermion5Dcache.h:172-230)
  static cplx<R> cf_at(const std::vector<C>& v, int s, int dag) { return cplx<R>(dag ? cj(v[s]) : v[s]); }
  static cplx<R> inv_dee(const std::vector<C>& d, int s, int dag) {
    const C x = C(1.0) / d[s];
    return cplx<R>(dag ? cj(x) : x);
  }
  void MooeeInv(const Field<R>& psi, Field<R>& chi) override { mooee_inv(psi, chi, 0); }
  void MooeeInvDag(const Field<R>& psi, Field<R>& chi) override { mooee_inv(psi, chi, 1); }
  void mooee_inv(const Field<R>& psi, Field<R>& chi, int dag) {
    chi.resize(psi.size());
    const auto& lee = dag ? cf.uee : cf.lee;    // dag: roles of (lee,leem) and (uee,ueem)
    const auto& leem = dag ? cf.ueem : cf.leem; // swap and the chiralities swap
    const auto& uee = dag ? cf.lee : cf.uee;
    const auto& ueem = dag ? cf.leem : cf.ueem;
    const auto& dee = cf.dee;
    int64_t n = n4(psi);
#pragma omp parallel for
    for (int64_t x = 0; x < n; x++) {
      for (int k = 0; k < Nsc; k++) {
        // chirality of the component: "first" = the projector applied in the forward
        // sweep (P+ non-dag, P- dag), "second" = the other one
        bool upper_spin = k < 6;
        bool first = dag ? !upper_spin : upper_spin;
        auto at = [&](int s) -> size_t { return (size_t(x) * Ls + s) * Nsc + k; };
        // forward: res_s = psi_s - lee[s-1] P_first res_{s-1};  acc += leem[s] P_second res_s
        cplx<R> prev = 0, acc = 0;
        for (int s = 0; s < Ls - 1; s++) {
          cplx<R> r = psi[at(s)];
          if (s > 0 && first) r -= cf_at(lee, s - 1, dag) * prev;
          if (!first) acc += cf_at(leem, s, dag) * r;
          chi[at(s)] = r;
          prev = r;
        }
        cplx<R> r = psi[at(Ls - 1)];
        if (first) r -= cf_at(lee, Ls - 2, dag) * prev;
        else r -= acc;
        // backward: chi_{Ls-1} = r / dee ; chi_s = chi_s/dee[s] - uee[s] P_second chi_{s+1}
        //                                               - ueem[s] P_first chi_{Ls-1}
        r = inv_dee(dee, Ls - 1, dag) * r;
        chi[at(Ls - 1)] = r;
        cplx<R> last = r, nxt = r;
        for (int s = Ls - 2; s >= 0; s--) {
          cplx<R> v = inv_dee(dee, s, dag) * chi[at(s)];
          if (!first) v -= cf_at(uee, s, dag) * nxt;
          else v -= cf_at(ueem, s, dag) * last;
          chi[at(s)] = v;
          nxt = v;
        }
      }
    }
  }
  void Meooe(const Field<R>& in, Field<R>& out, int p) override {
    Field<R> t; Meooe5D(in, t); this->DhopCB(t, out, p, 0);
  }
  void MeooeDag(const Field<R>& in, Field<R>& out, int p) override {
    Field<R> t; this->DhopCB(in, t, p, 1); MeooeDag5D(t, out);
  }
  void M(const Field<R>& psi, Field<R>& chi) override {
    Field<R> Din; Meooe5D(psi, Din);
    DW(Din, chi, 0);
    axpy<R>(chi, R(1), chi, psi);
    std::vector<double> diag(Ls, 1.0), upper(Ls, -1.0), lower(Ls, -1.0);
    upper[Ls - 1] = cf.mf; lower[0] = cf.mf;
    m5d<R>(n4(psi), Ls, psi, chi, chi, lower, diag, upper, 0);
  }
  void Mdag(const Field<R>& psi, Field<R>& chi) override {
    Field<R> Din; DW(psi, Din, 1);
    MeooeDag5D(Din, chi);
    std::vector<double> diag(Ls, 1.0), upper(Ls, -1.0), lower(Ls, -1.0);
    upper[Ls - 1] = cf.mf; lower[0] = cf.mf;
    m5d<R>(n4(psi), Ls, psi, chi, chi, lower, diag, upper, 1);
    axpy<R>(chi, R(1), chi, psi);
  }
};

// ---------------------------------------------------------------------------------------
// ConjugateGradient (ConjugateGradient.h:68-257), same sequence of operations.
// ---------------------------------------------------------------------------------------
struct CGResult {
  int iterations = 0;
  int reliable_updates = 0;
  int cleanup_iterations = 0;
  double true_residual = 0;
  int converged = 0;
};

template <class R, class HermOp>
CGResult cg(HermOp&& A, const Field<R>& src, Field<R>& psi, double tol, int maxit) {
  CGResult res;
  size_t n = src.size();
  psi.resize(n);
  Field<R> p(n), mmp(n), r(n);
  double ssq = norm2(src), guess = norm2(psi), a, cp, c, d, b;
  if (guess == 0.0) { r = src; p = r; a = ssq; }
  else { A(psi, mmp); for (size_t i = 0; i < n; i++) r[i] = src[i] - mmp[i]; p = r; a = norm2(p); }
  cp = a;
  if (ssq == 0.0) { std::fill(psi.begin(), psi.end(), cplx<R>(0)); res.iterations = 1; res.converged = 1; return res; }
  double rsq = tol * tol * ssq;
  if (cp <= rsq) { res.true_residual = std::sqrt(a / ssq); res.converged = 1; return res; }
  for (int k = 1; k <= maxit; k++) {
    c = cp;
    A(p, mmp);
    d = inner(p, mmp).real();
    a = c / d;
    // cp = axpy_norm(r, -a, mmp, r)
    for (size_t i = 0; i < n; i++) r[i] = R(-a) * mmp[i] + r[i];
    cp = norm2(r);
    b = cp / c;
    for (size_t i = 0; i < n; i++) { psi[i] = R(a) * p[i] + psi[i]; p[i] = R(b) * p[i] + r[i]; }
    if (cp <= rsq) {
      A(psi, mmp);
      for (size_t i = 0; i < n; i++) p[i] = mmp[i] - src[i];
      res.true_residual = std::sqrt(norm2(p)) / std::sqrt(norm2(src));
      res.iterations = k;
      res.converged = 1;
      return res;
    }
  }
  res.iterations = maxit;
  A(psi, mmp);
  for (size_t i = 0; i < n; i++) p[i] = mmp[i] - src[i];
  res.true_residual = std::sqrt(norm2(p) / ssq);
  return res;
}

// ConjugateGradientMultiShift (ConjugateGradientMultiShift.h:76-330): (A + m_s) psi_s = src
// for every shift, m_0 the lightest; the same sequence of operations as Grid's.
struct MultiShiftResult {
  int iterations = 0;
  int converged = 0;
  std::vector<int> iterations_shift;
  std::vector<double> true_residual;
};

template <class HermOp>
MultiShiftResult cg_multishift(HermOp&& A, const Field<double>& src, std::vector<Field<double>>& psi,
                               const std::vector<double>& mass, const std::vector<double>& tol, int maxit) {
  MultiShiftResult res;
  const int ns = int(mass.size());
  const size_t n = src.size();
  psi.assign(ns, Field<double>(n));
  res.iterations_shift.assign(ns, 0);
  res.true_residual.assign(ns, 0.0);
  std::vector<Field<double>> ps(ns, src);
  std::vector<double> bs(ns), rsq(ns);
  std::vector<std::array<double, 2>> z(ns);
  std::vector<int> conv(ns, 0);
  Field<double> r = src, p = src, mmp(n), tmp(n);
  double cp = norm2(src);
  if (cp == 0.0) {
    for (int s = 0; s < ns; s++) res.iterations_shift[s] = 1;
    res.converged = 1;
    return res;
  }
  const double ssq = cp;
  for (int s = 0; s < ns; s++) rsq[s] = cp * tol[s] * tol[s];
  auto apply = [&](const Field<double>& x, Field<double>& y, double m) {  // y = (A + m) x ; returns <x,y>
    A(x, y);
    for (size_t i = 0; i < n; i++) y[i] += m * x[i];
    return inner(x, y).real();
  };
  double d = apply(p, mmp, mass[0]);
  double b = -cp / d, a = 0, c = 0, bp = 0;
  int iz = 0;
  z[0][0] = z[0][1] = 1.0;
  bs[0] = b;
  for (int s = 1; s < ns; s++) {
    z[s][1 - iz] = 1.0;
    z[s][iz] = 1.0 / (1.0 - b * (mass[s] - mass[0]));
    bs[s] = b * z[s][iz];
  }
  for (size_t i = 0; i < n; i++) r[i] += b * mmp[i];
  c = norm2(r);
  for (int s = 0; s < ns; s++)
    for (size_t i = 0; i < n; i++) psi[s][i] = -bs[s] * src[i];
  for (int k = 1; k <= maxit; k++) {
    a = c / cp;
    for (size_t i = 0; i < n; i++) p[i] = a * p[i] + r[i];
    for (int s = 0; s < ns; s++) {
      if (conv[s]) continue;
      if (s == 0) {
        for (size_t i = 0; i < n; i++) ps[s][i] = a * ps[s][i] + r[i];
      } else {
        const double as = a * z[s][iz] * bs[s] / (z[s][1 - iz] * b);
        for (size_t i = 0; i < n; i++) ps[s][i] = z[s][iz] * r[i] + as * ps[s][i];
      }
    }
    cp = c;
    d = apply(p, mmp, mass[0]);
    bp = b;
    b = -cp / d;
    for (size_t i = 0; i < n; i++) r[i] += b * mmp[i];
    c = norm2(r);
    bs[0] = b;
    iz = 1 - iz;
    for (int s = 1; s < ns; s++) {
      if (conv[s]) continue;
      const double z0 = z[s][1 - iz], z1 = z[s][iz];
      z[s][iz] = z0 * z1 * bp / (b * a * (z1 - z0) + z1 * bp * (1 - (mass[s] - mass[0]) * b));
      bs[s] = b * z[s][iz] / z0;
    }
    for (int s = 0; s < ns; s++)
      if (!conv[s])
        for (size_t i = 0; i < n; i++) psi[s][i] -= bs[s] * ps[s][i];
    int all = 1;
    for (int s = 0; s < ns; s++) {
      if (conv[s]) continue;
      res.iterations_shift[s] = k;
      if (c * z[s][iz] * z[s][iz] < rsq[s]) conv[s] = 1;
      else all = 0;
    }
    res.iterations = k;
    if (all) { res.converged = 1; break; }
  }
  for (int s = 0; s < ns; s++) {
    apply(psi[s], mmp, mass[s]);
    for (size_t i = 0; i < n; i++) tmp[i] = mmp[i] - src[i];
    res.true_residual[s] = std::sqrt(norm2(tmp) / ssq);
  }
  return res;
}

template <class A, class B> inline void precision_change(Field<A>& out, const Field<B>& in) {
  out.resize(in.size());
  for (size_t i = 0; i < in.size(); i++) out[i] = cplx<A>(in[i]);
}

// ConjugateGradientReliableUpdate (ConjugateGradientReliableUpdate.h:77-269) with the
// optional extra rule "reliable update at least every relup_every iterations"
// (relup_every <= 0 disables it) and the final FP64 cleanup CG.
template <class HermD, class HermF>
CGResult cg_reliable(HermD&& Ad, HermF&& Af, const Field<double>& src, Field<double>& psi, double tol, int maxit,
                     double delta, int relup_every, bool cleanup) {
  CGResult res;
  size_t n = src.size();
  psi.resize(n);
  Field<double> p(n), mmp(n), r(n);
  Ad(psi, mmp);
  for (size_t i = 0; i < n; i++) r[i] = src[i] - mmp[i];
  p = r;
  double a = norm2(p), cp = a, ssq = norm2(src), c, d, b;
  double rsq = tol * tol * ssq;
  if (cp <= rsq) { res.converged = 1; return res; }
  Field<float> r_f, psi_f(n, 0), p_f, mmp_f(n);
  precision_change(r_f, r);
  p_f = r_f;
  double maxres = cp;
  int l = 0, since = 0;
  for (int k = 1; k <= maxit; k++) {
    c = cp;
    Af(p_f, mmp_f);
    d = inner(p_f, mmp_f).real();
    a = c / d;
    for (size_t i = 0; i < n; i++) r_f[i] = float(-a) * mmp_f[i] + r_f[i];
    cp = norm2(r_f);
    b = cp / c;
    for (size_t i = 0; i < n; i++) psi_f[i] = float(a) * p_f[i] + psi_f[i];
    since++;
    if (cp > maxres) maxres = cp;
    if (cp <= rsq) {
      for (size_t i = 0; i < n; i++) psi[i] += cplx<double>(psi_f[i]);
      res.iterations = k;
      res.reliable_updates = l;
      if (cleanup) {
        CGResult c2 = cg<double>(Ad, src, psi, tol, maxit);
        res.cleanup_iterations = c2.iterations;
        res.true_residual = c2.true_residual;
        res.converged = c2.converged;
      } else {
        Ad(psi, mmp);
        for (size_t i = 0; i < n; i++) p[i] = mmp[i] - src[i];
        res.true_residual = std::sqrt(norm2(p) / ssq);
        res.converged = 1;
      }
      return res;
    } else if (cp < delta * maxres || (relup_every > 0 && since >= relup_every)) {
      for (size_t i = 0; i < n; i++) psi[i] += cplx<double>(psi_f[i]);
      Ad(psi, mmp);
      for (size_t i = 0; i < n; i++) r[i] = src[i] - mmp[i];
      std::fill(psi_f.begin(), psi_f.end(), cplx<float>(0));
      precision_change(r_f, r);
      cp = norm2(r);
      maxres = cp;
      b = cp / c;
      l++;
      since = 0;
    }
    for (size_t i = 0; i < n; i++) p_f[i] = float(b) * p_f[i] + r_f[i];
  }
  res.iterations = maxit;
  res.reliable_updates = l;
  return res;
}

}  // namespace orc
