// oracle_capi.cpp -- extern "C" face of the CPU oracle (TEST INFRASTRUCTURE ONLY).
//
// Every array is the canonical host layout described in oracle.hpp, complex<double>
// interleaved (re, im).  Operators built with prec = 1 compute in float: inputs are
// rounded to float, outputs widened back to double.
#include "oracle.hpp"

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace orc;

namespace {

struct Handle {
  int kind;  // 0 = Wilson, 1 = Moebius
  int prec;  // 0 = double, 1 = float
  Op<double>* d = nullptr;
  Op<float>* f = nullptr;
  ~Handle() { delete d; delete f; }
};

template <class R> Field<R> load(const double* p, size_t n) {
  Field<R> f(n);
  for (size_t i = 0; i < n; i++) f[i] = cplx<R>(R(p[2 * i]), R(p[2 * i + 1]));
  return f;
}
template <class R> void store(const Field<R>& f, double* p) {
  for (size_t i = 0; i < f.size(); i++) { p[2 * i] = double(f[i].real()); p[2 * i + 1] = double(f[i].imag()); }
}

enum Opcode {
  OP_M = 0, OP_MDAG = 1, OP_DHOP = 2, OP_DHOP_DAG = 3, OP_MEOOE = 4, OP_MEOOE_DAG = 5, OP_MOOEE = 6,
  OP_MOOEE_DAG = 7, OP_MOOEE_INV = 8, OP_MOOEE_INV_DAG = 9, OP_MPC = 10, OP_MPC_DAG = 11,
  OP_MPCDAGMPC = 12, OP_MDAGM = 13, OP_MEOOE5D = 14, OP_MEOOE_DAG5D = 15, OP_DMINUS = 16,
  OP_DMINUS_DAG = 17, OP_P = 18, OP_PDAG = 19
};

// returns the input length (in complex numbers) that the opcode expects
template <class R> size_t in_len(Op<R>* op, int opcode) {
  switch (opcode) {
    case OP_M: case OP_MDAG: case OP_DHOP: case OP_DHOP_DAG: case OP_MDAGM: case OP_DMINUS: case OP_DMINUS_DAG:
    case OP_P: case OP_PDAG:
      return op->full_len();
    default: return op->half_len();
  }
}

template <class R> int apply(Op<R>* op, int kind, int opcode, const double* in, double* out, int parity) {
  size_t n = in_len(op, opcode);
  Field<R> a = load<R>(in, n), b;
  switch (opcode) {
    case OP_M: op->M(a, b); break;
    case OP_MDAG: op->Mdag(a, b); break;
    case OP_DHOP: op->Dhop(a, b, 0); break;
    case OP_DHOP_DAG: op->Dhop(a, b, 1); break;
    case OP_MEOOE: op->Meooe(a, b, parity); break;
    case OP_MEOOE_DAG: op->MeooeDag(a, b, parity); break;
    case OP_MOOEE: op->Mooee(a, b); break;
    case OP_MOOEE_DAG: op->MooeeDag(a, b); break;
    case OP_MOOEE_INV: op->MooeeInv(a, b); break;
    case OP_MOOEE_INV_DAG: op->MooeeInvDag(a, b); break;
    case OP_MPC: op->Mpc(a, b); break;
    case OP_MPC_DAG: op->MpcDag(a, b); break;
    case OP_MPCDAGMPC: op->MpcDagMpc(a, b); break;
    case OP_MDAGM: op->MdagM(a, b); break;
    case OP_MEOOE5D:
    case OP_MEOOE_DAG5D: {
      if (kind == 0) return 1;
      auto* m = static_cast<CayleyBase<R>*>(op);
      if (opcode == OP_MEOOE5D) m->Meooe5D(a, b); else m->MeooeDag5D(a, b);
      break;
    }
    case OP_DMINUS:
    case OP_DMINUS_DAG: {
      if (kind == 0) return 1;
      static_cast<CayleyBase<R>*>(op)->Dminus(a, b, opcode == OP_DMINUS_DAG);
      break;
    }
    case OP_P:
    case OP_PDAG: {
      if (kind == 0) return 1;
      static_cast<CayleyBase<R>*>(op)->P(a, b, opcode == OP_PDAG);
      break;
    }
    default: return 1;
  }
  store<R>(b, out);
  return 0;
}

template <class R> Op<R>* make(int kind, const int* dims, int L5, const double* par) {
  if (kind == 0) return new Wilson<R>(dims, L5, par[0]);
  if (kind == 1) return new Mobius<R>(dims, L5, par[0], par[1], par[2], par[3]);
  // ZMobius: par[4 + 2 s], par[5 + 2 s] = gamma_s
  std::vector<cplx<double>> gamma(L5);
  for (int s = 0; s < L5; s++) gamma[s] = cplx<double>(par[4 + 2 * s], par[5 + 2 * s]);
  return new Mobius<R, cplx<double>>(dims, L5, par[0], par[1], par[2], par[3], gamma);
}

}  // namespace

extern "C" {

void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}
int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// kind 0: Wilson, par = {mf}; kind 1: Moebius, par = {mf, M5, b, c}, L5 = Ls; kind 2:
// ZMobius, par = {mf, M5, b, c, gamma_0 (re, im), ..., gamma_{Ls-1}}.
// U: canonical gauge field; phases: 4 complex boundary phases.
void* orc_create(int kind, int prec, const int* dims, int L5, const double* par, const double* U,
                 const double* phases) {
  Handle* h = new Handle;
  h->kind = kind;
  h->prec = prec;
  const cplx<double>* Uc = reinterpret_cast<const cplx<double>*>(U);
  const cplx<double>* ph = reinterpret_cast<const cplx<double>*>(phases);
  if (prec == 0) { h->d = make<double>(kind, dims, L5, par); h->d->import_gauge(Uc, ph); }
  else { h->f = make<float>(kind, dims, L5, par); h->f->import_gauge(Uc, ph); }
  return h;
}
void orc_free(void* p) { delete static_cast<Handle*>(p); }

// SetMass: the operator's mass (and, for Cayley operators, its coefficients) changes
int orc_set_mass(void* p, double mass) {
  Handle* h = static_cast<Handle*>(p);
  if (h->prec == 0) h->d->set_mass(mass);
  else h->f->set_mass(mass);
  return 0;
}

// parity = parity of the input field for the half-checkerboard opcodes
int orc_apply(void* p, int opcode, const double* in, double* out, int parity) {
  Handle* h = static_cast<Handle*>(p);
  if (h->prec == 0) return apply<double>(h->d, h->kind, opcode, in, out, parity);
  return apply<float>(h->f, h->kind, opcode, in, out, parity);
}

// 4D <-> 5D surface fields of a Moebius operator (CayleyFermion5DImplementation.h:57-129).
// mode 0: ImportPhysicalFermionSource, 1: ImportUnphysicalFermion (in4: full 4D field,
// out5: full 5D field); mode 2: ExportPhysicalFermionSolution, 3: ExportPhysicalFermionSource
// (in = 5D, out = 4D).
int orc_physical(void* p, int mode, const double* in, double* out) {
  Handle* h = static_cast<Handle*>(p);
  if (h->kind == 0 || h->prec != 0) return 1;
  auto* m = static_cast<CayleyBase<double>*>(h->d);
  const size_t n5 = m->full_len(), n4 = n5 / size_t(m->L5);
  Field<double> a = load<double>(in, mode < 2 ? n4 : n5), b;
  switch (mode) {
    case 0: m->ImportPhysicalSource(a, b); break;
    case 1: m->ImportUnphysical(a, b); break;
    case 2: m->ExportPhysical(a, b, true); break;
    case 3: m->ExportPhysical(a, b, false); break;
    default: return 1;
  }
  store<double>(b, out);
  return 0;
}

// DhopEO / DhopOE: in has parity in_parity, out the other one
int orc_dhop_cb(void* p, const double* in, double* out, int in_parity, int dag) {
  Handle* h = static_cast<Handle*>(p);
  if (h->prec == 0) {
    Field<double> a = load<double>(in, h->d->half_len()), b;
    h->d->DhopCB(a, b, in_parity, dag);
    store<double>(b, out);
  } else {
    Field<float> a = load<float>(in, h->f->half_len()), b;
    h->f->DhopCB(a, b, in_parity, dag);
    store<float>(b, out);
  }
  return 0;
}

// doubled links (canonical site order, [site][8][3][3]) as stored by the operator
void orc_doubled_links(void* p, double* Ud) {
  Handle* h = static_cast<Handle*>(p);
  if (h->prec == 0) store<double>(h->d->Ud, Ud);
  else store<float>(h->f->Ud, Ud);
}

void orc_dhop_naive(const int* dims, int L5, const double* U, const double* phases, const double* in, double* out,
                    int dag) {
  Geom g(dims);
  size_t n = size_t(g.vol) * L5 * Nsc;
  Field<double> a = load<double>(in, n), b;
  dhop_naive<double>(g, L5, reinterpret_cast<const cplx<double>*>(U), reinterpret_cast<const cplx<double>*>(phases),
                     a, b, dag);
  store<double>(b, out);
}

// out: 9*Ls doubles = bs, cs, bee, cee, dee, lee, leem, uee, ueem
void orc_cayley_coeffs(int Ls, double mf, double M5, double b, double c, double* out) {
  Cayley cf;
  cf.setup(Ls, mf, M5, b, c);
  const std::vector<double>* v[9] = {&cf.bs, &cf.cs, &cf.bee, &cf.cee, &cf.dee, &cf.lee, &cf.leem, &cf.uee, &cf.ueem};
  for (int k = 0; k < 9; k++) std::copy(v[k]->begin(), v[k]->end(), out + k * Ls);
}

// CG on kind 0: MdagM (full field) or kind 1: Schur MpcDagMpc (odd half field).
// psi holds the initial guess on entry.  info = {iterations, converged}; resid = true residual.
int orc_cg(void* p, int kind, const double* src, double* psi, double tol, int maxit, int* info, double* resid) {
  Handle* h = static_cast<Handle*>(p);
  CGResult r;
  if (h->prec == 0) {
    Op<double>* op = h->d;
    size_t n = kind == 0 ? op->full_len() : op->half_len();
    Field<double> s = load<double>(src, n), x = load<double>(psi, n);
    if (kind == 0) r = cg<double>([&](const Field<double>& a, Field<double>& b) { op->MdagM(a, b); }, s, x, tol, maxit);
    else r = cg<double>([&](const Field<double>& a, Field<double>& b) { op->MpcDagMpc(a, b); }, s, x, tol, maxit);
    store<double>(x, psi);
  } else {
    Op<float>* op = h->f;
    size_t n = kind == 0 ? op->full_len() : op->half_len();
    Field<float> s = load<float>(src, n), x = load<float>(psi, n);
    if (kind == 0) r = cg<float>([&](const Field<float>& a, Field<float>& b) { op->MdagM(a, b); }, s, x, tol, maxit);
    else r = cg<float>([&](const Field<float>& a, Field<float>& b) { op->MpcDagMpc(a, b); }, s, x, tol, maxit);
    store<float>(x, psi);
  }
  info[0] = r.iterations;
  info[1] = r.converged;
  *resid = r.true_residual;
  return r.converged ? 0 : 5;
}

// SchurRedBlackDiagMooeeSolve with CG (SchurRedBlack.h:236-291,373-436) in double.
// src, sol: full fields.  resid[0] = CG true residual, resid[1] = unpreconditioned
// true residual |M sol - src| / |src|.  guess (full field, or NULL for zero): the odd
// checkerboard's starting vector of the CG, as Grid's solver takes the incoming solution's
// odd sites (SchurRedBlack.h:261-265); it changes the work, not what the CG converges to.
int orc_schur_solve_guess(void* p, const double* src, const double* guess, double* sol, double tol, int maxit,
                          int* info, double* resid);
int orc_schur_solve(void* p, const double* src, double* sol, double tol, int maxit, int* info, double* resid) {
  return orc_schur_solve_guess(p, src, nullptr, sol, tol, maxit, info, resid);
}
int orc_schur_solve_guess(void* p, const double* src, const double* guess, double* sol, double tol, int maxit,
                          int* info, double* resid) {
  Handle* h = static_cast<Handle*>(p);
  if (h->prec != 0) return 1;
  Op<double>* op = h->d;
  Field<double> in = load<double>(src, op->full_len()), src_e, src_o, tmp, Mtmp, t2, sol_o, sol_e, out;
  pick_cb<double>(op->g, op->L5, 0, in, src_e);
  pick_cb<double>(op->g, op->L5, 1, in, src_o);
  op->MooeeInv(src_e, tmp);
  op->Meooe(tmp, Mtmp, 0);
  for (size_t i = 0; i < Mtmp.size(); i++) tmp[i] = src_o[i] - Mtmp[i];
  op->MpcDag(tmp, src_o);
  sol_o.assign(src_o.size(), cplx<double>(0));
  if (guess) pick_cb<double>(op->g, op->L5, 1, load<double>(guess, op->full_len()), sol_o);
  CGResult r = cg<double>([&](const Field<double>& a, Field<double>& b) { op->MpcDagMpc(a, b); }, src_o, sol_o, tol, maxit);
  op->Meooe(sol_o, tmp, 1);
  for (size_t i = 0; i < tmp.size(); i++) t2.push_back(src_e[i] - tmp[i]);
  op->MooeeInv(t2, sol_e);
  out.assign(op->full_len(), cplx<double>(0));
  set_cb<double>(op->g, op->L5, 0, sol_e, out);
  set_cb<double>(op->g, op->L5, 1, sol_o, out);
  Field<double> Mout;
  op->M(out, Mout);
  for (size_t i = 0; i < Mout.size(); i++) Mout[i] -= in[i];
  store<double>(out, sol);
  info[0] = r.iterations;
  info[1] = r.converged;
  resid[0] = r.true_residual;
  resid[1] = std::sqrt(norm2(Mout) / norm2(in));
  return r.converged ? 0 : 5;
}

// Reliable-update mixed-precision CG (double outer, float inner) on kind 0 (MdagM) or
// kind 1 (Schur MpcDagMpc).  pd: double handle, pf: float handle on the same gauge field.
// info = {iterations, reliable_updates, cleanup_iterations, converged}.
int orc_cg_reliable(void* pd, void* pf, int kind, const double* src, double* psi, double tol, int maxit, double delta,
                    int relup_every, int cleanup, int* info, double* resid) {
  Handle* hd = static_cast<Handle*>(pd);
  Handle* hf = static_cast<Handle*>(pf);
  if (hd->prec != 0 || hf->prec != 1) return 1;
  Op<double>* od = hd->d;
  Op<float>* of = hf->f;
  size_t n = kind == 0 ? od->full_len() : od->half_len();
  Field<double> s = load<double>(src, n), x = load<double>(psi, n);
  CGResult r;
  auto Ad = [&](const Field<double>& a, Field<double>& b) { if (kind == 0) od->MdagM(a, b); else od->MpcDagMpc(a, b); };
  auto Af = [&](const Field<float>& a, Field<float>& b) { if (kind == 0) of->MdagM(a, b); else of->MpcDagMpc(a, b); };
  r = cg_reliable(Ad, Af, s, x, tol, maxit, delta, relup_every, cleanup != 0);
  store<double>(x, psi);
  info[0] = r.iterations;
  info[1] = r.reliable_updates;
  info[2] = r.cleanup_iterations;
  info[3] = r.converged;
  *resid = r.true_residual;
  return r.converged ? 0 : 5;
}

}  // extern "C"

extern "C" {
// ConjugateGradientMultiShift in double (ConjugateGradientMultiShift.h:76-330): kind 0
// MdagM (full field), 1 MpcDagMpc (odd half field).  psi: nshift fields back to back.
// info = {iterations, converged, iterations of shift 0, 1, ...}; resid: true residual per shift.
int orc_cg_multishift(void* p, int kind, const double* src, int nshift, const double* mass, const double* tol,
                      int maxit, double* psi, int* info, double* resid) {
  Handle* h = static_cast<Handle*>(p);
  if (h->prec != 0) return 1;
  Op<double>* op = h->d;
  const size_t n = kind == 0 ? op->full_len() : op->half_len();
  Field<double> s = load<double>(src, n);
  std::vector<Field<double>> x;
  std::vector<double> m(mass, mass + nshift), t(tol, tol + nshift);
  MultiShiftResult r;
  if (kind == 0)
    r = cg_multishift([&](const Field<double>& a, Field<double>& b) { op->MdagM(a, b); }, s, x, m, t, maxit);
  else
    r = cg_multishift([&](const Field<double>& a, Field<double>& b) { op->MpcDagMpc(a, b); }, s, x, m, t, maxit);
  for (int k = 0; k < nshift; k++) {
    store<double>(x[k], psi + size_t(k) * n * 2);
    info[2 + k] = r.iterations_shift[k];
    resid[k] = r.true_residual[k];
  }
  info[0] = r.iterations;
  info[1] = r.converged;
  return r.converged ? 0 : 5;
}
}

extern "C" {
// DhopDeriv / MDeriv in double on full canonical fields (DhopDeriv: A, B as given;
// MDeriv of a Moebius operator: B -> Meooe5D B (dag = 0) or A -> Meooe5D A (dag = 1),
// CayleyFermion5DImplementation.h:346-391).  out_parity < 0: all sites (the full-field
// form); 0 / 1: only the sites of that parity (DerivEO / DerivOE with A on that parity).
// mat: [site][mu][3][3] complex.
int orc_deriv(void* p, int mderiv, const double* A, const double* B, int dag, int out_parity, double* mat) {
  Handle* h = static_cast<Handle*>(p);
  if (h->prec != 0) return 1;
  Op<double>* op = h->d;
  const size_t n = op->full_len();
  Field<double> a = load<double>(A, n), b = load<double>(B, n), t;
  if (mderiv && h->kind != 0) {
    auto* m = static_cast<CayleyBase<double>*>(op);
    if (!dag) { m->Meooe5D(b, t); b = t; }
    else { m->Meooe5D(a, t); a = t; }
  }
  std::vector<cplx<double>> M(size_t(op->g.vol) * 36, cplx<double>(0));
  dhop_deriv(op->g, op->L5, op->Ud, a, b, M, dag, out_parity);
  store<double>(M, mat);
  return 0;
}
}
