// gb_madwf.cu -- MADWF's defect-correction loop and the Pauli-Villars inverters it runs
// with: one implementation behind the C ABI, which the C++ and Python interfaces call.
//
// MADWF (Grid/qcd/action/fermion/MADWF.h:47-209) solves an outer (Moebius) system through
// two solvers handed to it as functions: a Pauli-Villars (mass 1) inverse of the outer
// operator and a red-black solve of a cheaper inner operator.  The Pauli-Villars inverters
// of PauliVillarsInverters.h:32-88 are provided here as such functions; the Fourier
// accelerated one restates FourierAcceleratedPV.h:56-237.  Everything runs on the
// operators' streams; the only kernel of this file negates a 4D surface field.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "gb_ops.h"

struct gb_pv_fourier_s {
  const double* U = nullptr;  // canonical FP64 gauge field in host memory (borrowed)
  gb_cg_params cg{};
  int group_in_s = 2;
  gb_cg_result result{};
  // the twisted-mass operator of the last call and what it was built for
  gb_op_t tm = nullptr;
  int dims[4] = {0, 0, 0, 0};
  int prec = -1;
  cudaStream_t stream = nullptr;
  std::complex<double> phases[4];
};

namespace gb {
namespace {

// a full field of op owned for the length of one call
struct TmpField {
  gb_field_t f = nullptr;
  ~TmpField() {
    if (f) gb_field_destroy(f);
  }
  int make(gb_op_t op) { return gb_field_create(op, GB_FULL, op->prec, &f); }
};

// the masses of one or two operators, put back when the guard goes
struct MassGuard {
  gb_op_t a, b;
  double ma, mb;
  MassGuard(gb_op_t a_, gb_op_t b_) : a(a_), b(b_), ma(a_ ? a_->mass : 0.0), mb(b_ ? b_->mass : 0.0) {}
  int set(double m) {
    if (a) GB_TRY(gb_op_set_mass(a, m));
    if (b) GB_TRY(gb_op_set_mass(b, m));
    return GB_OK;
  }
  ~MassGuard() {
    if (a) gb_op_set_mass(a, ma);
    if (b) gb_op_set_mass(b, mb);
  }
};

// a device buffer allocated on a stream for the length of one call
struct StreamBuffer {
  double* p = nullptr;
  cudaStream_t s = nullptr;
  ~StreamBuffer() {
    if (p) cudaFreeAsync(p, s);
  }
};

__global__ void negate_kernel(const double* __restrict__ in, double* __restrict__ out, size_t n) {
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x)
    out[i] = -in[i];
}

// sum over the visible right-hand sides of |f|^2
int norm2_sum(gb_field_t f, double* out) {
  std::vector<double> v(size_t(std::max(f->op->nrhs, 1)), 0.0);
  GB_TRY(gb_field_norm2(f, v.data()));
  double s = 0;
  for (int r = 0; r < f->op->nrhs_user; r++) s += v[size_t(r)];
  *out = s;
  return GB_OK;
}

// work queued on `to` after this point waits for the work queued on `from` so far
int order_streams(cudaStream_t from, cudaStream_t to, cudaEvent_t ev) {
  if (from == to) return GB_OK;
  GB_CHECK_CUDA(cudaEventRecord(ev, from));
  GB_CHECK_CUDA(cudaStreamWaitEvent(to, ev, 0));
  return GB_OK;
}

struct EventGuard {
  cudaEvent_t e = nullptr;
  ~EventGuard() {
    if (e) cudaEventDestroy(e);
  }
};

bool full_field_of(gb_field_t f, const Op* op) { return f && f->full() && ops_conformable(f->op, op); }

void merge_result(gb_cg_result& total, const gb_cg_result& r) {
  total.iterations += r.iterations;
  total.reliable_updates += r.reliable_updates;
  total.cleanup_iterations += r.cleanup_iterations;
  total.converged = total.converged && r.converged;
  total.true_residual = std::max(total.true_residual, r.true_residual);
  total.seconds += r.seconds;
  total.flops += r.flops;
}

}  // namespace
}  // namespace gb

using namespace gb;

extern "C" {

// SchurRedBlackDiagMooeeSolve(CG) (SchurRedBlack.h:236-291); the solve zeroes its odd
// initial guess itself, which is ZeroGuesser's guess
int gb_solver_schur(void* user, gb_op_t op, gb_field_t src, gb_field_t sol) {
  auto* s = static_cast<gb_cg_solver*>(user);
  if (!s || !op) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  std::vector<double> unprec(size_t(std::max(op->nrhs_user, 1)), 0.0);
  gb_cg_result r{};
  const int rc = gb_schur_solve(op, s->op_lo, src, sol, &s->cg, &r, unprec.data());
  s->result = r;
  s->unprec_residual = *std::max_element(unprec.begin(), unprec.end());
  return rc;
}

// PauliVillarsSolverUnprec (PauliVillarsInverters.h:32-52): at mass 1, A = Mdag src and CG
// on Mdag M from sol
int gb_solver_pv_unprec(void* user, gb_op_t op, gb_field_t src, gb_field_t sol) {
  auto* s = static_cast<gb_cg_solver*>(user);
  if (!s || !op) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (s->op_lo) { set_error("PauliVillarsSolverUnprec: a plain CG (op_lo NULL)"); return GB_ERR_UNSUPPORTED; }
  TmpField A;
  GB_TRY(A.make(op));
  MassGuard mass(op, nullptr);
  GB_TRY(mass.set(1.0));
  GB_TRY(gb_Mdag(op, src, A.f));
  gb_cg_result r{};
  const int rc = gb_cg_mdagm(op, A.f, sol, &s->cg, &r);
  s->result = r;
  return rc;
}

// PauliVillarsSolverRBprec (PauliVillarsInverters.h:54-72): the Schur solve at mass 1; a
// mixed-precision solve's inner operator is moved to mass 1 with it
int gb_solver_pv_rbprec(void* user, gb_op_t op, gb_field_t src, gb_field_t sol) {
  auto* s = static_cast<gb_cg_solver*>(user);
  if (!s || !op) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  MassGuard mass(op, s->op_lo);
  GB_TRY(mass.set(1.0));
  gb_cg_result r{};
  const int rc = gb_schur_solve(op, s->op_lo, src, sol, &s->cg, &r, nullptr);
  s->result = r;
  return rc;
}

int gb_pv_fourier_create(const double* U, const gb_cg_params* cg, int group_in_s, gb_pv_fourier_t* out) {
  if (!U || !cg || !out) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (group_in_s < 1 || 2 * group_in_s > kMaxSlots) {
    set_error("FourierAcceleratedPV: group_in_s in [1, %d]", kMaxSlots / 2);
    return GB_ERR_BAD_ARG;
  }
  auto* pv = new (std::nothrow) gb_pv_fourier_s;
  if (!pv) { set_error("host allocation failed"); return GB_ERR_OOM; }
  pv->U = U;
  pv->cg = *cg;
  pv->group_in_s = group_in_s;
  *out = pv;
  return GB_OK;
}

int gb_pv_fourier_destroy(gb_pv_fourier_t pv) {
  if (!pv) return GB_OK;
  if (pv->tm) gb_op_destroy(pv->tm);
  delete pv;
  return GB_OK;
}

int gb_pv_fourier_set_params(gb_pv_fourier_t pv, const gb_cg_params* cg) {
  if (!pv || !cg) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  pv->cg = *cg;
  return GB_OK;
}

int gb_pv_fourier_result(gb_pv_fourier_t pv, gb_cg_result* res) {
  if (!pv || !res) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  *res = pv->result;
  return GB_OK;
}

// FourierAcceleratedPV::pvInv (FourierAcceleratedPV.h:56-237).  With p = pi (2 s + 1) / Ls
// and den = b^2 + c^2 + 2 b c cos p, Fourier mode s of the mass-1 Cayley operator is the
// 4D Wilson operator at
//   mass = -(b^2 M5 + c (1 - cos p + c M5) + b (cos p - 1 + 2 c M5 cos p)) / den,
//   mu = (b + c) sin p / den,
// times (pA + pB gamma5), pA = b + c cos p, pB = -i c sin p; modes s and Ls-1-s carry
// opposite mu and are solved as the two slices of one twisted-mass pair.
int gb_solver_pv_fourier(void* user, gb_op_t op, gb_field_t src, gb_field_t sol) {
  auto* pv = static_cast<gb_pv_fourier_s*>(user);
  if (!pv || !op) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (op->kind != 1 || op->zmobius) {
    set_error("FourierAcceleratedPV: a Moebius operator with constant real b, c");
    return GB_ERR_UNSUPPORTED;
  }
  if (op->nrhs_user != 1) { set_error("FourierAcceleratedPV: one right-hand side"); return GB_ERR_UNSUPPORTED; }
  if (op->prec == GB_F16) { set_error("FourierAcceleratedPV: FP64 or FP32"); return GB_ERR_UNSUPPORTED; }
  const int Ls = op->Ls, g = pv->group_in_s;
  if (Ls % (2 * g) != 0) { set_error("FourierAcceleratedPV: Ls = %d is not a multiple of 2 group_in_s = %d", Ls, 2 * g); return GB_ERR_BAD_ARG; }
  if (!full_field_of(src, op) || !full_field_of(sol, op)) {
    set_error("FourierAcceleratedPV: full fields of the operator expected");
    return GB_ERR_BAD_ARG;
  }
  if (src == sol) { set_error("FourierAcceleratedPV: src and sol must be distinct"); return GB_ERR_BAD_ARG; }
  const double b = op->b, c = op->c, M5 = op->M5, pi = 3.14159265358979323846;

  // rotatePV: the twist e^{-i pi s / Ls} then the Ls-point DFT, and its inverse
  std::vector<std::complex<double>> T(size_t(Ls) * Ls), B(size_t(Ls) * Ls);
  for (int k = 0; k < Ls; k++)
    for (int s = 0; s < Ls; s++) {
      T[size_t(k) * Ls + s] = std::polar(1.0, -2 * pi * k * s / Ls - pi * s / Ls);
      B[size_t(s) * Ls + k] = std::polar(1.0 / Ls, 2 * pi * k * s / Ls + pi * s / Ls);
    }
  TmpField src_diag, dst_diag;
  GB_TRY(src_diag.make(op));
  GB_TRY(dst_diag.make(op));
  GB_TRY(gb_field_dft_s(src, src_diag.f, reinterpret_cast<const double*>(T.data())));

  // the twisted-mass pair operator, rebuilt only when the lattice it must match changes
  bool same = pv->tm && pv->prec == op->prec && pv->stream == op->stream;
  for (int k = 0; k < 4 && same; k++) same = pv->dims[k] == op->dims[k] && pv->phases[k] == op->phases[k];
  if (!same) {
    if (pv->tm) gb_op_destroy(pv->tm);
    pv->tm = nullptr;
    std::vector<double> zero(size_t(2 * g), 0.0), ph(8);
    for (int k = 0; k < 4; k++) { ph[2 * k] = op->phases[k].real(); ph[2 * k + 1] = op->phases[k].imag(); }
    GB_TRY(gb_wilson_tm5d_create(op->dims, 2 * g, zero.data(), zero.data(), ph.data(), op->prec, op->stream, 0, &pv->tm));
    std::copy(op->dims, op->dims + 4, pv->dims);
    std::copy(op->phases, op->phases + 4, pv->phases);
    pv->prec = op->prec;
    pv->stream = op->stream;
  }
  gb_op_t tm = pv->tm;
  GB_TRY(gb_op_import_gauge(tm, pv->U));
  TmpField ts, tx, ty;
  GB_TRY(ts.make(tm));
  GB_TRY(tx.make(tm));
  GB_TRY(ty.make(tm));

  gb_cg_result total{};
  total.converged = 1;
  std::vector<double> vmass(size_t(2 * g)), vmu(size_t(2 * g)), coef(size_t(8) * g);
  for (int sgroup = 0; sgroup < Ls / 2 / g; sgroup++) {
    for (int sidx = 0; sidx < g; sidx++) {
      const int s = sgroup * g + sidx;
      const double p = pi / Ls * (2.0 * s + 1.0), cp = std::cos(p), sp = std::sin(p);
      const double den = b * b + c * c + 2.0 * b * c * cp;
      const double mass = -(b * b * M5 + c * (1.0 - cp + c * M5) + b * (-1.0 + cp + 2.0 * c * cp * M5)) / den;
      const double mu = (b + c) * sp / den;
      vmass[size_t(2 * sidx)] = vmass[size_t(2 * sidx + 1)] = mass;
      vmu[size_t(2 * sidx)] = mu;
      vmu[size_t(2 * sidx + 1)] = -mu;
      const std::complex<double> pA(b + c * cp, 0.0), pB(0.0, -c * sp), pden = pA * pA - pB * pB;
      const std::complex<double> lo = (pA - pB) / pden, hi = (pA + pB) / pden;
      // slice 2 sidx: (pA - pB gamma5) / pden; slice 2 sidx + 1: (pA + pB gamma5) / pden
      const std::complex<double> cf[4] = {lo, hi, hi, lo};
      for (int q = 0; q < 4; q++) {
        coef[size_t(8) * sidx + 2 * q] = cf[q].real();
        coef[size_t(8) * sidx + 2 * q + 1] = cf[q].imag();
      }
      GB_TRY(gb_field_copy_slice5(ts.f, 2 * sidx, src_diag.f, s));
      GB_TRY(gb_field_copy_slice5(ts.f, 2 * sidx + 1, src_diag.f, Ls - s - 1));
    }
    GB_TRY(gb_op_tm_update(tm, vmass.data(), vmu.data()));
    GB_TRY(gb_field_zero(tx.f));
    gb_cg_result r{};
    const int rc = gb_schur_solve(tm, nullptr, ts.f, tx.f, &pv->cg, &r, nullptr);
    merge_result(total, r);
    pv->result = total;
    GB_TRY(rc);
    GB_TRY(gb_field_chiral_scale(tx.f, ty.f, coef.data()));
    for (int sidx = 0; sidx < g; sidx++) {
      const int s = sgroup * g + sidx;
      GB_TRY(gb_field_copy_slice5(dst_diag.f, s, ty.f, 2 * sidx));
      GB_TRY(gb_field_copy_slice5(dst_diag.f, Ls - s - 1, ty.f, 2 * sidx + 1));
    }
  }
  GB_TRY(gb_field_dft_s(dst_diag.f, sol, reinterpret_cast<const double*>(B.data())));
  return GB_OK;
}

// MADWF::operator() (MADWF.h:94-209)
int gb_madwf(gb_op_t outer, gb_op_t inner, gb_solver_fn pv, void* pv_user, gb_solver_fn inner_solve,
             void* inner_user, gb_field_t src5, gb_field_t sol5, double resid, int maxiter, gb_madwf_callback callback,
             void* callback_user, int* iterations, double* final_resid) {
  if (iterations) *iterations = 0;
  if (final_resid) *final_resid = 0;
  if (!outer || !inner || !pv || !inner_solve || !src5 || !sol5) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (outer->kind != 1 || inner->kind != 1) {
    set_error("MADWF: Moebius or ZMobius outer and inner operators");
    return GB_ERR_UNSUPPORTED;
  }
  for (int k = 0; k < 4; k++)
    if (outer->dims[k] != inner->dims[k]) { set_error("MADWF: outer and inner operators on different 4D lattices"); return GB_ERR_BAD_ARG; }
  if (outer->nrhs_user != inner->nrhs_user) { set_error("MADWF: outer and inner right-hand sides differ"); return GB_ERR_BAD_ARG; }
  if (!full_field_of(src5, outer) || !full_field_of(sol5, outer)) {
    set_error("MADWF: src5 and sol5 must be full fields of the outer operator");
    return GB_ERR_BAD_ARG;
  }
  if (maxiter < 0) { set_error("MADWF: maxiter < 0"); return GB_ERR_BAD_ARG; }

  TmpField A, B, bf, c, defect, ci, yi, xi, srci, Ai;
  for (TmpField* f : {&A, &B, &bf, &c, &defect}) GB_TRY(f->make(outer));
  for (TmpField* f : {&ci, &yi, &xi, &srci, &Ai}) GB_TRY(f->make(inner));
  // the s = 0 surface: y0 and -y0, canonical FP64 4D fields on the outer stream
  const size_t n4 = size_t(outer->vol4) * outer->nrhs_user * 24;
  StreamBuffer surf;
  surf.s = outer->stream;
  GB_CHECK_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&surf.p), 2 * n4 * sizeof(double), outer->stream));
  double* y0 = surf.p;
  double* neg_y0 = surf.p + n4;
  EventGuard ev;
  GB_CHECK_CUDA(cudaEventCreateWithFlags(&ev.e, cudaEventDisableTiming));
  const int nblocks = int(std::min<size_t>((n4 + 255) / 256, size_t(8) * 152));
  const double m_inner = inner->mass;
  MassGuard keep_inner(inner, nullptr);

  GB_TRY(gb_field_copy(bf.f, src5));
  double nb = 0;
  GB_TRY(norm2_sum(bf.f, &nb));
  GB_TRY(gb_field_zero(sol5));
  if (nb == 0) return GB_OK;  // the zero source has the zero solution
  GB_TRY(gb_field_copy(defect.f, bf.f));
  double r = 0;
  for (int i = 0; i < maxiter; i++) {
    // c0: the s = 0 slice of Pdag PV^-1 defect
    GB_TRY(pv(pv_user, outer, defect.f, A.f));
    GB_TRY(gb_P(outer, A.f, c.f, 1));
    GB_TRY(gb_extract_slice(outer, c.f, 0, y0, 1));
    GB_TRY(order_streams(outer->stream, inner->stream, ev.e));
    // the inner system with surface term c0: Dwm P y = D(1) P (c0, 0, ..., 0)^T
    GB_TRY(gb_field_zero(ci.f));
    GB_TRY(gb_insert_slice(inner, y0, 1, ci.f, 0));
    GB_TRY(gb_P(inner, ci.f, Ai.f, 0));
    GB_TRY(gb_op_set_mass(inner, 1.0));
    const int rc_m = gb_M(inner, Ai.f, srci.f);
    GB_TRY(gb_op_set_mass(inner, m_inner));
    GB_TRY(rc_m);
    GB_TRY(gb_field_zero(xi.f));
    GB_TRY(inner_solve(inner_user, inner, srci.f, xi.f));
    GB_TRY(gb_P(inner, xi.f, yi.f, 1));
    GB_TRY(gb_extract_slice(inner, yi.f, 0, y0, 1));
    GB_TRY(order_streams(inner->stream, outer->stream, ev.e));
    // the bulk of the outer solution: Pdag PV^-1 Dm P (-y0, c_1, ..., c_{Ls-1}), then the
    // surface solution y0 back in and P back to x
    negate_kernel<<<nblocks, 256, 0, outer->stream>>>(y0, neg_y0, n4);
    GB_CHECK_CUDA(cudaGetLastError());
    GB_TRY(gb_insert_slice(outer, neg_y0, 1, c.f, 0));
    GB_TRY(gb_P(outer, c.f, B.f, 0));
    GB_TRY(gb_M(outer, B.f, A.f));
    GB_TRY(pv(pv_user, outer, A.f, B.f));
    GB_TRY(gb_P(outer, B.f, A.f, 1));
    GB_TRY(gb_insert_slice(outer, y0, 1, A.f, 0));
    GB_TRY(gb_P(outer, A.f, B.f, 0));
    GB_TRY(gb_field_axpy(sol5, 1.0, B.f, sol5));  // sol5 += M^-1 defect
    GB_TRY(gb_M(outer, sol5, A.f));
    GB_TRY(gb_field_axpby(defect.f, 1.0, -1.0, bf.f, A.f));  // defect = src5 - M sol5
    double nd = 0;
    GB_TRY(norm2_sum(defect.f, &nd));
    r = std::sqrt(nd / nb);
    if (iterations) *iterations = i + 1;
    if (final_resid) *final_resid = r;
    if (callback) GB_TRY(callback(callback_user, i + 1, r));
    if (r < resid) return GB_OK;
  }
  set_error("MADWF: not converged in %d iterations (residual %.3e)", maxiter, r);
  return GB_ERR_NOT_CONVERGED;
}

}  // extern "C"
