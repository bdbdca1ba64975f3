// gb_solvers.cpp -- ConjugateGradient, ConjugateGradientReliableUpdate and the
// SchurRedBlackDiagMooeeSolve driver on device-resident fields.
//
// Iteration (Grid/algorithms/iterative/ConjugateGradient.h:151-200), per right-hand side:
//   c = cp ; mmp = A p ; d = <p|mmp> ; a = c/d ; r -= a mmp ; cp = |r|^2 ; b = cp/c ;
//   psi += a p ; p = b p + r ; stop when cp <= tol^2 |src|^2
// with A = Mdag M or MpcDag Mpc, d = <p|A p> is reduced as |M p|^2 (|Mpc p|^2): the same
// number, from the intermediate field, by the kernel that writes it where it can.  As in
// Grid, psi and p are updated in one pass after the residual.
// All scalars live on the device (one set per right-hand side); the host only polls the
// "all converged" flag every check_every iterations, so an iteration issues no host
// synchronisation.  A right-hand side that converges freezes (a = b = 0) while the
// others continue, which gives the same per-rhs iterates as independent solves.
#include <cuda_runtime.h>

#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "gb_ops.h"

namespace gb {

namespace {

struct Timer {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double seconds() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

// partial-buffer geometry of one reduction over a (full or half) field
struct Parts {
  int g;       // CTAs per half
  int halves;
};
Parts parts_of(Op* op, const Field* f) {
  return Parts{red_parts(op, f->prec), f->full() ? 2 : 1};
}

// d = |ap|^2 (ap = M p or Mpc p) -> a
int cg_alpha_norm(Op* op, Field* ap) {
  Parts P = parts_of(op, ap);
  for (int h = 0; h < P.halves; h++)
    GB_TRY(launch_norm2_partial(op, half_view(ap, h), ap->n5, op->d_partial + size_t(h) * P.g * op->nrhs));
  return launch_cg_alpha(op, op->d_partial, P.g * P.halves, 1);
}
// r -= a mmp ; cp = |r|^2 -> b
int cg_r_update(Op* op, Field* r, Field* mmp) {
  Parts P = parts_of(op, r);
  for (int h = 0; h < P.halves; h++)
    GB_TRY(launch_cg_r_update(op, half_view(r, h), half_view(mmp, h), r->n5,
                              op->d_partial + size_t(h) * P.g * op->nrhs));
  return launch_cg_beta(op, op->d_partial, P.g * P.halves);
}
// One CG matrix step on p: A = MdagM (kind 0) or MpcDagMpc (kind 1) with d = |M p|^2
// (|Mpc p|^2) -> a, then r -= a A p, cp = |r|^2 -> b.  For a FP32 / FP16 Moebius Schur
// operator the norm comes from the kernel that stores Mpc p, and MpcDag's last kernel
// updates r in place of storing A p (mmp is then not written).
int cg_matrix_step(Op* op, int kind, Field* p, Field* mmp, Field* r) {
  int rparts = 0;
  if (kind == 0) {
    Field* mp = nullptr;
    GB_TRY(op_mdagm(op, p, mmp, &mp));
    GB_TRY(cg_alpha_norm(op, mp));
  } else {
    Field* z;
    GB_TRY(ws_get(op, GB_ODD, p->prec, WS_MPCDAGMPC, &z));
    int dparts = 0;
    GB_TRY(op_mpc(op, p, z, 0, &dparts));
    if (dparts > 0) GB_TRY(launch_cg_alpha(op, op->d_partial, dparts, 1));
    else GB_TRY(cg_alpha_norm(op, z));
    GB_TRY(op_mpc(op, z, mmp, 1, nullptr, r, &rparts));
  }
  if (rparts > 0) return launch_cg_beta(op, op->d_partial, rparts);
  return cg_r_update(op, r, mmp);
}
// psi += a p ; with update_p also p = b p + r
int cg_xp_update(Op* op, Field* psi, Field* p, Field* r, int update_p) {
  const int halves = p->full() ? 2 : 1;
  for (int h = 0; h < halves; h++)
    GB_TRY(launch_cg_xp_update(op, half_view(psi, h), half_view(p, h), half_view(r, h), p->n5, update_p));
  return GB_OK;
}
int cg_p_update(Op* op, Field* p, Field* r) {
  const int halves = p->full() ? 2 : 1;
  for (int h = 0; h < halves; h++) GB_TRY(launch_cg_p_update(op, half_view(p, h), half_view(r, h), p->n5));
  return GB_OK;
}

// flags[0..3] = op->d_all_done (converged, reliable update wanted, chunks the last device
// loop ran, its cap)
int fetch_scalars(Op* op, int* flags) {
  GB_CHECK_CUDA(cudaMemcpyAsync(op->h_cg, op->d_cg, size_t(op->nrhs) * sizeof(CGScalars), cudaMemcpyDeviceToHost,
                                op->stream));
  int* hf = reinterpret_cast<int*>(reinterpret_cast<char*>(op->h_cg) + size_t(op->nrhs) * sizeof(CGScalars));
  GB_CHECK_CUDA(cudaMemcpyAsync(hf, op->d_all_done, 4 * sizeof(int), cudaMemcpyDeviceToHost, op->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  for (int i = 0; i < 4; i++) flags[i] = hf[i];
  return GB_OK;
}

// true residual |A psi - src| / |src| per rhs into res[]
int true_residual(Op* op, int kind, Field* src, Field* psi, Field* mmp, Field* tmp, double* res) {
  GB_TRY(op_hermop(op, kind, psi, mmp));
  GB_TRY(field_axpby(tmp, 1.0, -1.0, mmp, src));
  std::vector<double> nr(op->nrhs), ns(op->nrhs);
  GB_TRY(field_norm2(tmp, nr.data()));
  GB_TRY(field_norm2(src, ns.data()));
  for (int r = 0; r < op->nrhs; r++) res[r] = ns[r] > 0 ? std::sqrt(nr[r] / ns[r]) : 0.0;
  return GB_OK;
}

}  // namespace

// flops per CG iteration in Grid's model: 1452 per half-checkerboard 5D site for each of
// the four Meooe of MpcDagMpc plus 336 of linear algebra (Test_dwf_mixedcg_prec.cc:138-140,
// ConjugateGradient.h:204-205); Wilson: 1320 per Dhop site; MdagM: two full M.
double hermop_flops(const Op* op, int kind) {
  const double half5 = double(op->half4) * op->L5;
  if (kind == 0) return 2 * half5 * (2 * 1320.0 + (op->kind ? 2 * 120.0 : 48.0)) + 2 * half5 * 336.0;
  return half5 * (4 * (op->kind ? 1452.0 : 1320.0) + 336.0);
}

namespace {

int field_for(Op* op, int kind, int subset_half, int prec, int slot_half, int slot_full, Field** out) {
  if (kind == 0) return ws_get(op, GB_FULL, prec, slot_full, out);
  return ws_get(op, subset_half, prec, slot_half, out);
}

// m CG iterations on op's stream.  A chunk starts with p = b p + r (p = r at the start of a
// solve, where b = 0; after a reliable update with the new r and b, as Grid's
// ConjugateGradientReliableUpdate does), its iterations update psi and p in one pass, and
// its last one updates psi only, so the host can replace r between chunks.  Every chunk of
// `chunk` iterations is the same launch sequence, so it is captured once as a CUDA graph
// and replayed: the first chunk runs as direct launches (it allocates the workspace), the
// following full chunks replay the graph.
struct ChunkRunner {
  Op* op;
  int kind;
  Field *p, *mmp, *r, *psi;
  int chunk;
  bool graphs;
  int runs = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // use_graphs == 2: the loop graph, WHILE (condition) { chunk iterations; check }
  cudaGraph_t lgraph = nullptr;
  cudaGraphExec_t lexec = nullptr;
  ~ChunkRunner() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (lexec) cudaGraphExecDestroy(lexec);
    if (lgraph) cudaGraphDestroy(lgraph);
  }
  // whether the device-resident loop can run now: a non-legacy stream, and a first chunk
  // already run directly (the workspace it allocates cannot be allocated inside the loop)
  bool loop_ready() const { return op->stream != nullptr && runs > 0; }
  // up to max_chunks chunks of `chunk` iterations on the device, stopping after the chunk in
  // which every right-hand side converged or a reliable update became due
  int loop(int max_chunks) {
    if (!lexec) {
      GB_CHECK_CUDA(cudaGraphCreate(&lgraph, 0));
      cudaGraphConditionalHandle h;
      GB_CHECK_CUDA(cudaGraphConditionalHandleCreate(&h, lgraph, 1, cudaGraphCondAssignDefault));
      cudaGraphNodeParams np = {};
      np.type = cudaGraphNodeTypeConditional;
      np.conditional.handle = h;
      np.conditional.type = cudaGraphCondTypeWhile;
      np.conditional.size = 1;
      cudaGraphNode_t node;
      GB_CHECK_CUDA(cudaGraphAddNode(&node, lgraph, nullptr, nullptr, 0, &np));
      cudaGraph_t body = np.conditional.phGraph_out[0];
      GB_CHECK_CUDA(cudaStreamBeginCaptureToGraph(op->stream, body, nullptr, nullptr, 0,
                                                  cudaStreamCaptureModeThreadLocal));
      int rc = launch(chunk);
      if (rc == GB_OK) rc = launch_cg_loop_check(op, h);
      cudaGraph_t got = nullptr;
      const cudaError_t e = cudaStreamEndCapture(op->stream, &got);
      if (rc != GB_OK) return rc;
      if (e != cudaSuccess) { set_error("CG loop capture: %s", cudaGetErrorString(e)); return GB_ERR_CUDA; }
      GB_CHECK_CUDA(cudaGraphInstantiate(&lexec, lgraph, 0));
    }
    GB_TRY(launch_cg_loop_arm(op, max_chunks));
    GB_CHECK_CUDA(cudaGraphLaunch(lexec, op->stream));
    runs++;
    return GB_OK;
  }
  int launch(int m) {
    GB_TRY(cg_p_update(op, p, r));
    for (int j = 0; j < m; j++) {
      GB_TRY(cg_matrix_step(op, kind, p, mmp, r));
      GB_TRY(cg_xp_update(op, psi, p, r, j + 1 < m));
    }
    return GB_OK;
  }
  int iterate(int m) {
    const bool use = graphs && m == chunk && runs > 0 && op->stream != nullptr;
    runs++;
    if (!use) return launch(m);
    if (!exec) {
      GB_CHECK_CUDA(cudaStreamBeginCapture(op->stream, cudaStreamCaptureModeThreadLocal));
      const int rc = launch(m);
      cudaGraph_t g = nullptr;
      const cudaError_t e = cudaStreamEndCapture(op->stream, &g);
      if (rc != GB_OK) { if (g) cudaGraphDestroy(g); return rc; }
      if (e != cudaSuccess) { set_error("CG graph capture: %s", cudaGetErrorString(e)); return GB_ERR_CUDA; }
      graph = g;
      GB_CHECK_CUDA(cudaGraphInstantiate(&exec, graph, 0));
    }
    GB_CHECK_CUDA(cudaGraphLaunch(exec, op->stream));
    return GB_OK;
  }
};

// a private stream for a graph-captured solve on an operator bound to the legacy
// default stream (which cannot be captured); restored and released on scope exit
struct SolveStream {
  // the solver's operators and the operators owning the caller's fields (which may be
  // other operators of the same geometry and stream): all move to the private stream
  Op* ops[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaStream_t saved[4] = {nullptr, nullptr, nullptr, nullptr};
  cudaStream_t own = nullptr;
  SolveStream(Op* a, Op* b, Field* f0, Field* f1, bool want) {
    Op* cand[4] = {a, b, f0 ? f0->op : nullptr, f1 ? f1->op : nullptr};
    int n = 0;
    for (Op* o : cand) {
      bool seen = !o;
      for (int i = 0; i < n; i++) seen = seen || ops[i] == o;
      if (!seen) { ops[n] = o; saved[n] = o->stream; n++; }
    }
    if (!want || (a && a->stream)) return;
    cudaDeviceSynchronize();
    if (cudaStreamCreateWithFlags(&own, cudaStreamNonBlocking) != cudaSuccess) { own = nullptr; return; }
    for (Op* o : ops) if (o) o->stream = own;
  }
  ~SolveStream() {
    if (!own) return;
    cudaStreamSynchronize(own);
    for (int i = 0; i < 4; i++) if (ops[i]) ops[i]->stream = saved[i];
    cudaStreamDestroy(own);
  }
};

}  // namespace

// Plain CG in op's precision.  psi holds the initial guess on entry.
int cg_solve(Op* op, int kind, Field* src, Field* psi, const gb_cg_params* P, gb_cg_result* R) {
  Timer tm;
  const int n = op->nrhs;
  Field *p, *mmp, *r, *t;
  GB_TRY(field_for(op, kind, GB_ODD, src->prec, WS_CG_P, WS_FCG_P, &p));
  GB_TRY(field_for(op, kind, GB_ODD, src->prec, WS_CG_MMP, WS_FCG_MMP, &mmp));
  GB_TRY(field_for(op, kind, GB_ODD, src->prec, WS_CG_R, WS_FCG_R, &r));
  GB_TRY(field_for(op, kind, GB_ODD, src->prec, WS_CG_T, WS_FCG_T, &t));
  double* d_ssq = op->d_result + 2 * n;
  double* d_cp = op->d_result + 3 * n;
  GB_TRY(field_norm2_dev(src, d_ssq));
  std::vector<double> guess(n);
  GB_TRY(field_norm2(psi, guess.data()));
  bool zero_guess = true;
  for (double g : guess) {
    if (std::isnan(g)) { set_error("CG: NaN in the initial guess"); return GB_ERR_BAD_ARG; }
    if (g != 0.0) zero_guess = false;
  }
  if (zero_guess) {
    GB_TRY(field_copy(r, src));
  } else {
    GB_TRY(op_hermop(op, kind, psi, mmp));
    GB_TRY(field_axpby(r, 1.0, -1.0, src, mmp));
  }
  GB_TRY(field_copy(p, r));
  GB_TRY(field_norm2_dev(r, d_cp));
  GB_TRY(launch_cg_init(op, d_ssq, d_cp, P->tolerance, 0.0));
  const int chunk = P->check_every > 0 ? P->check_every : 8;
  int flags[4] = {0, 0, 0, 0};
  GB_TRY(fetch_scalars(op, flags));
  int k = 0;
  ChunkRunner runner{op, kind, p, mmp, r, psi, chunk, P->use_graphs != 0};
  while (!flags[0] && k < P->max_iterations) {
    const int full_chunks = (P->max_iterations - k) / chunk;
    if (P->use_graphs == 2 && runner.loop_ready() && full_chunks > 0) {
      GB_TRY(runner.loop(full_chunks));
      GB_TRY(fetch_scalars(op, flags));
      k += flags[2] * chunk;
    } else {
      const int m = std::min(chunk, P->max_iterations - k);
      GB_TRY(runner.iterate(m));
      k += m;
      GB_TRY(fetch_scalars(op, flags));
    }
    GB_TRY(check_device_error(op));
  }
  std::vector<double> res(n);
  if (k == 0) {
    // no iteration ran (the guess already meets the tolerance, as for the final cleanup of
    // a reliable-update solve): r = src - A psi is the true residual, the same numbers a
    // second application of A to the unchanged psi would give
    std::vector<double> nr(n), ns(n);
    GB_TRY(field_norm2(r, nr.data()));
    GB_TRY(field_norm2(src, ns.data()));
    for (int i = 0; i < n; i++) res[i] = ns[i] > 0 ? std::sqrt(nr[i] / ns[i]) : 0.0;
  } else {
    GB_TRY(true_residual(op, kind, src, psi, mmp, t, res.data()));
  }
  R->iterations = 0;
  R->true_residual = 0;
  R->converged = flags[0];
  for (int i = 0; i < n; i++) {
    op->last_iters[i] = op->h_cg[i].iter;
    op->last_resid[i] = res[i];
    if (i >= op->nrhs_user) continue;  // padding right-hand side
    R->iterations = std::max(R->iterations, op->h_cg[i].iter);
    R->true_residual = std::max(R->true_residual, res[i]);
  }
  R->reliable_updates = 0;
  R->cleanup_iterations = 0;
  R->seconds = tm.seconds();
  R->flops = hermop_flops(op, kind) * R->iterations;
  if (!flags[0]) {
    set_error("CG did not converge in %d iterations", P->max_iterations);
    return GB_ERR_NOT_CONVERGED;
  }
  return GB_OK;
}

// ConjugateGradientReliableUpdate (ConjugateGradientReliableUpdate.h:77-269):
// FP64 op_d, lower-precision op_f on the same gauge field.  src, psi are op_d fields.
int cg_reliable(Op* od, Op* of, int kind, Field* src, Field* psi, const gb_cg_params* P, gb_cg_result* R) {
  Timer tm;
  const int n = od->nrhs;
  if (of->nrhs != n || of->n5() != od->n5()) { set_error("reliable CG: operators differ in shape"); return GB_ERR_BAD_ARG; }
  cudaStream_t saved = of->stream;
  of->stream = od->stream;
  struct Restore { Op* o; cudaStream_t s; ~Restore() { o->stream = s; } } restore{of, saved};
  const int lp = of->prec;
  Field *mmp_d, *r_d, *t_d;
  GB_TRY(field_for(od, kind, GB_ODD, GB_F64, WS_CG_MMP, WS_FCG_MMP, &mmp_d));
  GB_TRY(field_for(od, kind, GB_ODD, GB_F64, WS_CG_R, WS_FCG_R, &r_d));
  GB_TRY(field_for(od, kind, GB_ODD, GB_F64, WS_CG_T, WS_FCG_T, &t_d));
  Field *p_f, *mmp_f, *r_f, *x_f;
  GB_TRY(field_for(of, kind, GB_ODD, lp, WS_RU_PF, WS_FRU_PF, &p_f));
  GB_TRY(field_for(of, kind, GB_ODD, lp, WS_RU_MMPF, WS_FRU_MMPF, &mmp_f));
  GB_TRY(field_for(of, kind, GB_ODD, lp, WS_RU_RF, WS_FRU_RF, &r_f));
  // the inner solution accumulates in FP32 even when r, p, mmp are FP16-stored
  GB_TRY(field_for(of, kind, GB_ODD, lp == GB_F16 ? GB_F32 : lp, WS_RU_XF, WS_FRU_XF, &x_f));
  if (!src->full()) {
    mmp_d->subset = r_d->subset = t_d->subset = src->subset;
    p_f->subset = mmp_f->subset = r_f->subset = x_f->subset = src->subset;
  }
  double* d_ssq = of->d_result + 2 * n;
  double* d_cp = of->d_result + 3 * n;
  double* d_cpt = od->d_result + 4 * n;
  // r = src - A psi as Grid does, cp = |r|^2; for a zero initial guess A psi = 0 and
  // r = src exactly, so the FP64 operator is not applied
  std::vector<double> guess(n);
  GB_TRY(field_norm2(psi, guess.data()));
  bool zero_guess = true;
  for (double g : guess) {
    if (std::isnan(g)) { set_error("reliable-update CG: NaN in the initial guess"); return GB_ERR_BAD_ARG; }
    if (g != 0.0) zero_guess = false;
  }
  if (zero_guess) {
    GB_TRY(field_copy(r_d, src));
  } else {
    GB_TRY(op_hermop(od, kind, psi, mmp_d));
    GB_TRY(field_axpby(r_d, 1.0, -1.0, src, mmp_d));
  }
  GB_TRY(field_norm2_dev(src, od->d_result + 5 * n));
  GB_TRY(field_norm2_dev(r_d, d_cpt));
  GB_CHECK_CUDA(cudaMemcpyAsync(d_ssq, od->d_result + 5 * n, n * sizeof(double), cudaMemcpyDeviceToDevice, od->stream));
  GB_CHECK_CUDA(cudaMemcpyAsync(d_cp, d_cpt, n * sizeof(double), cudaMemcpyDeviceToDevice, od->stream));
  GB_TRY(launch_copy(of, half_view(r_f, 0), half_view(r_d, 0), r_d->n5));
  if (r_d->full()) GB_TRY(launch_copy(of, half_view(r_f, 1), half_view(r_d, 1), r_d->n5));
  GB_TRY(field_copy(p_f, r_f));
  GB_TRY(field_zero(x_f));
  GB_TRY(launch_cg_init(of, d_ssq, d_cp, P->tolerance, P->delta > 0 ? P->delta : 0.0));
  const int chunk = P->check_every > 0 ? P->check_every : 8;
  int flags[4] = {0, 0, 0, 0};
  GB_TRY(fetch_scalars(of, flags));
  int k = 0, l = 0, since = 0;
  auto promote = [&]() -> int {  // psi += (double) x_f
    GB_TRY(field_copy(mmp_d, x_f));
    return field_axpby(psi, 1.0, 1.0, psi, mmp_d);
  };
  ChunkRunner runner{of, kind, p_f, mmp_f, r_f, x_f, chunk, P->use_graphs != 0};
  while (!flags[0] && k < P->max_iterations) {
    int full_chunks = (P->max_iterations - k) / chunk;
    if (P->relup_every > 0) full_chunks = std::min(full_chunks, (P->relup_every - since + chunk - 1) / chunk);
    if (P->use_graphs == 2 && runner.loop_ready() && full_chunks > 0) {
      GB_TRY(runner.loop(full_chunks));
      GB_TRY(fetch_scalars(of, flags));
      k += flags[2] * chunk;
      since += flags[2] * chunk;
    } else {
      const int m = std::min(chunk, P->max_iterations - k);
      GB_TRY(runner.iterate(m));
      k += m;
      since += m;
      GB_TRY(fetch_scalars(of, flags));
    }
    GB_TRY(check_device_error(of));
    if (flags[0]) break;
    if (flags[1] > 0 || (P->relup_every > 0 && since >= P->relup_every)) {
      // reliable update: psi += x_f ; r = src - A psi in FP64 ; x_f = 0 ; r_f = r
      GB_TRY(promote());
      GB_TRY(op_hermop(od, kind, psi, mmp_d));
      GB_TRY(field_axpby(r_d, 1.0, -1.0, src, mmp_d));
      GB_TRY(field_norm2_dev(r_d, d_cpt));
      GB_TRY(field_zero(x_f));
      GB_TRY(launch_copy(of, half_view(r_f, 0), half_view(r_d, 0), r_d->n5));
      if (r_d->full()) GB_TRY(launch_copy(of, half_view(r_f, 1), half_view(r_d, 1), r_d->n5));
      GB_TRY(launch_cg_relup_reset(of, d_cpt));
      l++;
      since = 0;
    }
  }
  GB_TRY(promote());
  R->iterations = 0;
  for (int i = 0; i < n; i++) R->iterations = std::max(R->iterations, of->h_cg[i].iter);
  R->reliable_updates = l;
  R->cleanup_iterations = 0;
  int rc = GB_OK;
  if (!flags[0]) {
    set_error("reliable-update CG did not converge in %d iterations", P->max_iterations);
    rc = GB_ERR_NOT_CONVERGED;
  }
  std::vector<int> inner_iters(n);
  for (int i = 0; i < n; i++) inner_iters[i] = of->h_cg[i].iter;
  if (rc == GB_OK && P->final_cleanup) {
    gb_cg_result R2;
    gb_cg_params P2 = *P;
    rc = cg_solve(od, kind, src, psi, &P2, &R2);
    R->cleanup_iterations = R2.iterations;
    R->true_residual = R2.true_residual;
    R->converged = R2.converged;
  } else {
    std::vector<double> res(n);
    GB_TRY(true_residual(od, kind, src, psi, mmp_d, t_d, res.data()));
    R->true_residual = 0;
    for (int i = 0; i < n; i++) {
      od->last_resid[i] = res[i];
      R->true_residual = std::max(R->true_residual, res[i]);
    }
    R->converged = flags[0];
  }
  for (int i = 0; i < n; i++) od->last_iters[i] = inner_iters[i];
  R->seconds = tm.seconds();
  R->flops = hermop_flops(od, kind) * (R->iterations + R->cleanup_iterations);
  return rc;
}

// SchurRedBlackDiagMooeeSolve (SchurRedBlack.h:236-291,373-436)
int schur_solve(Op* op, Op* olo, Field* src, Field* sol, const gb_cg_params* P, gb_cg_result* R, double* unprec) {
  const int n = op->nrhs;
  const int pr = src->prec;
  Field *src_e, *src_o, *tmp, *sol_o, *res;
  GB_TRY(ws_get(op, GB_EVEN, pr, WS_SCHUR_A, &src_e));
  GB_TRY(ws_get(op, GB_ODD, pr, WS_SCHUR_B, &src_o));
  GB_TRY(ws_get(op, GB_EVEN, pr, WS_SCHUR_C, &tmp));
  GB_TRY(ws_get(op, GB_ODD, pr, WS_SCHUR_D, &sol_o));
  Field* Mtmp;
  GB_TRY(ws_get(op, GB_ODD, pr, WS_CG_T, &Mtmp));
  // RedBlackSource: src_o' = MpcDag (src_o - Meooe MooeeInv src_e)
  GB_TRY(launch_copy(op, half_view(src_e, 0), half_view(src, GB_EVEN), src->n5));
  GB_TRY(launch_copy(op, half_view(src_o, 0), half_view(src, GB_ODD), src->n5));
  GB_TRY(op_mooee_inv(op, src_e, tmp, 0));
  GB_TRY(op_meooe(op, tmp, Mtmp, 0));
  GB_TRY(field_axpby(Mtmp, 1.0, -1.0, src_o, Mtmp));  // Mtmp = src_o - Mtmp
  GB_TRY(op_mpc(op, Mtmp, src_o, 1));
  GB_TRY(field_zero(sol_o));
  sol_o->subset = GB_ODD;
  int rc = olo ? cg_reliable(op, olo, 1, src_o, sol_o, P, R) : cg_solve(op, 1, src_o, sol_o, P, R);
  if (rc != GB_OK && rc != GB_ERR_NOT_CONVERGED) return rc;
  // RedBlackSolution: sol_e = MooeeInv (src_e - Meooe sol_o)
  GB_TRY(op_meooe(op, sol_o, tmp, 0));
  GB_TRY(field_axpby(tmp, 1.0, -1.0, src_e, tmp));
  GB_TRY(launch_copy(op, half_view(src_e, 0), half_view(tmp, 0), src->n5));
  src_e->subset = GB_EVEN;
  Field* sol_e = tmp;
  GB_TRY(op_mooee_inv(op, src_e, sol_e, 0));
  GB_TRY(launch_copy(op, half_view(sol, GB_EVEN), half_view(sol_e, 0), src->n5));
  GB_TRY(launch_copy(op, half_view(sol, GB_ODD), half_view(sol_o, 0), src->n5));
  if (unprec) {
    GB_TRY(ws_get(op, GB_FULL, pr, WS_SCHUR_RES, &res));
    GB_TRY(op_m(op, sol, res, 0));
    GB_TRY(field_axpby(res, 1.0, -1.0, res, src));
    std::vector<double> nr(n), ns(n);
    GB_TRY(field_norm2(res, nr.data()));
    GB_TRY(field_norm2(src, ns.data()));
    for (int i = 0; i < op->nrhs_user; i++) unprec[i] = ns[i] > 0 ? std::sqrt(nr[i] / ns[i]) : 0.0;
  }
  return rc;
}

}  // namespace gb

using namespace gb;

extern "C" {

void gb_cg_params_default(gb_cg_params* p) {
  if (!p) return;
  p->tolerance = 1e-10;
  p->max_iterations = 10000;
  p->err_on_no_conv = 1;
  p->delta = 1e-6;
  p->relup_every = 100;
  p->final_cleanup = 1;
  p->check_every = 10;
  p->use_graphs = 0;
}

static int solve_checks(gb_op_t op, gb_field_t a, gb_field_t b, const gb_cg_params* p, gb_cg_result* r) {
  if (!op || !a || !b || !p || !r) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (!op->gauge_loaded) { set_error("operator has no gauge field"); return GB_ERR_BAD_ARG; }
  if (!ops_conformable(a->op, op) || !ops_conformable(b->op, op)) {
    set_error("field is not conformable to the operator");
    return GB_ERR_BAD_ARG;
  }
  if (a->prec != op->prec || b->prec != op->prec) { set_error("field precision differs from the operator's"); return GB_ERR_BAD_ARG; }
  if (p->tolerance <= 0 || p->max_iterations < 1) { set_error("bad tolerance or max_iterations"); return GB_ERR_BAD_ARG; }
  std::memset(r, 0, sizeof(*r));
  return GB_OK;
}

// MixedPrecisionConjugateGradient (ConjugateGradientMixedPrec.h:68-166) and, with
// nrhs > 1 operators, its batched form (ConjugateGradientMixedPrecBatched.h:37-209) with
// all right-hand sides in one inner multi-RHS CG.  Outer loop: r = src - A psi in FP64;
// stop when |r|^2 < outer_mult * tol^2 |src|^2 for every right-hand side; raise the inner
// tolerance until |r|^2 t^2 >= tol^2 |src|^2; solve A e = r in FP32 from zero to t (the
// smallest over right-hand sides); psi += e.  Then an FP64 CG from psi to tol.
static int cg_mixed(Op* od, Op* of, int kind, Field* src, Field* psi, const gb_cg_params* P, const gb_mixed_params* M,
             gb_cg_result* R) {
  Timer tm;
  const int n = od->nrhs_user;
  if (of->nrhs != od->nrhs || of->n5() != od->n5()) { set_error("mixed CG: operators differ in shape"); return GB_ERR_BAD_ARG; }
  cudaStream_t saved = of->stream;
  of->stream = od->stream;
  struct Restore { Op* o; cudaStream_t s; ~Restore() { o->stream = s; } } restore{of, saved};
  Field *tmp_d, *res_d, *src_f, *sol_f;
  GB_TRY(field_for(od, kind, GB_ODD, GB_F64, WS_CG_T, WS_FCG_T, &tmp_d));
  GB_TRY(field_for(od, kind, GB_ODD, GB_F64, WS_CG_R, WS_FCG_R, &res_d));
  GB_TRY(field_for(of, kind, GB_ODD, of->prec, WS_RU_RF, WS_FRU_RF, &src_f));
  GB_TRY(field_for(of, kind, GB_ODD, of->prec, WS_RU_XF, WS_FRU_XF, &sol_f));
  if (!src->full()) tmp_d->subset = res_d->subset = src_f->subset = sol_f->subset = src->subset;
  const double tol = P->tolerance;
  const double mult = M->outer_loop_norm_mult > 0 ? M->outer_loop_norm_mult : 100.0;
  std::vector<double> stop(od->nrhs), nr(od->nrhs), t(n, M->inner_tolerance > 0 ? M->inner_tolerance : tol);
  GB_TRY(field_norm2(src, stop.data()));
  for (double& v : stop) v *= tol * tol;
  int total_inner = 0, outer = 0;
  for (; outer < M->max_outer_iterations; outer++) {
    GB_TRY(op_hermop(od, kind, psi, tmp_d));
    GB_TRY(field_axpby(res_d, 1.0, -1.0, src, tmp_d));
    GB_TRY(field_norm2(res_d, nr.data()));
    bool done = true;
    for (int i = 0; i < n; i++) done = done && nr[i] < mult * stop[i];
    if (done) break;
    double inner = 1.0;
    for (int i = 0; i < n; i++) {
      while (nr[i] * t[i] * t[i] < stop[i]) t[i] *= 2;
      inner = std::min(inner, t[i]);
    }
    GB_TRY(field_copy(src_f, res_d));
    GB_TRY(field_zero(sol_f));
    gb_cg_params Pi = *P;
    Pi.tolerance = inner;
    Pi.max_iterations = M->max_inner_iterations;
    Pi.err_on_no_conv = 0;
    gb_cg_result Ri;
    const int rc = cg_solve(of, kind, src_f, sol_f, &Pi, &Ri);
    if (rc != GB_OK && rc != GB_ERR_NOT_CONVERGED) return rc;
    total_inner += Ri.iterations;
    GB_TRY(field_copy(tmp_d, sol_f));
    GB_TRY(field_axpby(psi, 1.0, 1.0, psi, tmp_d));
  }
  gb_cg_params Pd = *P;
  Pd.max_iterations = M->max_patchup_iterations > 0 ? M->max_patchup_iterations : M->max_inner_iterations;
  gb_cg_result Rd;
  const int rc = cg_solve(od, kind, src, psi, &Pd, &Rd);
  R->iterations = total_inner;
  R->reliable_updates = outer;
  R->cleanup_iterations = Rd.iterations;
  R->true_residual = Rd.true_residual;
  R->converged = Rd.converged;
  R->seconds = tm.seconds();
  R->flops = hermop_flops(od, kind) * (total_inner + Rd.iterations + outer);
  return rc;
}

static int finish(int rc, const gb_cg_params* p) {
  if (rc == GB_ERR_NOT_CONVERGED && !p->err_on_no_conv) return GB_OK;
  return rc;
}

int gb_cg_mdagm(gb_op_t op, gb_field_t src, gb_field_t psi, const gb_cg_params* p, gb_cg_result* res) {
  GB_TRY(solve_checks(op, src, psi, p, res));
  if (!src->full() || !psi->full()) { set_error("MdagM CG: full fields expected"); return GB_ERR_BAD_PARITY; }
  SolveStream ss(op, nullptr, src, psi, p->use_graphs != 0);
  return finish(cg_solve(op, 0, src, psi, p, res), p);
}

int gb_cg_schur(gb_op_t op, gb_field_t src, gb_field_t psi, const gb_cg_params* p, gb_cg_result* res) {
  GB_TRY(solve_checks(op, src, psi, p, res));
  if (src->subset != GB_ODD) { set_error("Schur CG: odd source expected"); return GB_ERR_BAD_PARITY; }
  psi->subset = GB_ODD;
  SolveStream ss(op, nullptr, src, psi, p->use_graphs != 0);
  return finish(cg_solve(op, 1, src, psi, p, res), p);
}

int gb_cg_last_per_rhs(gb_op_t op, int* iterations, double* true_residual) {
  if (!op) return GB_ERR_BAD_ARG;
  for (int i = 0; i < op->nrhs_user; i++) {
    if (iterations) iterations[i] = op->last_iters[i];
    if (true_residual) true_residual[i] = op->last_resid[i];
  }
  return GB_OK;
}

int gb_cg_reliable(gb_op_t op_d, gb_op_t op_lo, int kind, gb_field_t src, gb_field_t psi, const gb_cg_params* p,
                   gb_cg_result* res) {
  GB_TRY(solve_checks(op_d, src, psi, p, res));
  if (!op_lo || op_lo->prec == GB_F64 || op_d->prec != GB_F64) { set_error("reliable CG: need FP64 op_d and FP32/FP16 op_lo"); return GB_ERR_BAD_ARG; }
  if (!op_lo->gauge_loaded) { set_error("op_lo has no gauge field"); return GB_ERR_BAD_ARG; }
  if (kind == 0 && (!src->full() || !psi->full())) { set_error("reliable CG: full fields expected"); return GB_ERR_BAD_PARITY; }
  if (kind == 1 && src->subset != GB_ODD) { set_error("reliable CG: odd source expected"); return GB_ERR_BAD_PARITY; }
  if (kind == 1) psi->subset = GB_ODD;
  SolveStream ss(op_d, op_lo, src, psi, p->use_graphs != 0);
  return finish(cg_reliable(op_d, op_lo, kind, src, psi, p, res), p);
}

void gb_mixed_params_default(gb_mixed_params* m) {
  if (!m) return;
  m->inner_tolerance = 0.0;
  m->max_inner_iterations = 10000;
  m->max_outer_iterations = 100;
  m->max_patchup_iterations = 0;
  m->outer_loop_norm_mult = 100.0;
}

int gb_cg_mixed(gb_op_t op_d, gb_op_t op_f, int kind, gb_field_t src, gb_field_t psi, const gb_cg_params* p,
                const gb_mixed_params* m, gb_cg_result* res) {
  GB_TRY(solve_checks(op_d, src, psi, p, res));
  if (!m) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (!op_f || op_d->prec != GB_F64 || op_f->prec != GB_F32) { set_error("mixed CG: need FP64 op_d and FP32 op_f"); return GB_ERR_BAD_ARG; }
  if (!op_f->gauge_loaded) { set_error("op_f has no gauge field"); return GB_ERR_BAD_ARG; }
  if (kind != 0 && kind != 1) { set_error("kind must be 0 (MdagM) or 1 (MpcDagMpc)"); return GB_ERR_BAD_ARG; }
  if (kind == 0 && (!src->full() || !psi->full())) { set_error("mixed CG: full fields expected"); return GB_ERR_BAD_PARITY; }
  if (kind == 1 && src->subset != GB_ODD) { set_error("mixed CG: odd source expected"); return GB_ERR_BAD_PARITY; }
  if (m->max_inner_iterations < 1 || m->max_outer_iterations < 0) { set_error("mixed CG: bad iteration limits"); return GB_ERR_BAD_ARG; }
  if (kind == 1) psi->subset = GB_ODD;
  SolveStream ss(op_d, op_f, src, psi, p->use_graphs != 0);
  return finish(cg_mixed(op_d, op_f, kind, src, psi, p, m, res), p);
}

int gb_schur_solve(gb_op_t op, gb_op_t op_lo, gb_field_t src, gb_field_t sol, const gb_cg_params* p, gb_cg_result* res,
                   double* unprec_resid) {
  GB_TRY(solve_checks(op, src, sol, p, res));
  if (!src->full() || !sol->full()) { set_error("Schur solve: full fields expected"); return GB_ERR_BAD_PARITY; }
  if (op_lo && (op->prec != GB_F64 || op_lo->prec == GB_F64)) { set_error("Schur solve: mixed needs FP64 op and FP32/FP16 op_lo"); return GB_ERR_BAD_ARG; }
  SolveStream ss(op, op_lo, src, sol, p->use_graphs != 0);
  return finish(schur_solve(op, op_lo, src, sol, p, res, unprec_resid), p);
}

}  // extern "C"
