// gb_api.cpp -- C ABI: library, operators, fields, field algebra and the operator call
// sequences of Grid's WilsonFermion / CayleyFermion5D (host side).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>
#include <new>

#include "gb_ops.h"

namespace gb {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

size_t Op::link_bytes_per_parity() const { return size_t(half4) * 8 * (recon12 ? 12 : 18) * (prec == GB_F64 ? 8 : 4); }

size_t Field::half_bytes() const { return n5 * spinor_bytes(prec); }
void* Field::half_ptr(int parity) const {
  if (!full()) return data;
  return static_cast<char*>(data) + (parity ? half_bytes() : 0);
}
float* Field::half_norms(int parity) const {
  if (!norms) return nullptr;
  if (!full()) return norms;
  return norms + (parity ? n5 : 0);
}

static int check_op(const Op* op) {
  if (!op) { set_error("null operator"); return GB_ERR_BAD_ARG; }
  if (!op->gauge_loaded) { set_error("operator has no gauge field: call gb_op_import_gauge"); return GB_ERR_BAD_ARG; }
  return GB_OK;
}
// for calls that use only the geometry (and coefficients) of the operator, not its links
static int check_op_geometry(const Op* op) {
  if (!op) { set_error("null operator"); return GB_ERR_BAD_ARG; }
  return GB_OK;
}
static int check_conf(const Field* a, const Field* b) {
  if (!a || !b) { set_error("null field"); return GB_ERR_BAD_ARG; }
  if (!ops_conformable(a->op, b->op) || a->n5 != b->n5) { set_error("fields are not conformable"); return GB_ERR_BAD_ARG; }
  return GB_OK;
}
static int check_subset(const Field* f, int subset, const char* what) {
  if (f->subset != subset) {
    set_error("%s: field is on the wrong checkerboard (subset %d, expected %d)", what, f->subset, subset);
    return GB_ERR_BAD_PARITY;
  }
  return GB_OK;
}

// ---------------------------------------------------------------------------------------
// Allocation.  Device memory of operators and fields comes from the stream-ordered
// allocator on the operator's stream (cudaMallocAsync / cudaFreeAsync), and the device's
// default memory pool keeps freed blocks for reuse: creating or destroying an operator
// then neither synchronises the device nor calls into the driver's allocator once the
// pool holds enough, so one stream's set-up does not stall another stream's kernels (the
// propagator service creates operators per request while other requests run).  Small
// page-locked host buffers come from a process-wide pool for the same reason:
// cudaFreeHost synchronises the device.
// ---------------------------------------------------------------------------------------
static void keep_pool_memory(int device) {
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> lk(mu);
  for (int d : done)
    if (d == device) return;
  done.push_back(device);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = ~uint64_t(0);  // never trim at synchronisation points
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
}
static cudaError_t dev_alloc(void** p, size_t n, cudaStream_t s) { return cudaMallocAsync(p, n, s); }
static void dev_free(void* p, cudaStream_t s) {
  if (p) cudaFreeAsync(p, s);
}

namespace {
struct PinnedPool {
  std::mutex mu;
  std::multimap<size_t, void*> free_blocks;  // size class -> block
  std::map<void*, size_t> sizes;
};
PinnedPool& pinned_pool() {
  static PinnedPool* pp = new PinnedPool;  // process lifetime: blocks stay page-locked until exit
  return *pp;
}
}  // namespace
static void* pinned_get(size_t bytes) {
  const size_t cls = (bytes + 255) & ~size_t(255);
  PinnedPool& pp = pinned_pool();
  {
    std::lock_guard<std::mutex> lk(pp.mu);
    auto it = pp.free_blocks.find(cls);
    if (it != pp.free_blocks.end()) {
      void* p = it->second;
      pp.free_blocks.erase(it);
      return p;
    }
  }
  void* p = nullptr;
  if (cudaMallocHost(&p, cls) != cudaSuccess) return nullptr;
  std::lock_guard<std::mutex> lk(pp.mu);
  pp.sizes[p] = cls;
  return p;
}
static void pinned_put(void* p) {
  if (!p) return;
  PinnedPool& pp = pinned_pool();
  std::lock_guard<std::mutex> lk(pp.mu);
  pp.free_blocks.emplace(pp.sizes[p], p);
}

int field_alloc(Op* op, int subset, int prec, Field** out) {
  Field* f = new (std::nothrow) gb_field_s;
  if (!f) { set_error("host allocation failed"); return GB_ERR_OOM; }
  f->op = op;
  f->subset = subset;
  f->prec = prec;
  f->n5 = op->n5();
  const size_t halves = subset == GB_FULL ? 2 : 1;
  cudaError_t e = dev_alloc(&f->data, halves * f->half_bytes(), op->stream);
  if (e != cudaSuccess) {
    delete static_cast<gb_field_s*>(f);
    set_error("device allocation of %zu bytes failed: %s", halves * f->n5 * spinor_bytes(prec), cudaGetErrorString(e));
    return GB_ERR_OOM;
  }
  // zero on the operator's stream: a non-blocking stream does not wait for work on the
  // legacy default stream, so a plain cudaMemset could land after this stream's kernels
  // have written the (lazily allocated) field
  cudaMemsetAsync(f->data, 0, halves * f->half_bytes(), op->stream);
  if (prec == GB_F16) {
    e = dev_alloc(reinterpret_cast<void**>(&f->norms), halves * f->n5 * sizeof(float), op->stream);
    if (e != cudaSuccess) {
      dev_free(f->data, op->stream);
      delete static_cast<gb_field_s*>(f);
      set_error("device allocation of norms failed: %s", cudaGetErrorString(e));
      return GB_ERR_OOM;
    }
    cudaMemsetAsync(f->norms, 0, halves * f->n5 * sizeof(float), op->stream);
  }
  *out = f;
  return GB_OK;
}

void field_free(Field* f) {
  if (!f) return;
  if (f->owned) {
    dev_free(f->data, f->op->stream);
    dev_free(f->norms, f->op->stream);
  }
  delete static_cast<gb_field_s*>(f);
}

// workspace: the slot-th cached field of (full or half, precision); a half workspace
// field is relabelled to the requested checkerboard
int ws_get(Op* op, int subset, int prec, int slot, Field** out) {
  const bool want_full = subset == GB_FULL;
  for (Field* f : op->ws) {
    if (f->full() == want_full && f->prec == prec && f->ws_slot == slot) {
      if (!want_full) f->subset = subset;
      *out = f;
      return GB_OK;
    }
  }
  Field* f = nullptr;
  GB_TRY(field_alloc(op, subset, prec, &f));
  f->ws_slot = slot;
  op->ws.push_back(f);
  *out = f;
  return GB_OK;
}

// ---------------------------------------------------------------------------------------
// reductions on whole fields (both halves of a full field), results to host
// ---------------------------------------------------------------------------------------
int field_norm2_dev(Field* f, double* d_out) {
  Op* op = f->op;
  const int g = red_parts(op, f->prec);
  const int halves = f->full() ? 2 : 1;
  for (int h = 0; h < halves; h++)
    GB_TRY(launch_norm2_partial(op, half_view(f, h), f->n5, op->d_partial + size_t(h) * g * op->nrhs));
  return launch_reduce_final(op, op->d_partial, g * halves, 1, d_out);
}

int field_inner_dev(Field* a, Field* b, double* d_out) {
  Op* op = a->op;
  const int g = red_parts(op, a->prec);
  const int halves = a->full() ? 2 : 1;
  for (int h = 0; h < halves; h++)
    GB_TRY(launch_inner_partial(op, half_view(a, h), half_view(b, h), a->n5, op->d_partial + size_t(h) * g * op->nrhs * 2));
  return launch_reduce_final(op, op->d_partial, g * halves, 2, d_out);
}

static int fetch(Op* op, const double* d_src, double* host, size_t n) {
  GB_CHECK_CUDA(cudaMemcpyAsync(op->h_result, d_src, n * sizeof(double), cudaMemcpyDeviceToHost, op->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  std::memcpy(host, op->h_result, n * sizeof(double));
  return GB_OK;
}

int field_norm2(Field* f, double* out) {
  GB_TRY(field_norm2_dev(f, f->op->d_result));
  return fetch(f->op, f->op->d_result, out, f->op->nrhs);
}
int field_inner(Field* a, Field* b, double* out) {
  GB_TRY(field_inner_dev(a, b, a->op->d_result));
  return fetch(a->op, a->op->d_result, out, size_t(a->op->nrhs) * 2);
}

int field_axpby(Field* z, double a, double b, Field* x, Field* y) {
  const int halves = z->full() ? 2 : 1;
  for (int h = 0; h < halves; h++)
    GB_TRY(launch_axpby(z->op, half_view(z, h), a, half_view(x, h), b, half_view(y, h), z->n5));
  return GB_OK;
}
int field_scale(Field* z, double a, Field* x) {
  const int halves = z->full() ? 2 : 1;
  for (int h = 0; h < halves; h++) GB_TRY(launch_scale(z->op, half_view(z, h), a, half_view(x, h), z->n5));
  return GB_OK;
}
int field_copy(Field* dst, Field* src) {
  if (dst == src) return GB_OK;
  const int halves = dst->full() ? 2 : 1;
  for (int h = 0; h < halves; h++) GB_TRY(launch_copy(dst->op, half_view(dst, h), half_view(src, h), dst->n5));
  return GB_OK;
}
int field_zero(Field* z) {
  const int halves = z->full() ? 2 : 1;
  for (int h = 0; h < halves; h++) GB_TRY(launch_zero(z->op, half_view(z, h), z->n5));
  return GB_OK;
}

// ---------------------------------------------------------------------------------------
// Operator call sequences
// ---------------------------------------------------------------------------------------
// 5D coefficient sets (CayleyFermion5DImplementation.h:155-271)
void coeffs_meooe5d(const Op* op, int dag, std::vector<double>& l, std::vector<double>& d, std::vector<double>& u) {
  const int Ls = op->Ls;
  d = op->bs;
  u.assign(Ls, 0);
  l.assign(Ls, 0);
  if (!dag) {
    u = op->cs;
    l = op->cs;
    u[Ls - 1] = -op->mass * u[Ls - 1];
    l[0] = -op->mass * l[0];
  } else {
    for (int s = 0; s < Ls; s++) {
      if (s == 0) { u[s] = op->cs[s + 1]; l[s] = -op->mass * op->cs[Ls - 1]; }
      else if (s == Ls - 1) { u[s] = -op->mass * op->cs[0]; l[s] = op->cs[s - 1]; }
      else { u[s] = op->cs[s + 1]; l[s] = op->cs[s - 1]; }
    }
  }
}
void coeffs_mooee(const Op* op, int dag, std::vector<double>& l, std::vector<double>& d, std::vector<double>& u) {
  const int Ls = op->Ls;
  d = op->bee;
  u.assign(Ls, 0);
  l.assign(Ls, 0);
  if (!dag) {
    for (int i = 0; i < Ls; i++) { u[i] = -op->cee[i]; l[i] = -op->cee[i]; }
    u[Ls - 1] = -op->mass * u[Ls - 1];
    l[0] = -op->mass * l[0];
  } else {
    for (int s = 0; s < Ls; s++) {
      if (s == 0) { u[s] = -op->cee[s + 1]; l[s] = op->mass * op->cee[Ls - 1]; }
      else if (s == Ls - 1) { u[s] = op->mass * op->cee[0]; l[s] = -op->cee[s - 1]; }
      else { u[s] = -op->cee[s + 1]; l[s] = -op->cee[s - 1]; }
    }
  }
}
// M5D / M5Ddag with unit diagonal used by M and Mdag (CayleyFermion5DImplementation.h:130-231)
void coeffs_m5d_unit(const Op* op, std::vector<double>& l, std::vector<double>& d, std::vector<double>& u) {
  const int Ls = op->Ls;
  d.assign(Ls, 1.0);
  u.assign(Ls, -1.0);
  l.assign(Ls, -1.0);
  u[Ls - 1] = op->mass;
  l[0] = op->mass;
}

// (norm_parts: |chi|^2 partial sums into op->d_partial where the kernel can, one
// checkerboard half only; see launch_m5d_pair)
static int m5d_field(Op* op, Field* psi, Field* phi, Field* chi, const std::vector<double>& l,
                     const std::vector<double>& d, const std::vector<double>& u, int dag, Field* z, double zc,
                     int* norm_parts = nullptr) {
  const int halves = chi->full() ? 2 : 1;
  if (norm_parts) *norm_parts = 0;
  for (int h = 0; h < halves; h++) {
    HalfView zv = z ? half_view(z, h) : HalfView{nullptr, nullptr, chi->prec};
    GB_TRY(launch_m5d_z(op, half_view(psi, h), half_view(phi, h), half_view(chi, h), l.data(), d.data(), u.data(), dag,
                        chi->n5, z ? &zv : nullptr, zc, halves == 1 ? norm_parts : nullptr));
  }
  return GB_OK;
}

// a fused s-column program on every checkerboard half of the fields (FP32 Moebius)
// (r_upd: the CG's residual update in place of storing out where the kernel can, one
// checkerboard half only; see launch_col)
static int col_field(Op* op, int opa, int opb, int dag, Field* x, Field* y, Field* out, double zc,
                     const ColCoefsHost& h, Field* r_upd = nullptr, int* r_parts = nullptr) {
  const int halves = out->full() ? 2 : 1;
  if (r_parts) *r_parts = 0;
  for (int k = 0; k < halves; k++) {
    const HalfView yv = y ? half_view(y, k) : HalfView{nullptr, nullptr, x->prec};
    HalfView rv = r_upd ? half_view(r_upd, k) : HalfView{};
    const bool fuse = r_upd && halves == 1;
    GB_TRY(launch_col(op, opa, opb, dag, half_view(x, k), yv, half_view(out, k), zc, h, fuse ? &rv : nullptr,
                      fuse ? r_parts : nullptr));
  }
  return GB_OK;
}

// ---- ZMobius: the same coefficient sets with complex bs, cs (CayleyFermion5DImplementation.h:
// 155-271); the dagger forms are conjugated as Grid assembles them ----
using cplxd = std::complex<double>;
static void conj_all(std::vector<cplxd>& v) {
  for (auto& x : v) x = std::conj(x);
}
static void zcoeffs_meooe5d(const Op* op, int dag, ZCoefsHost& h) {
  const int Ls = op->Ls;
  const double mf = op->mass;
  h.d = op->zbs;
  h.u.assign(Ls, 0);
  h.l.assign(Ls, 0);
  if (!dag) {
    h.u = op->zcs;
    h.l = op->zcs;
    h.u[Ls - 1] = -mf * h.u[Ls - 1];
    h.l[0] = -mf * h.l[0];
    return;
  }
  for (int s = 0; s < Ls; s++) {
    if (s == 0) { h.u[s] = op->zcs[s + 1]; h.l[s] = -mf * op->zcs[Ls - 1]; }
    else if (s == Ls - 1) { h.u[s] = -mf * op->zcs[0]; h.l[s] = op->zcs[s - 1]; }
    else { h.u[s] = op->zcs[s + 1]; h.l[s] = op->zcs[s - 1]; }
  }
  conj_all(h.d); conj_all(h.u); conj_all(h.l);
}
static void zcoeffs_mooee(const Op* op, int dag, ZCoefsHost& h) {
  const int Ls = op->Ls;
  const double mf = op->mass;
  h.d = op->zbee;
  h.u.assign(Ls, 0);
  h.l.assign(Ls, 0);
  if (!dag) {
    for (int i = 0; i < Ls; i++) { h.u[i] = -op->zcee[i]; h.l[i] = -op->zcee[i]; }
    h.u[Ls - 1] = -mf * h.u[Ls - 1];
    h.l[0] = -mf * h.l[0];
    return;
  }
  for (int s = 0; s < Ls; s++) {
    if (s == 0) { h.u[s] = -op->zcee[s + 1]; h.l[s] = mf * op->zcee[Ls - 1]; }
    else if (s == Ls - 1) { h.u[s] = mf * op->zcee[0]; h.l[s] = -op->zcee[s - 1]; }
    else { h.u[s] = -op->zcee[s + 1]; h.l[s] = -op->zcee[s - 1]; }
  }
  conj_all(h.d); conj_all(h.u); conj_all(h.l);
}
// MooeeInv / MooeeInvDag (CayleyFermion5Dcache.h:117-230): the dagger swaps the L and U
// factors and conjugates them
static void zcoeffs_inv(const Op* op, int dag, ZCoefsHost& h) {
  const int Ls = op->Ls;
  h.dinv.resize(Ls);
  for (int s = 0; s < Ls; s++) h.dinv[s] = 1.0 / op->zdee[s];
  if (!dag) {
    h.lee = op->zlee; h.leem = op->zleem; h.uee = op->zuee; h.ueem = op->zueem;
    return;
  }
  h.lee = op->zuee; h.leem = op->zueem; h.uee = op->zlee; h.ueem = op->zleem;
  conj_all(h.lee); conj_all(h.leem); conj_all(h.uee); conj_all(h.ueem); conj_all(h.dinv);
}
static int zcol_field(Op* op, int prog, int dag, Field* x, Field* y, Field* out, double zc, const ZCoefsHost& h) {
  const int halves = out->full() ? 2 : 1;
  for (int k = 0; k < halves; k++) {
    const HalfView yv = y ? half_view(y, k) : HalfView{nullptr, nullptr, x->prec};
    GB_TRY(launch_zcol(op, prog, dag, half_view(x, k), y ? &yv : nullptr, half_view(out, k), zc, h));
  }
  return GB_OK;
}

int op_meooe5d(Op* op, Field* in, Field* out, int dag) {
  if (op->zmobius) {
    ZCoefsHost h;
    zcoeffs_meooe5d(op, dag, h);
    return zcol_field(op, ZPROG_M5D, dag, in, nullptr, out, 0.0, h);
  }
  std::vector<double> l, d, u;
  coeffs_meooe5d(op, dag, l, d, u);
  return m5d_field(op, in, in, out, l, d, u, dag, nullptr, 0);
}

int op_dhop_cb(Op* op, Field* in, Field* out, int dag) {
  // in: half field of parity p ; out: parity 1-p
  if (in->full() || out->full()) { set_error("DhopEO/OE: half fields expected"); return GB_ERR_BAD_PARITY; }
  const int p = in->subset;
  out->subset = 1 - p;
  return launch_dhop(op, half_view(in, 0), half_view(out, 0), 1 - p, dag);
}

int op_dhop_full(Op* op, Field* in, Field* out, int dag) {
  if (!in->full() || !out->full()) { set_error("Dhop: full fields expected"); return GB_ERR_BAD_PARITY; }
  // both checkerboards in one launch: blockIdx.z selects the output parity
  return launch_dhop_full(op, half_view(in, 1), half_view(out, 0), half_view(in, 0), half_view(out, 1), dag);
}

int op_meooe(Op* op, Field* in, Field* out, int dag) {
  if (in->full()) { set_error("Meooe: half field expected"); return GB_ERR_BAD_PARITY; }
  if (op->kind == 0) return op_dhop_cb(op, in, out, dag);
  Field* t;
  if (!dag) {  // Meooe = DhopEO/OE (Meooe5D in)
    GB_TRY(ws_get(op, in->subset, in->prec, WS_MEOOE_A, &t));
    GB_TRY(op_meooe5d(op, in, t, 0));
    return op_dhop_cb(op, t, out, 0);
  }
  // MeooeDag = MeooeDag5D (DhopEO/OE^dag in)
  GB_TRY(ws_get(op, 1 - in->subset, in->prec, WS_MEOOE_B, &t));
  GB_TRY(op_dhop_cb(op, in, t, 1));
  out->subset = 1 - in->subset;
  return op_meooe5d(op, t, out, 1);
}

// the per-slot chiral diagonal of a twisted-mass operator (WilsonTMFermion5D.h:82-135):
// Mooee = (4 + m) + i mu gamma5, MooeeInv = ((4 + m) - i mu gamma5) / ((4 + m)^2 + mu^2);
// the daggers conjugate
static int tm_diag(Op* op, Field* in, Field* out, int dag, int inverse, Field* z, double zc) {
  const int L5 = op->L5;
  std::vector<double> ur(L5), ui(L5), dr(L5), di(L5);
  for (int s = 0; s < L5; s++) {
    const double m = 4.0 + op->tm_mass[s], mu = op->tm_mu[s];
    double re = m, im = mu;  // P+ component of Mooee
    if (inverse) { const double q = m * m + mu * mu; re = m / q; im = -mu / q; }
    if (dag) im = -im;
    ur[s] = re; ui[s] = im;  // spins 0,1: gamma5 = +1
    dr[s] = re; di[s] = -im; // spins 2,3: gamma5 = -1
  }
  const int halves = in->full() ? 2 : 1;
  for (int h = 0; h < halves; h++) {
    HalfView zv = z ? half_view(z, h) : HalfView{};
    GB_TRY(launch_chiral_scale(op, half_view(in, h), z ? &zv : nullptr, zc, half_view(out, h), ur.data(), ui.data(),
                               dr.data(), di.data()));
  }
  return GB_OK;
}

int op_mooee(Op* op, Field* in, Field* out, int dag, Field* z, double zc, int* norm_parts) {
  if (norm_parts) *norm_parts = 0;
  if (in->full() != out->full()) { set_error("Mooee: in and out must both be full or both half fields"); return GB_ERR_BAD_PARITY; }
  out->subset = in->subset;
  if (op->tm) return tm_diag(op, in, out, dag, 0, z, zc);
  if (op->kind == 0) {
    if (z) return field_axpby(out, op->diag_mass, zc, in, z);
    return field_scale(out, op->diag_mass, in);
  }
  if (op->zmobius) {
    ZCoefsHost h;
    zcoeffs_mooee(op, dag, h);
    return zcol_field(op, ZPROG_M5D, dag, in, z, out, zc, h);
  }
  std::vector<double> l, d, u;
  coeffs_mooee(op, dag, l, d, u);
  return m5d_field(op, in, in, out, l, d, u, dag, z, zc, norm_parts);
}

int op_mooee_inv(Op* op, Field* in, Field* out, int dag) {
  if (in->full() != out->full()) { set_error("MooeeInv: in and out must both be full or both half fields"); return GB_ERR_BAD_PARITY; }
  out->subset = in->subset;
  if (op->tm) return tm_diag(op, in, out, dag, 1, nullptr, 0.0);
  if (op->kind == 0) return field_scale(out, 1.0 / op->diag_mass, in);
  if (op->zmobius) {
    ZCoefsHost h;
    zcoeffs_inv(op, dag, h);
    return zcol_field(op, ZPROG_INV, dag, in, nullptr, out, 0.0, h);
  }
  if (col_available(op, in->prec)) return col_field(op, COL_INV, COLB_NONE, dag, in, nullptr, out, 0.0, ColCoefsHost());
  const int halves = in->full() ? 2 : 1;
  for (int h = 0; h < halves; h++)
    GB_TRY(launch_mooee_inv(op, half_view(in, h), half_view(out, h), dag, size_t(op->half4)));
  return GB_OK;
}

// SchurDiagMooeeOperator::Mpc / MpcDag (LinearOperator.h:330-349).  With norm_parts (Mpc
// of a FP32 / FP16 Moebius operator) the last kernel also reduces |out|^2 per right-hand
// side (see launch_m5d_pair).  With r_upd (MpcDag of a FP32 / FP16 Moebius operator whose
// right-hand-side count divides 16) the last kernel applies r -= a out for the CG instead
// of storing out (see launch_col).
int op_mpc(Op* op, Field* in, Field* out, int dag, int* norm_parts, Field* r_upd, int* r_parts) {
  if (norm_parts) *norm_parts = 0;
  if (r_parts) *r_parts = 0;
  if (in->subset != GB_ODD) { set_error("Mpc: odd checkerboard expected"); return GB_ERR_BAD_PARITY; }
  Field *te1, *te2, *to;
  GB_TRY(ws_get(op, GB_EVEN, in->prec, WS_MPC_E1, &te1));
  GB_TRY(ws_get(op, GB_EVEN, in->prec, WS_MPC_E2, &te2));
  GB_TRY(ws_get(op, GB_ODD, in->prec, WS_MPC_O, &to));
  if (col_available(op, in->prec)) {
    // the same sequence with the 5D steps fused into s-column programs:
    //   Mpc    = Mooee in - DhopOE M5D MooeeInv DhopEO M5D in            (5 launches)
    //   MpcDag = MooeeDag in - M5Ddag DhopOE^dag MooeeInvDag M5Ddag DhopEO^dag in  (4)
    // (a lone M5D stays on the site-pair kernel, which is faster for it)
    ColCoefsHost meo;
    coeffs_meooe5d(op, dag, meo.l1, meo.d1, meo.u1);
    te1->subset = te2->subset = GB_EVEN;
    to->subset = out->subset = GB_ODD;
    if (!dag) {
      GB_TRY(op_meooe5d(op, in, to, 0));
      GB_TRY(op_dhop_cb(op, to, te1, 0));
      GB_TRY(col_field(op, COL_INV_M5D, COLB_NONE, 0, te1, nullptr, te2, 0.0, meo));
      // FP32 / FP16 (one right-hand side, or 16-slot column blocks of two rhs at most): the
      // second Dhop ends with Mooee in - (its result) and the norm, in one launch; otherwise
      // the Dhop and the Mooee kernel run separately
      std::vector<double> ml, md, mu;
      coeffs_mooee(op, 0, ml, md, mu);
      int fused = 0;
      GB_TRY(launch_dhop_mooee(op, half_view(te2, 0), half_view(in, 0), half_view(out, 0), GB_ODD, ml.data(),
                               md.data(), mu.data(), &fused));
      if (fused) {
        out->subset = GB_ODD;
        if (norm_parts) *norm_parts = fused;
        return GB_OK;
      }
      GB_TRY(op_dhop_cb(op, te2, to, 0));
      return op_mooee(op, in, out, 0, to, -1.0, norm_parts);
    }
    GB_TRY(op_dhop_cb(op, in, te1, 1));
    GB_TRY(col_field(op, COL_M5D_INV, COLB_NONE, 1, te1, nullptr, te2, 0.0, meo));
    GB_TRY(op_dhop_cb(op, te2, to, 1));
    ColCoefsHost h;
    coeffs_mooee(op, 1, h.l1, h.d1, h.u1);
    h.l2 = meo.l1; h.d2 = meo.d1; h.u2 = meo.u1;
    return col_field(op, COL_M5D, COLB_M5D, 1, in, to, out, -1.0, h, r_upd, r_parts);
  }
  GB_TRY(op_meooe(op, in, te1, dag));
  GB_TRY(op_mooee_inv(op, te1, te2, dag));
  GB_TRY(op_meooe(op, te2, to, dag));
  return op_mooee(op, in, out, dag, to, -1.0, dag ? nullptr : norm_parts);  // out = Mooee in - tmp
}

int op_mpcdagmpc(Op* op, Field* in, Field* out) {
  Field* t;
  GB_TRY(ws_get(op, GB_ODD, in->prec, WS_MPCDAGMPC, &t));
  GB_TRY(op_mpc(op, in, t, 0));
  return op_mpc(op, t, out, 1);
}

// M / Mdag on full fields (WilsonFermionImplementation.h:113-127,
// CayleyFermion5DImplementation.h:272-306)
int op_m(Op* op, Field* in, Field* out, int dag) {
  if (!in->full() || !out->full()) { set_error("M: full fields expected"); return GB_ERR_BAD_PARITY; }
  if (op->kind == 0) {
    GB_TRY(op_dhop_full(op, in, out, dag));
    if (op->tm) return tm_diag(op, in, out, dag, 0, out, 1.0);  // out = Mooee in + Dhop in
    return field_axpby(out, 1.0, op->diag_mass, out, in);
  }
  Field* Din;
  GB_TRY(ws_get(op, GB_FULL, in->prec, WS_M_DIN, &Din));
  Field* t;
  GB_TRY(ws_get(op, GB_FULL, in->prec, WS_M_T, &t));
  std::vector<double> l, d, u;
  coeffs_m5d_unit(op, l, d, u);
  if (!dag) {
    GB_TRY(op_meooe5d(op, in, Din, 0));            // Din = Meooe5D psi
    GB_TRY(op_dhop_full(op, Din, t, 0));           // t = Dhop Din
    GB_TRY(field_axpby(t, 1.0, 4.0 - op->M5, t, Din));  // t = DW Din
    return m5d_field(op, in, t, out, l, d, u, 0, in, 1.0);  // out = M5D(psi, t) + psi
  }
  GB_TRY(op_dhop_full(op, in, t, 1));
  GB_TRY(field_axpby(t, 1.0, 4.0 - op->M5, t, in));   // t = DW^dag psi
  GB_TRY(op_meooe5d(op, t, Din, 1));               // Din = MeooeDag5D t
  return m5d_field(op, in, Din, out, l, d, u, 1, in, 1.0);  // out = M5Ddag(psi, Din) + psi
}

int op_mdagm(Op* op, Field* in, Field* out, Field** m_in) {
  Field* t;
  GB_TRY(ws_get(op, GB_FULL, in->prec, WS_MDAGM, &t));
  GB_TRY(op_m(op, in, t, 0));
  if (m_in) *m_in = t;
  return op_m(op, t, out, 1);
}

// Dminus / DminusDag (CayleyFermion5DImplementation.h:131-153):
// chi = psi - cs (DW psi), DW = Dhop + (4 - M5); cs = c for every s of a Moebius operator.
int op_dminus(Op* op, Field* in, Field* out, int dag) {
  if (op->kind != 1) { set_error("Dminus: Moebius operators only"); return GB_ERR_UNSUPPORTED; }
  if (!in->full() || !out->full()) { set_error("Dminus: full fields expected"); return GB_ERR_BAD_PARITY; }
  Field* t;
  GB_TRY(ws_get(op, GB_FULL, in->prec, WS_DMINUS, &t));
  GB_TRY(op_dhop_full(op, in, t, dag));
  if (op->zmobius) {  // chi_s = psi_s - cs_s (DW psi)_s, conj(cs_s) for the dagger
    GB_TRY(field_axpby(t, 1.0, 4.0 - op->M5, t, in));
    ZCoefsHost h;
    h.e.resize(op->Ls);
    for (int s = 0; s < op->Ls; s++) h.e[s] = dag ? -std::conj(op->zcs[s]) : -op->zcs[s];
    return zcol_field(op, ZPROG_DIAG, dag, in, t, out, 0.0, h);
  }
  const double c = op->cs[0];
  return field_axpby(out, 1.0 - c * (4.0 - op->M5), -c, in, t);
}

// ---------------------------------------------------------------------------------------
// neighbour tables
// ---------------------------------------------------------------------------------------
int build_neighbours(Op* op) {
  const int* L = op->dims;
  std::vector<int> tab(size_t(op->half4) * 8);
  for (int p = 0; p < 2; p++) {
    for (int64_t site = 0; site < op->vol4; site++) {
      int x[4];
      int64_t r = site;
      for (int k = 0; k < 4; k++) { x[k] = int(r % L[k]); r /= L[k]; }
      if (((x[0] + x[1] + x[2] + x[3]) & 1) != p) continue;
      const int64_t xcb = site >> 1;
      for (int leg = 0; leg < 8; leg++) {
        const int mu = leg & 3;
        int y[4] = {x[0], x[1], x[2], x[3]};
        y[mu] = (y[mu] + (leg < 4 ? 1 : -1) + L[mu]) % L[mu];
        const int64_t ns = y[0] + int64_t(L[0]) * (y[1] + int64_t(L[1]) * (y[2] + int64_t(L[2]) * y[3]));
        tab[size_t(xcb) * 8 + leg] = int(ns >> 1);
      }
    }
    GB_CHECK_CUDA(cudaMemcpyAsync(op->nbr[p], tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice, op->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));  // tab is reused for the next parity
  }
  return GB_OK;
}

static void cayley_setup(Op* op) {
  const int Ls = op->Ls;
  const double b = op->b, c = op->c, M5 = op->M5, mf = op->mass;
  op->bs.assign(Ls, 0); op->cs.assign(Ls, 0); op->bee.assign(Ls, 0); op->cee.assign(Ls, 0);
  op->dee.assign(Ls, 0); op->lee.assign(Ls, 0); op->leem.assign(Ls, 0); op->uee.assign(Ls, 0); op->ueem.assign(Ls, 0);
  // Moebius tanh: omega_s = 1 (MobiusFermion.h:63-67, Zolotarev.cc:471-473)
  for (int i = 0; i < Ls; i++) {
    const double omega = 1.0;
    op->bs[i] = 0.5 * ((b + c) / omega + (b - c));
    op->cs[i] = 0.5 * ((b + c) / omega - (b - c));
    op->bee[i] = op->bs[i] * (4.0 - M5) + 1.0;
    op->cee[i] = 1.0 - op->cs[i] * (4.0 - M5);
  }
  const std::vector<double>& aee = op->cee;
  for (int i = 0; i < Ls; i++) {
    op->dee[i] = op->bee[i];
    if (i < Ls - 1) {
      op->lee[i] = -op->cee[i + 1] / op->bee[i];
      op->leem[i] = mf * op->cee[Ls - 1] / op->bee[0];
      for (int j = 0; j < i; j++) op->leem[i] *= aee[j] / op->bee[j + 1];
      op->uee[i] = -aee[i] / op->bee[i];
      op->ueem[i] = mf;
      for (int j = 1; j <= i; j++) op->ueem[i] *= op->cee[j] / op->bee[j];
      op->ueem[i] *= aee[0] / op->bee[0];
    }
  }
  double delta_d = mf * op->cee[Ls - 1];
  for (int j = 0; j < Ls - 1; j++) delta_d *= op->cee[j] / op->bee[j];
  op->dee[Ls - 1] += delta_d;
}

// SetCoefficientsInternal with complex omega_s = gamma_s (ZMobiusFermion.h,
// CayleyFermion5DImplementation.h:410-535)
static void zcayley_setup(Op* op) {
  const int Ls = op->Ls;
  const double b = op->b, c = op->c, M5 = op->M5, mf = op->mass;
  using C = std::complex<double>;
  op->zbs.assign(Ls, 0); op->zcs.assign(Ls, 0); op->zbee.assign(Ls, 0); op->zcee.assign(Ls, 0);
  op->zdee.assign(Ls, 0); op->zlee.assign(Ls, 0); op->zleem.assign(Ls, 0); op->zuee.assign(Ls, 0); op->zueem.assign(Ls, 0);
  for (int i = 0; i < Ls; i++) {
    const C omega = op->zgamma[i];
    op->zbs[i] = 0.5 * ((b + c) / omega + (b - c));
    op->zcs[i] = 0.5 * ((b + c) / omega - (b - c));
    op->zbee[i] = op->zbs[i] * (4.0 - M5) + 1.0;
    op->zcee[i] = 1.0 - op->zcs[i] * (4.0 - M5);
  }
  const std::vector<C>& aee = op->zcee;
  for (int i = 0; i < Ls; i++) {
    op->zdee[i] = op->zbee[i];
    if (i < Ls - 1) {
      op->zlee[i] = -op->zcee[i + 1] / op->zbee[i];
      op->zleem[i] = mf * op->zcee[Ls - 1] / op->zbee[0];
      for (int j = 0; j < i; j++) op->zleem[i] *= aee[j] / op->zbee[j + 1];
      op->zuee[i] = -aee[i] / op->zbee[i];
      op->zueem[i] = mf;
      for (int j = 1; j <= i; j++) op->zueem[i] *= op->zcee[j] / op->zbee[j];
      op->zueem[i] *= aee[0] / op->zbee[0];
    }
  }
  C delta_d = mf * op->zcee[Ls - 1];
  for (int j = 0; j < Ls - 1; j++) delta_d *= op->zcee[j] / op->zbee[j];
  op->zdee[Ls - 1] += delta_d;
}

static void op_release(Op* op) {
  for (auto& e : op->events)
    if (e) cudaEventDestroy(e);
  for (Field* f : op->ws) field_free(f);
  op->ws.clear();
  for (int p = 0; p < 2; p++) {
    dev_free(op->links[p], op->stream);
    dev_free(op->nbr[p], op->stream);
  }
  dev_free(op->d_err, op->stream);
  dev_free(op->d_partial, op->stream);
  dev_free(op->d_result, op->stream);
  pinned_put(op->h_result);
  dev_free(op->d_stage, op->stream);
  dev_free(op->d_cg, op->stream);
  pinned_put(op->h_cg);
  dev_free(op->d_all_done, op->stream);
}

static int op_create(int kind, const int dims[4], int Ls, double mass, double M5, double b, double c,
                     const double* phases, int precision, int nrhs, void* stream, unsigned flags, gb_op_t* out) {
  if (!dims || !out) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  for (int k = 0; k < 4; k++)
    if (dims[k] < 2 || (dims[k] & 1)) { set_error("dims[%d] = %d must be even and >= 2", k, dims[k]); return GB_ERR_BAD_ARG; }
  if (precision < GB_F64 || precision > GB_F16) { set_error("bad precision %d", precision); return GB_ERR_BAD_ARG; }
  if (nrhs < 1 || Ls < 1) { set_error("nrhs and Ls must be >= 1"); return GB_ERR_BAD_ARG; }
  if (kind == 1 && (Ls < 2 || Ls > kMaxLs)) { set_error("Ls = %d outside [2, %d]", Ls, kMaxLs); return GB_ERR_BAD_ARG; }
  if (kind == 1 && (Ls & 1)) { set_error("Ls = %d: the fifth dimension must be even", Ls); return GB_ERR_UNSUPPORTED; }
  if (Ls * nrhs > kMaxL5) { set_error("Ls*nrhs = %d exceeds %d", Ls * nrhs, kMaxL5); return GB_ERR_UNSUPPORTED; }
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { set_error("no CUDA device"); return GB_ERR_NO_DEVICE; }
  gb_op_s* op = new (std::nothrow) gb_op_s;
  if (!op) { set_error("host allocation failed"); return GB_ERR_OOM; }
  op->kind = kind;
  op->vol4 = 1;
  for (int k = 0; k < 4; k++) { op->dims[k] = dims[k]; op->vol4 *= dims[k]; }
  op->half4 = op->vol4 / 2;
  if (op->half4 * 8 > int64_t(0x7fffffff)) { delete op; set_error("lattice too large for 32-bit neighbour tables"); return GB_ERR_UNSUPPORTED; }
  op->Ls = kind == 1 ? Ls : 1;
  op->nrhs_user = nrhs;
  op->nrhs = ((op->Ls * nrhs) & 1) ? nrhs + 1 : nrhs;  // keep L5 even (site pairs)
  op->L5 = op->Ls * op->nrhs;
  nrhs = op->nrhs;
  op->prec = precision;
  op->mass = mass;
  op->M5 = M5;
  op->b = b;
  op->c = c;
  op->diag_mass = 4.0 + mass;
  op->flags = flags;
  op->stream = static_cast<cudaStream_t>(stream);
  cudaGetDevice(&op->device);
  for (int k = 0; k < 4; k++) {
    op->phases[k] = phases ? std::complex<double>(phases[2 * k], phases[2 * k + 1]) : std::complex<double>(1, 0);
    const std::complex<double> z = op->phases[k];
    if (!(z.imag() == 0 && (z.real() == 1 || z.real() == -1))) op->phases_pm1 = false;
  }
  op->recon12 = (flags & GB_FLAG_RECON12) != 0;
  if (op->recon12 && !op->phases_pm1) {
    delete op;
    set_error("12-real links need real boundary phases (+1 or -1)");
    return GB_ERR_UNSUPPORTED;
  }
  if ((flags & GB_FLAG_DF64) && (precision != GB_F64 || op->recon12)) {
    delete op;
    set_error("double-float arithmetic is for FP64 operators with 18-real links");
    return GB_ERR_UNSUPPORTED;
  }
  op->df64 = (flags & GB_FLAG_DF64) != 0;
  if (kind == 1) cayley_setup(op);
  keep_pool_memory(op->device);
  int rc = GB_OK;
  auto alloc = [&](void** p, size_t n) {
    if (rc != GB_OK) return;
    if (dev_alloc(p, n, op->stream) != cudaSuccess) { set_error("device allocation of %zu bytes failed", n); rc = GB_ERR_OOM; }
  };
  for (int p = 0; p < 2; p++) {
    alloc(&op->links[p], op->link_bytes_per_parity());
    alloc(reinterpret_cast<void**>(&op->nbr[p]), size_t(op->half4) * 8 * sizeof(int));
  }
  alloc(reinterpret_cast<void**>(&op->d_err), sizeof(int));
  // the reductions' [2 halves][kRedBlocks][nrhs][2]; an FP32 Moebius Dhop with the Mooee
  // epilogue writes nrhs sums per CTA
  op->partial_doubles = size_t(2) * kRedBlocks * nrhs * 2;
  if (op->prec != GB_F64 && op->kind == 1)
    op->partial_doubles = std::max(op->partial_doubles, dhop_pair_ctas(op) * nrhs);
  alloc(reinterpret_cast<void**>(&op->d_partial), op->partial_doubles * sizeof(double));
  alloc(reinterpret_cast<void**>(&op->d_result), size_t(nrhs) * 8 * sizeof(double));
  alloc(reinterpret_cast<void**>(&op->d_cg), size_t(nrhs) * sizeof(CGScalars));
  alloc(reinterpret_cast<void**>(&op->d_all_done), 4 * sizeof(int));
  if (rc == GB_OK && !(op->h_result = static_cast<double*>(pinned_get(size_t(nrhs) * 8 * sizeof(double))))) rc = GB_ERR_OOM;
  if (rc == GB_OK && !(op->h_cg = static_cast<CGScalars*>(pinned_get(size_t(nrhs) * sizeof(CGScalars) + 64)))) rc = GB_ERR_OOM;
  if (rc == GB_OK && cudaMemsetAsync(op->d_err, 0, sizeof(int), op->stream) != cudaSuccess) rc = GB_ERR_CUDA;
  if (rc == GB_OK) rc = build_neighbours(op);
  if (rc != GB_OK) {
    op_release(op);
    delete op;
    return rc;
  }
  op->last_iters.assign(nrhs, 0);
  op->last_resid.assign(nrhs, 0.0);
  *out = op;
  return GB_OK;
}

int op_import_gauge_dev(Op* op, const double* U_dev) {
  for (int p = 0; p < 2; p++) GB_TRY(launch_double_store(op, U_dev, p));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  op->gauge_loaded = true;
  return GB_OK;
}

int ensure_stage(Op* op, size_t bytes) {
  if (op->stage_bytes >= bytes) return GB_OK;
  dev_free(op->d_stage, op->stream);
  op->d_stage = nullptr;
  op->stage_bytes = 0;
  if (dev_alloc(reinterpret_cast<void**>(&op->d_stage), bytes, op->stream) != cudaSuccess) {
    set_error("device allocation of %zu staging bytes failed", bytes);
    return GB_ERR_OOM;
  }
  op->stage_bytes = bytes;
  return GB_OK;
}

size_t field_host_doubles(const Field* f) {
  const Op* op = f->op;
  const size_t n4 = f->full() ? size_t(op->vol4) : size_t(op->half4);
  return n4 * op->Ls * op->nrhs_user * 24;
}

int field_import_dev(Field* f, const void* dev, int canon_prec) {
  if (f->full()) {
    for (int p = 0; p < 2; p++) GB_TRY(launch_import_half(f->op, dev, canon_prec, half_view(f, p), p, 1));
  } else {
    GB_TRY(launch_import_half(f->op, dev, canon_prec, half_view(f, 0), f->subset, 0));
  }
  return GB_OK;
}
int field_export_dev(Field* f, void* dev, int canon_prec) {
  if (f->full()) {
    for (int p = 0; p < 2; p++) GB_TRY(launch_export_half(f->op, half_view(f, p), dev, canon_prec, p, 1));
  } else {
    GB_TRY(launch_export_half(f->op, half_view(f, 0), dev, canon_prec, f->subset, 0));
  }
  return GB_OK;
}

int check_device_error(Op* op) {
  int h = 0;
  GB_CHECK_CUDA(cudaMemcpyAsync(&h, op->d_err, sizeof(int), cudaMemcpyDeviceToHost, op->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  if (h) {
    op->poisoned = true;
    set_error("a bounded device wait timed out: this operator's results are untrusted; recreate it");
    cudaMemsetAsync(op->d_err, 0, sizeof(int), op->stream);
    return GB_ERR_TIMEOUT;
  }
  return GB_OK;
}

}  // namespace gb

using namespace gb;

// =======================================================================================
// C ABI
// =======================================================================================
extern "C" {

int gb_version(void) { return 100; }
const char* gb_last_error(void) { return gb::g_err; }
const char* gb_status_string(int s) {
  switch (s) {
    case GB_OK: return "ok";
    case GB_ERR_BAD_ARG: return "bad argument";
    case GB_ERR_BAD_PARITY: return "checkerboard mismatch";
    case GB_ERR_OOM: return "out of memory";
    case GB_ERR_CUDA: return "CUDA error";
    case GB_ERR_NOT_CONVERGED: return "not converged";
    case GB_ERR_TIMEOUT: return "device wait timed out";
    case GB_ERR_NO_DEVICE: return "no CUDA device";
    case GB_ERR_UNSUPPORTED: return "unsupported";
    case GB_ERR_IO: return "file I/O or format error";
    case GB_ERR_CANCELLED: return "cancelled";
  }
  return "unknown status";
}
int gb_device_count(int* n) {
  int k = 0;
  if (cudaGetDeviceCount(&k) != cudaSuccess) k = 0;
  if (n) *n = k;
  return GB_OK;
}

int gb_wilson_create(const int dims[4], double mass, const double* phases, int precision, int nrhs, void* stream,
                     unsigned flags, gb_op_t* out) {
  return op_create(0, dims, 1, mass, 0, 0, 0, phases, precision, nrhs, stream, flags, out);
}
int gb_mobius_create(const int dims[4], int Ls, double mf, double M5, double b, double c, const double* phases,
                     int precision, int nrhs, void* stream, unsigned flags, gb_op_t* out) {
  return op_create(1, dims, Ls, mf, M5, b, c, phases, precision, nrhs, stream, flags, out);
}
int gb_zmobius_create(const int dims[4], int Ls, double mf, double M5, const double* gamma, double b, double c,
                      const double* phases, int precision, int nrhs, void* stream, unsigned flags, gb_op_t* out) {
  if (!gamma || !out) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (precision == GB_F16) { set_error("ZMobius: FP64 or FP32 operators"); return GB_ERR_UNSUPPORTED; }
  if (!zmobius_ls_supported(Ls)) { set_error("ZMobius: Ls = %d is not supported", Ls); return GB_ERR_UNSUPPORTED; }
  for (int s = 0; s < Ls; s++)
    if (gamma[2 * s] == 0.0 && gamma[2 * s + 1] == 0.0) { set_error("ZMobius: gamma[%d] = 0", s); return GB_ERR_BAD_ARG; }
  GB_TRY(op_create(1, dims, Ls, mf, M5, b, c, phases, precision, nrhs, stream, flags, out));
  Op* op = *out;
  op->zmobius = true;
  op->zgamma.resize(Ls);
  for (int s = 0; s < Ls; s++) op->zgamma[s] = std::complex<double>(gamma[2 * s], gamma[2 * s + 1]);
  zcayley_setup(op);
  return GB_OK;
}
int gb_op_destroy(gb_op_t op) {
  if (!op) return GB_OK;
  cudaStreamSynchronize(op->stream);
  op_release(op);
  delete op;
  return GB_OK;
}
int gb_op_import_gauge(gb_op_t op, const double* U_host) {
  if (!op || !U_host) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  const size_t bytes = size_t(op->vol4) * 4 * 9 * 16;
  GB_TRY(ensure_stage(op, bytes));
  GB_CHECK_CUDA(cudaMemcpyAsync(op->d_stage, U_host, bytes, cudaMemcpyHostToDevice, op->stream));
  return op_import_gauge_dev(op, op->d_stage);
}
int gb_op_import_gauge_device(gb_op_t op, const double* U_device) {
  if (!op || !U_device) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  return op_import_gauge_dev(op, U_device);
}
int gb_op_info(gb_op_t op, int* Ls, int* nrhs, int64_t* half_sites4, int* precision) {
  if (!op) { set_error("null operator"); return GB_ERR_BAD_ARG; }
  if (Ls) *Ls = op->Ls;
  if (nrhs) *nrhs = op->nrhs_user;
  if (half_sites4) *half_sites4 = op->half4;
  if (precision) *precision = op->prec;
  return GB_OK;
}
int gb_op_set_stream(gb_op_t op, void* stream) {
  if (!op) { set_error("null operator"); return GB_ERR_BAD_ARG; }
  op->stream = static_cast<cudaStream_t>(stream);
  return GB_OK;
}
int gb_op_cayley_coeffs(gb_op_t op, double* out) {
  if (!op || !out || op->kind != 1) { set_error("not a Moebius operator"); return GB_ERR_BAD_ARG; }
  if (op->zmobius) { set_error("ZMobius coefficients are complex"); return GB_ERR_UNSUPPORTED; }
  const std::vector<double>* v[9] = {&op->bs, &op->cs, &op->bee, &op->cee, &op->dee, &op->lee, &op->leem, &op->uee, &op->ueem};
  for (int k = 0; k < 9; k++) std::memcpy(out + k * op->Ls, v[k]->data(), op->Ls * sizeof(double));
  return GB_OK;
}

int gb_field_create(gb_op_t op, int subset, int precision, gb_field_t* out) {
  if (!op || !out) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (subset < GB_EVEN || subset > GB_FULL) { set_error("bad subset %d", subset); return GB_ERR_BAD_ARG; }
  Field* f;
  GB_TRY(field_alloc(op, subset, precision, &f));
  *out = static_cast<gb_field_t>(f);
  return GB_OK;
}
int gb_field_destroy(gb_field_t f) {
  if (f) {
    cudaStreamSynchronize(f->op->stream);
    field_free(f);
  }
  return GB_OK;
}
int gb_field_subset(gb_field_t f, int* subset) {
  if (!f || !subset) return GB_ERR_BAD_ARG;
  *subset = f->subset;
  return GB_OK;
}
int gb_field_set_subset(gb_field_t f, int subset) {
  if (!f || f->full() || subset == GB_FULL || subset < 0) { set_error("only half fields can be relabelled"); return GB_ERR_BAD_ARG; }
  f->subset = subset;
  return GB_OK;
}
int gb_field_host_len(gb_field_t f, size_t* n) {
  if (!f || !n) return GB_ERR_BAD_ARG;
  *n = field_host_doubles(f);
  return GB_OK;
}
static int host_import(gb_field_t f, const void* host, int host_prec) {
  if (!f || !host) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  Op* op = f->op;
  const size_t bytes = field_host_doubles(f) * (host_prec == GB_F32 ? sizeof(float) : sizeof(double));
  GB_TRY(ensure_stage(op, bytes));
  GB_CHECK_CUDA(cudaMemcpyAsync(op->d_stage, host, bytes, cudaMemcpyHostToDevice, op->stream));
  GB_TRY(field_import_dev(f, op->d_stage, host_prec));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  return GB_OK;
}
static int host_export(gb_field_t f, void* host, int host_prec) {
  if (!f || !host) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  Op* op = f->op;
  const size_t bytes = field_host_doubles(f) * (host_prec == GB_F32 ? sizeof(float) : sizeof(double));
  GB_TRY(ensure_stage(op, bytes));
  GB_TRY(field_export_dev(f, op->d_stage, host_prec));
  GB_CHECK_CUDA(cudaMemcpyAsync(host, op->d_stage, bytes, cudaMemcpyDeviceToHost, op->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  return GB_OK;
}
int gb_field_import(gb_field_t f, const double* host) { return host_import(f, host, GB_F64); }
int gb_field_export(gb_field_t f, double* host) { return host_export(f, host, GB_F64); }
int gb_field_import_f32(gb_field_t f, const float* host) { return host_import(f, host, GB_F32); }
int gb_field_export_f32(gb_field_t f, float* host) { return host_export(f, host, GB_F32); }
int gb_field_import_device(gb_field_t f, const double* dev) {
  if (!f || !dev) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  return field_import_dev(f, dev, GB_F64);
}
int gb_field_export_device(gb_field_t f, double* dev) {
  if (!f || !dev) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  return field_export_dev(f, dev, GB_F64);
}

// ---- transfer queue: double-buffered staging, H2D and D2H on copy streams of their own ----
}  // extern "C"

struct gb_xfer_s {
  Op* op = nullptr;
  cudaStream_t h2d = nullptr, d2h = nullptr;
  struct Slot {
    void* buf = nullptr;
    size_t cap = 0;
    cudaEvent_t filled = nullptr, free = nullptr;
  };
  Slot in[2], out[2];
  int in_next = 0, out_next = 0;
};

static int xfer_slot_ensure(gb_xfer_s::Slot& s, size_t bytes) {
  if (s.cap >= bytes) return GB_OK;
  if (s.buf) {
    // the slot's last user is ordered before its free event
    GB_CHECK_CUDA(cudaEventSynchronize(s.free));
    cudaFree(s.buf);
    s.buf = nullptr;
    s.cap = 0;
  }
  GB_CHECK_CUDA(cudaMalloc(&s.buf, bytes));
  s.cap = bytes;
  return GB_OK;
}

static void xfer_release(gb_xfer_s* x) {
  if (x->h2d) cudaStreamSynchronize(x->h2d);
  if (x->d2h) cudaStreamSynchronize(x->d2h);
  if (x->op) cudaStreamSynchronize(x->op->stream);
  for (auto* set : {x->in, x->out})
    for (int k = 0; k < 2; k++) {
      cudaFree(set[k].buf);
      if (set[k].filled) cudaEventDestroy(set[k].filled);
      if (set[k].free) cudaEventDestroy(set[k].free);
    }
  if (x->h2d) cudaStreamDestroy(x->h2d);
  if (x->d2h) cudaStreamDestroy(x->d2h);
  delete x;
}

extern "C" {

int gb_xfer_create(gb_op_t op, gb_xfer_t* out) {
  if (!op || !out) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  gb_xfer_s* x = new (std::nothrow) gb_xfer_s;
  if (!x) { set_error("host allocation failed"); return GB_ERR_OOM; }
  x->op = op;
  cudaError_t e = cudaStreamCreateWithFlags(&x->h2d, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&x->d2h, cudaStreamNonBlocking);
  for (auto* set : {x->in, x->out})
    for (int k = 0; k < 2 && e == cudaSuccess; k++) {
      e = cudaEventCreateWithFlags(&set[k].filled, cudaEventDisableTiming);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&set[k].free, cudaEventDisableTiming);
    }
  if (e != cudaSuccess) {
    set_error("transfer queue: %s", cudaGetErrorString(e));
    xfer_release(x);
    return GB_ERR_CUDA;
  }
  *out = x;
  return GB_OK;
}
int gb_xfer_destroy(gb_xfer_t x) {
  if (x) xfer_release(x);
  return GB_OK;
}
int gb_xfer_import(gb_xfer_t x, gb_field_t f, const void* host, int host_prec) {
  if (!x || !f || !host) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (host_prec != GB_F64 && host_prec != GB_F32) { set_error("host precision must be GB_F64 or GB_F32"); return GB_ERR_BAD_ARG; }
  if (!ops_conformable(f->op, x->op)) { set_error("field is not conformable to the queue's operator"); return GB_ERR_BAD_ARG; }
  Op* op = x->op;
  gb_xfer_s::Slot& s = x->in[x->in_next];
  const size_t bytes = field_host_doubles(f) * (host_prec == GB_F32 ? sizeof(float) : sizeof(double));
  GB_TRY(xfer_slot_ensure(s, bytes));
  x->in_next ^= 1;
  GB_CHECK_CUDA(cudaStreamWaitEvent(x->h2d, s.free, 0));  // the slot's previous layout kernel is done
  GB_CHECK_CUDA(cudaMemcpyAsync(s.buf, host, bytes, cudaMemcpyHostToDevice, x->h2d));
  GB_CHECK_CUDA(cudaEventRecord(s.filled, x->h2d));
  GB_CHECK_CUDA(cudaStreamWaitEvent(op->stream, s.filled, 0));
  GB_TRY(field_import_dev(f, s.buf, host_prec));
  GB_CHECK_CUDA(cudaEventRecord(s.free, op->stream));
  return GB_OK;
}
int gb_xfer_export(gb_xfer_t x, gb_field_t f, void* host, int host_prec) {
  if (!x || !f || !host) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (host_prec != GB_F64 && host_prec != GB_F32) { set_error("host precision must be GB_F64 or GB_F32"); return GB_ERR_BAD_ARG; }
  if (!ops_conformable(f->op, x->op)) { set_error("field is not conformable to the queue's operator"); return GB_ERR_BAD_ARG; }
  Op* op = x->op;
  gb_xfer_s::Slot& s = x->out[x->out_next];
  const size_t bytes = field_host_doubles(f) * (host_prec == GB_F32 ? sizeof(float) : sizeof(double));
  GB_TRY(xfer_slot_ensure(s, bytes));
  x->out_next ^= 1;
  GB_CHECK_CUDA(cudaStreamWaitEvent(op->stream, s.free, 0));  // the slot's previous copy-out is done
  GB_TRY(field_export_dev(f, s.buf, host_prec));
  GB_CHECK_CUDA(cudaEventRecord(s.filled, op->stream));
  GB_CHECK_CUDA(cudaStreamWaitEvent(x->d2h, s.filled, 0));
  GB_CHECK_CUDA(cudaMemcpyAsync(host, s.buf, bytes, cudaMemcpyDeviceToHost, x->d2h));
  GB_CHECK_CUDA(cudaEventRecord(s.free, x->d2h));
  return GB_OK;
}
int gb_xfer_wait(gb_xfer_t x) {
  if (!x) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  GB_CHECK_CUDA(cudaStreamSynchronize(x->h2d));
  GB_CHECK_CUDA(cudaStreamSynchronize(x->op->stream));
  GB_CHECK_CUDA(cudaStreamSynchronize(x->d2h));
  return GB_OK;
}

int gb_field_zero(gb_field_t f) {
  if (!f) return GB_ERR_BAD_ARG;
  return field_zero(f);
}
int gb_field_copy(gb_field_t dst, gb_field_t src) {
  GB_TRY(check_conf(dst, src));
  if (dst->full() != src->full()) { set_error("copy: full/half mismatch"); return GB_ERR_BAD_PARITY; }
  dst->subset = src->subset;
  return field_copy(dst, src);
}
int gb_field_norm2(gb_field_t f, double* out) {
  if (!f || !out) return GB_ERR_BAD_ARG;
  std::vector<double> v(f->op->nrhs);
  GB_TRY(field_norm2(f, v.data()));
  std::memcpy(out, v.data(), f->op->nrhs_user * sizeof(double));
  return GB_OK;
}
int gb_field_inner(gb_field_t a, gb_field_t b, double* out) {
  GB_TRY(check_conf(a, b));
  if (!out) return GB_ERR_BAD_ARG;
  if (a->subset != b->subset) { set_error("innerProduct: checkerboard mismatch"); return GB_ERR_BAD_PARITY; }
  std::vector<double> v(2 * a->op->nrhs);
  GB_TRY(field_inner(a, b, v.data()));
  std::memcpy(out, v.data(), 2 * a->op->nrhs_user * sizeof(double));
  return GB_OK;
}
int gb_field_axpby(gb_field_t z, double a, double b, gb_field_t x, gb_field_t y) {
  GB_TRY(check_conf(z, x));
  GB_TRY(check_conf(z, y));
  if (x->subset != y->subset) { set_error("axpby: checkerboard mismatch"); return GB_ERR_BAD_PARITY; }
  if (z->full() != x->full()) { set_error("axpby: full/half mismatch"); return GB_ERR_BAD_PARITY; }
  z->subset = x->subset;
  return field_axpby(z, a, b, x, y);
}
int gb_field_axpy(gb_field_t z, double a, gb_field_t x, gb_field_t y) { return gb_field_axpby(z, a, 1.0, x, y); }
int gb_field_axpy_norm(gb_field_t z, double a, gb_field_t x, gb_field_t y, double* norm_out) {
  GB_TRY(check_conf(z, x));
  GB_TRY(check_conf(z, y));
  if (x->subset != y->subset) { set_error("axpy_norm: checkerboard mismatch"); return GB_ERR_BAD_PARITY; }
  Op* op = z->op;
  z->subset = x->subset;
  const int g = red_parts(op, z->prec);
  const int halves = z->full() ? 2 : 1;
  for (int h = 0; h < halves; h++)
    GB_TRY(launch_axpy_norm_partial(op, half_view(z, h), a, half_view(x, h), half_view(y, h), z->n5,
                                    op->d_partial + size_t(h) * g * op->nrhs));
  GB_TRY(launch_reduce_final(op, op->d_partial, g * halves, 1, op->d_result));
  std::vector<double> v(op->nrhs);
  GB_TRY(fetch(op, op->d_result, v.data(), op->nrhs));
  std::memcpy(norm_out, v.data(), op->nrhs_user * sizeof(double));
  return GB_OK;
}
// axpby_norm (Lattice_reduction.h:316-372): z = a x + b y and |z|^2 per rhs (here two
// passes: the axpby, then the norm)
int gb_field_axpby_norm(gb_field_t z, double a, double b, gb_field_t x, gb_field_t y, double* norm_out) {
  if (!norm_out) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  GB_TRY(gb_field_axpby(z, a, b, x, y));
  std::vector<double> v(z->op->nrhs);
  GB_TRY(field_norm2(z, v.data()));
  std::memcpy(norm_out, v.data(), z->op->nrhs_user * sizeof(double));
  return GB_OK;
}
// innerProductNorm (Lattice_reduction.h:374-410): <a|b> (re, im per rhs) and |a|^2 per rhs
int gb_field_inner_norm(gb_field_t a, gb_field_t b, double* inner_out, double* norm_out) {
  if (!inner_out || !norm_out) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  GB_TRY(check_conf(a, b));
  if (a->subset != b->subset) { set_error("innerProductNorm: checkerboard mismatch"); return GB_ERR_BAD_PARITY; }
  Op* op = a->op;
  std::vector<double> ip(size_t(op->nrhs) * 2), nr(op->nrhs);
  GB_TRY(field_inner(a, b, ip.data()));
  GB_TRY(field_norm2(a, nr.data()));
  std::memcpy(inner_out, ip.data(), size_t(op->nrhs_user) * 2 * sizeof(double));
  std::memcpy(norm_out, nr.data(), op->nrhs_user * sizeof(double));
  return GB_OK;
}
int gb_field_pick_checkerboard(gb_field_t half, gb_field_t full) {
  GB_TRY(check_conf(half, full));
  if (half->full() || !full->full()) { set_error("pickCheckerboard: (half, full) expected"); return GB_ERR_BAD_PARITY; }
  Field* f = full;
  return launch_copy(half->op, half_view(half, 0), half_view(f, half->subset), half->n5);
}
int gb_field_set_checkerboard(gb_field_t full, gb_field_t half) {
  GB_TRY(check_conf(half, full));
  if (half->full() || !full->full()) { set_error("setCheckerboard: (full, half) expected"); return GB_ERR_BAD_PARITY; }
  Field* f = full;
  return launch_copy(half->op, half_view(f, half->subset), half_view(half, 0), half->n5);
}

// ---- operators ----
#define GB_OP_PRE(op, in, out)                                                     \
  GB_TRY(check_op(op));                                                            \
  GB_TRY(check_conf(in, out));                                                     \
  if (!ops_conformable(in->op, op)) { set_error("field is not conformable to the operator"); return GB_ERR_BAD_ARG; } \
  if (in == out) { set_error("in and out must be distinct fields"); return GB_ERR_BAD_ARG; }

int gb_M(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); return op_m(op, in, out, 0); }
int gb_Mdag(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); return op_m(op, in, out, 1); }
int gb_MdagM(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); return op_mdagm(op, in, out); }
int gb_Dhop(gb_op_t op, gb_field_t in, gb_field_t out, int dag) {
  GB_OP_PRE(op, in, out);
  return op_dhop_full(op, in, out, dag);
}
int gb_DhopEO(gb_op_t op, gb_field_t in, gb_field_t out, int dag) {
  GB_OP_PRE(op, in, out);
  GB_TRY(check_subset(in, GB_ODD, "DhopEO"));
  return op_dhop_cb(op, in, out, dag);
}
int gb_DhopOE(gb_op_t op, gb_field_t in, gb_field_t out, int dag) {
  GB_OP_PRE(op, in, out);
  GB_TRY(check_subset(in, GB_EVEN, "DhopOE"));
  return op_dhop_cb(op, in, out, dag);
}
int gb_Meooe(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); return op_meooe(op, in, out, 0); }
int gb_MeooeDag(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); return op_meooe(op, in, out, 1); }
int gb_Mooee(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); return op_mooee(op, in, out, 0, nullptr, 0); }
int gb_MooeeDag(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); return op_mooee(op, in, out, 1, nullptr, 0); }
int gb_MooeeInv(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); return op_mooee_inv(op, in, out, 0); }
int gb_MooeeInvDag(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); return op_mooee_inv(op, in, out, 1); }
int gb_Mpc(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); out->subset = GB_ODD; return op_mpc(op, in, out, 0); }
int gb_MpcDag(gb_op_t op, gb_field_t in, gb_field_t out) { GB_OP_PRE(op, in, out); out->subset = GB_ODD; return op_mpc(op, in, out, 1); }
int gb_MpcDagMpc(gb_op_t op, gb_field_t in, gb_field_t out) {
  GB_OP_PRE(op, in, out);
  GB_TRY(check_subset(in, GB_ODD, "MpcDagMpc"));
  out->subset = GB_ODD;
  return op_mpcdagmpc(op, in, out);
}
int gb_Dminus(gb_op_t op, gb_field_t in, gb_field_t out, int dag) {
  GB_OP_PRE(op, in, out);
  return op_dminus(op, in, out, dag ? 1 : 0);
}

// ---- force terms (WilsonFermion5DImplementation.h:212-305, CayleyFermion5DImplementation.h:346-391) ----
static int deriv_launch(Op* op, Field* A, Field* B, int dag, double* mat) {
  if (A->full() != B->full()) { set_error("Deriv: A and B must both be full or both half fields"); return GB_ERR_BAD_PARITY; }
  if (A->full()) {
    for (int p = 0; p < 2; p++) GB_TRY(launch_deriv(op, half_view(A, p), half_view(B, 1 - p), p, dag, mat, 0));
    return GB_OK;
  }
  if (B->subset != 1 - A->subset) { set_error("DhopDerivEO/OE: B must be on the other checkerboard"); return GB_ERR_BAD_PARITY; }
  return launch_deriv(op, half_view(A, 0), half_view(B, 0), A->subset, dag, mat, 1);
}
static int deriv_entry(gb_op_t op, gb_field_t A, gb_field_t B, int dag, double* mat, int on_device, bool mderiv) {
  GB_TRY(check_op(op));
  if (!A || !B || !mat) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  GB_TRY(check_conf(A, B));
  if (!ops_conformable(A->op, op)) { set_error("field is not conformable to the operator"); return GB_ERR_BAD_ARG; }
  const size_t bytes = size_t(A->full() ? op->vol4 : op->half4) * 36 * 16;
  double* d = mat;
  if (!on_device) GB_CHECK_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&d), bytes, op->stream));
  struct Free { double* p; cudaStream_t s; ~Free() { if (p) cudaFreeAsync(p, s); } } guard{on_device ? nullptr : d, op->stream};
  Field* a = A;
  Field* b = B;
  if (mderiv && op->kind == 1) {
    // U d[D_w D5]/du V: Din = Meooe5D V (non-dag) or Meooe5D U (dag, the adjoint is implicit)
    Field* din;
    Field* src = dag ? A : B;
    GB_TRY(ws_get(op, src->full() ? GB_FULL : src->subset, src->prec, src->full() ? WS_DERIV_FULL : WS_DERIV, &din));
    din->subset = src->subset;
    GB_TRY(op_meooe5d(op, src, din, 0));
    (dag ? a : b) = din;
  }
  GB_TRY(deriv_launch(op, a, b, dag ? 1 : 0, d));
  if (!on_device) {
    GB_CHECK_CUDA(cudaMemcpyAsync(mat, d, bytes, cudaMemcpyDeviceToHost, op->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  }
  return GB_OK;
}
int gb_DhopDeriv(gb_op_t op, gb_field_t A, gb_field_t B, int dag, double* mat, int on_device) {
  return deriv_entry(op, A, B, dag, mat, on_device, false);
}
int gb_MDeriv(gb_op_t op, gb_field_t U, gb_field_t V, int dag, double* mat, int on_device) {
  return deriv_entry(op, U, V, dag, mat, on_device, true);
}

// ---- 4D <-> 5D surface fields (CayleyFermion5DImplementation.h:57-129) ----
static int surface_checks(gb_op_t op, gb_field_t f, const double* p4) {
  GB_TRY(check_op(op));
  if (!f || !p4) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (op->kind != 1) { set_error("physical fields: Moebius operators only"); return GB_ERR_UNSUPPORTED; }
  if (!ops_conformable(f->op, op)) { set_error("field is not conformable to the operator"); return GB_ERR_BAD_ARG; }
  if (!f->full()) { set_error("physical fields: a full 5D field expected"); return GB_ERR_BAD_PARITY; }
  return GB_OK;
}
static size_t surface_bytes(const Op* op) { return size_t(op->vol4) * op->nrhs_user * 24 * sizeof(double); }

static int import_surface(gb_op_t op, const double* src4d, int on_device, gb_field_t out, bool physical) {
  GB_TRY(surface_checks(op, out, src4d));
  const double* d = src4d;
  if (!on_device) {
    GB_TRY(ensure_stage(op, surface_bytes(op)));
    GB_CHECK_CUDA(cudaMemcpyAsync(op->d_stage, src4d, surface_bytes(op), cudaMemcpyHostToDevice, op->stream));
    d = op->d_stage;
  }
  Field* t = out;
  if (physical) GB_TRY(ws_get(op, GB_FULL, out->prec, WS_PHYS, &t));
  GB_TRY(field_zero(t));
  GB_TRY(launch_surface_insert(op, d, half_view(t, 0), half_view(t, 1)));
  if (physical) GB_TRY(op_dminus(op, t, out, 0));
  if (!on_device) GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  return GB_OK;
}
static int export_surface(gb_op_t op, gb_field_t in, double* out4d, int on_device, int solution) {
  GB_TRY(surface_checks(op, in, out4d));
  double* d = out4d;
  if (!on_device) {
    GB_TRY(ensure_stage(op, surface_bytes(op)));
    d = op->d_stage;
  }
  GB_TRY(launch_surface_extract(op, half_view(in, 0), half_view(in, 1), d, solution));
  if (!on_device) {
    GB_CHECK_CUDA(cudaMemcpyAsync(out4d, d, surface_bytes(op), cudaMemcpyDeviceToHost, op->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  }
  return GB_OK;
}
int gb_import_physical_source(gb_op_t op, const double* src4d, int on_device, gb_field_t out5d) {
  return import_surface(op, src4d, on_device, out5d, true);
}
int gb_import_unphysical_fermion(gb_op_t op, const double* src4d, int on_device, gb_field_t out5d) {
  return import_surface(op, src4d, on_device, out5d, false);
}
int gb_export_physical_solution(gb_op_t op, gb_field_t sol5d, double* out4d, int on_device) {
  return export_surface(op, sol5d, out4d, on_device, 1);
}
int gb_export_physical_source(gb_op_t op, gb_field_t src5d, double* out4d, int on_device) {
  return export_surface(op, src5d, out4d, on_device, 0);
}

// InsertSlice / ExtractSlice along the fifth dimension (Lattice_transfer.h:999-1070)
static int slice_checks(gb_op_t op, gb_field_t f, const double* p4, int s) {
  GB_TRY(check_op_geometry(op));
  if (!f || !p4) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (!ops_conformable(f->op, op)) { set_error("field is not conformable to the operator"); return GB_ERR_BAD_ARG; }
  if (!f->full()) { set_error("slices: a full 5D field expected"); return GB_ERR_BAD_PARITY; }
  if (s < 0 || s >= op->Ls) { set_error("slice %d outside [0, %d)", s, op->Ls); return GB_ERR_BAD_ARG; }
  return GB_OK;
}
int gb_insert_slice(gb_op_t op, const double* src4d, int on_device, gb_field_t f5d, int s) {
  GB_TRY(slice_checks(op, f5d, src4d, s));
  const double* d = src4d;
  if (!on_device) {
    GB_TRY(ensure_stage(op, surface_bytes(op)));
    GB_CHECK_CUDA(cudaMemcpyAsync(op->d_stage, src4d, surface_bytes(op), cudaMemcpyHostToDevice, op->stream));
    d = op->d_stage;
  }
  GB_TRY(launch_slice(op, const_cast<double*>(d), half_view(f5d, 0), half_view(f5d, 1), s, 1));
  if (!on_device) GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  return GB_OK;
}
int gb_extract_slice(gb_op_t op, gb_field_t f5d, int s, double* out4d, int on_device) {
  GB_TRY(slice_checks(op, f5d, out4d, s));
  double* d = out4d;
  if (!on_device) {
    GB_TRY(ensure_stage(op, surface_bytes(op)));
    d = op->d_stage;
  }
  GB_TRY(launch_slice(op, d, half_view(f5d, 0), half_view(f5d, 1), s, 0));
  if (!on_device) {
    GB_CHECK_CUDA(cudaMemcpyAsync(out4d, d, surface_bytes(op), cudaMemcpyDeviceToHost, op->stream));
    GB_CHECK_CUDA(cudaStreamSynchronize(op->stream));
  }
  return GB_OK;
}

// CayleyFermion5D::P / Pdag (CayleyFermion5DImplementation.h:70-88)
int gb_P(gb_op_t op, gb_field_t in, gb_field_t out, int dag) {
  GB_TRY(check_op_geometry(op));
  if (!in || !out) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (op->kind != 1) { set_error("P: Moebius operators only"); return GB_ERR_UNSUPPORTED; }
  if (in == out || in->data == out->data) { set_error("P: in and out must be distinct fields"); return GB_ERR_BAD_ARG; }
  GB_TRY(check_conf(in, out));
  if (!ops_conformable(in->op, op)) { set_error("field is not conformable to the operator"); return GB_ERR_BAD_ARG; }
  if (in->subset != out->subset) { set_error("P: in and out on different checkerboards"); return GB_ERR_BAD_PARITY; }
  if (in->full()) {
    for (int p = 0; p < 2; p++) GB_TRY(launch_chiral_shift(op, half_view(in, p), half_view(out, p), dag));
  } else {
    GB_TRY(launch_chiral_shift(op, half_view(in, in->subset), half_view(out, out->subset), dag));
  }
  return GB_OK;
}

// CayleyFermion5D::SetMass / Mass (CayleyFermion5D.h:71-83): the Cayley coefficients are
// rebuilt on the host; kernels take them by value at each launch, so the change applies to
// every operator call issued after this one
int gb_op_set_mass(gb_op_t op, double mass) {
  GB_TRY(check_op_geometry(op));
  op->mass = mass;
  op->diag_mass = 4.0 + mass;
  if (op->kind == 1) {
    if (op->zmobius) zcayley_setup(op);
    else cayley_setup(op);
  }
  return GB_OK;
}
// WilsonTMFermion5D (WilsonTMFermion5D.h:40-145): a Wilson operator on nslices slots
int gb_wilson_tm5d_create(const int dims[4], int nslices, const double* mass, const double* mu, const double* phases,
                          int precision, void* stream, unsigned flags, gb_op_t* out) {
  if (!mass || !mu || !out) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (nslices < 2 || (nslices & 1) || nslices > kMaxSlots) {
    set_error("WilsonTMFermion5D: an even number of slices in [2, %d]", kMaxSlots);
    return GB_ERR_BAD_ARG;
  }
  if (precision == GB_F16) { set_error("WilsonTMFermion5D: FP64 or FP32"); return GB_ERR_UNSUPPORTED; }
  GB_TRY(op_create(0, dims, 1, 0.0, 0.0, 0.0, 0.0, phases, precision, nslices, stream, flags, out));
  Op* op = *out;
  op->tm = true;
  op->tm_mass.assign(mass, mass + nslices);
  op->tm_mu.assign(mu, mu + nslices);
  return GB_OK;
}
int gb_op_tm_update(gb_op_t op, const double* mass, const double* mu) {
  GB_TRY(check_op_geometry(op));
  if (!op->tm || !mass || !mu) { set_error("tm update: a twisted-mass operator and both arrays"); return GB_ERR_BAD_ARG; }
  op->tm_mass.assign(mass, mass + op->L5);
  op->tm_mu.assign(mu, mu + op->L5);
  return GB_OK;
}

// the fifth-dimension transforms of the Fourier-accelerated Pauli-Villars solve
int gb_field_dft_s(gb_field_t in, gb_field_t out, const double* mat) {
  GB_TRY(check_conf(in, out));
  if (!mat || in == out) { set_error("DFT along s: a matrix and distinct fields"); return GB_ERR_BAD_ARG; }
  if (in->full() != out->full()) { set_error("DFT along s: full/half mismatch"); return GB_ERR_BAD_PARITY; }
  out->subset = in->subset;
  const int halves = in->full() ? 2 : 1;
  for (int h = 0; h < halves; h++) GB_TRY(launch_dft_s(in->op, half_view(in, h), half_view(out, h), mat));
  return GB_OK;
}
int gb_field_copy_slice5(gb_field_t dst, int t, gb_field_t src, int s) {
  if (!dst || !src) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  Op *od = dst->op, *os = src->op;
  for (int k = 0; k < 4; k++)
    if (od->dims[k] != os->dims[k]) { set_error("slice copy: different 4D extents"); return GB_ERR_BAD_ARG; }
  if (od->stream != os->stream) { set_error("slice copy: fields on different streams"); return GB_ERR_BAD_ARG; }
  if (dst->full() != src->full() || (!dst->full() && dst->subset != src->subset)) {
    set_error("slice copy: checkerboards differ");
    return GB_ERR_BAD_PARITY;
  }
  if (s < 0 || s >= os->L5 || t < 0 || t >= od->L5) { set_error("slice copy: slot out of range"); return GB_ERR_BAD_ARG; }
  const int halves = src->full() ? 2 : 1;
  for (int h = 0; h < halves; h++)
    GB_TRY(launch_copy_slot(od, half_view(src, h), os->L5, s, half_view(dst, h), od->L5, t));
  return GB_OK;
}
int gb_field_chiral_scale(gb_field_t in, gb_field_t out, const double* coef) {
  GB_TRY(check_conf(in, out));
  if (!coef) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  if (in->full() != out->full()) { set_error("chiral scale: full/half mismatch"); return GB_ERR_BAD_PARITY; }
  Op* op = in->op;
  const int L5 = op->L5;
  if (L5 > kMaxSlots) { set_error("chiral scale: L5 = %d above %d", L5, kMaxSlots); return GB_ERR_UNSUPPORTED; }
  std::vector<double> ur(L5), ui(L5), dr(L5), di(L5);
  for (int q = 0; q < L5; q++) { ur[q] = coef[4 * q]; ui[q] = coef[4 * q + 1]; dr[q] = coef[4 * q + 2]; di[q] = coef[4 * q + 3]; }
  out->subset = in->subset;
  const int halves = in->full() ? 2 : 1;
  for (int h = 0; h < halves; h++)
    GB_TRY(launch_chiral_scale(op, half_view(in, h), nullptr, 0.0, half_view(out, h), ur.data(), ui.data(), dr.data(),
                               di.data()));
  return GB_OK;
}

int gb_op_mass(gb_op_t op, double* mass) {
  GB_TRY(check_op_geometry(op));
  if (!mass) { set_error("null argument"); return GB_ERR_BAD_ARG; }
  *mass = op->mass;
  return GB_OK;
}

}  // extern "C"
