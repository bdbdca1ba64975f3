// gb_internal.h -- private types of the GB300 fermion library (host + device).
//
// Device layout of a fermion field (one checkerboard, "half"):
//   5D site index   i = s5 + L5 * x_cb,  s5 = rhs*Ls + s,  x_cb = site4 >> 1
//   FP64            12 planes of n5 double2, plane k = complex component spin*3+colour
//   FP32            12 planes of n5/2 float4: component k of the site pair (i, i+1),
//                   i even, as (re_i, re_i+1, im_i, im_i+1)
//   FP16            6 planes of n5/2 16-byte vectors: components 2q, 2q+1 of the site
//                   pair, each site scaled by its own float norm (one per 5D site)
//   A full field is the even half followed by the odd half.  The first half of the
//   planes holds spins 0,1 (the P+ chirality), the rest spins 2,3 (P-), so the 5D
//   chiral projections read half the planes.
// Gauge links (per output parity p): [x_cb][leg 0..7][3][3] complex in link precision,
//   legs 0..3 = Ud_mu(x) (forward), 4..7 = Ud_{mu}(x-mu)^dagger (backward), with the
//   -1/2 and boundary phases folded in (Grid's DoubleStore).  Neighbour table per parity:
//   [x_cb][leg] = x_cb of the neighbour in the other parity.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <complex>
#include <string>
#include <vector>

#include "gbdwf.h"

namespace gb {

constexpr int kMaxLs = 64;      // longest fifth dimension handled by the 5D kernels
constexpr int kMaxL5 = 1024;    // Ls * nrhs upper bound
constexpr int kMaxSlots = 64;   // L5 bound of the per-slot coefficient kernels
constexpr int kRedBlocks = 1216;  // 8 blocks per SM on 152 SMs for reductions

void set_error(const char* fmt, ...);

#define GB_CHECK_CUDA(call)                                                          \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      ::gb::set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
      return GB_ERR_CUDA;                                                            \
    }                                                                                \
  } while (0)

#define GB_TRY(call)              \
  do {                            \
    int rc_ = (call);             \
    if (rc_ != GB_OK) return rc_; \
  } while (0)

struct Field;

// Device-side per-right-hand-side scalars of a running CG (all FP64).
struct CGScalars {
  double c, d, a, cp, b, rsq, ssq, cprev, maxres, delta;
  int done, iter, relup, pad;
};

struct Op {
  int kind = 0;          // 0 Wilson, 1 Moebius
  int dims[4] = {0, 0, 0, 0};
  int64_t vol4 = 0, half4 = 0;
  // nrhs_user right-hand sides are visible at the ABI; internally nrhs is rounded up so
  // that L5 = Ls * nrhs is even (site pairs never straddle a 4D site).  The extra
  // right-hand side, when there is one, holds zeros: it converges at CG set-up and no
  // reduction result of it is returned.
  int Ls = 1, nrhs = 1, nrhs_user = 1, L5 = 1;
  int prec = GB_F64;     // arithmetic / storage precision of the operator
  double mass = 0, M5 = 0, b = 0, c = 0, diag_mass = 0;
  std::complex<double> phases[4];
  bool phases_pm1 = true;  // every phase is +1 or -1 (12-real reconstruction allowed)
  unsigned flags = 0;
  bool recon12 = false;
  bool df64 = false;     // FP64: the hopping term in double-float arithmetic (GB_FLAG_DF64)
  cudaStream_t stream = nullptr;
  int device = 0;
  bool gauge_loaded = false;

  void* links[2] = {nullptr, nullptr};  // per output parity
  int* nbr[2] = {nullptr, nullptr};
  int* d_err = nullptr;                 // device error flag of bounded waits
  // Set when the host finds d_err raised.  A Dhop CTA whose bounded wait for its TMA copy
  // gave up returns while that copy may still be writing into shared memory that the
  // next CTA on the SM receives, so no later result of this operator can be trusted:
  // every further Dhop on it returns GB_ERR_TIMEOUT until the operator is recreated.
  bool poisoned = false;

  // Cayley coefficients (Moebius) -- host copies
  std::vector<double> bs, cs, bee, cee, dee, lee, leem, uee, ueem;
  // ZMobius: complex omega_s, so complex Cayley coefficients (the real arrays above are
  // then unused)
  bool zmobius = false;
  // WilsonTMFermion5D (a Wilson operator, kind 0, whose L5 slots are the fifth dimension):
  // Mooee = (4 + m_s) + i mu_s gamma5 per slot
  bool tm = false;
  std::vector<double> tm_mass, tm_mu;
  std::vector<std::complex<double>> zgamma, zbs, zcs, zbee, zcee, zdee, zlee, zleem, zuee, zueem;

  // reduction scratch
  double* d_partial = nullptr;  // per-CTA partial sums, partial_doubles of them
  size_t partial_doubles = 0;    // 4 kRedBlocks nrhs, or a single-checkerboard Dhop's CTAs x nrhs if more
  double* d_result = nullptr;   // nrhs * 4
  double* h_result = nullptr;   // pinned, nrhs * 4
  // canonical FP64 staging buffer for import/export (device)
  double* d_stage = nullptr;
  size_t stage_bytes = 0;
  // CG device scalars
  CGScalars* d_cg = nullptr;   // nrhs
  CGScalars* h_cg = nullptr;   // pinned copy
  int* d_all_done = nullptr;
  std::vector<int> last_iters;
  std::vector<double> last_resid;

  // workspace fields keyed by (full|half, precision)
  std::vector<Field*> ws;
  cudaEvent_t events[16] = {};

  size_t n5() const { return size_t(half4) * L5; }
  size_t link_bytes_per_parity() const;
};

// Fields created on one operator may be used with another of the same geometry (4D
// extents, Ls, right-hand sides) on the same stream: the device layout is identical and
// the work of both is ordered on that one stream.
// A twisted-mass 5D operator keeps its slices in the slots where a Cayley operator keeps
// s, so its fields and those of a 5D grid with Ls = its slice count (one right-hand side)
// share one layout.
inline bool ops_conformable(const Op* a, const Op* b) {
  if (a == b) return true;
  if (!a || !b) return false;
  for (int k = 0; k < 4; k++)
    if (a->dims[k] != b->dims[k]) return false;
  if (a->stream != b->stream) return false;
  if (a->tm != b->tm) {
    const Op* t = a->tm ? a : b;
    const Op* o = a->tm ? b : a;
    return o->nrhs == 1 && o->L5 == t->L5;
  }
  return a->Ls == b->Ls && a->nrhs == b->nrhs && a->nrhs_user == b->nrhs_user;
}

struct Field {
  Op* op = nullptr;
  int subset = GB_EVEN;
  int prec = GB_F64;
  void* data = nullptr;   // plane 0 of the even (or only) half
  float* norms = nullptr; // FP16 per-site norms (even half first for full fields)
  bool owned = true;
  int ws_slot = -1;       // workspace slot of the owning operator (-1: a user field)
  size_t n5 = 0;          // 5D sites per checkerboard
  bool full() const { return subset == GB_FULL; }
  size_t half_bytes() const;   // bytes of one checkerboard's planes
  void* half_ptr(int parity) const;
  float* half_norms(int parity) const;
};

// bytes of one 16-byte vector plane set per 5D site
inline size_t spinor_bytes(int prec) { return prec == GB_F64 ? 192 : prec == GB_F32 ? 96 : 48; }

// ---- workspace ----
int ws_get(Op* op, int subset, int prec, int slot, Field** out);

// ---- kernel launchers (gb_dhop.cu, gb_5d.cu, gb_blas.cu) ----
struct HalfView {
  void* data;
  float* norms;
  int prec;
};
inline HalfView half_view(const Field* f, int parity) { return HalfView{f->half_ptr(parity), f->half_norms(parity), f->prec}; }

int launch_dhop(Op* op, HalfView in, HalfView out, int out_parity, int dag);
// FP32 / FP16: out = M5D(x5) - DhopEO/OE(in) in one launch (M5D with the given coefficients:
// Mooee for the end of Mpc), |out|^2 per CTA and right-hand side into op->d_partial
// ([CTA][nrhs], the norm partials' layout) and the CTA count into *parts.  Cases: one
// right-hand side, or several whose Dhop CTAs run 8-pair chunks of at most two right-hand
// sides each.  Otherwise it launches nothing and sets *parts = 0.
int launch_dhop_mooee(Op* op, HalfView in, HalfView x5, HalfView out, int out_parity, const double* lower,
                      const double* diag, const double* upper, int* parts);
// CTAs of one single-checkerboard launch of the FP32 / FP16 Dhop kernel
size_t dhop_pair_ctas(const Op* op);
int launch_dhop_full(Op* op, HalfView in_odd, HalfView out_even, HalfView in_even, HalfView out_odd, int dag);
// force term of the output parity's sites into mat (FP64 canonical gauge layout, indexed
// by x_cb when half_out, else by the lexicographic site); A has the output parity
int launch_deriv(Op* op, HalfView A, HalfView B, int out_parity, int dag, double* mat, int half_out);
// chi = diag*phi + upper*P(-/+) psi[s+1] + lower*P(+/-) psi[s-1]   (per rhs block of Ls)
int launch_m5d(Op* op, HalfView psi, HalfView phi, HalfView chi, const double* lower, const double* diag,
               const double* upper, int dag, size_t n5);
int launch_mooee_inv(Op* op, HalfView in, HalfView out, int dag, size_t n4);
// z = a*x + b*y (host scalars); x or y may alias z
int launch_axpby(Op* op, HalfView z, double a, HalfView x, double b, HalfView y, size_t n5);
int launch_scale(Op* op, HalfView z, double a, HalfView x, size_t n5);
int launch_copy(Op* op, HalfView dst, HalfView src, size_t n5);
int launch_zero(Op* op, HalfView z, size_t n5);
// reductions: per-rhs results into op->d_result; partial per half
int launch_norm2_partial(Op* op, HalfView x, size_t n5, double* partial);
int launch_inner_partial(Op* op, HalfView a, HalfView b, size_t n5, double* partial);
int launch_axpy_norm_partial(Op* op, HalfView z, double a, HalfView x, HalfView y, size_t n5, double* partial);
int launch_reduce_final(Op* op, const double* partial, int nparts, int nv, double* out);
int red_grid(Op* op, size_t n5, int* blocks, int* threads);
// pair-layout (FP32 / FP16) kernels, gb_pair.cu
int red_grid_pair(Op* op, size_t np, int* blocks, int* threads);
// norm_parts (non-null): with z and no dagger the kernel also writes per-CTA sums of
// |chi|^2 as stored into op->d_partial ([CTA][nrhs]) and their count into *norm_parts;
// otherwise *norm_parts = 0
int launch_m5d_pair(Op* op, HalfView psi, HalfView phi, HalfView chi, const double* lower, const double* diag,
                    const double* upper, int dag, size_t n5, const HalfView* z, double zc, int* norm_parts = nullptr);
// kind 0: |x|^2 ; 1: <x|y> ; 2: z = a x + y, |z|^2 ; 3: y -= a[rhs] x (the device CG
// scalars), |y|^2
int launch_reduce_pair(Op* op, int kind, HalfView x, HalfView y, HalfView z, double a, size_t n5, double* partial);
int launch_cg_p_pair(Op* op, HalfView p, HalfView r, size_t n5);
int launch_cg_xp_pair(Op* op, HalfView psi, HalfView p, HalfView r, size_t n5, int update_p);
int launch_axpby_pair(Op* op, HalfView z, double a, HalfView x, double b, HalfView y, size_t n5, int use_y);
// partial sums per checkerboard half that a reduction over a field of precision prec writes
inline int red_parts(Op* op, int prec) {
  int g = 1, B = 256;
  if (prec == GB_F64) red_grid(op, op->n5(), &g, &B);
  else red_grid_pair(op, op->n5() >> 1, &g, &B);
  return g;
}

// fused s-column programs of the Cayley 5D operators (gb_col.cu, FP32 Moebius):
// out = A(x) + zc * B(y), one dagger flag for the program
enum { COL_M5D = 0, COL_INV = 1, COL_INV_M5D = 2, COL_M5D_INV = 3 };  // A: M5D, INV, M5D(INV x), INV(M5D x)
enum { COLB_NONE = 0, COLB_IDENT = 1, COLB_M5D = 2 };                 // B: -, y, M5D(y)
struct ColCoefsHost {
  std::vector<double> l1, d1, u1;  // M5D of A (lower, diagonal, upper per s)
  std::vector<double> l2, d2, u2;  // M5D of B
};
bool col_available(const Op* op, int prec);
// complex-coefficient 5D programs of ZMobius operators (gb_zmobius.cu); coefficients as
// the operator applies them (conjugated / swapped for the dagger forms by the host)
struct ZCoefsHost {
  std::vector<std::complex<double>> d, u, l;                    // M5D
  std::vector<std::complex<double>> lee, leem, uee, ueem, dinv;  // MooeeInv
  std::vector<std::complex<double>> e;                          // DIAG: out = x + e y
};
enum { ZPROG_M5D = 0, ZPROG_INV = 2, ZPROG_DIAG = 3 };
bool zmobius_ls_supported(int Ls);
int launch_zcol(Op* op, int prog, int dag, HalfView x, const HalfView* y, HalfView out, double zc, const ZCoefsHost& h);
// With r_upd (FP32 or FP16, nrhs dividing 16, the program MooeeDag - M5Ddag z that ends MpcDag)
// the kernel does not store out: it applies the CG's residual update r -= a out (a per
// right-hand side from op->d_cg) and writes per-CTA sums of |r|^2 [CTA][nrhs] into
// op->d_partial, their count into *r_parts (0 when it could not fuse; out is then stored
// and the caller updates r).
int launch_col(Op* op, int opa, int opb, int dag, HalfView x, HalfView y, HalfView out, double zc,
               const ColCoefsHost& h, HalfView* r_upd = nullptr, int* r_parts = nullptr);

// layout conversion between canonical FP64 (device) and the device layout
// canonical host layout (complex double or, with canon_prec = GB_F32, complex float) <->
// device layout of one checkerboard half
int launch_import_half(Op* op, const void* canon, int canon_prec, HalfView out, int parity, int canon_is_full);
int launch_export_half(Op* op, HalfView in, void* canon, int canon_prec, int parity, int canon_is_full);
int launch_double_store(Op* op, const double* U_canon, int parity);
// 4D <-> 5D surface fields (Moebius): canonical FP64 4D field in device memory
int launch_surface_insert(Op* op, const double* c4, HalfView even, HalfView odd);
int launch_surface_extract(Op* op, HalfView even, HalfView odd, double* c4, int solution);
// 4D slice s of a full 5D field <-> canonical 4D field (device)
int launch_slice(Op* op, double* c4, HalfView even, HalfView odd, int s, int insert);
// CayleyFermion5D::P (dag = 0) / Pdag (dag = 1) on one checkerboard half
int launch_chiral_shift(Op* op, HalfView in, HalfView out, int dag);
// out = d(slot, chirality) x [+ zc z] with per-slot complex d for spins 0,1 and 2,3
int launch_chiral_scale(Op* op, HalfView x, const HalfView* z, double zc, HalfView out, const double* up_re,
                        const double* up_im, const double* dn_re, const double* dn_im);
// out_{r,k} = sum_s mat[k][s] in_{r,s} (complex Ls x Ls, row major) along each rhs block
int launch_dft_s(Op* op, HalfView in, HalfView out, const double* mat_host);
// slot t of dst (L5d slots) = slot s of src (L5s slots), one checkerboard half
int launch_copy_slot(Op* op, HalfView src, int L5s, int s, HalfView dst, int L5d, int t);
int build_neighbours(Op* op);

// CG kernels (gb_blas.cu)
// init from device arrays ssq[nrhs] and cp[nrhs]
int launch_cg_init(Op* op, const double* d_ssq, const double* d_cp, double tol, double delta);
// a = c / d per rhs, d from partial sums [nparts][nrhs][nv] (nv = 2: inner-product
// partials, real part first; nv = 1: norm partials)
int launch_cg_alpha(Op* op, const double* partial, int nparts, int nv);
// r -= a mmp ; partial |r|^2
int launch_cg_r_update(Op* op, HalfView r, HalfView mmp, size_t n5, double* partial);
// psi += a p ; with update_p also p = b p + r
int launch_cg_xp_update(Op* op, HalfView psi, HalfView p, HalfView r, size_t n5, int update_p);
int launch_cg_beta(Op* op, const double* partial_norm, int nparts);
// p = b p + r
int launch_cg_p_update(Op* op, HalfView p, HalfView r, size_t n5);
// after a reliable update: cp = c = maxres = cp_true ; b = cp_true / cprev
int launch_cg_relup_reset(Op* op, const double* d_cp_true);
// the device-resident CG loop's condition: arm before a graph launch (at most max_chunks
// chunks), check after every chunk inside the WHILE body (gb_blas.cu)
int launch_cg_loop_arm(Op* op, int max_chunks);
int launch_cg_loop_check(Op* op, cudaGraphConditionalHandle h);

}  // namespace gb

struct gb_op_s : gb::Op {};
struct gb_field_s : gb::Field {};
