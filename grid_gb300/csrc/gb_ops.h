// gb_ops.h -- host-side operator sequences and field helpers shared between the C-ABI
// translation units.
#pragma once

#include "gb_internal.h"

namespace gb {

// workspace slots (per (full|half, precision)); every nested use has its own slot
enum {
  WS_MPC_E1 = 0, WS_MPC_E2 = 1, WS_MPC_O = 2, WS_MPCDAGMPC = 3, WS_MEOOE_A = 4, WS_MEOOE_B = 5,
  WS_CG_P = 8, WS_CG_MMP = 9, WS_CG_R = 10, WS_CG_T = 11,
  WS_RU_PF = 12, WS_RU_MMPF = 13, WS_RU_RF = 14, WS_RU_XF = 15,
  WS_SCHUR_A = 16, WS_SCHUR_B = 17, WS_SCHUR_C = 18, WS_SCHUR_D = 19,
  WS_MS_P = 20, WS_MS_MMP = 21, WS_MS_R = 22, WS_MS_T = 23, WS_MS_PS = 24,  // WS_MS_PS + shift, < 24 + 32
  WS_DERIV = 56,
};
enum { WS_M_DIN = 0, WS_M_T = 1, WS_MDAGM = 2, WS_FCG_P = 3, WS_FCG_MMP = 4, WS_FCG_R = 5, WS_FCG_T = 6,
       WS_FRU_PF = 7, WS_FRU_MMPF = 8, WS_FRU_RF = 9, WS_FRU_XF = 10, WS_SCHUR_RES = 11, WS_DMINUS = 12,
       WS_PHYS = 13, WS_MS_P_FULL = 14, WS_MS_MMP_FULL = 15, WS_MS_R_FULL = 16, WS_MS_T_FULL = 17,
       WS_MS_PS_FULL = 18,  // WS_MS_PS_FULL + shift, < 18 + 32
       WS_DERIV_FULL = 50 };

int field_alloc(Op* op, int subset, int prec, Field** out);
void field_free(Field* f);
int field_norm2_dev(Field* f, double* d_out);
int field_inner_dev(Field* a, Field* b, double* d_out);
int field_norm2(Field* f, double* out);
int field_inner(Field* a, Field* b, double* out);
int field_axpby(Field* z, double a, double b, Field* x, Field* y);
int field_scale(Field* z, double a, Field* x);
int field_copy(Field* dst, Field* src);
int field_zero(Field* z);
size_t field_host_doubles(const Field* f);
// WilsonLoops::avgPlaquette / linkTrace of a canonical FP64 gauge field in device memory
int gauge_stats_device(const int dims[4], const double* Ud, cudaStream_t s, double* plaq, double* trace);
int field_import_dev(Field* f, const void* dev, int canon_prec);
int field_export_dev(Field* f, void* dev, int canon_prec);
int ensure_stage(Op* op, size_t bytes);
int check_device_error(Op* op);

int launch_m5d_z(Op* op, HalfView psi, HalfView phi, HalfView chi, const double* lower, const double* diag,
                 const double* upper, int dag, size_t n5, const HalfView* z, double zc, int* norm_parts = nullptr);

int op_meooe5d(Op* op, Field* in, Field* out, int dag);
int op_dhop_cb(Op* op, Field* in, Field* out, int dag);
int op_dhop_full(Op* op, Field* in, Field* out, int dag);
int op_meooe(Op* op, Field* in, Field* out, int dag);
int op_mooee(Op* op, Field* in, Field* out, int dag, Field* z, double zc, int* norm_parts = nullptr);
int op_mooee_inv(Op* op, Field* in, Field* out, int dag);
// norm_parts (Mpc only): when non-null, the last kernel may also reduce |out|^2 into
// op->d_partial ([CTA][nrhs], the layout of the norm partials) and sets *norm_parts to the
// number of CTA sums written, or to 0 when it did not.
// r_upd, r_parts (MpcDag only, for the CG): when both are non-null, the last kernel may
// instead of storing out apply r_upd -= a out (a: the CG scalars of op) and reduce
// |r_upd|^2 into op->d_partial ([CTA][nrhs]); *r_parts is the number of CTA sums written, or
// 0 when it stored out and left r_upd alone
int op_mpc(Op* op, Field* in, Field* out, int dag, int* norm_parts = nullptr, Field* r_upd = nullptr,
           int* r_parts = nullptr);
int op_mpcdagmpc(Op* op, Field* in, Field* out);
int op_m(Op* op, Field* in, Field* out, int dag);
// m_in: the workspace field that holds M in afterwards
int op_mdagm(Op* op, Field* in, Field* out, Field** m_in = nullptr);
int op_dminus(Op* op, Field* in, Field* out, int dag);
// flops of one application of MdagM (kind 0) or MpcDagMpc (kind 1) in Grid's model
double hermop_flops(const Op* op, int kind);

// kind 0: MdagM on full fields; kind 1: MpcDagMpc on odd half fields
inline int op_hermop(Op* op, int kind, Field* in, Field* out) {
  return kind == 0 ? op_mdagm(op, in, out) : op_mpcdagmpc(op, in, out);
}


}  // namespace gb
