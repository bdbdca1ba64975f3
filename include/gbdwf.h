/* gbdwf.h -- C ABI of the GB300-native Wilson / Moebius domain-wall fermion library.
 *
 * The library replaces the device hot path of Grid's fermion operators and their
 * conjugate-gradient drivers.  Every entry point returns an int status (GB_OK on
 * success) and never aborts; gb_last_error() returns a thread-local message for the
 * last failure.  Handles are opaque.  No entry point takes a C++ or torch type.
 *
 * Host layout at the boundary ("canonical"), complex<double> interleaved (re, im):
 *   4D site index  site = x + Lx*(y + Ly*(z + Lz*t))
 *   gauge field    U[site][mu][a][b], mu = x,y,z,t             (Grid LatticeGaugeField)
 *   fermion        psi[site][s][spin][colour], s innermost      (Grid sF = s + Ls*sU)
 *   half field     psi[site>>1][s][spin][colour] over the sites of one parity
 *   parity         (x+y+z+t) & 1, Even = 0; s takes no part     (WilsonFermion5D.h:37-61)
 * A multi-RHS operator (nrhs > 1) takes nrhs such fields back to back.
 *
 * Device layout is private to the library: structure-of-arrays, 5D site fastest, in
 * 16-byte vectors.
 */
#ifndef GBDWF_H
#define GBDWF_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
/* the library is built with hidden visibility: only these declarations are exported */
#pragma GCC visibility push(default)
#endif
#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (the error convention of Grid's asserts, as return values) ---- */
enum {
  GB_OK = 0,
  GB_ERR_BAD_ARG = 1,       /* conformable()/argument checks                         */
  GB_ERR_BAD_PARITY = 2,    /* checkerboard mismatch (WilsonFermion5DImplementation.h:426-435) */
  GB_ERR_OOM = 3,           /* device allocation failed or HBM budget exceeded       */
  GB_ERR_CUDA = 4,          /* a CUDA runtime error                                  */
  GB_ERR_NOT_CONVERGED = 5, /* CG hit MaxIterations (ConjugateGradient.h:254)        */
  GB_ERR_TIMEOUT = 6,       /* a bounded device wait gave up                         */
  GB_ERR_NO_DEVICE = 7,     /* no CUDA device visible                                */
  GB_ERR_UNSUPPORTED = 8,
  GB_ERR_IO = 9,            /* file I/O, format, or a checksum / plaquette mismatch (NerscIO.h asserts) */
  GB_ERR_CANCELLED = 10     /* a queued service request shed by gb_server_cancel_queued  */
};

/* ---- precisions and subsets ---- */
enum { GB_F64 = 0, GB_F32 = 1, GB_F16 = 2 };
enum { GB_EVEN = 0, GB_ODD = 1, GB_FULL = 2 };
enum { GB_DAG_NO = 0, GB_DAG_YES = 1 };

typedef struct gb_op_s* gb_op_t;       /* a fermion operator on one gauge field       */
typedef struct gb_field_s* gb_field_t; /* a device fermion field conformable to an op */

/* ---- library ---- */
int gb_version(void);
const char* gb_last_error(void);
const char* gb_status_string(int status);
int gb_device_count(int* n);

/* ---- operators ----------------------------------------------------------------
 * gb_wilson_create   ~ WilsonFermion(U, Fgrid, Hgrid, mass, ImplParams)
 *                      (Grid/qcd/action/fermion/WilsonFermion.h:139-142)
 * gb_mobius_create   ~ MobiusFermion(U, FGrid, FrbGrid, UGrid, UrbGrid, mf, M5, b, c, ImplParams)
 *                      (Grid/qcd/action/fermion/MobiusFermion.h:45-67)
 * dims: Lx, Ly, Lz, Lt (all even).  phases: 4 complex boundary phases (re, im),
 * ImplParams::boundary_phases (Grid/qcd/action/ActionParams.h:49-66); NULL = periodic.
 * precision: GB_F64 or GB_F32 (or GB_F16: FP16 spinors with per-site FP32 norms,
 * FP32 links and arithmetic).  nrhs >= 1 right-hand sides share the gauge field.
 * stream: a cudaStream_t (NULL = the default stream).
 * flags: GB_FLAG_RECON12 = store the doubled links as 12 reals (rows 0, 1) and rebuild
 * row 2 in the Dhop kernel (the optional 12-real reconstruction); needs real boundary
 * phases (+1 / -1), else GB_ERR_UNSUPPORTED.
 * GB_FLAG_DF64 (GB_F64 operators with 18-real links, else GB_ERR_UNSUPPORTED): the hopping
 * term computes in double-float arithmetic (pairs of floats, about 48 significant bits:
 * relative L2 error near 5e-15 per application) on the FP32 pipes instead of the FP64
 * pipe, which on GB300 runs at 1/64 of the FP32 rate; fields stay FP64.  Every other
 * FP64 kernel is unchanged.
 */
#define GB_FLAG_RECON12 1u
#define GB_FLAG_DF64 2u
int gb_wilson_create(const int dims[4], double mass, const double* phases, int precision, int nrhs, void* stream,
                     unsigned flags, gb_op_t* out);
int gb_mobius_create(const int dims[4], int Ls, double mf, double M5, double b, double c, const double* phases,
                     int precision, int nrhs, void* stream, unsigned flags, gb_op_t* out);
/* Approx::zolotarev(epsilon, n, type) (Grid/algorithms/approx/Zolotarev.cc:296-417): the
 * Cayley-form zeros gamma[0..n-1] of Zolotarev's optimal approximation to sgn(x) on
 * epsilon <= |x| <= 1 (type 0: R(0) = 0, type 1: R(0) = infinity) and its maximum error
 * (delta may be NULL).  MobiusZolotarevFermion(mf, M5, b, c, lo, hi) is the Cayley operator
 * with omega_s = hi * gamma_s of zolotarev(lo / hi, Ls, 0) (MobiusZolotarevFermion.h:45-70,
 * CayleyFermion5DImplementation.h:411-445): gb_zmobius_create with that omega. */
int gb_zolotarev(double epsilon, int n, int type, double* gamma, double* delta);
/* Approx::computeZmobiusGamma(gamma, bpc_out, Ls_out, bpc_in, Ls_in, lambda)
 * (Grid/algorithms/approx/ZMobius.cc:73-183): the Ls_out (even, <= 32) complex gamma_s of
 * the ZMobius operator whose sign function best approximates, on 0 <= x <= lambda, that
 * of the Moebius operator with Ls_in slices and b + c = bpc_in; gamma_s = bpc_out omega_s.
 * gamma: 2 Ls_out doubles (re, im); max_error (may be NULL): the minimax error. */
int gb_zmobius_gamma(int Ls_out, double bpc_out, int Ls_in, double bpc_in, double lambda_bound, double* gamma,
                     double* max_error);

/* ZMobiusFermion(U, FGrid, FrbGrid, UGrid, UrbGrid, mf, M5, gamma, b, c, ImplParams)
 * (Grid/qcd/action/fermion/ZMobiusFermion.h): complex omega_s = gamma[s] (Ls complex
 * numbers as re, im), hence complex Cayley coefficients.  FP64 or FP32; Ls even, 2..16,
 * 20, 24 or 32. */
int gb_zmobius_create(const int dims[4], int Ls, double mf, double M5, const double* gamma, double b, double c,
                      const double* phases, int precision, int nrhs, void* stream, unsigned flags, gb_op_t* out);
int gb_op_destroy(gb_op_t op);
/* ImportGauge (WilsonFermion5DImplementation.h:149-180): canonical FP64 host field. */
int gb_op_import_gauge(gb_op_t op, const double* U_host);
/* the same from a canonical FP64 field already in device memory */
int gb_op_import_gauge_device(gb_op_t op, const double* U_device);
/* geometry queries: Ls (1 for Wilson), nrhs, sites in one checkerboard (4D), precision */
int gb_op_info(gb_op_t op, int* Ls, int* nrhs, int64_t* half_sites4, int* precision);
int gb_op_set_stream(gb_op_t op, void* stream);
/* Cayley coefficients as the operator holds them: 9*Ls doubles
 * bs, cs, bee, cee, dee, lee, leem, uee, ueem (CayleyFermion5DImplementation.h:410-535) */
int gb_op_cayley_coeffs(gb_op_t op, double* out);

/* ---- fields ---------------------------------------------------------------------
 * Lattice<vobj>(grid) on the op's FermionGrid (GB_FULL) or FermionRedBlackGrid
 * (GB_EVEN / GB_ODD).  precision may differ from the op's (for precisionChange).
 * A field may be used with any operator of the same geometry (4D extents, Ls, nrhs) on
 * the same stream as the one that created it (Grid: fields belong to a grid, not to an
 * operator); the operator that created it must outlive it.
 */
int gb_field_create(gb_op_t op, int subset, int precision, gb_field_t* out);
int gb_field_destroy(gb_field_t f);
int gb_field_subset(gb_field_t f, int* subset);
int gb_field_set_subset(gb_field_t f, int subset); /* relabel a half field's checkerboard */
/* number of doubles in the canonical host form (all nrhs right-hand sides) */
int gb_field_host_len(gb_field_t f, size_t* n_doubles);
int gb_field_import(gb_field_t f, const double* host);
int gb_field_export(gb_field_t f, double* host);
int gb_field_import_device(gb_field_t f, const double* dev); /* canonical FP64 in device memory */
int gb_field_export_device(gb_field_t f, double* dev);
/* the canonical host form in single precision: complex<float> in the same order (Grid's
 * LatticeFermionF host data); n_doubles of gb_field_host_len floats */
int gb_field_import_f32(gb_field_t f, const float* host);
int gb_field_export_f32(gb_field_t f, float* host);

/* Transfer queue of an operator: host fields in and out without blocking the caller.
 * Each import is a host->device copy on the queue's own copy stream into one of two
 * staging buffers, then the layout kernel on the operator's stream, so operator calls
 * issued after gb_xfer_import see the field; each export is the layout kernel on the
 * operator's stream (after every call issued before it), then a device->host copy on a
 * second copy stream.  The copy of the next input and of the last result therefore
 * overlap each other and the operator's kernels.  Host buffers: canonical form in FP64
 * (host_prec GB_F64) or FP32 (GB_F32), page-locked for the copies to overlap, left
 * untouched (imports) or unread (exports) by the caller until gb_xfer_wait returns. */
typedef struct gb_xfer_s* gb_xfer_t;
int gb_xfer_create(gb_op_t op, gb_xfer_t* out);
int gb_xfer_destroy(gb_xfer_t x);
int gb_xfer_import(gb_xfer_t x, gb_field_t f, const void* host, int host_prec);
int gb_xfer_export(gb_xfer_t x, gb_field_t f, void* host, int host_prec);
int gb_xfer_wait(gb_xfer_t x); /* every queued import and export has completed */

/* ---- field linear algebra (Grid/lattice/Lattice_arith.h, Lattice_reduction.h) ----
 * Reductions return one value per right-hand side (arrays of length nrhs), in FP64.
 */
int gb_field_zero(gb_field_t f);
int gb_field_copy(gb_field_t dst, gb_field_t src);          /* also precisionChange */
int gb_field_norm2(gb_field_t f, double* out);              /* norm2               */
int gb_field_inner(gb_field_t a, gb_field_t b, double* out); /* innerProduct <a|b>: re,im per rhs */
int gb_field_axpy(gb_field_t z, double a, gb_field_t x, gb_field_t y);               /* z = a x + y   */
int gb_field_axpby(gb_field_t z, double a, double b, gb_field_t x, gb_field_t y);    /* z = a x + b y */
int gb_field_axpy_norm(gb_field_t z, double a, gb_field_t x, gb_field_t y, double* norm_out);
int gb_field_axpby_norm(gb_field_t z, double a, double b, gb_field_t x, gb_field_t y, double* norm_out);
/* innerProductNorm: <a|b> (re, im per rhs) and |a|^2 per rhs */
int gb_field_inner_norm(gb_field_t a, gb_field_t b, double* inner_out, double* norm_out);
int gb_field_pick_checkerboard(gb_field_t half, gb_field_t full); /* half's subset picks */
int gb_field_set_checkerboard(gb_field_t full, gb_field_t half);

/* gb_field_norm2_noalloc: the same per-rhs norm2 as gb_field_norm2, but it allocates
 * nothing.  It has no counterpart in the reference.  It is for callers that may not call
 * cudaMalloc/cudaFree while they work: a solve loop running under a fixed HBM budget
 * (its memory was reserved when the request was admitted and must not grow), or a thread
 * in a context where allocator calls are forbidden or would stall the device.  The
 * reduction's partial sums go to one static device array of 64.1 KB that every GPU which
 * loads the library keeps until the process exits.  Limit: at most 16 right-hand sides
 * per field, and Ls x right-hand sides at most 256 when there are several (larger fields
 * are rejected with GB_ERR_UNSUPPORTED); any lattice size.
 * The first call on a device looks up that array's device address (a one-time set-up
 * per device); make that first call before any stream capture.  All calls share the
 * array: calls whose work overlaps on the GPU (other streams or threads) race and must
 * be serialised by the caller.  `out` (nrhs doubles) may be host or device memory; the
 * call returns when it is written. */
int gb_field_norm2_noalloc(gb_field_t f, double* out);

/* ---- operator application (FermionOperator.h:40-192 / CayleyFermion5D) ----------
 * Full-field ops: M, Mdag, MdagM, Dhop.  Half-field ops pick DhopEO/DhopOE from the
 * input subset exactly as Grid does (Meooe: Odd in -> Even out).
 */
int gb_M(gb_op_t op, gb_field_t in, gb_field_t out);
int gb_Mdag(gb_op_t op, gb_field_t in, gb_field_t out);
int gb_MdagM(gb_op_t op, gb_field_t in, gb_field_t out);
int gb_Dhop(gb_op_t op, gb_field_t in, gb_field_t out, int dag);
int gb_DhopEO(gb_op_t op, gb_field_t in_odd, gb_field_t out_even, int dag);
int gb_DhopOE(gb_op_t op, gb_field_t in_even, gb_field_t out_odd, int dag);
int gb_Meooe(gb_op_t op, gb_field_t in, gb_field_t out);
int gb_MeooeDag(gb_op_t op, gb_field_t in, gb_field_t out);
int gb_Mooee(gb_op_t op, gb_field_t in, gb_field_t out);
int gb_MooeeDag(gb_op_t op, gb_field_t in, gb_field_t out);
int gb_MooeeInv(gb_op_t op, gb_field_t in, gb_field_t out);
int gb_MooeeInvDag(gb_op_t op, gb_field_t in, gb_field_t out);
/* SchurDiagMooeeOperator (Grid/algorithms/LinearOperator.h:325-349), odd checkerboard */
int gb_Mpc(gb_op_t op, gb_field_t in, gb_field_t out);
int gb_MpcDag(gb_op_t op, gb_field_t in, gb_field_t out);
int gb_MpcDagMpc(gb_op_t op, gb_field_t in, gb_field_t out);
/* CayleyFermion5D::Dminus / DminusDag (CayleyFermion5DImplementation.h:131-153), full
 * fields: chi = psi - c (DW psi), DW = Dhop + (4 - M5).  Moebius operators only. */
int gb_Dminus(gb_op_t op, gb_field_t in, gb_field_t out, int dag);

/* ---- force terms ---------------------------------------------------------------------
 * gb_DhopDeriv ~ WilsonFermion5D::DhopDeriv / DhopDerivEO / DhopDerivOE
 * (WilsonFermion5DImplementation.h:212-305) with WilsonImpl::InsertForce5D (WilsonImpl.h:193-238):
 *   mat[x][mu]_ab = sum_s sum_spin [(1 -+ gamma_mu) U~_mu(x) B(x+mu, s)]_{spin,a} conj(A(x,s)_{spin,b})
 * (minus sign: dag = 0), summed over all L5 slots (every right-hand side), U~ the doubled
 * link with -1/2 and the boundary phase.  A, B full fields (mat: full canonical gauge
 * layout [site][mu][3][3]) or half fields on opposite checkerboards (DerivEO: A even,
 * B odd; DerivOE: A odd, B even; mat indexed by site>>1 over A's checkerboard), FP64 out.
 * gb_MDeriv ~ CayleyFermion5D::MDeriv / MoeDeriv / MeoDeriv (CayleyFermion5DImplementation.h:346-391):
 * DhopDeriv(U, Meooe5D V) (dag = 0) or DhopDeriv(Meooe5D U, V) (dag = 1); for a Wilson
 * operator MDeriv = DhopDeriv.  FP64 or FP32 operators.  mat: host (on_device = 0) or device. */
int gb_DhopDeriv(gb_op_t op, gb_field_t A, gb_field_t B, int dag, double* mat, int on_device);
int gb_MDeriv(gb_op_t op, gb_field_t U, gb_field_t V, int dag, double* mat, int on_device);

/* ---- 4D <-> 5D surface fields (CayleyFermion5DImplementation.h:57-129) ------------
 * The 4D side is a canonical FP64 4D fermion (nrhs fields back to back), in host memory
 * (on_device = 0; the call returns when it is done) or device memory (on_device = 1; the
 * work is queued on the operator's stream).  The 5D side is a full field.  Moebius only.
 *   import_physical_source    ImportPhysicalFermionSource: P+ src at s=0, P- src at
 *                             s=Ls-1, then Dminus (P+- = (1 +- gamma5)/2)
 *   import_unphysical_fermion ImportUnphysicalFermion: the same without Dminus
 *   export_physical_solution  ExportPhysicalFermionSolution: P- psi(0) + P+ psi(Ls-1)
 *   export_physical_source    ExportPhysicalFermionSource:   P+ psi(0) + P- psi(Ls-1)  */
int gb_import_physical_source(gb_op_t op, const double* src4d, int on_device, gb_field_t out5d);
int gb_import_unphysical_fermion(gb_op_t op, const double* src4d, int on_device, gb_field_t out5d);
int gb_export_physical_solution(gb_op_t op, gb_field_t sol5d, double* out4d, int on_device);
int gb_export_physical_source(gb_op_t op, gb_field_t src5d, double* out4d, int on_device);

/* InsertSlice(lowDim, higherDim, s, 0) / ExtractSlice(lowDim, higherDim, s, 0)
 * (Grid/lattice/Lattice_transfer.h:999-1070) along the fifth dimension: the whole 4D
 * spinor field at slice s (0 <= s < Ls) of a full 5D field; 4D layout as for the surface
 * functions above.  Insert leaves every other slice untouched. */
int gb_insert_slice(gb_op_t op, const double* src4d, int on_device, gb_field_t f5d, int s);
int gb_extract_slice(gb_op_t op, gb_field_t f5d, int s, double* out4d, int on_device);

/* CayleyFermion5D::P / Pdag (CayleyFermion5DImplementation.h:70-88), the chiral
 * permutation of the MADWF method: chi_s = P- psi_s + P+ psi_{s+1} (dag = 0) or
 * P+ psi_{s-1} (dag = 1), s cyclic.  Full or half fields; in and out distinct. */
int gb_P(gb_op_t op, gb_field_t in, gb_field_t out, int dag);

/* WilsonTMFermion5D(U, FGrid, FrbGrid, UGrid, UrbGrid, mass, mu) (WilsonTMFermion5D.h:40-145):
 * nslices (even, <= 64) independent slices of the 4D Wilson hop with Mooee = (4 + m_s) +
 * i mu_s gamma5 per slice; the slices are the operator's right-hand-side slots, so its
 * fields are nslices-right-hand-side 4D Wilson fields and its CG converges each slice to
 * the tolerance.  FP64 or FP32.  gb_op_tm_update: TM update(mass, mu). */
int gb_wilson_tm5d_create(const int dims[4], int nslices, const double* mass, const double* mu, const double* phases,
                          int precision, void* stream, unsigned flags, gb_op_t* out);
int gb_op_tm_update(gb_op_t op, const double* mass, const double* mu);

/* Fifth-dimension transforms (FourierAcceleratedPV.h:56-237).  gb_field_dft_s: out_k =
 * sum_s mat[k][s] in_s on each rhs block of Ls slots, mat Ls x Ls complex row major (re,
 * im).  gb_field_copy_slice5: slot t of dst = slot s of src, fields of any Ls on the same
 * 4D geometry and stream.  gb_field_chiral_scale: out = c gamma-chirally per slot,
 * coef[4 q .. 4 q + 3] = (re, im) for spins 0,1 and (re, im) for spins 2,3 of slot q. */
int gb_field_dft_s(gb_field_t in, gb_field_t out, const double* mat);
int gb_field_copy_slice5(gb_field_t dst, int t, gb_field_t src, int s);
int gb_field_chiral_scale(gb_field_t in, gb_field_t out, const double* coef);

/* CayleyFermion5D::SetMass / Mass (CayleyFermion5D.h:71-83); WilsonFermion's mass for
 * Wilson operators.  The Cayley coefficients are rebuilt at once; later calls use them. */
int gb_op_set_mass(gb_op_t op, double mass);
int gb_op_mass(gb_op_t op, double* mass);

/* ---- solvers ------------------------------------------------------------------- */
typedef struct {
  double tolerance;      /* ConjugateGradient::Tolerance                                  */
  int max_iterations;    /* ConjugateGradient::MaxIterations                              */
  int err_on_no_conv;    /* ErrorOnNoConverge: return GB_ERR_NOT_CONVERGED (never aborts)  */
  double delta;          /* reliable update when |r|^2 < delta * max|r|^2 since the last  */
  int relup_every;       /* ... or at least every relup_every inner iterations (0 = off)  */
  int final_cleanup;     /* ConjugateGradientReliableUpdate::DoFinalCleanup               */
  int check_every;       /* host convergence poll interval in iterations (0 = default)    */
  int use_graphs;        /* 1: capture the iteration chunk in a CUDA graph; 2: the CG loop
                            itself on the device -- one graph whose conditional WHILE node
                            repeats the captured chunk until every right-hand side has
                            converged, a reliable update is due or the iteration cap is
                            reached, so the host steps in only at those points            */
} gb_cg_params;

typedef struct {
  int iterations;         /* IterationsToComplete (max over right-hand sides)            */
  int reliable_updates;   /* ReliableUpdatesPerformed                                    */
  int cleanup_iterations; /* IterationsToCleanup                                         */
  int converged;          /* 1 when every right-hand side converged                      */
  double true_residual;   /* TrueResidual (max over right-hand sides)                    */
  double seconds;         /* wall time of the solve                                      */
  double flops;           /* Grid's flop model for the solve                             */
} gb_cg_result;

void gb_cg_params_default(gb_cg_params* p);

/* MixedPrecisionConjugateGradient (ConjugateGradientMixedPrec.h:34-166): defect correction
 * with restarted FP32 inner CGs.  Outer loop: r = src - A psi in FP64; stop when |r|^2 <
 * outer_loop_norm_mult * tol^2 |src|^2; double the inner tolerance while |r|^2 t^2 <
 * tol^2 |src|^2; solve A e = r in FP32 from zero to t within max_inner_iterations; psi +=
 * e.  Then the final FP64 "patch-up" CG from psi to tol.  With nrhs > 1 operators this is
 * MixedPrecisionConjugateGradientBatched (ConjugateGradientMixedPrecBatched.h:37-209),
 * every right-hand side in one inner multi-RHS CG.  gb_cg_result: iterations =
 * TotalInnerIterations, reliable_updates = TotalOuterIterations, cleanup_iterations =
 * TotalFinalStepIterations, true_residual = TrueResidual.  p: tolerance, err_on_no_conv,
 * check_every, use_graphs (max_iterations is unused). */
typedef struct {
  double inner_tolerance;      /* InnerTolerance (0: the outer tolerance)             */
  int max_inner_iterations;    /* MaxInnerIterations                                  */
  int max_outer_iterations;    /* MaxOuterIterations                                  */
  int max_patchup_iterations;  /* MaxPatchupIterations (0: MaxInnerIterations)        */
  double outer_loop_norm_mult; /* OuterLoopNormMult (Grid: 100)                        */
} gb_mixed_params;
void gb_mixed_params_default(gb_mixed_params* m);
int gb_cg_mixed(gb_op_t op_d, gb_op_t op_f, int kind, gb_field_t src, gb_field_t psi, const gb_cg_params* p,
                const gb_mixed_params* m, gb_cg_result* res);

/* ConjugateGradient<Field>(MdagMLinearOperator) on a full field (Test_wilson_cg_unprec.cc) */
int gb_cg_mdagm(gb_op_t op, gb_field_t src, gb_field_t psi, const gb_cg_params* p, gb_cg_result* res);
/* ConjugateGradient<Field>(SchurDiagMooeeOperator) on an odd half field */
int gb_cg_schur(gb_op_t op, gb_field_t src_o, gb_field_t psi_o, const gb_cg_params* p, gb_cg_result* res);
/* per right-hand-side results of the last solve on this op: iterations and true residuals */
int gb_cg_last_per_rhs(gb_op_t op, int* iterations, double* true_residual);
/* ConjugateGradientReliableUpdate<FieldD,FieldF>: op_d FP64, op_lo FP32 or FP16 on the
 * same gauge field; kind 0 = MdagM (full fields), 1 = Schur (odd half fields). */
int gb_cg_reliable(gb_op_t op_d, gb_op_t op_lo, int kind, gb_field_t src, gb_field_t psi, const gb_cg_params* p,
                   gb_cg_result* res);
/* ConjugateGradientMultiShift (Grid/algorithms/iterative/ConjugateGradientMultiShift.h:76-330):
 * solves (A + shifts[s]) psi[s] = src for nshift <= GB_MAX_SHIFTS shifts at once, A = MdagM
 * (kind 0, full fields) or MpcDagMpc (kind 1, odd fields); shifts[0] must be the lightest
 * (MultiShiftFunction::poles), tolerances[s] is shift s's target |r_s|/|src|.  FP64 or
 * FP32 operators, one right-hand side.  psi[s] are outputs (no initial guess, as in Grid).
 * The rational sum psi = norm src + sum_s residues[s] psi[s] is left to the caller
 * (gb_field_axpby). */
#define GB_MAX_SHIFTS 32
typedef struct {
  int nshift;
  int iterations;                              /* IterationsToComplete                  */
  int converged;                               /* 1 when every shift converged          */
  int iterations_shift[GB_MAX_SHIFTS];         /* IterationsToCompleteShift             */
  double true_residual_shift[GB_MAX_SHIFTS];   /* TrueResidualShift                     */
  double seconds;
  double flops;                                /* Grid's flop model of the A applications */
} gb_multishift_result;
int gb_cg_multishift(gb_op_t op, int kind, gb_field_t src, int nshift, const double* shifts, const double* tolerances,
                     gb_field_t* psi, int max_iterations, int check_every, gb_multishift_result* res);

/* SchurRedBlackDiagMooeeSolve(CG)(M, src, sol) (SchurRedBlack.h:236-291,373-436).
 * op_lo == NULL: plain CG in op's precision; else mixed precision (reliable update).
 * unprec_resid (may be NULL): |M sol - src| / |src| per right-hand side of op (an array
 * of gb_op_info's nrhs doubles; the slices of a twisted-mass operator count as such). */
int gb_schur_solve(gb_op_t op, gb_op_t op_lo, gb_field_t src, gb_field_t sol, const gb_cg_params* p,
                   gb_cg_result* res, double* unprec_resid);

/* ---- MADWF and its Pauli-Villars inverters ------------------------------------------
 * A solver: solve op sol = src for full 5D fields of op; sol's contents on entry are the
 * initial guess where the solver takes one.  Returns a status; GB_OK to go on.  The
 * Grid template parameters PVinverter and SchurSolver of MADWF become a function and its
 * user pointer, so a caller may pass its own solver or one of those below. */
typedef int (*gb_solver_fn)(void* user, gb_op_t op, gb_field_t src, gb_field_t sol);

/* The state of the library's CG-based solvers (user pointer of the functions below): the
 * CG parameters, op_lo (NULL: plain CG in op's precision; else the mixed-precision inner
 * operator of a reliable-update CG, whose mass follows op's), and the results of the last
 * call (iterations summed over the CG solves it made; the largest true residual). */
typedef struct {
  gb_cg_params cg;
  gb_op_t op_lo;
  gb_cg_result result;
  double unprec_residual; /* gb_solver_schur: max over right-hand sides of |M sol - src|/|src| */
} gb_cg_solver;

/* SchurRedBlackDiagMooeeSolve(CG)(op, src, sol) (SchurRedBlack.h:236-291) with a zero
 * initial guess (ZeroGuesser, Guesser.h). */
int gb_solver_schur(void* user /* gb_cg_solver* */, gb_op_t op, gb_field_t src, gb_field_t sol);
/* PauliVillarsSolverUnprec(CG) (PauliVillarsInverters.h:32-52): M(mass 1) sol = src by CG
 * on Mdag M from sol's contents; op's mass is restored on every return. */
int gb_solver_pv_unprec(void* user /* gb_cg_solver*, op_lo NULL */, gb_op_t op, gb_field_t src, gb_field_t sol);
/* PauliVillarsSolverRBprec(SchurSolver) (PauliVillarsInverters.h:54-72): the red-black
 * Schur solve at mass 1 (op's and op_lo's masses restored on every return). */
int gb_solver_pv_rbprec(void* user /* gb_cg_solver* */, gb_op_t op, gb_field_t src, gb_field_t sol);

/* PauliVillarsSolverFourierAccel(Umu, CG) (PauliVillarsInverters.h:74-88) running
 * FourierAcceleratedPV::pvInv (FourierAcceleratedPV.h:56-237): the mass-1 inverse of a
 * Moebius operator with constant real b, c, one right-hand side, FP64 or FP32.  A twisted
 * DFT along s block-diagonalises it; modes s and Ls-1-s pair into 5D twisted-mass Wilson
 * systems (group_in_s pairs per red-black Schur CG) whose solutions are recombined with
 * (pA -+ pB gamma5) / (pA^2 - pB^2) and transformed back.  U: the canonical FP64 gauge
 * field in host memory, borrowed (it must stay valid while the handle is used) and read at
 * every call; the twisted-mass operator is built at the first call and kept while the
 * geometry, precision, stream and boundary phases stay the same.  Ls % (2 group_in_s)
 * must be 0. */
typedef struct gb_pv_fourier_s* gb_pv_fourier_t;
int gb_pv_fourier_create(const double* U, const gb_cg_params* cg, int group_in_s, gb_pv_fourier_t* out);
int gb_pv_fourier_destroy(gb_pv_fourier_t pv);
int gb_pv_fourier_set_params(gb_pv_fourier_t pv, const gb_cg_params* cg);
int gb_pv_fourier_result(gb_pv_fourier_t pv, gb_cg_result* res);
int gb_solver_pv_fourier(void* user /* gb_pv_fourier_t */, gb_op_t op, gb_field_t src, gb_field_t sol);

/* MADWF(Mato, Mati, PauliVillarsSolvero, SchurSolveri, Guesseri, resid, maxiter, callback)
 * (Grid/qcd/action/fermion/MADWF.h:47-209): solves outer sol5 = src5 (full 5D fields of
 * the Moebius or ZMobius outer operator; a 4D source goes in by gb_import_physical_source)
 * by defect correction.  Each step: c = Pdag PV^-1 defect; the inner system Dwm P y =
 * D(1) P (c_0, 0, ..., 0) solved by inner_solve from a zero guess; the bulk Pdag PV^-1 Dm
 * P (-y_0, c_1, ...) with y_0 put back at s = 0; sol5 += P of that; defect = src5 - M sol5.
 * pv solves the outer operator at its own mass (the Pauli-Villars solvers set mass 1),
 * inner_solve the inner operator at its mass.  After each step callback (may be NULL)
 * gets the step number (1-based) and |defect| / |src5| (sums over right-hand sides); a
 * non-zero return ends the solve with that status.  Stops when that residual is below
 * resid, else returns GB_ERR_NOT_CONVERGED after maxiter steps (where Grid asserts).  The
 * operators share the 4D lattice and the number of right-hand sides; the inner mass is
 * restored on every return.  iterations / final_resid (may be NULL): IterationsToComplete
 * and the last residual. */
typedef int (*gb_madwf_callback)(void* user, int iteration, double resid);
int gb_madwf(gb_op_t outer, gb_op_t inner, gb_solver_fn pv, void* pv_user, gb_solver_fn inner_solve,
             void* inner_user, gb_field_t src5, gb_field_t sol5, double resid, int maxiter, gb_madwf_callback callback,
             void* callback_user, int* iterations, double* final_resid);

/* ---- NERSC gauge configurations (Grid/parallelIO/NerscIO.h:62-300) ---------------
 * Canonical FP64 gauge fields U[site][mu][3][3] to and from NERSC files: DATATYPE
 * 4D_SU3_GAUGE (two rows stored, the third rebuilt) or 4D_SU3_GAUGE_3x3; FLOATING_POINT
 * IEEE32BIG, IEEE32, IEEE64BIG, IEEE64 / IEEE64LITTLE.  The byte swapping, row rebuild,
 * checksum (32-bit wrapping sum of the payload words in host order) and the plaquette /
 * link trace run on the device.  U may be host (on_device = 0) or device memory. */
typedef struct {
  int dims[4];
  int two_row;                  /* 1: 4D_SU3_GAUGE, 0: 4D_SU3_GAUGE_3x3                   */
  int bits;                     /* 32 or 64                                               */
  int big_endian;
  int sequence_number;
  int64_t data_start;           /* byte offset of the payload                             */
  double link_trace, plaquette; /* header values                                          */
  uint32_t checksum;            /* header value                                           */
  uint32_t checksum_computed;   /* gb_nersc_read: of the payload                          */
  double link_trace_computed, plaquette_computed;  /* gb_nersc_read: of the field read     */
  char data_type[64], floating_point[32], ensemble_id[64], ensemble_label[64], boundary[4][32];
} gb_nersc_header;
int gb_nersc_read_header(const char* path, gb_nersc_header* h);
/* readConfiguration: check != 0 returns GB_ERR_IO when the checksum differs, the
 * plaquette differs by >= 1e-5 or the link trace by >= 1e-6 (Grid asserts) */
int gb_nersc_read(const char* path, double* U, int on_device, gb_nersc_header* h, int check);
/* writeConfiguration: two_row selects 4D_SU3_GAUGE; bits 32/64; big_endian as IEEE*BIG */
int gb_nersc_write(const char* path, const double* U, int on_device, const int dims[4], int two_row, int bits,
                   int big_endian, const char* ensemble_id, const char* ensemble_label, int sequence_number);
/* ---- ILDG / SciDAC gauge files (Grid/parallelIO/IldgIO.h:611-950, IldgIOtypes.h) ----
 * LIME records; binary data site-lexicographic (x fastest), per site [mu][row][col]
 * complex, IEEE32BIG or IEEE64BIG; the SciDAC checksum (BinaryIO.h:139-192) is the XOR
 * over sites of the CRC-32 of the site's bytes rotated left by site % 29 (suma) and
 * site % 31 (sumb). */
typedef struct {
  int dims[4];                       /* lx ly lz lt of the ildg-format record      */
  int precision;                     /* 32 or 64                                   */
  char field[32];                    /* "su3gauge"                                 */
  char lfn[256];                     /* ildg-data-lfn                              */
  int has_checksum;                  /* a scidac-checksum record was found         */
  uint32_t scidac_suma, scidac_sumb; /* from the record                            */
  uint32_t scidac_suma_computed, scidac_sumb_computed; /* of the data (gb_ildg_read) */
  int has_plaquette;                 /* usqcdInfo (or grid-format) carried them    */
  double plaquette, link_trace;      /* from the file                              */
  double plaquette_computed, link_trace_computed;
  int64_t data_offset, data_bytes;   /* the ildg-binary-data record                */
} gb_ildg_header;
/* the records only (no GPU work) */
int gb_ildg_read_header(const char* path, gb_ildg_header* h);
/* IldgReader::readConfiguration into canonical U[site][mu][3][3] (host, or device memory
 * with on_device); check != 0 returns GB_ERR_IO when the checksum record is missing or
 * differs, or the plaquette / link trace differ from the file's by >= 1e-5 (Grid asserts) */
int gb_ildg_read(const char* path, double* U, int on_device, gb_ildg_header* h, int check);
/* IldgWriter::writeConfiguration: precision 32 or 64; lfn may be NULL */
int gb_ildg_write(const char* path, const double* U, int on_device, const int dims[4], int precision, const char* lfn);

/* ---- openQCD gauge files (Grid/parallelIO/OpenQcdIO.h:43-170; read only, as in Grid) ----
 * dims in Grid order (x, y, z, t); plaquette in Grid's normalisation (the header's / 3).
 * gb_openqcd_read: canonical U[site][mu][3][3] (host, or device memory with on_device);
 * check != 0 returns GB_ERR_IO when the field's plaquette differs from the header's by
 * >= 2e-15 (Grid asserts). */
int gb_openqcd_read_header(const char* path, int dims[4], double* plaquette);
int gb_openqcd_read(const char* path, double* U, int on_device, int dims[4], double* plaquette,
                    double* plaquette_computed, int check);

/* WilsonLoops::avgPlaquette and linkTrace (Grid/qcd/utils/WilsonLoops.h:88-126,203-218) */
int gb_gauge_stats(const int dims[4], const double* U, int on_device, double* plaquette, double* link_trace);

/* The bounded-wait contract of the library's device waits, on its own: a kernel polls a
 * device flag at most max_polls times (~1 us apart; max_polls <= 2^22).  set_flag != 0
 * sets the flag first (returns GB_OK); otherwise nothing sets it and the call returns
 * GB_ERR_TIMEOUT with the context still usable. */
int gb_bounded_wait_test(gb_op_t op, int set_flag, long long max_polls);

/* ---- seeded synthetic inputs (Grid: GridParallelRNG + SU3::HotConfiguration) ----
 * Counter-based generator keyed by (seed, site, element); independent of thread count.
 * gb_random_gauge: U = reunitarise(exp(i*eps*H)), H traceless Hermitian with Gaussian
 * entries, canonical layout.  gb_random_gaussian: n complex numbers with N(0,1) real
 * and imaginary parts.  gb_random_z2: (+-1 +-i)/sqrt(2) per complex number.
 */
int gb_random_gauge(const int dims[4], double eps, uint64_t seed, double* U);
/* the same constructions evaluated on the device into device memory (stream may be NULL) */
int gb_random_gauge_device(const int dims[4], double eps, uint64_t seed, double* U_dev, void* stream);
int gb_random_gaussian_device(size_t n_complex, uint64_t seed, double* out_dev, void* stream);
int gb_random_gaussian(size_t n_complex, uint64_t seed, double* out);
int gb_random_z2(size_t n_complex, uint64_t seed, double* out);
int gb_unit_gauge(const int dims[4], double* U);

/* ---- propagator-solve service (continuous batching under an HBM budget) -----------
 * No single Grid interface corresponds: a service loop in front of
 * SchurRedBlackDiagMooeeSolve(ConjugateGradientReliableUpdate) on MobiusFermion.
 * A request solves M x = b for nsrc Gaussian 5D sources on a seeded gauge field; its
 * sources share one multi-RHS operator.  Workers (slots) admit queued requests whose
 * memory estimate fits what the budget has left; solves of different requests overlap on
 * the device (each slot has its own stream, and the library's allocations are
 * stream-ordered, so a slot's set-up does not synchronise the device).
 * Admission (default): the first queued request, in arrival order, that fits; once the
 * oldest request has waited age_limit seconds (gb_server_set_age_limit, default 10 s)
 * nothing may pass it, so a large request is not starved.  A request that cannot fit the
 * whole budget even with one source is rejected at submission (status GB_ERR_OOM).
 * flags: bit 0 = dry run (no device work: each request sleeps dry_seconds),
 *        bit 1 = run each solve's CG loop on the device (gb_cg_params use_graphs = 2),
 *        bit 2 = strict FIFO admission (only the oldest request may be admitted),
 *        bit 3 = shortest first: among the requests that may be admitted, the one with
 *                the least work per CG iteration (volume x Ls x sources). */
typedef struct {
  int dims[4];
  int Ls;
  double mf, M5, b, c;
  double eps;           /* gauge field U = exp(i eps H), seeded by gauge_seed */
  uint64_t gauge_seed;
  int nsrc;             /* 1..: Gaussian sources seeded by src_seed */
  uint64_t src_seed;
  double tolerance;     /* CG tolerance (default 1e-10) */
  int max_iterations;
  int inner_precision;  /* GB_F32 or GB_F16 */
  double dry_seconds;   /* dry-run duration */
  double t_submit;      /* set by the server */
  double* solution;     /* optional host buffer: nsrc canonical full 5D fields */
} gb_request;

typedef struct {
  int64_t id;
  int status;           /* GB_OK, GB_ERR_OOM (does not fit the budget), solver status */
  int nsrc, chunk;      /* sources, and sources per multi-RHS solve */
  int iterations, reliable_updates, cleanup_iterations;
  double true_residual; /* max over sources of the CG true residual (Grid's TrueResidual) */
  double unprec_residual; /* max over sources of |M x - b| / |b| */
  double solution_norm2;
  double t_submit, t_start, t_end; /* seconds since the server was created */
  double dev_start, dev_end;      /* the request's device work on the GPU's clock (CUDA events
                                     on its slot's stream), seconds since the server was
                                     created; -1 without device work */
} gb_request_result;

typedef struct {
  size_t budget_bytes, used_bytes, peak_used_bytes;
  int running, max_running, queued;
  int64_t submitted, finished;
  double now;
  int64_t cancelled, rejected; /* shed by gb_server_cancel_queued; rejected at submission */
  int max_queued;
} gb_server_stats_t;

typedef struct gb_server_s* gb_server_t;
int gb_server_create(size_t hbm_budget_bytes, int slots, unsigned flags, gb_server_t* out);
int gb_server_submit(gb_server_t s, const gb_request* r, int64_t* id);
int gb_server_wait(gb_server_t s, int64_t finished_count, double timeout_s);
int gb_server_results(gb_server_t s, gb_request_result* out, int max, int* n);
int gb_server_stats(gb_server_t s, gb_server_stats_t* st);
int gb_server_destroy(gb_server_t s);
int gb_request_bytes(const gb_request* r, size_t* bytes); /* the admission estimate */
int gb_server_set_age_limit(gb_server_t s, double seconds);
/* Sheds every request still queued (not admitted): each finishes with GB_ERR_CANCELLED;
 * *n = how many.  Requests already running complete. */
int gb_server_cancel_queued(gb_server_t s, int64_t* n);
/* The queue depth over time: one sample (t, queued, running) at every submission,
 * admission and completion, oldest first; *n = samples copied (at most max). */
int gb_server_trace(gb_server_t s, double* t, int* queued, int* running, int max, int* n);

/* ---- device, stream and host-buffer utilities ------------------------------------ */
int gb_set_device(int device);                       /* cudaSetDevice for this thread        */
int gb_stream_create(void** stream);                 /* a non-blocking CUDA stream           */
int gb_stream_destroy(void* stream);
int gb_op_sync(gb_op_t op);                          /* wait for the op's stream             */
int gb_op_event_record(gb_op_t op, int slot);        /* slot in [0, 16): event on op stream  */
int gb_op_event_elapsed(gb_op_t op, int slot0, int slot1, double* ms); /* waits for slot1   */
int gb_host_alloc(size_t bytes, void** ptr);         /* page-locked host memory              */
int gb_host_free(void* ptr);

/* ---- timing helpers for benchmarks (CUDA events on the op's stream) --------------- */
/* Runs `reps` applications of kernel `which` rotating over n_pairs (in,out) field pairs,
 * returns the average device milliseconds per application.
 * which: 0 DhopEO, 1 DhopOE, 2 Mooee, 3 MooeeInv, 4 Meooe5D, 5 MpcDagMpc, 6 Dhop(full) */
int gb_bench_kernel(gb_op_t op, int which, gb_field_t* ins, gb_field_t* outs, int n_pairs, int reps, double* ms);

#ifdef __cplusplus
}
#endif
#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#endif /* GBDWF_H */
