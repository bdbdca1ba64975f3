// Grid-style program on the C++ adapter (include/gbgrid.h): the even-odd identities of
// tests/core/Test_mobius_even_odd.cc, the Schur red-black solve, the mixed-precision
// reliable-update CG of tests/Test_dwf_mixedcg_prec.cc, the multishift CG, the unpreconditioned Wilson CG of
// tests/solver/Test_wilson_cg_unprec.cc, a user-defined linear operator through the
// host-driven CG, the 4D <-> 5D surface fields, MADWF, the ZMobius even-odd identities and
// the double-float FP64 option.  Exit status 0 when every check holds.
#include <cstdio>
#include <cstdlib>

#include "gbgrid.h"

using namespace Grid;

static int failures = 0;
static void expect(bool ok, const char* what, double v) {
  std::printf("%-58s %-4s %.3e\n", what, ok ? "ok" : "FAIL", v);
  if (!ok) failures++;
}

// a user-defined Hermitian operator: MdagM + shift (no library counterpart)
template <class Matrix, class Field> class ShiftedMdagM : public LinearOperatorBase<Field> {
  Matrix& m_;
  RealD shift_;

 public:
  ShiftedMdagM(Matrix& m, RealD s) : m_(m), shift_(s) {}
  void Op(const Field& in, Field& out) override { HermOp(in, out); }
  void AdjOp(const Field& in, Field& out) override { HermOp(in, out); }
  void HermOp(const Field& in, Field& out) override {
    m_.MdagM(in, out);
    axpy(out, shift_, in, out);
  }
};

int main() {
  const int Ls = 8;
  const RealD mass = 0.05, M5 = 1.8, b = 1.5, c = 0.5;
  GridCartesian* UGrid = SpaceTimeGrid::makeFourDimGrid({8, 8, 8, 8}, GridDefaultSimd(Nd, 1), GridDefaultMpi());
  GridRedBlackCartesian* UrbGrid = SpaceTimeGrid::makeFourDimRedBlackGrid(UGrid);
  GridCartesian* FGrid = SpaceTimeGrid::makeFiveDimGrid(Ls, UGrid);
  GridRedBlackCartesian* FrbGrid = SpaceTimeGrid::makeFiveDimRedBlackGrid(Ls, UGrid);

  GridParallelRNG RNG4(UGrid), RNG5(FGrid);
  RNG4.SeedFixedIntegers({1, 2, 3, 4});
  RNG5.SeedFixedIntegers({5, 6, 7, 8});
  LatticeGaugeField Umu(UGrid);
  SU<Nc>::ExpiHConfiguration(RNG4, Umu, 0.5);
  LatticeGaugeFieldF UmuF(UGrid);
  precisionChange(UmuF, Umu);

  WilsonImplParams params;
  params.boundary_phases[3] = ComplexD(-1, 0);  // antiperiodic in time
  MobiusFermionD Ddwf(Umu, *FGrid, *FrbGrid, *UGrid, *UrbGrid, mass, M5, b, c, params);
  MobiusFermionF DdwfF(UmuF, *FGrid, *FrbGrid, *UGrid, *UrbGrid, mass, M5, b, c, params);

  // ---- even-odd identities (Test_mobius_even_odd.cc) ----
  LatticeFermion src(FGrid), phi(FGrid), ref(FGrid), tmp(FGrid);
  gaussian(RNG5, src);
  gaussian(RNG5, phi);
  LatticeFermion src_e(FrbGrid), src_o(FrbGrid), r_e(FrbGrid), r_o(FrbGrid), r_eo(FGrid);
  pickCheckerboard(Even, src_e, src);
  pickCheckerboard(Odd, src_o, src);
  Ddwf.Meooe(src_e, r_o);
  Ddwf.Meooe(src_o, r_e);
  LatticeFermion t_e(FrbGrid), t_o(FrbGrid);
  Ddwf.Mooee(src_e, t_e);
  Ddwf.Mooee(src_o, t_o);
  axpy(r_e, 1.0, t_e, r_e);
  axpy(r_o, 1.0, t_o, r_o);
  setCheckerboard(r_eo, r_e);
  setCheckerboard(r_eo, r_o);
  Ddwf.M(src, ref);
  tmp = ref - r_eo;
  expect(std::sqrt(norm2(tmp) / norm2(ref)) < 1e-13, "Meooe + Mooee == M", std::sqrt(norm2(tmp) / norm2(ref)));
  {
    // the library option through ImplParams: the double-float hopping term keeps M to 1e-13
    WilsonImplParams pdf = params;
    pdf.flags = GB_FLAG_DF64;
    MobiusFermionD Ddf(Umu, *FGrid, *FrbGrid, *UGrid, *UrbGrid, mass, M5, b, c, pdf);
    LatticeFermion mdf(FGrid);
    Ddf.M(src, mdf);
    tmp = ref - mdf;
    expect(std::sqrt(norm2(tmp) / norm2(ref)) < 1e-13, "M with GB_FLAG_DF64 == M", std::sqrt(norm2(tmp) / norm2(ref)));
  }

  Ddwf.Mooee(src_o, t_o);
  Ddwf.MooeeInv(t_o, r_o);
  LatticeFermion d_o = r_o - src_o;
  expect(std::sqrt(norm2(d_o) / norm2(src_o)) < 1e-13, "MooeeInv Mooee == 1", std::sqrt(norm2(d_o) / norm2(src_o)));

  LatticeFermion phi_o(FrbGrid), Mpc_src(FrbGrid), MpcDag_phi(FrbGrid);
  pickCheckerboard(Odd, phi_o, phi);
  SchurDiagMooeeOperator<MobiusFermionD, LatticeFermion> HermOpEO(Ddwf);
  HermOpEO.Mpc(src_o, Mpc_src);
  HermOpEO.MpcDag(phi_o, MpcDag_phi);
  const ComplexD pMs = innerProduct(phi_o, Mpc_src), Mdps = innerProduct(MpcDag_phi, src_o);
  expect(std::abs(pMs - Mdps) / std::abs(pMs) < 1e-12, "<phi|Mpc src> == <MpcDag phi|src>", std::abs(pMs - Mdps) / std::abs(pMs));

  // ---- fused reductions (Lattice_reduction.h) ----
  {
    LatticeFermion z(FGrid);
    const RealD nz = axpby_norm(z, 0.5, -2.0, src, phi);
    ComplexD ip;
    RealD nrm;
    innerProductNorm(ip, nrm, src, phi);
    const ComplexD ip2 = rankInnerProduct(src, phi);
    expect(std::abs(nz - norm2(z)) < 1e-12 * nz && std::abs(nrm - norm2(src)) < 1e-12 * nrm &&
               std::abs(ip - innerProduct(src, phi)) < 1e-12 * std::abs(ip) && ip2 == innerProduct(src, phi),
           "axpby_norm / innerProductNorm / rankInnerProduct", std::abs(nz - norm2(z)) / nz);
  }

  // ---- Schur red-black solve, FP64 and mixed precision ----
  ConjugateGradient<LatticeFermion> CG(1e-10, 10000);
  SchurRedBlackDiagMooeeSolve<LatticeFermion> SchurSolver(CG);
  LatticeFermion sol(FGrid), sol_mixed(FGrid);
  sol = Zero();
  SchurSolver(Ddwf, src, sol);
  Ddwf.M(sol, tmp);
  tmp = tmp - src;
  const RealD res = std::sqrt(norm2(tmp) / norm2(src));
  std::printf("Schur CG: %d iterations, true residual %.3e\n", CG.IterationsToComplete, CG.TrueResidual);
  expect(res < 1e-9, "Schur solve |M x - b| / |b|", res);

  sol_mixed = Zero();
  SchurSolver(Ddwf, DdwfF, src, sol_mixed);
  tmp = sol_mixed - sol;
  expect(std::sqrt(norm2(tmp) / norm2(sol)) < 1e-8, "mixed-precision Schur solve == FP64", std::sqrt(norm2(tmp) / norm2(sol)));

  // ConjugateGradientReliableUpdate on the Schur operator (Test_dwf_mixedcg_prec.cc)
  SchurDiagMooeeOperator<MobiusFermionF, LatticeFermionF> HermOpEO_f(DdwfF);
  ConjugateGradientReliableUpdate<LatticeFermion, LatticeFermionF> mCG(1e-10, 10000, 1e-6, FrbGrid, HermOpEO_f, HermOpEO);
  LatticeFermion psi_o(FrbGrid), psi_d(FrbGrid);
  psi_o = Zero();
  psi_o.Checkerboard() = Odd;
  mCG(src_o, psi_o);
  psi_d = Zero();
  psi_d.Checkerboard() = Odd;
  CG(HermOpEO, src_o, psi_d);
  LatticeFermion dpsi = psi_o - psi_d;
  std::printf("reliable update CG: %d iterations, %d updates; FP64 CG %d iterations\n", mCG.IterationsToComplete,
              mCG.ReliableUpdatesPerformed, CG.IterationsToComplete);
  expect(std::sqrt(norm2(dpsi) / norm2(psi_d)) < 1e-8, "ReliableUpdate CG == FP64 CG", std::sqrt(norm2(dpsi) / norm2(psi_d)));

  // ---- MixedPrecisionConjugateGradient (restarted FP32 inner CGs) ----
  {
    MixedPrecisionConjugateGradient<LatticeFermion, LatticeFermionF> rCG(1e-10, 10000, 50, FrbGrid, HermOpEO_f, HermOpEO);
    LatticeFermion psi_m(FrbGrid);
    psi_m = Zero();
    psi_m.Checkerboard() = Odd;
    rCG(src_o, psi_m);
    LatticeFermion dm = psi_m - psi_d;
    std::printf("mixed-precision CG: %d inner iterations, %d restarts, %d patch-up\n", rCG.TotalInnerIterations,
                rCG.TotalOuterIterations, rCG.TotalFinalStepIterations);
    expect(std::sqrt(norm2(dm) / norm2(psi_d)) < 1e-8 && rCG.TotalOuterIterations >= 1,
           "MixedPrecisionConjugateGradient == FP64 CG", std::sqrt(norm2(dm) / norm2(psi_d)));
  }

  // ---- user-defined operator: host-driven CG on device fields ----
  ShiftedMdagM<MobiusFermionD, LatticeFermion> Shifted(Ddwf, 0.5);
  ConjugateGradient<LatticeFermion> CGu(1e-10, 2000);
  LatticeFermion x(FGrid), Ax(FGrid);
  x = Zero();
  CGu(Shifted, src, x);
  Shifted.HermOp(x, Ax);
  Ax = Ax - src;
  expect(std::sqrt(norm2(Ax) / norm2(src)) < 1e-9, "host-driven CG on a user operator", std::sqrt(norm2(Ax) / norm2(src)));

  // ---- multishift CG on the Schur operator (tests/solver/Test_dwf_multishift_mixedprec.cc pattern) ----
  MultiShiftFunction Sqrt(3, 0.01, 10.0);
  Sqrt.poles = {0.01, 0.1, 1.0};
  Sqrt.residues = {0.3, 0.6, 1.1};
  Sqrt.tolerances = {1e-10, 1e-10, 1e-10};
  Sqrt.norm = 0.2;
  ConjugateGradientMultiShift<LatticeFermion> MSCG(5000, Sqrt);
  std::vector<LatticeFermion> shifted;
  for (int i = 0; i < 3; i++) {
    shifted.emplace_back(FrbGrid);
    shifted.back().Checkerboard() = Odd;
  }
  MSCG(HermOpEO, src_o, shifted);
  RealD worst = 0;
  for (int i = 0; i < 3; i++) {
    LatticeFermion chk(FrbGrid);
    HermOpEO.HermOp(shifted[i], chk);
    axpy(chk, Sqrt.poles[i], shifted[i], chk);
    chk = chk - src_o;
    worst = std::max(worst, std::sqrt(norm2(chk) / norm2(src_o)));
  }
  std::printf("multishift CG: %d iterations\n", MSCG.IterationsToComplete);
  expect(worst < 2e-10, "multishift (A + m_i) x_i == src", worst);
  LatticeFermion rat(FrbGrid);
  MSCG(HermOpEO, src_o, rat);
  LatticeFermion want(FrbGrid);
  axpby(want, Sqrt.norm, 0.0, src_o, src_o);
  for (int i = 0; i < 3; i++) axpby(want, 1.0, Sqrt.residues[i], want, shifted[i]);
  LatticeFermion drat = rat - want;
  expect(std::sqrt(norm2(drat) / norm2(want)) < 1e-12, "rational sum norm src + sum residues x_i",
         std::sqrt(norm2(drat) / norm2(want)));

  // ---- unpreconditioned Wilson CG (Test_wilson_cg_unprec.cc) ----
  WilsonFermionD Dw(Umu, *UGrid, *UrbGrid, 0.1, params);
  LatticeFermion wsrc(UGrid), wsol(UGrid), wtmp(UGrid);
  gaussian(RNG4, wsrc);
  wsol = Zero();
  MdagMLinearOperator<WilsonFermionD, LatticeFermion> HermOp(Dw);
  ConjugateGradient<LatticeFermion> CGw(1e-8, 10000);
  CGw(HermOp, wsrc, wsol);
  HermOp.HermOp(wsol, wtmp);
  wtmp = wtmp - wsrc;
  expect(std::sqrt(norm2(wtmp) / norm2(wsrc)) < 1e-7, "Wilson MdagM CG", std::sqrt(norm2(wtmp) / norm2(wsrc)));

  // ---- 4D <-> 5D surface fields ----
  LatticeFermion eta(UGrid), eta_back(UGrid), eta5(FGrid), prop5(FGrid), prop4(UGrid);
  gaussian(RNG4, eta);
  Ddwf.ImportUnphysicalFermion(eta, eta5);
  Ddwf.ExportPhysicalFermionSource(eta5, eta_back);
  eta_back = eta_back - eta;
  expect(norm2(eta_back) == 0.0, "ExportPhysicalFermionSource(ImportUnphysical(eta)) == eta", norm2(eta_back));
  Ddwf.ImportPhysicalFermionSource(eta, eta5);
  prop5 = Zero();
  SchurSolver(Ddwf, eta5, prop5);
  Ddwf.ExportPhysicalFermionSolution(prop5, prop4);
  expect(norm2(prop4) > 0 && SchurSolver.UnpreconditionedResidual < 1e-9, "physical propagator solve",
         SchurSolver.UnpreconditionedResidual);

  // ---- MADWF: outer Ls = 8, inner Ls = 4 (tests/solver/Test_zMADWF_prec.cc pattern) ----
  {
    GridCartesian* FGrid4 = SpaceTimeGrid::makeFiveDimGrid(4, UGrid);
    GridRedBlackCartesian* FrbGrid4 = SpaceTimeGrid::makeFiveDimRedBlackGrid(4, UGrid);
    MobiusFermionD Dinner(Umu, *FGrid4, *FrbGrid4, *UGrid, *UrbGrid, mass, M5, b, c, params);
    ConjugateGradient<LatticeFermion> CGpv(1e-12, 10000), CGin(1e-12, 10000, false);
    SchurRedBlackDiagMooeeSolve<LatticeFermion> SchurPV(CGpv), SchurIn(CGin);
    typedef PauliVillarsSolverRBprec<LatticeFermion, SchurRedBlackDiagMooeeSolve<LatticeFermion>> PVtype;
    PVtype PV(SchurPV);
    ZeroGuesser<LatticeFermion> Guess;
    // the Fourier-accelerated Pauli-Villars inverse equals the red-black one
    {
      ConjugateGradient<LatticeFermion> CGfa(1e-12, 10000);
      PauliVillarsSolverFourierAccel<LatticeFermion, LatticeGaugeField> PVfa(Umu, CGfa);
      LatticeFermion pa(FGrid), pb(FGrid);
      pa = Zero();
      pb = Zero();
      PVfa(Ddwf, src, pa);
      PV(Ddwf, src, pb);
      LatticeFermion dp = pa - pb;
      expect(std::sqrt(norm2(dp) / norm2(pb)) < 1e-9 && Ddwf.Mass() == mass,
             "PauliVillarsSolverFourierAccel == PauliVillarsSolverRBprec", std::sqrt(norm2(dp) / norm2(pb)));
    }
    struct Count : MADWFinnerIterCallbackBase {
      int calls = 0;
      void operator()(const RealD) override { calls++; }
    } count;
    MADWF<MobiusFermionD, MobiusFermionD, PVtype, SchurRedBlackDiagMooeeSolve<LatticeFermion>,
          ZeroGuesser<LatticeFermion>>
        madwf(Ddwf, Dinner, PV, SchurIn, Guess, 1e-9, 30, &count);
    LatticeFermion madwf_sol(FGrid);
    madwf(eta, madwf_sol);
    LatticeFermion dm = madwf_sol - prop5;
    const RealD rd = std::sqrt(norm2(dm) / norm2(prop5));
    std::printf("MADWF: %d outer iterations, residual %.3e\n", madwf.IterationsToComplete, madwf.FinalResidual);
    expect(rd < 1e-7 && count.calls == madwf.IterationsToComplete && Ddwf.Mass() == mass && Dinner.Mass() == mass,
           "MADWF solution == direct Schur solve", rd);
    delete FGrid4;
    delete FrbGrid4;
  }

  // ---- ZMobius, complex omega (tests/core/Test_zmobius_even_odd.cc pattern) ----
  const std::vector<ComplexD> omega = {1.45806438985048, 1.18231318389348, 0.830951166685955, 0.542352409156791,
                                       0.341985020453729, 0.21137902619029,
                                       ComplexD(0.0686324988446592, 0.0550658530827402),
                                       ComplexD(0.0686324988446592, -0.0550658530827402)};
  ZMobiusFermionD Dz(Umu, *FGrid, *FrbGrid, *UGrid, *UrbGrid, mass, M5, omega, 1.0, 0.0, params);
  Dz.Meooe(src_e, r_o);
  Dz.Meooe(src_o, r_e);
  Dz.Mooee(src_e, t_e);
  Dz.Mooee(src_o, t_o);
  axpy(r_e, 1.0, t_e, r_e);
  axpy(r_o, 1.0, t_o, r_o);
  setCheckerboard(r_eo, r_e);
  setCheckerboard(r_eo, r_o);
  Dz.M(src, ref);
  tmp = ref - r_eo;
  expect(std::sqrt(norm2(tmp) / norm2(ref)) < 1e-13, "ZMobius Meooe + Mooee == M", std::sqrt(norm2(tmp) / norm2(ref)));
  Dz.MooeeDag(src_o, t_o);
  Dz.MooeeInvDag(t_o, r_o);
  d_o = r_o - src_o;
  expect(std::sqrt(norm2(d_o) / norm2(src_o)) < 1e-13, "ZMobius MooeeInvDag MooeeDag == 1",
         std::sqrt(norm2(d_o) / norm2(src_o)));
  sol = Zero();
  SchurSolver(Dz, src, sol);
  Dz.M(sol, tmp);
  tmp = tmp - src;
  expect(std::sqrt(norm2(tmp) / norm2(src)) < 1e-9, "ZMobius Schur solve |M x - b| / |b|",
         std::sqrt(norm2(tmp) / norm2(src)));

  // ---- Zolotarev Cayley operator (MobiusZolotarevFermion.h) ----
  {
    Approx::zolotarev_data* z = Approx::zolotarev(0.1, Ls, 0);
    const bool zok = z->n == Ls && z->Delta > 0 && z->Delta < 1e-2;
    Approx::zolotarev_free(z);
    MobiusZolotarevFermionD Dzolo(Umu, *FGrid, *FrbGrid, *UGrid, *UrbGrid, mass, M5, b, c, 0.1, 2.0, params);
    sol = Zero();
    SchurSolver(Dzolo, src, sol);
    Dzolo.M(sol, tmp);
    tmp = tmp - src;
    const RealD rz = std::sqrt(norm2(tmp) / norm2(src));
    expect(zok && rz < 1e-9, "MobiusZolotarev Schur solve |M x - b| / |b|", rz);
  }

  // ---- errors come back as exceptions ----
  bool threw = false;
  try {
    Ddwf.DhopEO(src, tmp, DaggerNo);  // full fields where an odd half field is expected
  } catch (const GridError& e) {
    threw = e.status == GB_ERR_BAD_PARITY;
  }
  expect(threw, "checkerboard mismatch throws GridError", 0.0);

  std::printf("%s (%d failures)\n", failures ? "FAILED" : "PASSED", failures);
  return failures ? 1 : 0;
}
