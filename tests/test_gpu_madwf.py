"""MADWF on the GPU (Grid/qcd/action/fermion/MADWF.h, tests/solver/Test_zMADWF_prec.cc)
against the oracle: the chiral permutation P / Pdag (bit-exact data movement), SetMass,
InsertSlice / ExtractSlice, and the whole defect-correction loop -- its residual history
against the oracle's MADWF and its solution against the direct outer solve -- with a
Moebius and a ZMobius inner operator and both Pauli-Villars solvers."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import madwf as mw
from oracle import oracle as o
from tests._common import MOBIUS, fermion
from tests.test_oracle_pins import ZOMEGA, zparams

pytestmark = pytest.mark.gpu

DIMS = (4, 4, 4, 4)
VOL = 256
MF = 0.05


def mobius(U, Ls, prec=g.F64, nrhs=1, b=MOBIUS["b"], c=MOBIUS["c"]):
    return g.MobiusFermion(U, DIMS, Ls, MF, MOBIUS["M5"], b, c, precision=prec, nrhs=nrhs)


@pytest.mark.parametrize("prec", [g.F64, g.F32, g.F16])
@pytest.mark.parametrize("nrhs", [1, 3])
def test_p_pdag(gpu_available, prec, nrhs):
    U = g.random_gauge(DIMS, 0.3, 5)
    Ls = 6
    op = mobius(U, Ls, prec, nrhs)
    ref = o.OracleOp(1, 0, DIMS, Ls, [MF, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    xs = [fermion(VOL, Ls, 30 + r) for r in range(nrhs)]
    fin, fout = op.FermionField().import_(np.concatenate(xs)), op.FermionField()
    stored = fin.export().reshape(nrhs, -1)  # the inputs as the field holds them
    exact = prec != g.F16  # FP16 re-encodes each site with its new norm
    for name, code in (("P", o.OP_P), ("Pdag", o.OP_PDAG)):
        getattr(op, name)(fin, fout)
        got = fout.export().reshape(nrhs, -1)
        for r in range(nrhs):
            want = ref.apply(code, stored[r])
            if exact:
                assert np.array_equal(got[r], want), (name, r)
            else:
                assert o.rel_l2(got[r], want) < 2e-3, (name, r)
    # half fields: P acts within each 4D site
    xh = fermion(VOL // 2, Ls, 40)
    hin = op.FermionRedBlackField(g.ODD).import_(np.tile(xh, nrhs))
    hout = op.FermionRedBlackField(g.ODD)
    op.P(hin, hout)
    held = hin.export().reshape(nrhs, -1)[0]
    want = ref.apply(o.OP_P, np.concatenate([held, np.zeros_like(held)]))[:held.size]  # site-local: any padding works
    assert o.rel_l2(hout.export().reshape(nrhs, -1)[0], want) < (1e-15 if exact else 2e-3)
    with pytest.raises(g.GridError):
        op.P(fin, fin)


@pytest.mark.parametrize("kind", ["mobius", "zmobius", "wilson"])
def test_set_mass(gpu_available, kind):
    U = g.random_gauge(DIMS, 0.3, 6)
    if kind == "mobius":
        op = mobius(U, 6)
        ref = o.OracleOp(1, 0, DIMS, 6, [MF, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
        L5 = 6
    elif kind == "zmobius":
        op = g.ZMobiusFermion(U, DIMS, ZOMEGA, MF, MOBIUS["M5"], 1.0, 0.0)
        ref = o.OracleOp(2, 0, DIMS, 10, zparams(MF, MOBIUS["M5"], 1.0, 0.0, ZOMEGA), U, g.antiperiodic_t())
        L5 = 10
    else:
        op = g.WilsonFermion(U, DIMS, MF)
        ref = o.OracleOp(0, 0, DIMS, 1, [MF], U, g.antiperiodic_t())
        L5 = 1
    x = fermion(VOL, L5, 41)
    xh = fermion(VOL // 2, L5, 42)
    fin, fout = op.FermionField().import_(x), op.FermionField()
    hin, hout = op.FermionRedBlackField(g.ODD).import_(xh), op.FermionRedBlackField(g.ODD)
    for m in (1.0, 0.3, MF):
        op.SetMass(m)
        ref.set_mass(m)
        assert op.Mass() == m
        op.M(fin, fout)
        assert o.rel_l2(fout.export(), ref.apply(o.OP_M, x)) < 1e-13, (kind, m)
        op.MooeeInv(hin, hout)
        assert o.rel_l2(hout.export(), ref.apply(o.OP_MOOEE_INV, xh, 1)) < 1e-13, (kind, m)


def test_slices(gpu_available):
    U = g.random_gauge(DIMS, 0.3, 7)
    Ls = 6
    op = mobius(U, Ls)
    x = fermion(VOL, Ls, 43)
    f = op.FermionField().import_(x)
    for s in (0, 3, Ls - 1):
        assert np.array_equal(g.ExtractSlice(f, s), mw.extract_slice(x, Ls, s))
    y4 = fermion(VOL, 1, 44)
    g.InsertSlice(y4, f, 2)
    assert np.array_equal(f.export(), mw.insert_slice(y4, x, Ls, 2))
    with pytest.raises(g.GridError):
        g.ExtractSlice(f, Ls)
    with pytest.raises(g.GridError):
        g.InsertSlice(y4, op.FermionRedBlackField(g.ODD), 0)


def _outer_problem(Lo, b=MOBIUS["b"], c=MOBIUS["c"]):
    U = g.random_gauge(DIMS, 0.3, 5)
    outer = mobius(U, Lo, b=b, c=c)
    ref = o.OracleOp(1, 0, DIMS, Lo, [MF, MOBIUS["M5"], b, c], U, g.antiperiodic_t())
    eta = fermion(VOL, 1, 4)
    return U, outer, ref, eta


@pytest.mark.parametrize("pv", ["rbprec", "unprec"])
def test_madwf_mobius_inner_matches_oracle(gpu_available, pv):
    """Outer Moebius Ls = 8, inner Moebius Ls = 4: the residual history of each
    defect-correction step agrees with the oracle's MADWF, and the solution with the
    oracle's direct solve of the outer system."""
    Lo, Li = 8, 4
    U, outer, ref, eta = _outer_problem(Lo)
    inner = mobius(U, Li)
    ref_in = o.OracleOp(1, 0, DIMS, Li, [MF, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    b = ref.physical(o.IMPORT_PHYSICAL_SOURCE, eta)
    want_sol, want_hist = mw.madwf(ref, Lo, MF, ref_in, Li, MF, b, 1e-12, 1e-12, 1e-9, 20)

    cg_pv = g.ConjugateGradient(1e-12, 10000)
    pv_solver = (g.PauliVillarsSolverRBprec(g.SchurRedBlackDiagMooeeSolve(cg_pv)) if pv == "rbprec"
                 else g.PauliVillarsSolverUnprec(cg_pv))
    cg_in = g.ConjugateGradient(1e-12, 10000, False)
    seen = []
    madwf = g.MADWF(outer, inner, pv_solver, g.SchurRedBlackDiagMooeeSolve(cg_in), g.ZeroGuesser(), 1e-9, 20,
                    callback=seen.append)
    sol = outer.FermionField()
    madwf(eta, sol)
    hist = madwf.residuals
    assert seen == hist
    assert len(hist) == len(want_hist)
    for a, w in zip(hist, want_hist):
        assert abs(a - w) < 1e-3 * w + 1e-10, (hist, want_hist)
    assert outer.Mass() == MF and inner.Mass() == MF
    direct, _, _, _ = ref.schur_solve(b, 1e-11, 10000)
    assert o.rel_l2(sol.export(), direct) < 1e-8
    assert o.rel_l2(ref.apply(o.OP_M, sol.export()), b) < 1e-9


def test_madwf_zmobius_inner(gpu_available):
    """Test_zMADWF_prec.cc's pattern: outer Moebius Ls = 12 (b + c = 2), inner ZMobius
    Ls = 10 with complex omegas; a 5D source; the inner tolerance is relaxed by a callback
    as the outer residual falls (CGincreaseTol)."""
    Lo = 12
    U, outer, ref, eta = _outer_problem(Lo, 1.5, 0.5)
    inner = g.ZMobiusFermion(U, DIMS, ZOMEGA, MF, MOBIUS["M5"], 1.0, 0.0)
    b = ref.physical(o.IMPORT_PHYSICAL_SOURCE, eta)
    src = outer.FermionField().import_(b)
    cg_in = g.ConjugateGradient(1e-10, 10000, False)

    def increase_tol(resid):
        while cg_in.Tolerance < resid:
            cg_in.Tolerance *= 2

    madwf = g.MADWF(outer, inner, g.PauliVillarsSolverRBprec(g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000))),
                    g.SchurRedBlackDiagMooeeSolve(cg_in), g.ZeroGuesser(), 1e-9, 20, callback=increase_tol)
    sol = outer.FermionField()
    madwf(src, sol)
    assert madwf.iterations <= 8 and madwf.residuals[-1] < 1e-9
    direct, _, _, _ = ref.schur_solve(b, 1e-11, 10000)
    assert o.rel_l2(sol.export(), direct) < 1e-8


def test_madwf_not_converged_raises(gpu_available):
    Lo, Li = 8, 4
    U, outer, ref, eta = _outer_problem(Lo)
    inner = mobius(U, Li)
    pv_solver = g.PauliVillarsSolverRBprec(g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000)))
    madwf = g.MADWF(outer, inner, pv_solver, g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000, False)),
                    g.ZeroGuesser(), 1e-12, 2)
    with pytest.raises(g.GridError):
        madwf(eta, outer.FermionField())
    assert outer.Mass() == MF and inner.Mass() == MF


def test_madwf_with_computed_zmobius_gammas(gpu_available):
    """Test_zMADWF_prec.cc's workflow end to end: the inner ZMobius gammas come from
    Approx::computeZmobiusGamma(b+c = 1, Ls_in = 8, outer b+c = 2, Ls_out = 12, lambda =
    1.42), the inner operator has b = 1, c = 0, and MADWF reproduces the outer solve."""
    Lo, Li = 12, 8
    U, outer, ref, eta = _outer_problem(Lo, 1.5, 0.5)
    gamma, err = g.computeZmobiusGamma(1.0, Li, 2.0, Lo, 1.42)
    assert err < 1e-2
    inner = g.ZMobiusFermion(U, DIMS, list(gamma), MF, MOBIUS["M5"], 1.0, 0.0)
    pv = g.PauliVillarsSolverRBprec(g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000)))
    madwf = g.MADWF(outer, inner, pv, g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000, False)),
                    g.ZeroGuesser(), 1e-9, 20)
    sol = outer.FermionField()
    madwf(eta, sol)
    assert madwf.residuals[-1] < 1e-9 and madwf.iterations <= 10
    b = ref.physical(o.IMPORT_PHYSICAL_SOURCE, eta)
    direct, _, _, _ = ref.schur_solve(b, 1e-11, 10000)
    assert o.rel_l2(sol.export(), direct) < 1e-8


def _c_solver(name):
    return g.api._SOLVER_FN((name, g.api.lib))


def test_madwf_library_solvers_through_the_c_abi(gpu_available):
    """gb_madwf driven with the library's own solver functions as C function pointers (no
    host-language callback in the loop) gives the residual history of the MADWF class."""
    Lo, Li = 8, 4
    U, outer, ref, eta = _outer_problem(Lo)
    inner = mobius(U, Li)
    madwf = g.MADWF(outer, inner, g.PauliVillarsSolverRBprec(g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000))),
                    g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000, False)), g.ZeroGuesser(), 1e-9, 20)
    want = outer.FermionField()
    madwf(eta, want)
    b = outer.FermionField()
    outer.ImportPhysicalFermionSource(eta, b)
    pv_st, in_st = g.api.CGSolver(), g.api.CGSolver()
    pv_st.cg = g.ConjugateGradient(1e-12, 10000).params()
    in_st.cg = g.ConjugateGradient(1e-12, 10000, False).params()
    seen = []
    cb = g.api._MADWF_CB(lambda user, it, r: seen.append((it, r)) or 0)
    sol = outer.FermionField()
    it, fr = g.api.C.c_int(), g.api.C.c_double()
    rc = g.api.lib.gb_madwf(outer.h, inner.h, _c_solver("gb_solver_pv_rbprec"), g.api.C.addressof(pv_st),
                            _c_solver("gb_solver_schur"), g.api.C.addressof(in_st), b.h, sol.h, 1e-9, 20, cb, None,
                            g.api.C.byref(it), g.api.C.byref(fr))
    assert rc == 0
    assert [r for _, r in seen] == madwf.residuals and it.value == madwf.iterations == len(seen)
    assert fr.value == madwf.residuals[-1]
    assert o.rel_l2(sol.export(), want.export()) < 1e-14
    assert in_st.result.iterations > 0 and in_st.unprec_residual < 1e-9
    assert outer.Mass() == MF and inner.Mass() == MF


def test_madwf_solver_exception_propagates(gpu_available):
    """An exception raised by a host-language solver ends the library's loop and is raised
    again to the caller; both operators keep their masses."""
    Lo, Li = 8, 4
    U, outer, ref, eta = _outer_problem(Lo)
    inner = mobius(U, Li)
    pv = g.PauliVillarsSolverRBprec(g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000)))
    calls = []

    def failing_pv(matrix, src, sol):
        calls.append(1)
        if len(calls) == 3:
            raise ValueError("planted")
        pv(matrix, src, sol)

    madwf = g.MADWF(outer, inner, failing_pv, g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000, False)),
                    g.ZeroGuesser(), 1e-9, 20)
    with pytest.raises(ValueError, match="planted"):
        madwf(eta, outer.FermionField())
    assert len(calls) == 3 and madwf.iterations == 1
    assert outer.Mass() == MF and inner.Mass() == MF


def test_madwf_operators_on_different_streams(gpu_available):
    """Outer operator on its own stream, inner on the default stream: the surface slices
    pass between the streams in order, and the result is the single-stream one."""
    Lo, Li = 8, 4
    U, outer, ref, eta = _outer_problem(Lo)
    inner = mobius(U, Li)
    st = g.Stream()
    outer_s = g.MobiusFermion(U, DIMS, Lo, MF, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], stream=st.ptr)

    def run(o_op):
        madwf = g.MADWF(o_op, inner, g.PauliVillarsSolverRBprec(g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000))),
                        g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-12, 10000, False)), g.ZeroGuesser(), 1e-9, 20)
        sol = o_op.FermionField()
        madwf(eta, sol)
        return madwf.residuals, sol.export()

    h1, x1 = run(outer)
    h2, x2 = run(outer_s)
    del outer_s  # before its stream
    assert h1 == h2
    assert np.array_equal(x1, x2)
