"""Parity of the CUDA path (through the C ABI) with the CPU oracle on the same seeded
inputs.  Tolerances (relative L2): FP64 1e-13, FP32 1e-6 for every operator, the
composites (M, MdagM, Mooee, MooeeInv, Mpc, MpcDagMpc) included (FP32 measures 1.3e-7 at
most); solvers are checked by the true residual |A x - b| / |b| measured with the
oracle's FP64 operator."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o
from tests._common import MOBIUS, fermion

pytestmark = pytest.mark.gpu

TOL = {g.F64: 1e-13, g.F32: 1e-6}


def mobius_pair(dims, Ls, mf, prec, eps=0.5, seed=1, nrhs=1, flags=0):
    U = g.random_gauge(dims, eps, seed)
    op = g.MobiusFermion(U, dims, Ls, mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], precision=prec, nrhs=nrhs,
                         flags=flags)
    ref = o.OracleOp(1, 0, dims, Ls, [mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    return op, ref, U


def wilson_pair(dims, mass, prec, eps=0.3, seed=2, nrhs=1):
    U = g.random_gauge(dims, eps, seed)
    op = g.WilsonFermion(U, dims, mass, precision=prec, nrhs=nrhs)
    ref = o.OracleOp(0, 0, dims, nrhs, [mass], U, g.antiperiodic_t())
    return op, ref, U


def half(op, cb, data):
    f = op.FermionRedBlackField(cb)
    f.import_(data)
    return f


@pytest.mark.parametrize("prec", [g.F64, g.F32])
@pytest.mark.parametrize("dag", [0, 1])
@pytest.mark.parametrize("case", ["wilson8", "wilson_odd_shape", "mobius8", "mobius12"])
def test_dhop_eo_oe(gpu_available, prec, dag, case):
    if case.startswith("wilson"):
        dims = (8, 8, 8, 8) if case == "wilson8" else (6, 4, 2, 10)
        op, ref, U = wilson_pair(dims, 0.1, prec)
        L5 = 1
    else:
        dims = (4, 4, 4, 8) if case == "mobius8" else (4, 6, 4, 4)
        L5 = 8 if case == "mobius8" else 12
        op, ref, U = mobius_pair(dims, L5, 0.01, prec)
    nh = int(np.prod(dims)) // 2
    for in_cb in (1, 0):
        x = fermion(nh, L5, 10 + in_cb)
        fin = half(op, in_cb, x)
        fout = op.FermionRedBlackField(1 - in_cb)
        (op.DhopEO if in_cb == 1 else op.DhopOE)(fin, fout, dag)
        assert fout.checkerboard == 1 - in_cb
        assert o.rel_l2(fout.export(), ref.dhop_cb(x, in_cb, dag)) < TOL[prec]


@pytest.mark.parametrize("prec", [g.F64, g.F32])
def test_full_dhop_and_M(gpu_available, prec):
    dims = (4, 4, 4, 6)
    op, ref, U = mobius_pair(dims, 6, 0.05, prec)
    x = fermion(int(np.prod(dims)), 6, 20)
    fin = op.FermionField().import_(x)
    fout = op.FermionField()
    for name, code in (("M", o.OP_M), ("Mdag", o.OP_MDAG), ("MdagM", o.OP_MDAGM)):
        getattr(op, name)(fin, fout)
        assert o.rel_l2(fout.export(), ref.apply(code, x)) < TOL[prec], name
    for dag, code in ((0, o.OP_DHOP), (1, o.OP_DHOP_DAG)):
        op.Dhop(fin, fout, dag)
        assert o.rel_l2(fout.export(), ref.apply(code, x)) < TOL[prec]


@pytest.mark.parametrize("prec", [g.F64, g.F32])
@pytest.mark.parametrize("Ls", [4, 6, 8, 12, 16, 18])
def test_mobius_half_ops(gpu_available, prec, Ls):
    dims = (4, 4, 4, 4)
    op, ref, U = mobius_pair(dims, Ls, 0.01, prec, seed=Ls)
    nh = 128
    x = fermion(nh, Ls, 30 + Ls)
    for name, code, cb in (("Mooee", o.OP_MOOEE, 1), ("MooeeDag", o.OP_MOOEE_DAG, 1), ("MooeeInv", o.OP_MOOEE_INV, 1),
                           ("MooeeInvDag", o.OP_MOOEE_INV_DAG, 1), ("Meooe", o.OP_MEOOE, 1),
                           ("Meooe", o.OP_MEOOE, 0), ("MeooeDag", o.OP_MEOOE_DAG, 1),
                           ("MeooeDag", o.OP_MEOOE_DAG, 0), ("Mpc", o.OP_MPC, 1), ("MpcDag", o.OP_MPC_DAG, 1),
                           ("MpcDagMpc", o.OP_MPCDAGMPC, 1)):
        fin = half(op, cb, x)
        fout = op.FermionRedBlackField(cb)
        getattr(op, name)(fin, fout)
        assert o.rel_l2(fout.export(), ref.apply(code, x, cb)) < TOL[prec], (name, cb)


def test_fp16_storage_operators(gpu_available):
    """FP16 spinors with per-site FP32 norms, FP32 links and arithmetic: every operator
    agrees with the FP64 oracle to FP16 rounding.  Single operators: relative L2 below
    3e-3 (one FP16 store); the Schur composites store four FP16 intermediates and
    subtract two O(1) terms, below 3e-2."""
    dims = (4, 4, 4, 4)
    Ls = 8
    op, ref, U = mobius_pair(dims, Ls, 0.01, g.F16)
    x = fermion(128, Ls, 35)
    for name, code, tol in (("Mooee", o.OP_MOOEE, 3e-3), ("MooeeDag", o.OP_MOOEE_DAG, 3e-3),
                            ("MooeeInv", o.OP_MOOEE_INV, 3e-3), ("MooeeInvDag", o.OP_MOOEE_INV_DAG, 3e-3),
                            ("Meooe", o.OP_MEOOE, 3e-3), ("MeooeDag", o.OP_MEOOE_DAG, 3e-3),
                            ("Mpc", o.OP_MPC, 3e-2), ("MpcDagMpc", o.OP_MPCDAGMPC, 3e-2)):
        fin = half(op, 1, x)
        fout = op.FermionRedBlackField(1)
        getattr(op, name)(fin, fout)
        assert o.rel_l2(fout.export(), ref.apply(code, x, 1)) < tol, name
    fin = half(op, 1, x)
    fout = op.FermionRedBlackField(0)
    op.DhopEO(fin, fout, 0)
    assert o.rel_l2(fout.export(), ref.dhop_cb(x, 1, 0)) < 3e-3


@pytest.mark.parametrize("prec", [g.F64, g.F32])
def test_wilson_half_ops(gpu_available, prec):
    dims = (4, 4, 4, 4)
    op, ref, U = wilson_pair(dims, 0.2, prec)
    x = fermion(128, 1, 40)
    for name, code in (("Mooee", o.OP_MOOEE), ("MooeeInv", o.OP_MOOEE_INV), ("Meooe", o.OP_MEOOE),
                       ("MeooeDag", o.OP_MEOOE_DAG), ("Mpc", o.OP_MPC), ("MpcDag", o.OP_MPC_DAG),
                       ("MpcDagMpc", o.OP_MPCDAGMPC)):
        fin = half(op, 1, x)
        fout = op.FermionRedBlackField(1)
        getattr(op, name)(fin, fout)
        assert o.rel_l2(fout.export(), ref.apply(code, x, 1)) < TOL[prec], name


@pytest.mark.parametrize("prec", [g.F64, g.F32])
def test_multi_rhs_wilson_dhop(gpu_available, prec):
    """nrhs right-hand sides share each link read; each equals its own single solve."""
    dims = (4, 4, 4, 8)
    nrhs = 5
    op, ref, U = wilson_pair(dims, 0.02, prec, nrhs=nrhs)
    nh = int(np.prod(dims)) // 2
    xs = [fermion(nh, 1, 50 + r) for r in range(nrhs)]
    fin = half(op, 1, np.concatenate(xs))
    fout = op.FermionRedBlackField(0)
    op.DhopEO(fin, fout, 0)
    got = fout.export().reshape(nrhs, -1)
    single = o.OracleOp(0, 0, dims, 1, [0.02], U, g.antiperiodic_t())
    for r in range(nrhs):
        assert o.rel_l2(got[r], single.dhop_cb(xs[r], 1)) < TOL[prec]


def test_multi_rhs_mobius_ops(gpu_available):
    dims = (4, 4, 4, 4)
    nrhs, Ls = 3, 8
    op, ref, U = mobius_pair(dims, Ls, 0.01, g.F64, nrhs=nrhs)
    xs = [fermion(128, Ls, 60 + r) for r in range(nrhs)]
    fin = half(op, 1, np.concatenate(xs))
    fout = op.FermionRedBlackField(1)
    op.MpcDagMpc(fin, fout)
    got = fout.export().reshape(nrhs, -1)
    for r in range(nrhs):
        assert o.rel_l2(got[r], ref.apply(o.OP_MPCDAGMPC, xs[r], 1)) < 1e-12
    n2 = fin.norm2()
    for r in range(nrhs):
        assert abs(n2[r] - np.vdot(xs[r], xs[r]).real) < 1e-12 * n2[r]


@pytest.mark.parametrize("prec", [g.F64, g.F32, g.F16])
def test_reductions_and_axpy(gpu_available, prec):
    dims = (8, 4, 4, 4)
    op, ref, U = mobius_pair(dims, 8, 0.01, g.F64 if prec == g.F64 else g.F32)
    x = fermion(256, 8, 70)
    y = fermion(256, 8, 71)
    fx = op.FermionRedBlackField(1, precision=prec).import_(x)
    fy = op.FermionRedBlackField(1, precision=prec).import_(y)
    tol = {g.F64: 1e-13, g.F32: 1e-6, g.F16: 2e-3}[prec]
    assert abs(fx.norm2()[0] / np.vdot(x, x).real - 1) < tol
    ip = fx.inner(fy)[0]
    ref_ip = np.vdot(x, y)
    assert abs(ip - ref_ip) < tol * 10 * np.sqrt(np.vdot(x, x).real * np.vdot(y, y).real)
    fz = op.FermionRedBlackField(1, precision=prec)
    nz = g.api.axpy_norm(fz, -0.7, fx, fy)[0]
    z = -0.7 * x + y
    assert abs(nz / np.vdot(z, z).real - 1) < tol * 10
    assert o.rel_l2(fz.export(), z) < tol * 5
    # precision change round trip
    f64 = op.FermionRedBlackField(1, precision=g.F64)
    f64.copy_from(fx)
    assert o.rel_l2(f64.export(), x) < tol


def test_checkerboard_pick_set(gpu_available):
    dims = (4, 4, 4, 4)
    op, ref, U = mobius_pair(dims, 4, 0.01, g.F64)
    x = fermion(256, 4, 80)
    full = op.FermionField().import_(x)
    e = op.FermionRedBlackField(0)
    od = op.FermionRedBlackField(1)
    g.api.pickCheckerboard(0, e, full)
    g.api.pickCheckerboard(1, od, full)
    assert np.array_equal(e.export(), o.pick(dims, 4, x, 0))
    assert np.array_equal(od.export(), o.pick(dims, 4, x, 1))
    full2 = op.FermionField().zero()
    g.api.setCheckerboard(full2, e)
    g.api.setCheckerboard(full2, od)
    assert np.array_equal(full2.export(), x)


def test_wrong_checkerboard_is_an_error(gpu_available):
    dims = (4, 4, 4, 4)
    op, ref, U = mobius_pair(dims, 4, 0.01, g.F64)
    fe = op.FermionRedBlackField(0).zero()
    fo = op.FermionRedBlackField(1)
    with pytest.raises(g.GridError) as ei:
        op.DhopEO(fe, fo, 0)  # DhopEO needs an odd input
    assert ei.value.status == 2
    with pytest.raises(g.GridError):
        op.MpcDagMpc(fe, fo)


# ---- solvers -----------------------------------------------------------------------------
def test_cg_wilson_unprec_config1(gpu_available):
    """Wilson 8^4, antiperiodic t, m = 0.1, unpreconditioned CG on MdagM to 1e-8
    (tests/solver/Test_wilson_cg_unprec.cc); checked against the oracle's CG."""
    dims = (8, 8, 8, 8)
    op, ref, U = wilson_pair(dims, 0.1, g.F64)
    src = fermion(4096, 1, 90)
    fs = op.FermionField().import_(src)
    fx = op.FermionField().zero()
    cg = g.ConjugateGradient(1e-8, 10000)
    cg(g.MdagMLinearOperator(op), fs, fx)
    x = fx.export()
    xr, it_ref, res_ref = ref.cg(0, src, 1e-8, 10000)
    assert abs(cg.IterationsToComplete - it_ref) <= 2
    r = ref.apply(o.OP_MDAGM, x) - src
    assert np.linalg.norm(r) / np.linalg.norm(src) < 1e-8 * 1.5
    assert abs(cg.TrueResidual - res_ref) < 1e-9
    assert o.rel_l2(x, xr) < 1e-6


def test_cg_not_converged_raises_and_flag(gpu_available):
    dims = (4, 4, 4, 4)
    op, ref, U = wilson_pair(dims, 0.01, g.F64)
    src = fermion(256, 1, 91)
    fs = op.FermionField().import_(src)
    fx = op.FermionField().zero()
    with pytest.raises(g.GridError) as ei:
        g.ConjugateGradient(1e-12, 5)(g.MdagMLinearOperator(op), fs, fx)
    assert ei.value.status == 5
    fx.zero()
    cg = g.ConjugateGradient(1e-12, 5, err_on_no_conv=False)
    r = cg(g.MdagMLinearOperator(op), fs, fx)
    assert r.converged == 0 and cg.IterationsToComplete == 5


def test_cg_nonzero_guess_matches_oracle(gpu_available):
    dims = (4, 4, 4, 4)
    op, ref, U = wilson_pair(dims, 0.1, g.F64)
    src = fermion(256, 1, 92)
    x0 = 0.1 * fermion(256, 1, 93)
    fs = op.FermionField().import_(src)
    fx = op.FermionField().import_(x0)
    cg = g.ConjugateGradient(1e-10, 1000)
    cg(g.MdagMLinearOperator(op), fs, fx)
    xr, it, res = ref.cg(0, src, 1e-10, 1000, psi0=x0)
    assert abs(cg.IterationsToComplete - it) <= 1
    assert o.rel_l2(fx.export(), xr) < 1e-8


def test_schur_solve_mobius_fp64(gpu_available):
    dims = (4, 4, 4, 8)
    Ls = 8
    op, ref, U = mobius_pair(dims, Ls, 0.01, g.F64)
    src = fermion(512, Ls, 100)
    fs = op.FermionField().import_(src)
    fx = op.FermionField().zero()
    solver = g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-10, 5000))
    solver(op, fs, fx)
    x = fx.export()
    xr, it, r_cg, r_un = ref.schur_solve(src, 1e-10, 5000)
    assert abs(solver.solver.IterationsToComplete - it) <= 2
    assert o.rel_l2(ref.apply(o.OP_M, x), src) < 1e-9
    assert solver.unprec_residual[0] < 1e-9
    assert o.rel_l2(x, xr) < 1e-7


def test_cg_converged_guess_reports_the_same_true_residual(gpu_available):
    """A CG whose guess already meets the tolerance runs no iteration and reports the true
    residual of the r = b - A x it starts from; it equals, bit for bit, the true residual
    the converged solve reported after applying A to the same x."""
    dims, Ls = (4, 4, 4, 8), 8
    op, ref, U = mobius_pair(dims, Ls, 0.01, g.F64)
    nh = 256
    b = op.FermionRedBlackField(1).import_(fermion(nh, Ls, 101))
    x = op.FermionRedBlackField(1).zero()
    lin = g.SchurDiagMooeeOperator(op)
    c1 = g.ConjugateGradient(1e-10, 5000)
    c1(lin, b, x)
    assert c1.IterationsToComplete > 0
    c2 = g.ConjugateGradient(1e-10, 5000)
    c2(lin, b, x)
    assert c2.IterationsToComplete == 0
    assert c2.TrueResidual == c1.TrueResidual
    got = x.export()
    bh = fermion(nh, Ls, 101)
    assert abs(o.rel_l2(ref.apply(o.OP_MPCDAGMPC, got, 1), bh) - c2.TrueResidual) < 1e-3 * c2.TrueResidual


@pytest.mark.parametrize("lo", [g.F32, g.F16])
def test_mixed_precision_schur_reaches_1e10(gpu_available, lo):
    """FP32 (or FP16-stored) inner CG with FP64 reliable updates reaches a true residual
    1e-10; the solution agrees with the oracle's FP64 solve."""
    dims = (4, 4, 4, 8)
    Ls = 8
    U = g.random_gauge(dims, 0.6, 5)
    od = g.MobiusFermion(U, dims, Ls, 0.01, 1.8, 1.5, 0.5, precision=g.F64)
    of = g.MobiusFermion(U, dims, Ls, 0.01, 1.8, 1.5, 0.5, precision=lo)
    ref = o.OracleOp(1, 0, dims, Ls, [0.01, 1.8, 1.5, 0.5], U, g.antiperiodic_t())
    src = fermion(512, Ls, 110)
    fs = od.FermionField().import_(src)
    fx = od.FermionField().zero()
    cg = g.ConjugateGradientReliableUpdate(1e-10, 20000, 1e-6, g.SchurDiagMooeeOperator(of),
                                           g.SchurDiagMooeeOperator(od), relup_every=100)
    solver = g.SchurRedBlackDiagMooeeSolve(cg)
    solver(od, fs, fx)
    x = fx.export()
    assert cg.TrueResidual < 1e-10
    assert cg.ReliableUpdatesPerformed >= 1
    xr, it, r_cg, r_un = ref.schur_solve(src, 1e-10, 5000)
    assert o.rel_l2(ref.apply(o.OP_M, x), src) < 1e-9
    assert o.rel_l2(x, xr) < 1e-7


@pytest.mark.parametrize("lo,nrhs", [(g.F32, 4), (g.F16, 4), (g.F32, 3)])
def test_multi_rhs_mobius_mixed_cg_each_equals_single(gpu_available, lo, nrhs):
    """A multi-RHS Moebius operator pair through the mixed-precision Schur CG: the per-rhs
    reductions fused into the operator (|Mpc p|^2 in Mpc's last kernel, and MpcDag's
    residual update when the rhs count divides the column kernel's 16-column tiles; 3 takes
    the separate update pass) keep every right-hand side on its own solve.  Each solution
    meets the tolerance against the oracle's FP64 M and agrees with its single-RHS solve."""
    dims, Ls = (4, 4, 4, 8), 8
    U = g.random_gauge(dims, 0.6, 5)
    srcs = [fermion(512, Ls, 130 + r) for r in range(nrhs)]
    ref = o.OracleOp(1, 0, dims, Ls, [0.01, 1.8, 1.5, 0.5], U, g.antiperiodic_t())

    def solve(n, src):
        od = g.MobiusFermion(U, dims, Ls, 0.01, 1.8, 1.5, 0.5, precision=g.F64, nrhs=n)
        of = g.MobiusFermion(U, dims, Ls, 0.01, 1.8, 1.5, 0.5, precision=lo, nrhs=n)
        fs = od.FermionField().import_(src)
        fx = od.FermionField().zero()
        cg = g.ConjugateGradientReliableUpdate(1e-10, 20000, 1e-6, g.SchurDiagMooeeOperator(of),
                                               g.SchurDiagMooeeOperator(od), relup_every=100, use_graphs=1)
        g.SchurRedBlackDiagMooeeSolve(cg)(od, fs, fx)
        return fx.export(), cg

    xb, cb = solve(nrhs, np.concatenate(srcs))
    got = xb.reshape(nrhs, -1)
    for r in range(nrhs):
        x1, c1 = solve(1, srcs[r])
        assert cb.per_rhs_true_residual[r] < 1e-10 and c1.TrueResidual < 1e-10
        assert abs(cb.per_rhs_iterations[r] - c1.IterationsToComplete) <= 0.1 * c1.IterationsToComplete
        assert o.rel_l2(ref.apply(o.OP_M, got[r]), srcs[r]) < 1e-9
        assert o.rel_l2(got[r], x1) < 1e-7


def test_multi_rhs_cg_each_equals_single(gpu_available):
    """Batched CG keeps independent alpha/beta per right-hand side (CGmultiRHS semantics,
    BlockConjugateGradient.h:412-540): each result equals its own single solve."""
    dims = (4, 4, 4, 8)
    nrhs = 4
    U = g.random_gauge(dims, 0.5, 9)
    op = g.WilsonFermion(U, dims, 0.05, precision=g.F64, nrhs=nrhs)
    one = g.WilsonFermion(U, dims, 0.05, precision=g.F64, nrhs=1)
    nh = 256
    srcs = [fermion(nh, 1, 120 + r) for r in range(nrhs)]
    fs = op.FermionRedBlackField(1).import_(np.concatenate(srcs))
    fx = op.FermionRedBlackField(1).zero()
    cg = g.ConjugateGradient(1e-10, 5000)
    cg(g.SchurDiagMooeeOperator(op), fs, fx)
    got = fx.export().reshape(nrhs, -1)
    for r in range(nrhs):
        f1 = one.FermionRedBlackField(1).import_(srcs[r])
        x1 = one.FermionRedBlackField(1).zero()
        c1 = g.ConjugateGradient(1e-10, 5000)
        c1(g.SchurDiagMooeeOperator(one), f1, x1)
        # same iterates up to reduction-order rounding: iteration counts within one,
        # both true residuals below the tolerance, solutions equal to ~cond * 1e-10
        assert abs(cg.per_rhs_iterations[r] - c1.IterationsToComplete) <= 1
        assert cg.per_rhs_true_residual[r] < 1e-10 * 1.5 and c1.TrueResidual < 1e-10 * 1.5
        assert o.rel_l2(got[r], x1.export()) < 1e-8


@pytest.mark.parametrize("prec", [g.F64, g.F32])
@pytest.mark.parametrize("nrhs", [1, 2])
def test_dminus_and_physical_fields(gpu_available, prec, nrhs):
    """Dminus/DminusDag and the 4D <-> 5D surface fields (CayleyFermion5DImplementation.h:57-153)
    against the oracle, one right-hand side at a time for nrhs = 2."""
    dims, Ls = (4, 4, 4, 6), 8
    op, ref, U = mobius_pair(dims, Ls, 0.05, prec, nrhs=nrhs)
    vol = int(np.prod(dims))
    xs = [fermion(vol, Ls, 40 + r) for r in range(nrhs)]
    fin = op.FermionField().import_(np.concatenate(xs))
    fout = op.FermionField()
    for name, code in (("Dminus", o.OP_DMINUS), ("DminusDag", o.OP_DMINUS_DAG)):
        getattr(op, name)(fin, fout)
        got = fout.export().reshape(nrhs, -1)
        for r in range(nrhs):
            assert o.rel_l2(got[r], ref.apply(code, xs[r])) < TOL[prec], (name, r)
    etas = [fermion(vol, 1, 50 + r) for r in range(nrhs)]
    for fn, mode in ((op.ImportPhysicalFermionSource, o.IMPORT_PHYSICAL_SOURCE),
                     (op.ImportUnphysicalFermion, o.IMPORT_UNPHYSICAL)):
        fn(np.concatenate(etas), fout)
        got = fout.export().reshape(nrhs, -1)
        for r in range(nrhs):
            assert o.rel_l2(got[r], ref.physical(mode, etas[r])) < TOL[prec], (mode, r)
    for fn, mode in ((op.ExportPhysicalFermionSolution, o.EXPORT_PHYSICAL_SOLUTION),
                     (op.ExportPhysicalFermionSource, o.EXPORT_PHYSICAL_SOURCE)):
        got = fn(fin).reshape(nrhs, -1)
        for r in range(nrhs):
            assert o.rel_l2(got[r], ref.physical(mode, xs[r])) < TOL[prec], (mode, r)


def test_fields_shared_between_operators(gpu_available):
    """A field created on one operator works with another of the same geometry and stream
    (Grid fields belong to a grid), and is refused by an operator on another stream."""
    dims, Ls = (4, 4, 4, 4), 8
    op_a, _, U = mobius_pair(dims, Ls, 0.05, g.F64)
    op_b = g.MobiusFermion(U, dims, Ls, 0.2, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], precision=g.F64)
    ref_b = o.OracleOp(1, 0, dims, Ls, [0.2, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    x = fermion(int(np.prod(dims)), Ls, 60)
    fin = op_a.FermionField().import_(x)
    fout = op_a.FermionField()
    op_b.M(fin, fout)
    assert o.rel_l2(fout.export(), ref_b.apply(o.OP_M, x)) < TOL[g.F64]
    s = g.Stream()
    op_c = g.MobiusFermion(U, dims, Ls, 0.2, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], precision=g.F64, stream=s.ptr)
    with pytest.raises(g.GridError):
        op_c.M(fin, fout)
    del op_c


@pytest.mark.parametrize("prec", [g.F64, g.F32, g.F16])
@pytest.mark.parametrize("kind", ["wilson", "mobius"])
@pytest.mark.parametrize("antiperiodic", [True, False])
def test_recon12_links(gpu_available, prec, kind, antiperiodic):
    """12-real links (rows 0, 1 stored, row 2 rebuilt with the -1/2 and the boundary sign)
    give the same Dhop as the full links."""
    dims = (4, 6, 4, 8)
    ph = g.antiperiodic_t() if antiperiodic else g.periodic()
    U = g.random_gauge(dims, 0.5, 17)
    if kind == "wilson":
        op = g.WilsonFermion(U, dims, 0.1, phases=ph, precision=prec, flags=g.RECON12)
        ref = o.OracleOp(0, 0, dims, 1, [0.1], U, ph)
        L5 = 1
    else:
        op = g.MobiusFermion(U, dims, 8, 0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], phases=ph, precision=prec,
                             flags=g.RECON12)
        ref = o.OracleOp(1, 0, dims, 8, [0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, ph)
        L5 = 8
    tol = {g.F64: 1e-13, g.F32: 1e-6, g.F16: 3e-3}[prec]
    vol = int(np.prod(dims))
    x = fermion(vol, L5, 70)
    fin = op.FermionField().import_(x)
    fout = op.FermionField()
    for dag, code in ((0, o.OP_DHOP), (1, o.OP_DHOP_DAG)):
        op.Dhop(fin, fout, dag)
        assert o.rel_l2(fout.export(), ref.apply(code, x)) < tol, dag
    xh = fermion(vol // 2, L5, 71)
    out = op.FermionRedBlackField(g.EVEN)
    op.DhopEO(half(op, g.ODD, xh), out, 0)
    assert o.rel_l2(out.export(), ref.dhop_cb(xh, 1, 0)) < tol


def test_recon12_needs_real_phases(gpu_available):
    dims = (4, 4, 4, 4)
    ph = np.array([1, 0, 1, 0, 1, 0, 0, 1], dtype=np.float64)  # a complex phase in time
    with pytest.raises(g.GridError) as e:
        g.WilsonFermion(g.random_gauge(dims, 0.3, 1), dims, 0.1, phases=ph, flags=g.RECON12)
    assert e.value.status == 8


@pytest.mark.parametrize("prec", [g.F64, g.F32])
def test_axpby_norm_and_inner_product_norm(gpu_available, prec):
    """axpby_norm and innerProductNorm (Lattice_reduction.h:316-410) per right-hand side,
    against numpy on the values the fields hold."""
    dims, Ls, nrhs = (4, 4, 4, 4), 4, 2
    op, _, _ = mobius_pair(dims, Ls, 0.1, prec, nrhs=nrhs)
    vol = int(np.prod(dims))
    fx = op.FermionField().import_(fermion(vol * nrhs, Ls, 101))
    fy = op.FermionField().import_(fermion(vol * nrhs, Ls, 102))
    x = fx.export().reshape(nrhs, -1)
    y = fy.export().reshape(nrhs, -1)
    fz = op.FermionField()
    n = g.axpby_norm(fz, 0.5, -1.25, fx, fy)
    z = fz.export().reshape(nrhs, -1)
    tol = 1e-13 if prec == g.F64 else 1e-6
    assert o.rel_l2(z, 0.5 * x - 1.25 * y) < tol
    # FP32 fields: per-site products in FP32, sums in FP64
    rt = 1e-12 if prec == g.F64 else 1e-6
    for r in range(nrhs):
        assert abs(n[r] - np.vdot(z[r], z[r]).real) < rt * n[r]
    ip, nr = g.innerProductNorm(fx, fy)
    for r in range(nrhs):
        assert abs(ip[r] - np.vdot(x[r], y[r])) < rt * np.sqrt(nr[r] * np.vdot(y[r], y[r]).real)
        assert abs(nr[r] - np.vdot(x[r], x[r]).real) < rt * nr[r]
    assert np.allclose(g.rankInnerProduct(fx, fy), g.innerProduct(fx, fy))
