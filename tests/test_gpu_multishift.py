"""ConjugateGradientMultiShift on the GPU against the oracle's restatement of Grid's
recurrence (ConjugateGradientMultiShift.h:76-330) on the same seeded inputs: per-shift
solutions agree to relative L2 1e-8 (FP64) and every true residual |(A + m_s) x_s - b|/|b|,
measured with the oracle's FP64 operator, meets its tolerance; iteration counts match the
oracle's within one check interval's worth of rounding (+-1)."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o
from tests._common import MOBIUS, fermion

pytestmark = pytest.mark.gpu


def _solve(linop, src, shifts, tols, maxit=3000):
    psi = [linop.op.FermionField() if src.checkerboard == g.FULL else linop.op.FermionRedBlackField(g.ODD)
           for _ in shifts]
    cg = g.ConjugateGradientMultiShift(maxit, g.MultiShiftFunction(shifts, tolerances=tols), check_every=5)
    cg(linop, src, psi)
    return cg, [f.export() for f in psi]


def test_multishift_wilson_mdagm_fp64(gpu_available):
    dims, mass = (8, 8, 8, 8), 0.1
    U = g.random_gauge(dims, 0.3, 5)
    op = g.WilsonFermion(U, dims, mass, precision=g.F64)
    ref = o.OracleOp(0, 0, dims, 1, [mass], U, g.antiperiodic_t())
    eta = g.random_gaussian(4096 * 12, 6)
    shifts, tols = [0.0, 0.02, 0.2, 2.0], [1e-10, 1e-10, 1e-11, 1e-12]
    cg, xs = _solve(g.MdagMLinearOperator(op), op.FermionField().import_(eta), shifts, tols)
    rx, it, conv, its, res = ref.cg_multishift(0, eta, shifts, tols, 3000)
    assert conv == 1 and abs(cg.IterationsToComplete - it) <= 1
    for k, s in enumerate(shifts):
        assert abs(cg.IterationsToCompleteShift[k] - its[k]) <= 1
        assert cg.TrueResidualShift[k] < 1.5 * tols[k]
        r = o.rel_l2(ref.apply(o.OP_MDAGM, xs[k]) + s * xs[k], eta)
        assert r < 1.5 * tols[k], (s, r)
        assert o.rel_l2(xs[k], rx[k]) < 1e-8, s


@pytest.mark.parametrize("prec", [g.F64, g.F32])
def test_multishift_mobius_schur(gpu_available, prec):
    dims, Ls, mf = (4, 4, 4, 8), 8, 0.05
    U = g.random_gauge(dims, 0.5, 7)
    op = g.MobiusFermion(U, dims, Ls, mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], precision=prec)
    ref = o.OracleOp(1, 0, dims, Ls, [mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    eta = fermion(int(np.prod(dims)) // 2, Ls, 8)
    src = op.FermionRedBlackField(g.ODD).import_(eta)
    shifts = [0.0, 0.01, 0.1, 0.5, 1.0]
    tol = 1e-10 if prec == g.F64 else 1e-5
    cg, xs = _solve(g.SchurDiagMooeeOperator(op), src, shifts, [tol] * len(shifts))
    rx, it, conv, its, res = ref.cg_multishift(1, eta, shifts, [tol] * len(shifts), 3000)
    for k, s in enumerate(shifts):
        r = o.rel_l2(ref.apply(o.OP_MPCDAGMPC, xs[k], 1) + s * xs[k], eta)
        assert r < (1.5 * tol if prec == g.F64 else 1e-4), (s, r)
        assert o.rel_l2(xs[k], rx[k]) < (1e-8 if prec == g.F64 else 1e-4), s
    if prec == g.F64:
        assert abs(cg.IterationsToComplete - it) <= 1


def test_multishift_rational_sum(gpu_available):
    """psi = norm src + sum_s residues[s] (A + poles[s])^-1 src (the RHMC use)."""
    dims, mass = (4, 4, 4, 4), 0.2
    U = g.random_gauge(dims, 0.3, 9)
    op = g.WilsonFermion(U, dims, mass, precision=g.F64)
    ref = o.OracleOp(0, 0, dims, 1, [mass], U, g.antiperiodic_t())
    eta = g.random_gaussian(256 * 12, 10)
    f = g.MultiShiftFunction([0.01, 0.1, 1.0], residues=[0.5, 0.25, 2.0], tolerances=1e-11, norm=0.3)
    out = op.FermionField()
    g.ConjugateGradientMultiShift(2000, f)(g.MdagMLinearOperator(op), op.FermionField().import_(eta), out)
    rx, *_ = ref.cg_multishift(0, eta, f.poles, f.tolerances, 2000)
    want = f.norm * eta + sum(r * x for r, x in zip(f.residues, rx))
    assert o.rel_l2(out.export(), want) < 1e-9


def test_multishift_rejects_bad_shifts(gpu_available):
    dims = (4, 4, 4, 4)
    op = g.WilsonFermion(g.random_gauge(dims, 0.3, 1), dims, 0.1, precision=g.F64)
    src = op.FermionField().import_(g.random_gaussian(256 * 12, 2))
    with pytest.raises(g.GridError):  # the primary shift must be the lightest
        _solve(g.MdagMLinearOperator(op), src, [0.1, 0.0], [1e-8, 1e-8])
