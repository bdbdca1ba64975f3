"""ZMobius (complex omega_s; ZMobiusFermion.h) on the GPU against the oracle, with the
Ls = 10 omegas of Grid's tests/core/Test_zmobius_even_odd.cc: every Cayley operator, the
Schur operator, Dminus, M / Mdag, and a Schur red-black CG solve, FP64 (relative L2
1e-13) and FP32 (1e-6)."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o
from tests._common import fermion
from tests.test_oracle_pins import ZOMEGA, zparams

pytestmark = pytest.mark.gpu

DIMS = (4, 4, 4, 6)
VOL = int(np.prod(DIMS))
M5 = 1.8


def pair(prec, gamma=ZOMEGA, b=1.0, c=0.0, mf=0.05):
    U = g.random_gauge(DIMS, 0.5, 61)
    op = g.ZMobiusFermion(U, DIMS, gamma, mf, M5, b, c, precision=prec)
    ref = o.OracleOp(2, 0, DIMS, len(gamma), zparams(mf, M5, b, c, gamma), U, g.antiperiodic_t())
    return op, ref


@pytest.mark.parametrize("prec", [g.F64, g.F32])
def test_zmobius_operators(gpu_available, prec):
    op, ref = pair(prec)
    Ls = len(ZOMEGA)
    tol = {g.F64: 1e-13, g.F32: 1e-6}[prec]
    x = fermion(VOL, Ls, 62)
    fin, fout = op.FermionField().import_(x), op.FermionField()
    for name, code in (("M", o.OP_M), ("Mdag", o.OP_MDAG), ("MdagM", o.OP_MDAGM), ("Dminus", o.OP_DMINUS),
                       ("DminusDag", o.OP_DMINUS_DAG)):
        getattr(op, name)(fin, fout)
        assert o.rel_l2(fout.export(), ref.apply(code, x)) < 10 * tol, name
    xh = fermion(VOL // 2, Ls, 63)
    for name, code in (("Mooee", o.OP_MOOEE), ("MooeeDag", o.OP_MOOEE_DAG), ("MooeeInv", o.OP_MOOEE_INV),
                       ("MooeeInvDag", o.OP_MOOEE_INV_DAG), ("Meooe", o.OP_MEOOE), ("MeooeDag", o.OP_MEOOE_DAG),
                       ("Mpc", o.OP_MPC), ("MpcDag", o.OP_MPC_DAG), ("MpcDagMpc", o.OP_MPCDAGMPC)):
        hin = op.FermionRedBlackField(g.ODD).import_(xh)
        hout = op.FermionRedBlackField(g.ODD)
        getattr(op, name)(hin, hout)
        assert o.rel_l2(hout.export(), ref.apply(code, xh, 1)) < 10 * tol, name


@pytest.mark.parametrize("prec", [g.F64, g.F32])
def test_zmobius_physical_fields_and_force(gpu_available, prec):
    """ImportPhysicalFermionSource (Dminus with complex cs), the exports, and MDeriv with the
    complex Meooe5D folded in."""
    op, ref = pair(prec)
    Ls = len(ZOMEGA)
    tol = {g.F64: 1e-13, g.F32: 1e-6}[prec]
    eta = fermion(VOL, 1, 65)
    fout = op.FermionField()
    for fn, mode in ((op.ImportPhysicalFermionSource, o.IMPORT_PHYSICAL_SOURCE),
                     (op.ImportUnphysicalFermion, o.IMPORT_UNPHYSICAL)):
        fn(eta, fout)
        assert o.rel_l2(fout.export(), ref.physical(mode, eta)) < 10 * tol, mode
    A, B = fermion(VOL, Ls, 66), fermion(VOL, Ls, 67)
    fa, fb = op.FermionField().import_(A), op.FermionField().import_(B)
    assert o.rel_l2(op.ExportPhysicalFermionSolution(fa), ref.physical(o.EXPORT_PHYSICAL_SOLUTION, A)) < tol
    for dag in (0, 1):
        assert o.rel_l2(op.MDeriv(fa, fb, dag), ref.deriv(A, B, dag, mderiv=True)) < 10 * tol, dag


def test_zmobius_schur_solve(gpu_available):
    op, ref = pair(g.F64)
    Ls = len(ZOMEGA)
    src = fermion(VOL, Ls, 64)
    fs, fx = op.FermionField().import_(src), op.FermionField().zero()
    cg = g.ConjugateGradient(1e-10, 5000)
    g.SchurRedBlackDiagMooeeSolve(cg)(op, fs, fx)
    x = fx.export()
    assert o.rel_l2(ref.apply(o.OP_M, x), src) < 1e-9


def test_zmobius_rejects_fp16(gpu_available):
    with pytest.raises(g.GridError):
        g.ZMobiusFermion(g.random_gauge(DIMS, 0.5, 1), DIMS, ZOMEGA, 0.05, M5, 1.0, 0.0, precision=g.F16)
    op, _ = pair(g.F64)
    with pytest.raises(g.GridError):
        op.cayley_coeffs()


def test_zolotarev_and_scaled_shamir_operators(gpu_available):
    """MobiusZolotarevFermion = the Cayley operator with omega_s = hi * gamma_s of
    zolotarev(lo / hi, Ls, 0); ScaledShamirFermion = Moebius with b + c = scale, b - c = 1:
    both against the oracle, and a Schur solve of the Zolotarev operator."""
    U = g.random_gauge(DIMS, 0.5, 61)
    Ls, lo, hi = 8, 0.1, 2.0
    op = g.MobiusZolotarevFermion(U, DIMS, Ls, 0.05, M5, 1.5, 0.5, lo, hi)
    gamma, _ = g.zolotarev(lo / hi, Ls)
    ref = o.OracleOp(2, 0, DIMS, Ls, zparams(0.05, M5, 1.5, 0.5, list(hi * gamma)), U, g.antiperiodic_t())
    x = fermion(VOL, Ls, 68)
    fin, fout = op.FermionField().import_(x), op.FermionField()
    for name, code in (("M", o.OP_M), ("Mdag", o.OP_MDAG)):
        getattr(op, name)(fin, fout)
        assert o.rel_l2(fout.export(), ref.apply(code, x)) < 1e-12, name
    fx = op.FermionField().zero()
    g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-10, 5000))(op, fin, fx)
    assert o.rel_l2(ref.apply(o.OP_M, fx.export()), x) < 1e-9
    sh = g.ScaledShamirFermion(U, DIMS, Ls, 0.05, M5, 2.0)
    ref2 = o.OracleOp(1, 0, DIMS, Ls, [0.05, M5, 1.5, 0.5], U, g.antiperiodic_t())
    sh.M(fin, fout)
    assert o.rel_l2(fout.export(), ref2.apply(o.OP_M, x)) < 1e-13
