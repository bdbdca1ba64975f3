"""FP64 operators created with GB_FLAG_DF64: the hopping term runs in double-float
arithmetic (pairs of floats) on the FP32 pipes, fields stay FP64.  Against the oracle's
FP64 operators on the same seeded inputs, every Dhop form and every composite built on it
keeps the FP64 bound of the parity tests (relative L2 1e-13); the Schur CG converges in
the oracle's iteration count, a mixed-precision solve with a DF64 outer operator reaches
the true residual 1e-10, and the flag is refused where it does not apply."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o
from tests._common import MOBIUS, fermion

pytestmark = pytest.mark.gpu

TOL = 1e-13


def pair(kind, dims, flags=g.DF64, precision=g.F64, L5=8, mass=0.05, seed=31):
    U = g.random_gauge(dims, 0.5, seed)
    ph = g.antiperiodic_t()
    if kind == "wilson":
        op = g.WilsonFermion(U, dims, mass, phases=ph, precision=precision, flags=flags)
        ref = o.OracleOp(0, 0, dims, 1, [mass], U, ph)
        return op, ref, 1, U
    op = g.MobiusFermion(U, dims, L5, mass, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], phases=ph, precision=precision,
                         flags=flags)
    ref = o.OracleOp(1, 0, dims, L5, [mass, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, ph)
    return op, ref, L5, U


@pytest.mark.parametrize("kind,dims", [("wilson", (8, 8, 8, 8)), ("wilson", (6, 4, 2, 10)), ("mobius", (4, 4, 4, 8)),
                                       ("mobius", (4, 6, 4, 4))])
def test_df64_operators(gpu_available, kind, dims):
    op, ref, L5, U = pair(kind, dims)
    vol = int(np.prod(dims))
    for in_cb in (1, 0):
        x = fermion(vol // 2, L5, 40 + in_cb)
        fin = op.FermionRedBlackField(in_cb).import_(x)
        fout = op.FermionRedBlackField(1 - in_cb)
        for dag in (0, 1):
            (op.DhopEO if in_cb == 1 else op.DhopOE)(fin, fout, dag)
            assert o.rel_l2(fout.export(), ref.dhop_cb(x, in_cb, dag)) < TOL, (in_cb, dag)
    x = fermion(vol, L5, 42)
    fin, fout = op.FermionField().import_(x), op.FermionField()
    for name, code in (("M", o.OP_M), ("Mdag", o.OP_MDAG), ("MdagM", o.OP_MDAGM)):
        getattr(op, name)(fin, fout)
        assert o.rel_l2(fout.export(), ref.apply(code, x)) < TOL, name
    for dag, code in ((0, o.OP_DHOP), (1, o.OP_DHOP_DAG)):
        op.Dhop(fin, fout, dag)
        assert o.rel_l2(fout.export(), ref.apply(code, x)) < TOL, dag
    xh = fermion(vol // 2, L5, 43)
    for name, code in (("Meooe", o.OP_MEOOE), ("Mpc", o.OP_MPC), ("MpcDag", o.OP_MPC_DAG),
                       ("MpcDagMpc", o.OP_MPCDAGMPC)):
        fin = op.FermionRedBlackField(g.ODD).import_(xh)
        fout = op.FermionRedBlackField(g.EVEN if name == "Meooe" else g.ODD)
        getattr(op, name)(fin, fout)
        assert o.rel_l2(fout.export(), ref.apply(code, xh, 1)) < TOL, name


def test_df64_matches_native_fp64(gpu_available):
    """The double-float Dhop differs from the native FP64 kernel by its ~2^-48 rounding."""
    dims = (8, 8, 8, 8)
    a, _, L5, U = pair("mobius", dims, L5=12)
    b, _, _, _ = pair("mobius", dims, flags=0, L5=12)
    vol = int(np.prod(dims))
    x = fermion(vol // 2, L5, 44)
    outs = []
    for op in (a, b):
        fin = op.FermionRedBlackField(g.ODD).import_(x)
        fout = op.FermionRedBlackField(g.EVEN)
        op.DhopEO(fin, fout, 0)
        outs.append(fout.export())
    assert 0 < o.rel_l2(outs[0], outs[1]) < 2e-14


def test_df64_schur_solve(gpu_available):
    dims, Ls = (4, 4, 4, 8), 8
    op, ref, _, U = pair("mobius", dims, L5=Ls, mass=0.01)
    src = fermion(512, Ls, 100)
    fs = op.FermionField().import_(src)
    fx = op.FermionField().zero()
    solver = g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(1e-10, 5000))
    solver(op, fs, fx)
    x = fx.export()
    xr, it, r_cg, r_un = ref.schur_solve(src, 1e-10, 5000)
    assert abs(solver.solver.IterationsToComplete - it) <= 2
    assert o.rel_l2(ref.apply(o.OP_M, x), src) < 1e-9
    assert o.rel_l2(x, xr) < 1e-8


def test_df64_outer_operator_of_the_mixed_solve(gpu_available):
    """FP32 inner CG, DF64 outer operator for the reliable updates: true residual 1e-10 as
    measured by the oracle's FP64 operator."""
    dims, Ls = (4, 4, 4, 8), 8
    U = g.random_gauge(dims, 0.6, 5)
    od = g.MobiusFermion(U, dims, Ls, 0.01, 1.8, 1.5, 0.5, precision=g.F64, flags=g.DF64)
    of = g.MobiusFermion(U, dims, Ls, 0.01, 1.8, 1.5, 0.5, precision=g.F32)
    ref = o.OracleOp(1, 0, dims, Ls, [0.01, 1.8, 1.5, 0.5], U, g.antiperiodic_t())
    src = fermion(512, Ls, 110)
    fs = od.FermionField().import_(src)
    fx = od.FermionField().zero()
    cg = g.ConjugateGradientReliableUpdate(1e-10, 20000, 1e-6, g.SchurDiagMooeeOperator(of),
                                           g.SchurDiagMooeeOperator(od), relup_every=100)
    g.SchurRedBlackDiagMooeeSolve(cg)(od, fs, fx)
    x = fx.export()
    assert cg.TrueResidual < 1e-10 and cg.ReliableUpdatesPerformed >= 1
    assert o.rel_l2(ref.apply(o.OP_M, x), src) < 1e-9


@pytest.mark.parametrize("precision,flags", [(g.F32, g.DF64), (g.F16, g.DF64), (g.F64, g.DF64 | g.RECON12)])
def test_df64_flag_is_refused_where_it_does_not_apply(gpu_available, precision, flags):
    dims = (4, 4, 4, 4)
    with pytest.raises(g.GridError) as e:
        g.WilsonFermion(g.random_gauge(dims, 0.3, 1), dims, 0.1, precision=precision, flags=flags)
    assert e.value.status == 8
