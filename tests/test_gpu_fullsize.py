"""Parity at the workloads' full sizes, against the oracle on the same seeded inputs.

The small-volume parity tests pin the arithmetic; these run the CUDA path at the sizes
the benchmarks quote, where field offsets pass 2^31 bytes and grids span many waves:
- Moebius 16^4 x Ls16 (b 1.5, c 0.5, M5 1.8, mf 0.01, eps 0.5), FP64 and FP32: DhopEO,
  DhopOE and the full Dhop with and without dagger, Mooee, MooeeInv and their daggers,
  MpcDagMpc;
- Moebius 24^4 x Ls12 (mf 0.005, eps 0.6), FP32: the full Dhop and MpcDagMpc, and the
  mixed-precision red-black solve to a true residual of 1e-10 measured with the oracle's
  FP64 operator (the assertion of Grid's tests/Test_dwf_mixedcg_prec.cc);
- Wilson 32^3 x 64 (m 0.02, eps 0.5), 16 right-hand sides in one FP32 field: DhopEO of
  every right-hand side against the oracle's single-field DhopEO.
Tolerances (relative L2): FP64 1e-13, FP32 1e-6 per operator, ten times that for
MpcDagMpc (four hops and the 5D programs)."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o
from tests._common import MOBIUS, fermion

pytestmark = pytest.mark.gpu

TOL = {g.F64: 1e-13, g.F32: 1e-6}


def _rounded(x, prec):
    """The input as the operator stores it (FP32 fields hold the rounded values)."""
    return x.astype(np.complex64).astype(np.complex128) if prec == g.F32 else x


@pytest.mark.parametrize("prec", [g.F64, g.F32])
def test_mobius_16x16_operators(gpu_available, prec):
    dims, Ls, mf = (16, 16, 16, 16), 16, 0.01
    U = g.random_gauge(dims, 0.5, 201)
    op = g.MobiusFermion(U, dims, Ls, mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], precision=prec)
    ref = o.OracleOp(1, 0, dims, Ls, [mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    vol = int(np.prod(dims))
    x = _rounded(fermion(vol, Ls, 202), prec)
    fin = op.FermionField().import_(x)
    fout = op.FermionField()
    for dag, code in ((0, o.OP_DHOP), (1, o.OP_DHOP_DAG)):
        op.Dhop(fin, fout, dag)
        assert o.rel_l2(fout.export(), ref.apply(code, x)) < TOL[prec], ("Dhop", dag)
    del fin, fout
    for cb in (1, 0):
        h = _rounded(fermion(vol // 2, Ls, 203 + cb), prec)
        hin = op.FermionRedBlackField(cb).import_(h)
        hout = op.FermionRedBlackField(1 - cb)
        for dag in (0, 1):
            (op.DhopEO if cb == 1 else op.DhopOE)(hin, hout, dag)
            assert o.rel_l2(hout.export(), ref.dhop_cb(h, cb, dag)) < TOL[prec], ("Dhop cb", cb, dag)
    h = _rounded(fermion(vol // 2, Ls, 205), prec)
    hin = op.FermionRedBlackField(1).import_(h)
    hout = op.FermionRedBlackField(1)
    for name, code, tol in (("Mooee", o.OP_MOOEE, 1), ("MooeeDag", o.OP_MOOEE_DAG, 1),
                            ("MooeeInv", o.OP_MOOEE_INV, 1), ("MooeeInvDag", o.OP_MOOEE_INV_DAG, 1),
                            ("MpcDagMpc", o.OP_MPCDAGMPC, 10)):
        getattr(op, name)(hin, hout)
        assert o.rel_l2(hout.export(), ref.apply(code, h, 1)) < TOL[prec] * tol, name


def test_mobius_24x12_operators_and_mixed_solve(gpu_available):
    dims, Ls, mf = (24, 24, 24, 24), 12, 0.005
    U = g.random_gauge(dims, 0.6, 211)
    params = (mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"])
    of = g.MobiusFermion(U, dims, Ls, *params, precision=g.F32)
    ref = o.OracleOp(1, 0, dims, Ls, list(params), U, g.antiperiodic_t())
    vol = int(np.prod(dims))
    x = _rounded(fermion(vol, Ls, 212), g.F32)
    fin = of.FermionField().import_(x)
    fout = of.FermionField()
    of.Dhop(fin, fout, 0)
    assert o.rel_l2(fout.export(), ref.apply(o.OP_DHOP, x)) < TOL[g.F32]
    del fin, fout
    h = _rounded(fermion(vol // 2, Ls, 213), g.F32)
    hin = of.FermionRedBlackField(1).import_(h)
    hout = of.FermionRedBlackField(1)
    of.MpcDagMpc(hin, hout)
    assert o.rel_l2(hout.export(), ref.apply(o.OP_MPCDAGMPC, h, 1)) < TOL[g.F32] * 10
    del hin, hout

    od = g.MobiusFermion(U, dims, Ls, *params, precision=g.F64)
    src = fermion(vol, Ls, 214)
    fs = od.FermionField().import_(src)
    fx = od.FermionField().zero()
    cg = g.ConjugateGradientReliableUpdate(1e-10, 20000, 1e-6, g.SchurDiagMooeeOperator(of),
                                           g.SchurDiagMooeeOperator(od), relup_every=100)
    g.SchurRedBlackDiagMooeeSolve(cg)(od, fs, fx)
    assert cg.TrueResidual < 1e-10
    assert cg.ReliableUpdatesPerformed >= 1
    # the red-black solve returns the unpreconditioned solution: |M x - b| / |b| in FP64
    assert o.rel_l2(ref.apply(o.OP_M, fx.export()), src) < 1e-9


def test_wilson_32x64_16rhs_dhop(gpu_available):
    dims, nrhs, mass = (32, 32, 32, 64), 16, 0.02
    U = g.random_gauge(dims, 0.5, 221)
    op = g.WilsonFermion(U, dims, mass, precision=g.F32, nrhs=nrhs)
    single = o.OracleOp(0, 0, dims, 1, [mass], U, g.antiperiodic_t())
    nh = int(np.prod(dims)) // 2
    per = nh * 12
    x = np.empty(nrhs * per, dtype=np.complex64)  # 1.6 GB of canonical FP32 host data
    for r in range(nrhs):
        x[r * per:(r + 1) * per] = g.random_gaussian(per, 230 + r)
    fin = op.FermionRedBlackField(1).import_f32(x)
    fout = op.FermionRedBlackField(0)
    op.DhopEO(fin, fout, 0)
    got = fout.export_f32()
    del fin, fout
    for r in range(nrhs):
        want = single.dhop_cb(x[r * per:(r + 1) * per].astype(np.complex128), 1)
        assert o.rel_l2(got[r * per:(r + 1) * per].astype(np.complex128), want) < TOL[g.F32], r


@pytest.mark.parametrize("inner", [g.F32, g.F16])
def test_mixed_schur_solution_vs_oracle_fp64_12x12(gpu_available, inner):
    """The config of the mixed-precision benchmark (Moebius, Ls = 12, mf = 0.005, gauge
    eps = 0.6, reliable updates every 100 iterations or when |r| drops by 1e-3) at 12^4,
    the largest lattice whose FP64 oracle solve fits the test's time: the mixed solve
    reaches a Schur-system true residual of 1e-10, and its error against the oracle's
    FP64 solution is stated.  The oracle's red-black CG starts from the GPU's solution and
    runs to 1e-12 (the start changes its work, not what it converges to), so the
    difference is the GPU solution's error to within the oracle's own 1e-12 residual.
    Measured on GB300: 5.0e-9 (FP32 inner) and 4.6e-9 (FP16 inner); a 1e-10 residual on
    this operator allows errors of that size (the oracle's own 1e-10 and 1e-12 solutions
    at 8^4 differ by 3.2e-9).  The bound is 2e-8."""
    dims, Ls, mf = (12, 12, 12, 12), 12, 0.005
    U = g.random_gauge(dims, 0.6, 311)
    params = (mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"])
    od = g.MobiusFermion(U, dims, Ls, *params, precision=g.F64)
    of = g.MobiusFermion(U, dims, Ls, *params, precision=inner)
    ref = o.OracleOp(1, 0, dims, Ls, list(params), U, g.antiperiodic_t())
    src = fermion(int(np.prod(dims)), Ls, 312)
    fs = od.FermionField().import_(src)
    fx = od.FermionField().zero()
    cg = g.ConjugateGradientReliableUpdate(1e-10, 30000, 1e-6, g.SchurDiagMooeeOperator(of),
                                           g.SchurDiagMooeeOperator(od), relup_every=100)
    solver = g.SchurRedBlackDiagMooeeSolve(cg)
    solver(od, fs, fx)
    x = fx.export()
    assert cg.TrueResidual < 1e-10
    xr, it, r_cg, r_un = ref.schur_solve(src, 1e-12, 5000, guess=x)
    assert r_cg < 1e-12
    err = o.rel_l2(x, xr)
    print(f"12^4x12 mixed ({'fp32' if inner == g.F32 else 'fp16'} inner): {cg.IterationsToComplete} iterations, "
          f"Schur residual {cg.TrueResidual:.2e}, unpreconditioned {solver.unprec_residual[0]:.2e}, "
          f"error vs the oracle FP64 solution {err:.2e} (oracle: {it} more iterations from the GPU solution)")
    assert err < 2e-8
