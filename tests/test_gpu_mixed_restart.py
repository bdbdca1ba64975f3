"""MixedPrecisionConjugateGradient (ConjugateGradientMixedPrec.h:34-166) on the GPU: FP32
inner CGs restarted from FP64 residuals, then the FP64 patch-up CG.  The solution equals
the oracle's FP64 CG solution and its true residual (the oracle's operator) meets the
tolerance; with nrhs = 2 operators (the batched form) every right-hand side does."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o
from tests._common import MOBIUS, fermion

pytestmark = pytest.mark.gpu


def test_mixed_restart_schur_mobius(gpu_available):
    dims, Ls, mf = (4, 4, 4, 8), 8, 0.02
    U = g.random_gauge(dims, 0.5, 91)
    od = g.MobiusFermion(U, dims, Ls, mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], precision=g.F64)
    of = g.MobiusFermion(U, dims, Ls, mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], precision=g.F32)
    ref = o.OracleOp(1, 0, dims, Ls, [mf, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, g.antiperiodic_t())
    vol = int(np.prod(dims))
    src = fermion(vol // 2, Ls, 92)
    fs = od.FermionRedBlackField(g.ODD).import_(src)
    fx = od.FermionRedBlackField(g.ODD).zero()
    cg = g.MixedPrecisionConjugateGradient(1e-10, 10000, 50, None, g.SchurDiagMooeeOperator(of),
                                           g.SchurDiagMooeeOperator(od))
    cg(fs, fx)
    assert cg.TotalOuterIterations >= 1 and cg.TotalInnerIterations > 0
    x = fx.export()
    assert o.rel_l2(ref.apply(o.OP_MPCDAGMPC, x, 1), src) < 1.5e-10
    want, _, _ = ref.cg(1, src, 1e-11, 10000)
    assert o.rel_l2(x, want) < 1e-8
    assert cg.TrueResidual < 1.5e-10


def test_mixed_restart_batched_wilson(gpu_available):
    dims, mass, nrhs = (4, 4, 4, 8), 0.05, 2
    U = g.random_gauge(dims, 0.3, 93)
    od = g.WilsonFermion(U, dims, mass, precision=g.F64, nrhs=nrhs)
    of = g.WilsonFermion(U, dims, mass, precision=g.F32, nrhs=nrhs)
    ref = o.OracleOp(0, 0, dims, 1, [mass], U, g.antiperiodic_t())
    vol = int(np.prod(dims))
    srcs = [fermion(vol, 1, 94 + r) for r in range(nrhs)]
    fs = od.FermionField().import_(np.concatenate(srcs))
    fx = od.FermionField().zero()
    cg = g.MixedPrecisionConjugateGradientBatched(1e-10, 10000, 50, None, g.MdagMLinearOperator(of),
                                                  g.MdagMLinearOperator(od))
    cg(fs, fx)
    got = fx.export().reshape(nrhs, -1)
    for r in range(nrhs):
        assert o.rel_l2(ref.apply(o.OP_MDAGM, got[r]), srcs[r]) < 1.5e-10, r


def test_mixed_restart_rejects_fp16_inner(gpu_available):
    dims = (4, 4, 4, 4)
    U = g.random_gauge(dims, 0.3, 95)
    od = g.WilsonFermion(U, dims, 0.1, precision=g.F64)
    oh = g.WilsonFermion(U, dims, 0.1, precision=g.F16)
    fs, fx = od.FermionField().import_(fermion(256, 1, 96)), od.FermionField().zero()
    with pytest.raises(g.GridError):
        g.MixedPrecisionConjugateGradient(1e-10, 1000, 10, None, g.MdagMLinearOperator(oh),
                                          g.MdagMLinearOperator(od))(fs, fx)
