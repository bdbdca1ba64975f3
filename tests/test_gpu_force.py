"""Force terms on the GPU against the oracle (itself pinned as the link derivative of
<A|Dhop|B>): DhopDeriv on full fields, DhopDerivEO / DhopDerivOE on half fields, MDeriv of
Moebius (Meooe5D folded in) and Wilson operators, both daggers, FP64 (relative L2 1e-13)
and FP32 (1e-6), with full and 12-real links."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o
from tests._common import MOBIUS, fermion

pytestmark = pytest.mark.gpu

DIMS = (4, 4, 6, 4)
VOL = int(np.prod(DIMS))
TOL = {g.F64: 1e-13, g.F32: 1e-6}


def pick(dims, L5, parity, full):
    """the sites of one parity of a full canonical field, in site>>1 order"""
    f = full.reshape(int(np.prod(dims)), -1)
    idx = [s for s in range(f.shape[0]) if sum(np.unravel_index(s, dims[::-1])) % 2 == parity]
    return f[idx].reshape(-1)


def parity_mask(dims):
    return np.array([sum(np.unravel_index(s, dims[::-1])) % 2 for s in range(int(np.prod(dims)))])


@pytest.mark.parametrize("prec", [g.F64, g.F32])
@pytest.mark.parametrize("kind", ["wilson", "mobius"])
@pytest.mark.parametrize("flags", [0, g.RECON12])
def test_deriv_full_and_half(gpu_available, prec, kind, flags):
    U = g.random_gauge(DIMS, 0.5, 41)
    ph = g.antiperiodic_t()
    if kind == "wilson":
        op = g.WilsonFermion(U, DIMS, 0.1, precision=prec, flags=flags)
        ref = o.OracleOp(0, 0, DIMS, 1, [0.1], U, ph)
        L5 = 1
    else:
        op = g.MobiusFermion(U, DIMS, 6, 0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], precision=prec, flags=flags)
        ref = o.OracleOp(1, 0, DIMS, 6, [0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"]], U, ph)
        L5 = 6
    A, B = fermion(VOL, L5, 42), fermion(VOL, L5, 43)
    fa, fb = op.FermionField().import_(A), op.FermionField().import_(B)
    par = parity_mask(DIMS)
    for dag in (0, 1):
        for name, mder in (("DhopDeriv", False), ("MDeriv", True)):
            got = getattr(op, name)(fa, fb, dag)
            want = ref.deriv(A, B, dag, mderiv=mder)
            assert o.rel_l2(got, want) < TOL[prec], (name, dag)
            # the checkerboarded forms: A on parity p, B on 1 - p
            for p in (0, 1):
                ha = op.FermionRedBlackField(p).import_(pick(DIMS, L5, p, A))
                hb = op.FermionRedBlackField(1 - p).import_(pick(DIMS, L5, 1 - p, B))
                Ap = np.where(np.repeat(par == p, L5 * 12), A, 0)
                Bq = np.where(np.repeat(par == 1 - p, L5 * 12), B, 0)
                w = ref.deriv(Ap, Bq, dag, mderiv=mder, out_parity=p)
                got_h = getattr(op, name)(ha, hb, dag)
                assert o.rel_l2(got_h, pick(DIMS, 1, p, w)) < TOL[prec], (name, dag, p)
