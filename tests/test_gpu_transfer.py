"""Host transfers on the GPU: the single-precision canonical form (gb_field_import_f32 /
export_f32) and the transfer queue (gb_xfer_*), whose imports and exports overlap each
other and the operator's kernels.  Results must equal the synchronous path bit for bit."""
import numpy as np
import pytest

import grid_gb300 as g
from tests._common import MOBIUS, fermion

pytestmark = pytest.mark.gpu

DIMS = (4, 4, 4, 8)
VOL = 512
LS = 8


def make(prec, nrhs=1):
    U = g.random_gauge(DIMS, 0.5, 71)
    return g.MobiusFermion(U, DIMS, LS, 0.05, MOBIUS["M5"], MOBIUS["b"], MOBIUS["c"], precision=prec, nrhs=nrhs)


@pytest.mark.parametrize("prec", [g.F64, g.F32, g.F16])
def test_f32_host_form(gpu_available, prec):
    op = make(prec)
    x = fermion(VOL, LS, 72).astype(np.complex64)
    a = op.FermionField().import_f32(x)
    b = op.FermionField().import_(x.astype(np.complex128))
    assert np.array_equal(a.export(), b.export())
    assert np.array_equal(a.export_f32(), a.export().astype(np.complex64))
    if prec != g.F16:  # FP16 storage rounds
        assert np.array_equal(a.export_f32(), x)
    h = op.FermionRedBlackField(g.ODD).import_f32(x[: x.size // 2])
    hb = op.FermionRedBlackField(g.ODD).import_(x[: x.size // 2].astype(np.complex128))
    assert np.array_equal(h.export(), hb.export())
    with pytest.raises(g.GridError):
        op.FermionField().import_f32(x[:-1])


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("nrhs", [1, 2])
def test_transfer_queue_pipeline_matches_synchronous_path(gpu_available, dtype, nrhs):
    op = make(g.F32, nrhs)
    n = VOL * LS * 12 * nrhs
    steps = 5
    ins = [g.PinnedArray(n, dtype) for _ in range(steps)]
    outs = [g.PinnedArray(n, dtype) for _ in range(steps)]
    for i in range(steps):
        ins[i].array[:] = fermion(VOL * nrhs, LS, 80 + i).astype(dtype)
    q = g.TransferQueue(op)
    fin, fout = op.FermionField(), op.FermionField()
    for i in range(steps):  # nothing waits between steps: the copies overlap
        q.import_(fin, ins[i].array)
        op.Dhop(fin, fout, 0)
        q.export(fout, outs[i].array)
    q.wait()
    sin, sout = op.FermionField(), op.FermionField()
    for i in range(steps):
        if dtype == np.complex64:
            sin.import_f32(ins[i].array)
            op.Dhop(sin, sout, 0)
            want = sout.export_f32()
        else:
            sin.import_(ins[i].array)
            op.Dhop(sin, sout, 0)
            want = sout.export()
        assert np.array_equal(outs[i].array, want), i
    with pytest.raises(g.GridError):
        q.import_(fin, np.zeros(n - 1, dtype=dtype))
