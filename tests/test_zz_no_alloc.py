"""gb_field_norm2_noalloc through the C ABI: the allocation-free norm2 for callers that
may not call cudaMalloc/cudaFree while they run (a solve under a fixed HBM budget, or a
thread where allocator calls are forbidden or would stall the device).  It must give the
same per-rhs norms as the allocating gb_field_norm2, on consecutive calls that share the
static scratch array.  This file is collected last so that a run stopping at the first
failure has run every other test already."""
import ctypes as C

import numpy as np
import pytest

import grid_gb300 as g

pytestmark = pytest.mark.gpu

g.lib.gb_field_norm2_noalloc.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
g.lib.gb_field_norm2_noalloc.restype = C.c_int

REL_TOL = {g.F64: 1e-12, g.F32: 1e-6, g.F16: 1e-6}


def noalloc_norm2(f):
    out = np.zeros(f.op.nrhs, dtype=np.float64)
    rc = g.lib.gb_field_norm2_noalloc(f.h, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0, g.lib.gb_last_error()
    return out


def test_noalloc_norm2_matches_norm2_on_consecutive_calls(gpu_available):
    dims = (8, 8, 8, 8)
    U = g.random_gauge(dims, 0.5, 3)
    cases = []
    # a large FP64 full field, then a small FP32 half field with 3 rhs, then FP16:
    # the second and third calls see the first call's partial sums in the shared array
    op1 = g.MobiusFermion(U, dims, 8, 0.01, 1.8, 1.5, 0.5, precision=g.F64)
    f1 = op1.FermionField().import_(g.random_gaussian(int(np.prod(dims)) * 8 * 12, 1))
    cases.append((f1, g.F64))
    op2 = g.MobiusFermion(U, dims, 4, 0.01, 1.8, 1.5, 0.5, precision=g.F32, nrhs=3)
    f2 = op2.FermionRedBlackField(g.ODD).import_(g.random_gaussian(int(np.prod(dims)) // 2 * 4 * 3 * 12, 2))
    cases.append((f2, g.F32))
    f3 = op2.FermionRedBlackField(g.EVEN, precision=g.F16).import_(
        g.random_gaussian(int(np.prod(dims)) // 2 * 4 * 3 * 12, 4))
    cases.append((f3, g.F16))
    for f, prec in cases + cases:  # two calls in a row on every field
        ref = f.norm2()
        got = noalloc_norm2(f)
        assert got.shape == ref.shape
        assert np.all(np.abs(got / ref - 1) < REL_TOL[prec]), (got, ref)


def test_noalloc_norm2_rejects_too_many_rhs(gpu_available):
    dims = (4, 4, 4, 4)
    U = g.random_gauge(dims, 0.5, 5)
    op = g.WilsonFermion(U, dims, 0.1, precision=g.F32, nrhs=17)
    f = op.FermionRedBlackField(g.ODD).zero()
    out = np.zeros(17, dtype=np.float64)
    rc = g.lib.gb_field_norm2_noalloc(f.h, out.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 8  # GB_ERR_UNSUPPORTED
    assert b"16" in g.lib.gb_last_error()
