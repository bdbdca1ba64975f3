"""Failure detection without a GPU fault: a device wait on a flag that nothing sets runs
out of its (short) poll budget and reports GB_ERR_TIMEOUT to the host, after which the
same context and operator keep working (a Dhop afterwards matches the oracle); with the
flag set the same wait returns at once."""
import time

import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o
from tests._common import fermion

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_context_survives(gpu_available):
    dims = (4, 4, 4, 4)
    U = g.random_gauge(dims, 0.3, 111)
    op = g.WilsonFermion(U, dims, 0.1, precision=g.F64)
    assert g.lib.gb_bounded_wait_test(op.h, 1, 1000) == 0
    t0 = time.perf_counter()
    rc = g.lib.gb_bounded_wait_test(op.h, 0, 20000)  # about 20-40 ms of polling
    assert rc == 6  # GB_ERR_TIMEOUT
    assert b"gave up" in g.lib.gb_last_error()
    assert time.perf_counter() - t0 < 5.0
    # the context is intact: an operator call afterwards is correct
    ref = o.OracleOp(0, 0, dims, 1, [0.1], U, g.antiperiodic_t())
    x = fermion(256, 1, 112)
    fin, fout = op.FermionField().import_(x), op.FermionField()
    op.M(fin, fout)
    assert o.rel_l2(fout.export(), ref.apply(o.OP_M, x)) < 1e-13
    assert g.lib.gb_bounded_wait_test(op.h, 0, 0) == 1  # GB_ERR_BAD_ARG: no poll budget
