"""The propagator-solve service on the GPU: a request's result is the same alone and in
a mix of concurrent requests (tolerance: relative L2 1e-12; every solve reaches the true
residual 1e-10), agrees with the oracle's FP64 Schur solve of the same seeded inputs, and
CUDA-graph capture of the CG chunks does not change it.  The concurrent requests' device
work overlaps on the GPU's own clock (CUDA events on each slot's stream)."""
import numpy as np
import pytest

import grid_gb300 as g
from oracle import oracle as o

pytestmark = pytest.mark.gpu

GB = 1 << 30


def run(server, reqs):
    ids = [server.submit(r) for r in reqs]
    assert server.wait(len(ids), 600)
    res = {x.id: x for x in server.results()}
    return [res[i] for i in ids]


def sol_buffer(dims, Ls, nsrc):
    return np.zeros(int(np.prod(dims)) * Ls * 12 * nsrc, dtype=np.complex128)


def test_same_alone_and_in_the_mix(gpu_available):
    dims, Ls = (8, 8, 8, 8), 8
    alone = sol_buffer(dims, Ls, 2)
    s = g.Server(40 * GB, slots=1)
    (r0,) = run(s, [g.make_request(dims, Ls, 0.05, 0.5, 11, 2, 12, solution=alone)])
    s.close()
    assert r0.status == 0 and r0.true_residual < 1e-10 and r0.unprec_residual < 1e-9
    mixed = sol_buffer(dims, Ls, 2)
    s = g.Server(40 * GB, slots=4)
    others = [g.make_request((8, 8, 8, 16), 12, 0.02, 0.4, 21, 3, 22),
              g.make_request((12, 12, 12, 12), 8, 0.1, 0.6, 31, 1, 32, inner=g.F16),
              g.make_request((8, 8, 8, 8), 16, 0.01, 0.3, 41, 4, 42)]
    res = run(s, others[:2] + [g.make_request(dims, Ls, 0.05, 0.5, 11, 2, 12, solution=mixed)] + others[2:])
    st = s.stats()
    s.close()
    assert all(x.status == 0 for x in res)
    assert all(x.true_residual < 1e-10 and x.unprec_residual < 1e-9 for x in res)
    assert st.max_running >= 2
    # the device intervals of different requests overlap on the GPU timeline
    iv = [(x.dev_start, x.dev_end) for x in res]
    assert all(0 <= a < b for a, b in iv)
    overlaps = [(i, j) for i in range(len(iv)) for j in range(i + 1, len(iv))
                if min(iv[i][1], iv[j][1]) - max(iv[i][0], iv[j][0]) > 0]
    assert overlaps, iv
    assert o.rel_l2(mixed, alone) < 1e-12
    assert res[2].iterations == r0.iterations


def test_service_solution_matches_oracle(gpu_available):
    dims, Ls, mf = (8, 8, 8, 8), 8, 0.05
    sol = sol_buffer(dims, Ls, 1)
    s = g.Server(40 * GB, slots=2)
    (r,) = run(s, [g.make_request(dims, Ls, mf, 0.5, 7, 1, 8, solution=sol)])
    s.close()
    assert r.status == 0 and r.true_residual < 1e-10 and r.unprec_residual < 1e-9
    U = g.random_gauge(dims, 0.5, 7)
    src = g.random_gaussian(int(np.prod(dims)) * Ls * 12, 8)
    ref = o.OracleOp(1, 0, dims, Ls, [mf, 1.8, 1.5, 0.5], U, g.antiperiodic_t())
    assert o.rel_l2(ref.apply(o.OP_M, sol), src) < 1e-9
    xr, it, rc, ru = ref.schur_solve(src, 1e-11, 5000)
    assert o.rel_l2(sol, xr) < 1e-8


def test_graph_capture_gives_the_same_solve(gpu_available):
    dims, Ls = (8, 8, 8, 8), 8
    a = sol_buffer(dims, Ls, 3)
    b = sol_buffer(dims, Ls, 3)
    s = g.Server(40 * GB, slots=1)
    (ra,) = run(s, [g.make_request(dims, Ls, 0.02, 0.5, 5, 3, 6, solution=a)])
    s.close()
    s = g.Server(40 * GB, slots=1, flags=g.Server.GRAPHS)
    (rb,) = run(s, [g.make_request(dims, Ls, 0.02, 0.5, 5, 3, 6, solution=b)])
    s.close()
    assert ra.status == 0 and rb.status == 0
    assert ra.iterations == rb.iterations
    assert o.rel_l2(a, b) < 1e-12


def test_cg_with_graphs_matches_direct(gpu_available):
    dims = (8, 8, 8, 8)
    U = g.random_gauge(dims, 0.3, 3)
    op = g.WilsonFermion(U, dims, 0.1, precision=g.F64)
    src = g.random_gaussian(4096 * 12, 4)
    out = []
    for graphs in (0, 1):
        fs = op.FermionField().import_(src)
        fx = op.FermionField().zero()
        cg = g.ConjugateGradient(1e-8, 5000, use_graphs=graphs)
        cg(g.MdagMLinearOperator(op), fs, fx)
        out.append((cg.IterationsToComplete, fx.export()))
    assert out[0][0] == out[1][0]
    assert o.rel_l2(out[0][1], out[1][1]) < 1e-14


@pytest.mark.parametrize("solver", ["plain_fp64", "reliable_fp32"])
def test_device_resident_cg_loop_matches_host_loop(gpu_available, solver):
    """use_graphs = 2 runs the CG loop on the device (a graph's conditional WHILE node
    repeats the captured chunk until convergence or a reliable update is due): the same
    kernels in the same order as the host-driven loop, so the same iterations and the same
    solution to rounding."""
    dims, Ls = (8, 8, 8, 8), 8
    U = g.random_gauge(dims, 0.5, 17)
    od = g.MobiusFermion(U, dims, Ls, 0.02, 1.8, 1.5, 0.5, precision=g.F64)
    of = g.MobiusFermion(U, dims, Ls, 0.02, 1.8, 1.5, 0.5, precision=g.F32)
    src = g.random_gaussian(int(np.prod(dims)) * Ls * 12, 18)
    out = []
    for graphs in (0, 2):
        fs = od.FermionField().import_(src)
        fx = od.FermionField().zero()
        if solver == "plain_fp64":
            cg = g.ConjugateGradient(1e-10, 5000, check_every=10, use_graphs=graphs)
        else:
            cg = g.ConjugateGradientReliableUpdate(1e-10, 20000, 1e-6, g.SchurDiagMooeeOperator(of),
                                                   g.SchurDiagMooeeOperator(od), relup_every=100, check_every=10,
                                                   use_graphs=graphs)
        solver_ = g.SchurRedBlackDiagMooeeSolve(cg)
        r = solver_(od, fs, fx)
        out.append((int(r.iterations), float(r.true_residual), fx.export()))
    assert out[0][0] == out[1][0]
    assert out[1][1] < 1e-10
    assert o.rel_l2(out[0][2], out[1][2]) < 1e-13
