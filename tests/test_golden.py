"""Known answers (tests/golden/known_answers.json, written by make_known_answers.py from
the CPU oracle's FP64 operators): every Wilson, Moebius and ZMobius operator of the path
and the red-black Schur solve on seeded 4^4 lattices.

The CPU test re-derives the answers with the oracle (a regression lock on the oracle).
The GPU test runs the CUDA path through the library's public API on the same seeded
inputs and checks it against the stored numbers alone, with no oracle call.  A stored
answer y holds |y|^2, four inner products <w_k, y> and sixteen entries; a result y' with
rel_l2(y', y) <= tol satisfies
  | |y'|^2 - |y|^2 | <= (2 tol + tol^2) |y|^2,  |<w, y'> - <w, y>| <= tol |w| |y|,
  |y'_i - y_i| <= tol |y|,
and those are the checks.  Tolerances (relative L2): FP64 1e-13 (native, and with the
double-float hopping term of GB_FLAG_DF64), FP32 1e-6 for Wilson and Moebius, ten times
that for ZMobius; the Schur solution 1e-8 (solved to 1e-12)."""
import json
from pathlib import Path

import numpy as np
import pytest

import grid_gb300 as g

GOLDEN = json.loads((Path(__file__).resolve().parent / "golden" / "known_answers.json").read_text())
CASES = {c["name"]: c for c in GOLDEN["cases"]}


def check_functionals(got, ans, tol, what, gaussian):
    """got (the functionals of a result y') against ans, for rel_l2(y', y) <= tol;
    gaussian(n, seed) regenerates the probe vectors for their norms."""
    assert got["n"] == ans["n"], (what, "length")
    n2 = ans["norm2"]
    ny = np.sqrt(n2)
    assert abs(got["norm2"] - n2) <= (2 * tol + tol * tol) * n2 * 1.001, (what, "norm2")
    for k, (a, b) in enumerate(zip(got["probes"], ans["probes"])):
        wn = np.linalg.norm(gaussian(ans["n"], GOLDEN["probe_seed"] + k))
        assert abs(complex(*a) - complex(*b)) <= tol * wn * ny * 1.001, (what, "probe", k)
    for a, b in zip(got["samples"], ans["samples"]):
        assert a[0] == b[0] and abs(complex(a[1], a[2]) - complex(b[1], b[2])) <= tol * ny * 1.001, (what, a[0])


def functionals(y):
    """The stored functionals of y, computed with the library's own generator."""
    y = np.asarray(y, dtype=np.complex128).reshape(-1)
    probes = []
    for k in range(GOLDEN["nprobe"]):
        p = np.vdot(g.random_gaussian(y.size, GOLDEN["probe_seed"] + k), y)
        probes.append([p.real, p.imag])
    idx = [(7919 * j + 13) % y.size for j in range(GOLDEN["nsample"])]
    return {"n": y.size, "norm2": float(np.vdot(y, y).real), "probes": probes,
            "samples": [[i, y[i].real, y[i].imag] for i in idx]}


def check(y, ans, tol, what):
    check_functionals(functionals(y), ans, tol, what, g.random_gaussian)


def test_oracle_reproduces_known_answers():
    """The oracle's answers today equal the stored ones (FP64: 1e-12, room for another
    host's rounding)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_golden_make", Path(__file__).resolve().parent / "golden"
                                                  / "make_known_answers.py")
    mk = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mk)
    for case in mk.CASES:
        stored = CASES[case["name"]]["answers"]
        got = mk.compute(case)
        for name, ans in stored["operators"].items():
            check_functionals(got["operators"][name], ans, 1e-12, (case["name"], name), mk.o.random_gaussian)
        s_got, s_ans = got["schur_solve"], stored["schur_solve"]
        assert abs(s_got["iterations"] - s_ans["iterations"]) <= max(2, s_ans["iterations"] // 50)
        check_functionals(s_got, s_ans, 1e-8, (case["name"], "schur_solve"), mk.o.random_gaussian)


def make_op(case, prec, flags=0):
    dims = case["dims"]
    U = g.random_gauge(dims, case["gauge"]["eps"], case["gauge"]["seed"])
    ph = np.asarray(GOLDEN["phases"], dtype=np.float64)
    if case["kind"] == "wilson":
        return g.WilsonFermion(U, dims, case["mass"], phases=ph, precision=prec, flags=flags)
    if case["kind"] == "mobius":
        return g.MobiusFermion(U, dims, case["L5"], case["mass"], case["M5"], case["b"], case["c"], phases=ph,
                               precision=prec, flags=flags)
    gamma = [complex(re, im) for re, im in case["gamma"]]
    return g.ZMobiusFermion(U, dims, gamma, case["mass"], case["M5"], case["b"], case["c"], phases=ph,
                            precision=prec, flags=flags)


def apply(op, name, x, domain):
    if domain == "full":
        fin, fout = op.FermionField().import_(x), op.FermionField()
        if name in ("Dhop", "DhopDag"):
            op.Dhop(fin, fout, 1 if name == "DhopDag" else 0)
        else:
            getattr(op, name)(fin, fout)
    else:
        fin = op.FermionRedBlackField(g.ODD).import_(x)
        fout = op.FermionRedBlackField(g.EVEN if name.startswith("Meooe") else g.ODD)
        getattr(op, name)(fin, fout)
    return fout.export()


@pytest.mark.gpu
@pytest.mark.parametrize("prec,flags", [(g.F64, 0), (g.F64, g.DF64), (g.F32, 0)])
@pytest.mark.parametrize("name", sorted(CASES))
def test_cuda_path_matches_known_answers(gpu_available, name, prec, flags):
    case = CASES[name]
    tol = {g.F64: 1e-13, g.F32: 1e-6}[prec] * (10 if case["kind"] == "zmobius" else 1)
    op = make_op(case, prec, flags)
    vol = int(np.prod(case["dims"]))
    seeds = GOLDEN["field_seeds"]
    full = g.random_gaussian(vol * case["L5"] * 12, seeds["full"])
    odd = g.random_gaussian(vol // 2 * case["L5"] * 12, seeds["odd"])
    domains = {"Meooe": "odd", "MeooeDag": "odd", "Mooee": "odd", "MooeeDag": "odd", "MooeeInv": "odd",
               "MooeeInvDag": "odd", "Mpc": "odd", "MpcDag": "odd", "MpcDagMpc": "odd"}
    for opname, ans in case["answers"]["operators"].items():
        dom = domains.get(opname, "full")
        check(apply(op, opname, full if dom == "full" else odd, dom), ans, tol, (name, opname))
    if prec == g.F64:
        ans = case["answers"]["schur_solve"]
        fs = op.FermionField().import_(g.random_gaussian(vol * case["L5"] * 12, seeds["solve_source"]))
        fx = op.FermionField().zero()
        solver = g.SchurRedBlackDiagMooeeSolve(g.ConjugateGradient(ans["tol"], 20000))
        solver(op, fs, fx)
        check(fx.export(), ans, 1e-8, (name, "schur_solve"))
        assert abs(solver.solver.IterationsToComplete - ans["iterations"]) <= max(2, ans["iterations"] // 50)
        assert solver.unprec_residual[0] < 1e-10
