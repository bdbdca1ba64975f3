"""Writes known_answers.json beside this file: the CPU oracle's FP64 answers for every
operator of the path and for the red-black Schur solve, on small seeded lattices.

TEST INFRASTRUCTURE ONLY.  Grid ships no golden data for these operators and cannot be
built without Eigen, OpenSSL and GMP, so these answers come from the oracle (the C++
restatement under oracle/, itself pinned by tests/test_oracle_pins.py).  They lock the
oracle against regressions and let the GPU tests check the CUDA path against fixed
numbers instead of a live oracle run.

Each case names its operator (Wilson, Moebius, ZMobius), lattice, parameters and the
seeds of the library's generator (gauge field: random_gauge(dims, eps, seed); fields:
random_gaussian(n, seed), restated bit for bit by the oracle).  Each answer y is stored as
  norm2    |y|^2
  probes   <w_k, y> for w_k = random_gaussian(len(y), PROBE_SEED + k), k < 4
  samples  y[i] at SAMPLE indices (i_j = (7919 j + 13) mod len(y), j < 16)
(and its length n), so that rel_l2(y', y) <= tol bounds every stored number
(Cauchy-Schwarz for the probes).

Usage: python tests/golden/make_known_answers.py   (rewrites the JSON)
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from oracle import oracle as o  # noqa: E402

PROBE_SEED = 7000
NPROBE = 4
NSAMPLE = 16
PHASES = [1, 0, 1, 0, 1, 0, -1, 0]  # antiperiodic in time (ImplParams::boundary_phases)

# the Ls = 10 omegas of Grid's tests/core/Test_zmobius_even_odd.cc:97-106 (b = 1, c = 0)
ZOMEGA = [1.45806438985048, 1.18231318389348, 0.830951166685955, 0.542352409156791, 0.341985020453729,
          0.21137902619029, 0.126074299502912, 0.0990136651962626, 0.0686324988446592 + 0.0550658530827402j,
          0.0686324988446592 - 0.0550658530827402j]

CASES = [
    {"name": "wilson_4^4", "kind": "wilson", "dims": [4, 4, 4, 4], "L5": 1, "mass": 0.1,
     "gauge": {"eps": 0.3, "seed": 7}},
    {"name": "mobius_4^4xLs8", "kind": "mobius", "dims": [4, 4, 4, 4], "L5": 8, "mass": 0.01,
     "M5": 1.8, "b": 1.5, "c": 0.5, "gauge": {"eps": 0.5, "seed": 11}},
    {"name": "zmobius_4^4xLs10", "kind": "zmobius", "dims": [4, 4, 4, 4], "L5": 10, "mass": 0.05,
     "M5": 1.8, "b": 1.0, "c": 0.0, "gamma": [[complex(z).real, complex(z).imag] for z in ZOMEGA],
     "gauge": {"eps": 0.5, "seed": 13}},
]

# (answer name, oracle opcode, input domain): "full" = a full field, "odd" = the odd
# checkerboard (Meooe maps it to the even one, the other half-field operators to itself)
OPERATORS = [
    ("Dhop", o.OP_DHOP, "full"), ("DhopDag", o.OP_DHOP_DAG, "full"), ("M", o.OP_M, "full"),
    ("Mdag", o.OP_MDAG, "full"), ("MdagM", o.OP_MDAGM, "full"),
    ("Meooe", o.OP_MEOOE, "odd"), ("MeooeDag", o.OP_MEOOE_DAG, "odd"),
    ("Mooee", o.OP_MOOEE, "odd"), ("MooeeDag", o.OP_MOOEE_DAG, "odd"),
    ("MooeeInv", o.OP_MOOEE_INV, "odd"), ("MooeeInvDag", o.OP_MOOEE_INV_DAG, "odd"),
    ("Mpc", o.OP_MPC, "odd"), ("MpcDag", o.OP_MPC_DAG, "odd"), ("MpcDagMpc", o.OP_MPCDAGMPC, "odd"),
]
FULL_SEED, ODD_SEED, SOLVE_SEED = 101, 102, 103
SOLVE_TOL = 1e-12


def sample_indices(n):
    return [(7919 * j + 13) % n for j in range(NSAMPLE)]


def functionals(y):
    y = np.asarray(y, dtype=np.complex128).reshape(-1)
    probes = []
    for k in range(NPROBE):
        p = np.vdot(o.random_gaussian(y.size, PROBE_SEED + k), y)
        probes.append([float(p.real), float(p.imag)])
    return {"n": int(y.size), "norm2": float(np.vdot(y, y).real), "probes": probes,
            "samples": [[i, float(y[i].real), float(y[i].imag)] for i in sample_indices(y.size)]}


def oracle_op(case):
    U = o.random_gauge(case["dims"], case["gauge"]["eps"], case["gauge"]["seed"])
    if case["kind"] == "wilson":
        return o.OracleOp(0, 0, case["dims"], case["L5"], [case["mass"]], U, PHASES)
    params = [case["mass"], case["M5"], case["b"], case["c"]]
    if case["kind"] == "mobius":
        return o.OracleOp(1, 0, case["dims"], case["L5"], params, U, PHASES)
    params += [v for z in case["gamma"] for v in z]
    return o.OracleOp(2, 0, case["dims"], case["L5"], params, U, PHASES)


def compute(case):
    """The oracle's answers for one case (also called by the CPU test that re-derives them)."""
    op = oracle_op(case)
    full = o.random_gaussian(op.full_len(), FULL_SEED)
    odd = o.random_gaussian(op.half_len(), ODD_SEED)
    ops = {}
    for name, code, dom in OPERATORS:
        ops[name] = functionals(op.apply(code, full) if dom == "full" else op.apply(code, odd, 1))
    src = o.random_gaussian(op.full_len(), SOLVE_SEED)
    sol, iters, r_cg, r_unprec = op.schur_solve(src, SOLVE_TOL, 20000)
    solve = functionals(sol)
    solve.update({"tol": SOLVE_TOL, "iterations": int(iters), "unprec_residual": float(r_unprec)})
    return {"operators": ops, "schur_solve": solve}


def main():
    out = {"about": "FP64 answers of the CPU oracle (not of Grid, which cannot be built here); "
                    "written by tests/golden/make_known_answers.py",
           "phases": PHASES, "probe_seed": PROBE_SEED, "nprobe": NPROBE, "nsample": NSAMPLE,
           "field_seeds": {"full": FULL_SEED, "odd": ODD_SEED, "solve_source": SOLVE_SEED}, "cases": []}
    for case in CASES:
        out["cases"].append(dict(case, answers=compute(case)))
    (HERE / "known_answers.json").write_text(json.dumps(out, indent=1) + "\n")


if __name__ == "__main__":
    main()
