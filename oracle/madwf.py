"""MADWF restated on the CPU oracle (TEST INFRASTRUCTURE ONLY: the checker for the
library's MADWF; only tests/ use it).

Follows Grid/qcd/action/fermion/MADWF.h:87-209 (the defect-correction loop) with the
Pauli-Villars solve of PauliVillarsInverters.h:54-72 (red-black Schur solve at mass 1).
Fields are numpy complex128 arrays in the oracle's canonical layout: a 5D field is
[site][s][spin][colour], a 4D field [site][spin][colour].
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as o


def extract_slice(f5, Ls, s):
    """ExtractSlice(lowDim, higherDim, s, 0) (Lattice_transfer.h:999-1070)."""
    return np.ascontiguousarray(f5.reshape(-1, Ls, 12)[:, s, :]).reshape(-1)


def insert_slice(f4, f5, Ls, s):
    """InsertSlice(lowDim, higherDim, s, 0): f5 with slice s replaced by f4 (a new array)."""
    out = f5.reshape(-1, Ls, 12).copy()
    out[:, s, :] = f4.reshape(-1, 12)
    return out.reshape(-1)


def pv_solve(op: o.OracleOp, mass, src, tol, maxit):
    """PauliVillarsSolverRBprec: solve M(1) sol = src, then restore the mass."""
    op.set_mass(1.0)
    try:
        sol, _, _, _ = op.schur_solve(src, tol, maxit)
    finally:
        op.set_mass(mass)
    return sol


def madwf(outer: o.OracleOp, Ls_o, mass_o, inner: o.OracleOp, Ls_i, mass_i, b, pv_tol, inner_tol, resid, maxiter,
          pv_maxit=10000, inner_maxit=10000):
    """Solve outer.M sol5 = b (full 5D source b); returns (sol5, residual history)."""
    nb = np.vdot(b, b).real
    defect = b.copy()
    sol5 = np.zeros_like(b)
    history = []
    for _ in range(maxiter):
        A = pv_solve(outer, mass_o, defect, pv_tol, pv_maxit)
        c = outer.apply(o.OP_PDAG, A)
        c0 = extract_slice(c, Ls_o, 0)
        n4 = c0.size
        ci = insert_slice(c0, np.zeros(n4 * Ls_i, dtype=np.complex128), Ls_i, 0)
        Ai = inner.apply(o.OP_P, ci)
        inner.set_mass(1.0)
        try:
            srci = inner.apply(o.OP_M, Ai)
        finally:
            inner.set_mass(mass_i)
        xi, _, _, _ = inner.schur_solve(srci, inner_tol, inner_maxit)
        yi = inner.apply(o.OP_PDAG, xi)
        y0 = extract_slice(yi, Ls_i, 0)
        c = insert_slice(-y0, c, Ls_o, 0)
        B = outer.apply(o.OP_P, c)
        A = outer.apply(o.OP_M, B)
        B = pv_solve(outer, mass_o, A, pv_tol, pv_maxit)
        A = outer.apply(o.OP_PDAG, B)
        A = insert_slice(y0, A, Ls_o, 0)
        B = outer.apply(o.OP_P, A)
        sol5 = sol5 + B
        defect = b - outer.apply(o.OP_M, sol5)
        r = float(np.sqrt(np.vdot(defect, defect).real / nb))
        history.append(r)
        if r < resid:
            break
    return sol5, history
