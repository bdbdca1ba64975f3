"""ctypes wrapper of the CPU oracle (oracle.hpp / oracle_capi.cpp).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA library.  Only tests/, the smoke
check and bench.py's CPU-baseline / reference leg use it; the product never does.
Arrays are numpy complex128 in the canonical layout of include/gbdwf.h.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"

OP_M, OP_MDAG, OP_DHOP, OP_DHOP_DAG = 0, 1, 2, 3
OP_MEOOE, OP_MEOOE_DAG, OP_MOOEE, OP_MOOEE_DAG = 4, 5, 6, 7
OP_MOOEE_INV, OP_MOOEE_INV_DAG, OP_MPC, OP_MPC_DAG = 8, 9, 10, 11
OP_MPCDAGMPC, OP_MDAGM, OP_MEOOE5D, OP_MEOOE_DAG5D = 12, 13, 14, 15
OP_DMINUS, OP_DMINUS_DAG = 16, 17
OP_P, OP_PDAG = 18, 19  # CayleyFermion5D::P / Pdag
# orc_physical modes (CayleyFermion5DImplementation.h:57-129)
IMPORT_PHYSICAL_SOURCE, IMPORT_UNPHYSICAL, EXPORT_PHYSICAL_SOLUTION, EXPORT_PHYSICAL_SOURCE = 0, 1, 2, 3


def build():
    """Compile liboracle.so with the committed Makefile (g++ + OpenMP)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        vp, i, d = C.c_void_p, C.c_int, C.c_double
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.orc_create.argtypes = [i, i, ip, i, dp, dp, dp]
        L.orc_create.restype = vp
        L.orc_free.argtypes = [vp]
        L.orc_set_mass.argtypes = [vp, C.c_double]
        L.orc_apply.argtypes = [vp, i, dp, dp, i]
        L.orc_dhop_cb.argtypes = [vp, dp, dp, i, i]
        L.orc_doubled_links.argtypes = [vp, dp]
        L.orc_dhop_naive.argtypes = [ip, i, dp, dp, dp, dp, i]
        L.orc_cayley_coeffs.argtypes = [i, d, d, d, d, dp]
        L.orc_cg.argtypes = [vp, i, dp, dp, d, i, ip, dp]
        L.orc_schur_solve.argtypes = [vp, dp, dp, d, i, ip, dp]
        L.orc_schur_solve_guess.argtypes = [vp, dp, dp, dp, d, i, ip, dp]
        L.orc_cg_reliable.argtypes = [vp, vp, i, dp, dp, d, i, d, i, i, ip, dp]
        L.orc_physical.argtypes = [vp, i, dp, dp]
        L.orc_cg_multishift.argtypes = [vp, i, dp, i, dp, dp, i, dp, ip, dp]
        L.orc_deriv.argtypes = [vp, i, dp, dp, i, i, dp]
        L.orc_set_threads.argtypes = [i]
        L.orc_max_threads.restype = i
        L.orc_random_gauge.argtypes = [ip, d, C.c_uint64, dp]
        L.orc_random_gaussian.argtypes = [C.c_int64, C.c_uint64, dp]
        L.orc_hs_create.argtypes = [ip, i, dp, dp]
        L.orc_hs_create.restype = vp
        L.orc_hs_free.argtypes = [vp]
        L.orc_hs_set.argtypes = [vp, i, dp]
        L.orc_hs_get.argtypes = [vp, i, dp]
        L.orc_hs_dhop.argtypes = [vp, i, i]
        _lib = L
    return _lib


def _p(a):
    assert a.flags["C_CONTIGUOUS"] and a.dtype in (np.complex128, np.float64)
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _dims(d):
    return (C.c_int * 4)(*[int(x) for x in d])


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def max_threads() -> int:
    return lib().orc_max_threads()


def phases_array(ph):
    return np.ascontiguousarray(ph, dtype=np.float64)


class OracleOp:
    """kind 0: Wilson (params = [mass]); kind 1: Moebius (params = [mf, M5, b, c]).
    prec 0 double, 1 float.  L5 = Ls for Moebius, number of stacked rhs for Wilson."""

    def __init__(self, kind, prec, dims, L5, params, U, phases):
        self.kind, self.prec, self.dims, self.L5 = kind, prec, tuple(dims), int(L5)
        self.vol = int(np.prod(dims))
        par = np.ascontiguousarray(params, dtype=np.float64)
        self._U = np.ascontiguousarray(U, dtype=np.complex128)
        ph = phases_array(phases)
        self.h = lib().orc_create(kind, prec, _dims(dims), self.L5, _p(par), _p(self._U), _p(ph))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_free(self.h)
            self.h = None

    def full_len(self):
        return self.vol * self.L5 * 12

    def half_len(self):
        return self.vol // 2 * self.L5 * 12

    def set_mass(self, mass):
        """SetMass (CayleyFermion5D.h:75-78)."""
        assert lib().orc_set_mass(self.h, float(mass)) == 0

    def apply(self, opcode, x, parity=1):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        out = np.empty_like(x)
        rc = lib().orc_apply(self.h, opcode, _p(x), _p(out), parity)
        assert rc == 0
        return out

    def dhop_cb(self, x, in_parity, dag=0):
        x = np.ascontiguousarray(x, dtype=np.complex128)
        out = np.empty_like(x)
        lib().orc_dhop_cb(self.h, _p(x), _p(out), in_parity, dag)
        return out

    def physical(self, mode, x):
        """4D <-> 5D surface fields (Moebius, FP64): modes IMPORT_* take a 4D field and
        return a 5D one, EXPORT_* the reverse."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        n = self.vol * 12 * (self.L5 if mode < 2 else 1)
        out = np.empty(n, dtype=np.complex128)
        assert lib().orc_physical(self.h, mode, _p(x), _p(out)) == 0
        return out

    def deriv(self, A, B, dag=0, mderiv=False, out_parity=-1):
        """DhopDeriv (or MDeriv) force of full fields A, B: [site][mu][3][3] complex; only the
        sites of out_parity when >= 0 (zero elsewhere)."""
        A = np.ascontiguousarray(A, dtype=np.complex128)
        B = np.ascontiguousarray(B, dtype=np.complex128)
        mat = np.zeros(self.vol * 36, dtype=np.complex128)
        assert lib().orc_deriv(self.h, int(mderiv), _p(A), _p(B), int(dag), int(out_parity), _p(mat)) == 0
        return mat

    def doubled_links(self):
        out = np.empty(self.vol * 8 * 9, dtype=np.complex128)
        lib().orc_doubled_links(self.h, _p(out))
        return out

    def cg(self, kind, src, tol, maxit, psi0=None):
        src = np.ascontiguousarray(src, dtype=np.complex128)
        psi = np.zeros_like(src) if psi0 is None else np.ascontiguousarray(psi0, dtype=np.complex128).copy()
        info = (C.c_int * 2)()
        res = C.c_double()
        lib().orc_cg(self.h, kind, _p(src), _p(psi), float(tol), int(maxit), info, C.byref(res))
        return psi, info[0], res.value

    def cg_multishift(self, kind, src, shifts, tols, maxit):
        """(A + shifts[s]) psi_s = src for every shift (FP64); returns (psi list, iterations,
        converged, iterations per shift, true residual per shift)."""
        src = np.ascontiguousarray(src, dtype=np.complex128)
        ns = len(shifts)
        psi = np.zeros((ns, src.size), dtype=np.complex128)
        info = (C.c_int * (2 + ns))()
        res = (C.c_double * ns)()
        m = np.ascontiguousarray(shifts, dtype=np.float64)
        t = np.ascontiguousarray(tols, dtype=np.float64)
        lib().orc_cg_multishift(self.h, kind, _p(src), ns, _p(m), _p(t), int(maxit), _p(psi), info, res)
        return list(psi), info[0], info[1], list(info[2:]), list(res)

    def schur_solve(self, src, tol, maxit, guess=None):
        """Red-black Schur solve in FP64; guess (a full field) starts the odd-checkerboard
        CG, which converges to the same solution with fewer iterations."""
        src = np.ascontiguousarray(src, dtype=np.complex128)
        sol = np.zeros_like(src)
        info = (C.c_int * 2)()
        res = (C.c_double * 2)()
        if guess is None:
            lib().orc_schur_solve(self.h, _p(src), _p(sol), float(tol), int(maxit), info, res)
        else:
            gs = np.ascontiguousarray(guess, dtype=np.complex128)
            lib().orc_schur_solve_guess(self.h, _p(src), _p(gs), _p(sol), float(tol), int(maxit), info, res)
        return sol, info[0], res[0], res[1]


def cg_reliable(op_d: OracleOp, op_f: OracleOp, kind, src, tol, maxit, delta, relup_every=0, cleanup=True):
    src = np.ascontiguousarray(src, dtype=np.complex128)
    psi = np.zeros_like(src)
    info = (C.c_int * 4)()
    res = C.c_double()
    lib().orc_cg_reliable(op_d.h, op_f.h, kind, _p(src), _p(psi), float(tol), int(maxit), float(delta),
                          int(relup_every), 1 if cleanup else 0, info, C.byref(res))
    return psi, list(info), res.value


def dhop_naive(dims, L5, U, phases, x, dag=0):
    x = np.ascontiguousarray(x, dtype=np.complex128)
    U = np.ascontiguousarray(U, dtype=np.complex128)
    out = np.empty_like(x)
    lib().orc_dhop_naive(_dims(dims), int(L5), _p(U), _p(phases_array(phases)), _p(x), _p(out), dag)
    return out


def cayley_coeffs(Ls, mf, M5, b, c) -> dict:
    out = np.empty(9 * Ls, dtype=np.float64)
    lib().orc_cayley_coeffs(int(Ls), float(mf), float(M5), float(b), float(c), _p(out))
    names = ["bs", "cs", "bee", "cee", "dee", "lee", "leem", "uee", "ueem"]
    return {n: out[k * Ls:(k + 1) * Ls].copy() for k, n in enumerate(names)}


# ---- canonical-layout helpers (pure numpy) -------------------------------------------
def site_parity(dims):
    Lx, Ly, Lz, Lt = dims
    t, z, y, x = np.meshgrid(np.arange(Lt), np.arange(Lz), np.arange(Ly), np.arange(Lx), indexing="ij")
    return ((x + y + z + t) & 1).reshape(-1)


def pick(dims, L5, full, parity):
    f = full.reshape(-1, L5 * 12)
    return np.ascontiguousarray(f[site_parity(dims) == parity].reshape(-1))


def setcb(dims, L5, half, parity, full=None):
    vol = int(np.prod(dims))
    out = np.zeros((vol, L5 * 12), dtype=np.complex128) if full is None else full.reshape(vol, L5 * 12).copy()
    out[site_parity(dims) == parity] = half.reshape(-1, L5 * 12)
    return out.reshape(-1)


def rel_l2(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


# ---- the reference arm's inputs and CPU Dhop (cpu_dhop.cpp) ----
def random_gauge(dims, eps: float, seed: int) -> np.ndarray:
    """The seeded gauge field of the CUDA library's generator, restated (bit for bit):
    canonical U[site][mu][3][3] complex128."""
    vol = int(np.prod(dims))
    U = np.empty(vol * 4 * 9, dtype=np.complex128)
    lib().orc_random_gauge(_dims(dims), float(eps), int(seed), _p(U))
    return U


def random_gaussian(n: int, seed: int) -> np.ndarray:
    """n complex numbers with N(0,1) parts, the library generator's stream, restated."""
    out = np.empty(int(n), dtype=np.complex128)
    lib().orc_random_gaussian(int(n), int(seed), _p(out))
    return out


class HalfSpinorDhop:
    """Grid's CPU hopping-term algorithm on one checkerboard in FP32 (half-spinor
    projection, SU(3) x two-spinor, reconstruction; OpenMP over 4D sites, the fifth
    dimension vectorised).  set()/get() convert a canonical half field outside the timed
    dhop() call."""

    def __init__(self, dims, L5: int, U: np.ndarray, phases):
        ph = np.ascontiguousarray(np.asarray(phases, dtype=np.float64))
        self.h = lib().orc_hs_create(_dims(dims), int(L5), _p(np.ascontiguousarray(U)), _p(ph))
        if not self.h:
            raise ValueError("L5 must be in [1, 64]")
        self.n = int(np.prod(dims)) // 2 * int(L5) * 12

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_hs_free(self.h)

    def set(self, parity: int, x: np.ndarray):
        assert x.size == self.n
        lib().orc_hs_set(self.h, int(parity), _p(np.ascontiguousarray(x)))

    def get(self, parity: int) -> np.ndarray:
        out = np.empty(self.n, dtype=np.complex128)
        lib().orc_hs_get(self.h, int(parity), _p(out))
        return out

    def dhop(self, out_parity: int, dag: int = 0):
        lib().orc_hs_dhop(self.h, int(out_parity), int(dag))
