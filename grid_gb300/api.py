"""ctypes mirror of Grid's fermion-operator / linear-operator / CG interfaces over the
C ABI of libgbdwf.so.

Names, argument meaning and error behaviour follow Grid:
  * WilsonFermion(U, dims, mass, ...)                 Grid/qcd/action/fermion/WilsonFermion.h:139-142
  * MobiusFermion(U, dims, Ls, mf, M5, b, c, ...)     Grid/qcd/action/fermion/MobiusFermion.h:45-67
  * M, Mdag, Dhop, DhopEO, DhopOE, Meooe, MeooeDag, Mooee, MooeeDag, MooeeInv, MooeeInvDag
                                                      Grid/qcd/action/fermion/FermionOperator.h:40-192
  * MdagMLinearOperator, SchurDiagMooeeOperator       Grid/algorithms/LinearOperator.h:74-105,325-349
  * ConjugateGradient(tol, maxit, err_on_no_conv)     Grid/algorithms/iterative/ConjugateGradient.h:55-59
  * ConjugateGradientReliableUpdate(tol, maxit, delta, linop_f, linop_d)
                                                      Grid/algorithms/iterative/ConjugateGradientReliableUpdate.h:58-69
  * SchurRedBlackDiagMooeeSolve(solver)(op, src, sol) Grid/algorithms/iterative/SchurRedBlack.h:373-436
Grid asserts where this raises GridError (status code + message); a CG that does not
converge raises when err_on_no_conv is set, as Grid's ErrorOnNoConverge asserts.

Host arrays are numpy complex128 in the canonical layout of include/gbdwf.h.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().with_name("libgbdwf.so")

F64, F32, F16 = 0, 1, 2
RECON12 = 1  # gb_*_create flag GB_FLAG_RECON12: 12-real links
DF64 = 2  # gb_*_create flag GB_FLAG_DF64: FP64 hopping term in double-float arithmetic
EVEN, ODD, FULL = 0, 1, 2
DaggerNo, DaggerYes = 0, 1


class GridError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


def _load():
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is not built: run `python grid_gb300/build.py` (the CUDA library is required; "
            "there is no CPU fallback)")
    return C.CDLL(str(LIB_PATH))


lib = _load()

_vp, _i, _d, _u64, _sz = C.c_void_p, C.c_int, C.c_double, C.c_uint64, C.c_size_t
_ip, _dp = C.POINTER(C.c_int), C.POINTER(C.c_double)


class CGParams(C.Structure):
    _fields_ = [("tolerance", C.c_double), ("max_iterations", C.c_int), ("err_on_no_conv", C.c_int),
                ("delta", C.c_double), ("relup_every", C.c_int), ("final_cleanup", C.c_int),
                ("check_every", C.c_int), ("use_graphs", C.c_int)]


class CGResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("reliable_updates", C.c_int), ("cleanup_iterations", C.c_int),
                ("converged", C.c_int), ("true_residual", C.c_double), ("seconds", C.c_double),
                ("flops", C.c_double)]


def _proto(name, args, res=C.c_int):
    f = getattr(lib, name)
    f.argtypes = args
    f.restype = res
    return f


_proto("gb_last_error", [], C.c_char_p)
_proto("gb_status_string", [_i], C.c_char_p)
_proto("gb_device_count", [_ip])
_proto("gb_version", [])
_proto("gb_wilson_create", [_ip, _d, _dp, _i, _i, _vp, C.c_uint, C.POINTER(_vp)])
_proto("gb_mobius_create", [_ip, _i, _d, _d, _d, _d, _dp, _i, _i, _vp, C.c_uint, C.POINTER(_vp)])
_proto("gb_zmobius_create", [_ip, _i, _d, _d, _dp, _d, _d, _dp, _i, _i, _vp, C.c_uint, C.POINTER(_vp)])
_proto("gb_zolotarev", [_d, _i, _i, _dp, _dp])
_proto("gb_zmobius_gamma", [_i, _d, _i, _d, _d, _dp, _dp])
_proto("gb_op_destroy", [_vp])
_proto("gb_op_import_gauge", [_vp, _dp])
_proto("gb_op_import_gauge_device", [_vp, _vp])
_proto("gb_op_info", [_vp, _ip, _ip, C.POINTER(C.c_int64), _ip])
_proto("gb_op_set_stream", [_vp, _vp])
_proto("gb_op_cayley_coeffs", [_vp, _dp])
_proto("gb_field_create", [_vp, _i, _i, C.POINTER(_vp)])
_proto("gb_field_destroy", [_vp])
_proto("gb_field_subset", [_vp, _ip])
_proto("gb_field_set_subset", [_vp, _i])
_proto("gb_field_host_len", [_vp, C.POINTER(_sz)])
_proto("gb_field_import", [_vp, _dp])
_proto("gb_field_export", [_vp, _dp])
_proto("gb_field_import_device", [_vp, _vp])
_proto("gb_field_export_device", [_vp, _vp])
_proto("gb_field_import_f32", [_vp, _vp])
_proto("gb_field_export_f32", [_vp, _vp])
_proto("gb_xfer_create", [_vp, C.POINTER(_vp)])
_proto("gb_xfer_destroy", [_vp])
_proto("gb_xfer_import", [_vp, _vp, _vp, _i])
_proto("gb_xfer_export", [_vp, _vp, _vp, _i])
_proto("gb_xfer_wait", [_vp])
_proto("gb_field_zero", [_vp])
_proto("gb_field_copy", [_vp, _vp])
_proto("gb_field_norm2", [_vp, _dp])
_proto("gb_field_inner", [_vp, _vp, _dp])
_proto("gb_field_axpy", [_vp, _d, _vp, _vp])
_proto("gb_field_axpby", [_vp, _d, _d, _vp, _vp])
_proto("gb_field_axpy_norm", [_vp, _d, _vp, _vp, _dp])
_proto("gb_field_pick_checkerboard", [_vp, _vp])
_proto("gb_field_set_checkerboard", [_vp, _vp])
for _n in ("gb_M", "gb_Mdag", "gb_MdagM", "gb_Meooe", "gb_MeooeDag", "gb_Mooee", "gb_MooeeDag", "gb_MooeeInv",
           "gb_MooeeInvDag", "gb_Mpc", "gb_MpcDag", "gb_MpcDagMpc"):
    _proto(_n, [_vp, _vp, _vp])
for _n in ("gb_Dhop", "gb_DhopEO", "gb_DhopOE"):
    _proto(_n, [_vp, _vp, _vp, _i])
_proto("gb_cg_params_default", [C.POINTER(CGParams)], None)
_proto("gb_cg_mdagm", [_vp, _vp, _vp, C.POINTER(CGParams), C.POINTER(CGResult)])
_proto("gb_cg_schur", [_vp, _vp, _vp, C.POINTER(CGParams), C.POINTER(CGResult)])
_proto("gb_cg_last_per_rhs", [_vp, _ip, _dp])
_proto("gb_cg_reliable", [_vp, _vp, _i, _vp, _vp, C.POINTER(CGParams), C.POINTER(CGResult)])
_proto("gb_schur_solve", [_vp, _vp, _vp, _vp, C.POINTER(CGParams), C.POINTER(CGResult), _dp])
_proto("gb_random_gauge", [_ip, _d, _u64, _dp])
_proto("gb_random_gaussian", [_sz, _u64, _dp])
_proto("gb_random_z2", [_sz, _u64, _dp])
_proto("gb_unit_gauge", [_ip, _dp])
_proto("gb_bench_kernel", [_vp, _i, C.POINTER(_vp), C.POINTER(_vp), _i, _i, _dp])
_proto("gb_set_device", [_i])
_proto("gb_op_sync", [_vp])
_proto("gb_op_event_record", [_vp, _i])
_proto("gb_op_event_elapsed", [_vp, _i, _i, _dp])
_proto("gb_host_alloc", [_sz, C.POINTER(_vp)])
_proto("gb_host_free", [_vp])
_proto("gb_stream_create", [C.POINTER(_vp)])
_proto("gb_stream_destroy", [_vp])
_proto("gb_Dminus", [_vp, _vp, _vp, _i])
_proto("gb_insert_slice", [_vp, _vp, _i, _vp, _i])
_proto("gb_extract_slice", [_vp, _vp, _i, _vp, _i])
_proto("gb_P", [_vp, _vp, _vp, _i])
_proto("gb_op_set_mass", [_vp, _d])
_proto("gb_op_mass", [_vp, _dp])
for _n in ("gb_import_physical_source", "gb_import_unphysical_fermion"):
    _proto(_n, [_vp, _vp, _i, _vp])
for _n in ("gb_export_physical_solution", "gb_export_physical_source"):
    _proto(_n, [_vp, _vp, _vp, _i])
for _n in ("gb_DhopDeriv", "gb_MDeriv"):
    _proto(_n, [_vp, _vp, _vp, _i, _vp, _i])


def set_device(d: int):
    _check(lib.gb_set_device(int(d)))


class PinnedArray:
    """Page-locked host buffer viewed as a numpy complex128 (or, with dtype=np.complex64,
    complex64) array."""

    def __init__(self, n_complex: int, dtype=np.complex128):
        dtype = np.dtype(dtype)
        p = _vp()
        _check(lib.gb_host_alloc(int(n_complex) * dtype.itemsize, C.byref(p)))
        self.ptr = p
        buf = (C.c_char * (int(n_complex) * dtype.itemsize)).from_address(p.value)
        self.array = np.frombuffer(buf, dtype=dtype)

    def __del__(self):
        if getattr(self, "ptr", None):
            self.array = None
            lib.gb_host_free(self.ptr)
            self.ptr = None


class Stream:
    """A non-blocking CUDA stream owned by the library (for operators that should not use
    the legacy default stream); `ptr` is the cudaStream_t value."""

    def __init__(self):
        p = _vp()
        _check(lib.gb_stream_create(C.byref(p)))
        self.ptr = p.value

    def __del__(self):
        if getattr(self, "ptr", None):
            lib.gb_stream_destroy(_vp(self.ptr))
            self.ptr = None


def _check(rc: int):
    if rc != 0:
        raise GridError(rc, (lib.gb_last_error() or b"").decode() or lib.gb_status_string(rc).decode())


def _dptr(a: np.ndarray):
    assert a.dtype in (np.complex128, np.float64) and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def _dims(dims):
    d = (C.c_int * 4)(*[int(x) for x in dims])
    return d


def device_count() -> int:
    n = C.c_int(0)
    lib.gb_device_count(C.byref(n))
    return n.value


def periodic():
    return np.array([1, 0, 1, 0, 1, 0, 1, 0], dtype=np.float64)


def antiperiodic_t():
    """ImplParams::boundary_phases = {1,1,1,-1} (Test_mobius_bcg_nosplit.cc:51)."""
    return np.array([1, 0, 1, 0, 1, 0, -1, 0], dtype=np.float64)


# ---- seeded inputs ------------------------------------------------------------------
def random_gauge(dims, eps: float, seed: int) -> np.ndarray:
    vol = int(np.prod(dims))
    U = np.empty(vol * 4 * 9, dtype=np.complex128)
    _check(lib.gb_random_gauge(_dims(dims), float(eps), int(seed), _dptr(U)))
    return U


def unit_gauge(dims) -> np.ndarray:
    vol = int(np.prod(dims))
    U = np.empty(vol * 4 * 9, dtype=np.complex128)
    _check(lib.gb_unit_gauge(_dims(dims), _dptr(U)))
    return U


def random_gaussian(n_complex: int, seed: int) -> np.ndarray:
    a = np.empty(int(n_complex), dtype=np.complex128)
    _check(lib.gb_random_gaussian(int(n_complex), int(seed), _dptr(a)))
    return a


def random_z2(n_complex: int, seed: int) -> np.ndarray:
    a = np.empty(int(n_complex), dtype=np.complex128)
    _check(lib.gb_random_z2(int(n_complex), int(seed), _dptr(a)))
    return a


# ---- fields ---------------------------------------------------------------------------
class FermionField:
    """Lattice<SpinColourVector> on an operator's FermionGrid (FULL) or
    FermionRedBlackGrid (EVEN/ODD), device resident."""

    def __init__(self, op: "_FermionOperator", subset: int, precision: int | None = None):
        self.op = op
        h = _vp()
        _check(lib.gb_field_create(op.h, subset, op.precision if precision is None else precision, C.byref(h)))
        self.h = h
        self.precision = op.precision if precision is None else precision

    @classmethod
    def _view(cls, op: "_FermionOperator", h) -> "FermionField":
        """A field object over a handle the library owns (never destroyed through it)."""
        f = cls.__new__(cls)
        f.op, f.h, f.precision, f._borrowed = op, _vp(h), op.precision, True
        return f

    def __del__(self):
        h = getattr(self, "h", None)
        if h and not getattr(self, "_borrowed", False):
            lib.gb_field_destroy(h)
        self.h = None

    @property
    def _as_parameter_(self):
        return self.h

    @property
    def checkerboard(self) -> int:
        s = C.c_int()
        _check(lib.gb_field_subset(self.h, C.byref(s)))
        return s.value

    @checkerboard.setter
    def checkerboard(self, subset: int):
        _check(lib.gb_field_set_subset(self.h, subset))

    def host_len(self) -> int:
        n = _sz()
        _check(lib.gb_field_host_len(self.h, C.byref(n)))
        return n.value // 2

    def import_(self, a: np.ndarray) -> "FermionField":
        a = np.ascontiguousarray(a, dtype=np.complex128).reshape(-1)
        if a.size != self.host_len():
            raise GridError(1, f"host array has {a.size} complex numbers, field needs {self.host_len()}")
        _check(lib.gb_field_import(self.h, _dptr(a)))
        return self

    def export(self) -> np.ndarray:
        a = np.empty(self.host_len(), dtype=np.complex128)
        _check(lib.gb_field_export(self.h, _dptr(a)))
        return a

    def import_f32(self, a: np.ndarray) -> "FermionField":
        """The canonical form in single precision (complex64)."""
        a = np.ascontiguousarray(a, dtype=np.complex64).reshape(-1)
        if a.size != self.host_len():
            raise GridError(1, f"host array has {a.size} complex numbers, field needs {self.host_len()}")
        _check(lib.gb_field_import_f32(self.h, a.ctypes.data))
        return self

    def export_f32(self) -> np.ndarray:
        a = np.empty(self.host_len(), dtype=np.complex64)
        _check(lib.gb_field_export_f32(self.h, a.ctypes.data))
        return a

    def zero(self):
        _check(lib.gb_field_zero(self.h))
        return self

    def copy_from(self, other: "FermionField"):
        _check(lib.gb_field_copy(self.h, other.h))
        return self

    def norm2(self) -> np.ndarray:
        out = np.empty(self.op.nrhs, dtype=np.float64)
        _check(lib.gb_field_norm2(self.h, _dptr(out)))
        return out

    def inner(self, other: "FermionField") -> np.ndarray:
        out = np.empty(2 * self.op.nrhs, dtype=np.float64)
        _check(lib.gb_field_inner(self.h, other.h, _dptr(out)))
        return out[0::2] + 1j * out[1::2]


class TransferQueue:
    """gb_xfer_*: host fields in and out without blocking; the copy of the next input and of
    the last result overlap each other and the operator's kernels.  Arrays (complex128 or
    complex64, page-locked for overlap, e.g. PinnedArray) must stay alive and untouched
    until wait() returns."""

    def __init__(self, op: "_FermionOperator"):
        self.op = op
        h = _vp()
        _check(lib.gb_xfer_create(op.h, C.byref(h)))
        self.h = h
        self._held = []

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib.gb_xfer_destroy(h)
            self.h = None

    @staticmethod
    def _prec(a: np.ndarray) -> int:
        if a.dtype == np.complex128:
            return F64
        if a.dtype == np.complex64:
            return F32
        raise GridError(1, "host arrays must be complex128 or complex64")

    def import_(self, field: FermionField, a: np.ndarray):
        if not a.flags.c_contiguous or a.size != field.host_len():
            raise GridError(1, "host array must be contiguous with the field's canonical length")
        self._held.append(a)
        _check(lib.gb_xfer_import(self.h, field.h, a.ctypes.data, self._prec(a)))

    def export(self, field: FermionField, a: np.ndarray):
        if not a.flags.c_contiguous or a.size != field.host_len():
            raise GridError(1, "host array must be contiguous with the field's canonical length")
        self._held.append(a)
        _check(lib.gb_xfer_export(self.h, field.h, a.ctypes.data, self._prec(a)))

    def wait(self):
        _check(lib.gb_xfer_wait(self.h))
        self._held = []


def norm2(f: FermionField):
    return f.norm2()


def innerProduct(a: FermionField, b: FermionField):
    return a.inner(b)


def axpy(z: FermionField, a: float, x: FermionField, y: FermionField):
    _check(lib.gb_field_axpy(z.h, float(a), x.h, y.h))


def axpby(z: FermionField, a: float, b: float, x: FermionField, y: FermionField):
    _check(lib.gb_field_axpby(z.h, float(a), float(b), x.h, y.h))


def axpy_norm(z: FermionField, a: float, x: FermionField, y: FermionField):
    out = np.empty(z.op.nrhs, dtype=np.float64)
    _check(lib.gb_field_axpy_norm(z.h, float(a), x.h, y.h, _dptr(out)))
    return out


def InsertSlice(low, high: FermionField, slice_: int, orthog: int = 0):
    """InsertSlice(lowDim, higherDim, slice, 0) (Lattice_transfer.h:999-1070) along the
    fifth dimension: the 4D field `low` (canonical complex array, [site][spin][colour]
    per right-hand side) becomes slice s of the full 5D field `high`."""
    if orthog != 0:
        raise GridError(8, "InsertSlice: only the fifth dimension (orthog = 0) is supported")
    a = np.ascontiguousarray(low, dtype=np.complex128).reshape(-1)
    op = high.op
    if a.size != op.vol4 * 12 * op.nrhs:
        raise GridError(1, "4D field has the wrong size")
    _check(lib.gb_insert_slice(op.h, a.ctypes.data, 0, high.h, int(slice_)))


def ExtractSlice(high: FermionField, slice_: int, orthog: int = 0):
    """ExtractSlice(lowDim, higherDim, slice, 0): slice s of a full 5D field as a 4D
    canonical complex array."""
    if orthog != 0:
        raise GridError(8, "ExtractSlice: only the fifth dimension (orthog = 0) is supported")
    op = high.op
    out = np.empty(op.vol4 * 12 * op.nrhs, dtype=np.complex128)
    _check(lib.gb_extract_slice(op.h, high.h, int(slice_), out.ctypes.data, 0))
    return out


_proto("gb_bounded_wait_test", [_vp, _i, C.c_longlong])
_proto("gb_field_axpby_norm", [_vp, _d, _d, _vp, _vp, _dp])
_proto("gb_field_inner_norm", [_vp, _vp, _dp, _dp])


def axpby_norm(z: FermionField, a: float, b: float, x: FermionField, y: FermionField):
    """axpby_norm: z = a x + b y; returns |z|^2 per right-hand side."""
    out = np.empty(z.op.nrhs, dtype=np.float64)
    _check(lib.gb_field_axpby_norm(z.h, float(a), float(b), x.h, y.h, _dptr(out)))
    return out


def innerProductNorm(a: FermionField, b: FermionField):
    """innerProductNorm: (<a|b>, |a|^2) per right-hand side."""
    ip = np.empty(2 * a.op.nrhs, dtype=np.float64)
    nr = np.empty(a.op.nrhs, dtype=np.float64)
    _check(lib.gb_field_inner_norm(a.h, b.h, _dptr(ip), _dptr(nr)))
    return ip[0::2] + 1j * ip[1::2], nr


def rankInnerProduct(a: FermionField, b: FermionField):
    """One process, one GPU: the rank-local inner product is the global one."""
    return innerProduct(a, b)


def pickCheckerboard(cb: int, half: FermionField, full: FermionField):
    half.checkerboard = cb
    _check(lib.gb_field_pick_checkerboard(half.h, full.h))


def setCheckerboard(full: FermionField, half: FermionField):
    _check(lib.gb_field_set_checkerboard(full.h, half.h))


# ---- operators ------------------------------------------------------------------------
class _FermionOperator:
    h = None

    def _finish(self, h, U, stream):
        self.h = h
        Ls, nrhs, half4, prec = C.c_int(), C.c_int(), C.c_int64(), C.c_int()
        _check(lib.gb_op_info(h, C.byref(Ls), C.byref(nrhs), C.byref(half4), C.byref(prec)))
        self.Ls, self.nrhs, self.half_sites4, self.precision = Ls.value, nrhs.value, half4.value, prec.value
        if U is not None:
            self.ImportGauge(U)

    def __del__(self):
        if getattr(self, "h", None):
            lib.gb_op_destroy(self.h)
            self.h = None

    def ImportGauge(self, U: np.ndarray):
        U = np.ascontiguousarray(U, dtype=np.complex128).reshape(-1)
        if U.size != self.vol4 * 36:
            raise GridError(1, "gauge field has the wrong size")
        _check(lib.gb_op_import_gauge(self.h, _dptr(U)))

    def set_stream(self, stream_ptr: int):
        _check(lib.gb_op_set_stream(self.h, _vp(stream_ptr)))

    @property
    def vol4(self):
        return int(np.prod(self.dims))

    # grids
    def FermionField(self, precision=None):
        return FermionField(self, FULL, precision)

    def FermionRedBlackField(self, cb=ODD, precision=None):
        return FermionField(self, cb, precision)

    def Mass(self):
        return self.mass

    def SetMass(self, mass):
        """CayleyFermion5D::SetMass (CayleyFermion5D.h:75-78): rebuilds the Cayley
        coefficients; WilsonFermion: the mass term of M."""
        _check(lib.gb_op_set_mass(self.h, float(mass)))
        self.mass = float(mass)

    # FermionOperator interface
    def M(self, i, o): _check(lib.gb_M(self.h, i.h, o.h))
    def Mdag(self, i, o): _check(lib.gb_Mdag(self.h, i.h, o.h))
    def MdagM(self, i, o): _check(lib.gb_MdagM(self.h, i.h, o.h))
    def Dhop(self, i, o, dag): _check(lib.gb_Dhop(self.h, i.h, o.h, dag))
    def DhopEO(self, i, o, dag): _check(lib.gb_DhopEO(self.h, i.h, o.h, dag))
    def DhopOE(self, i, o, dag): _check(lib.gb_DhopOE(self.h, i.h, o.h, dag))
    def Meooe(self, i, o): _check(lib.gb_Meooe(self.h, i.h, o.h))
    def MeooeDag(self, i, o): _check(lib.gb_MeooeDag(self.h, i.h, o.h))
    def Mooee(self, i, o): _check(lib.gb_Mooee(self.h, i.h, o.h))
    def MooeeDag(self, i, o): _check(lib.gb_MooeeDag(self.h, i.h, o.h))
    def MooeeInv(self, i, o): _check(lib.gb_MooeeInv(self.h, i.h, o.h))
    def MooeeInvDag(self, i, o): _check(lib.gb_MooeeInvDag(self.h, i.h, o.h))
    def Mpc(self, i, o): _check(lib.gb_Mpc(self.h, i.h, o.h))
    def MpcDag(self, i, o): _check(lib.gb_MpcDag(self.h, i.h, o.h))
    def MpcDagMpc(self, i, o): _check(lib.gb_MpcDagMpc(self.h, i.h, o.h))

    # force terms (WilsonFermion5DImplementation.h:212-305, CayleyFermion5DImplementation.h:346-391)
    def _deriv(self, fn, A, B, dag):
        n = (self.vol4 if A.checkerboard == FULL else self.vol4 // 2) * 36
        mat = np.empty(n, dtype=np.complex128)
        _check(fn(self.h, A.h, B.h, int(dag), mat.ctypes.data, 0))
        return mat

    def DhopDeriv(self, A, B, dag):
        """force [site][mu][3][3] (full fields) or [site>>1][mu][3][3] (DerivEO/OE: half fields)"""
        return self._deriv(lib.gb_DhopDeriv, A, B, dag)

    DhopDerivEO = DhopDeriv
    DhopDerivOE = DhopDeriv

    def MDeriv(self, U, V, dag):
        return self._deriv(lib.gb_MDeriv, U, V, dag)

    MoeDeriv = MDeriv
    MeoDeriv = MDeriv

    def sync(self):
        _check(lib.gb_op_sync(self.h))

    def event(self, slot: int):
        _check(lib.gb_op_event_record(self.h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_double()
        _check(lib.gb_op_event_elapsed(self.h, a, b, C.byref(ms)))
        return ms.value

    def bench_kernel(self, which: int, ins, outs, reps: int) -> float:
        n = len(ins)
        a = (_vp * n)(*[f.h for f in ins])
        b = (_vp * n)(*[f.h for f in outs])
        ms = C.c_double()
        _check(lib.gb_bench_kernel(self.h, which, a, b, n, reps, C.byref(ms)))
        return ms.value


class WilsonFermion(_FermionOperator):
    """WilsonFermion<WilsonImplD/F>; nrhs > 1 packs right-hand sides that share U."""

    def __init__(self, U, dims, mass, phases=None, precision=F64, nrhs=1, stream=None, flags=0):
        self.dims = tuple(int(x) for x in dims)
        self.mass = float(mass)
        self.kind = 0
        ph = antiperiodic_t() if phases is None else np.ascontiguousarray(phases, dtype=np.float64)
        h = _vp()
        _check(lib.gb_wilson_create(_dims(dims), float(mass), _dptr(ph), int(precision), int(nrhs),
                                    _vp(stream or 0), int(flags), C.byref(h)))
        self._finish(h, U, stream)


_proto("gb_wilson_tm5d_create", [_ip, _i, _dp, _dp, _dp, _i, _vp, C.c_uint, C.POINTER(_vp)])
_proto("gb_op_tm_update", [_vp, _dp, _dp])
_proto("gb_field_dft_s", [_vp, _vp, _dp])
_proto("gb_field_copy_slice5", [_vp, _i, _vp, _i])
_proto("gb_field_chiral_scale", [_vp, _vp, _dp])


class WilsonTMFermion5D(_FermionOperator):
    """WilsonTMFermion5D(U, ..., mass, mu) (WilsonTMFermion5D.h:40-145): len(mass) slices
    of the 4D Wilson hop with Mooee = (4 + m_s) + i mu_s gamma5.  Its fields hold the
    slices as right-hand-side slots; its CG converges every slice."""

    def __init__(self, U, dims, mass, mu, phases=None, precision=F64, stream=None, flags=0):
        self.dims = tuple(int(x) for x in dims)
        self.kind = 0
        self.mass = 0.0
        ph = antiperiodic_t() if phases is None else np.ascontiguousarray(phases, dtype=np.float64)
        m = np.ascontiguousarray(mass, dtype=np.float64)
        u = np.ascontiguousarray(mu, dtype=np.float64)
        if m.shape != u.shape:
            raise GridError(1, "mass and mu differ in length")
        h = _vp()
        _check(lib.gb_wilson_tm5d_create(_dims(dims), int(m.size), _dptr(m), _dptr(u), _dptr(ph), int(precision),
                                         _vp(stream or 0), int(flags), C.byref(h)))
        self._finish(h, U, stream)
        self.nslices = int(m.size)

    def update(self, mass, mu):
        m = np.ascontiguousarray(mass, dtype=np.float64)
        u = np.ascontiguousarray(mu, dtype=np.float64)
        if m.size != self.nslices or u.size != self.nslices:
            raise GridError(1, "one mass and one mu per slice")
        _check(lib.gb_op_tm_update(self.h, _dptr(m), _dptr(u)))


def dft_s(src: FermionField, dst: FermionField, mat: np.ndarray):
    """dst_k = sum_s mat[k, s] src_s along the fifth dimension (complex Ls x Ls)."""
    m = np.ascontiguousarray(mat, dtype=np.complex128)
    _check(lib.gb_field_dft_s(src.h, dst.h, m.ctypes.data_as(_dp)))


def copy_slice5(dst: FermionField, t: int, src: FermionField, s: int):
    """slot t of dst = slot s of src (fields of any Ls on the same 4D lattice and stream)."""
    _check(lib.gb_field_copy_slice5(dst.h, int(t), src.h, int(s)))


def chiral_scale(src: FermionField, dst: FermionField, up, down):
    """dst = up[q] P+ src + down[q] P- src on every slot q (complex per slot)."""
    c = np.empty((len(up), 4), dtype=np.float64)
    c[:, 0], c[:, 1] = np.real(up), np.imag(up)
    c[:, 2], c[:, 3] = np.real(down), np.imag(down)
    _check(lib.gb_field_chiral_scale(src.h, dst.h, _dptr(np.ascontiguousarray(c.reshape(-1)))))


class CGSolver(C.Structure):
    """gb_cg_solver: the state of the library's CG-based solver functions."""
    _fields_ = [("cg", CGParams), ("op_lo", _vp), ("result", CGResult), ("unprec_residual", C.c_double)]


_SOLVER_FN = C.CFUNCTYPE(C.c_int, _vp, _vp, _vp, _vp)
_MADWF_CB = C.CFUNCTYPE(C.c_int, _vp, C.c_int, C.c_double)
for _n in ("gb_solver_schur", "gb_solver_pv_unprec", "gb_solver_pv_rbprec", "gb_solver_pv_fourier"):
    _proto(_n, [_vp, _vp, _vp, _vp])
_proto("gb_pv_fourier_create", [_dp, C.POINTER(CGParams), _i, C.POINTER(_vp)])
_proto("gb_pv_fourier_destroy", [_vp])
_proto("gb_pv_fourier_set_params", [_vp, C.POINTER(CGParams)])
_proto("gb_pv_fourier_result", [_vp, C.POINTER(CGResult)])
_proto("gb_madwf", [_vp, _vp, _SOLVER_FN, _vp, _SOLVER_FN, _vp, _vp, _vp, _d, _i, _MADWF_CB, _vp, _ip, _dp])


class _PVFourierHandle:
    """gb_pv_fourier_t: the library's Fourier-accelerated Pauli-Villars inverse, which keeps
    its twisted-mass operator between calls.  Holds the gauge array for the handle's life."""

    def __init__(self, Umu, cg, group_in_s):
        self.U = np.ascontiguousarray(Umu, dtype=np.complex128)
        self.cg = cg
        h = _vp()
        _check(lib.gb_pv_fourier_create(_dptr(self.U), C.byref(cg.params()), int(group_in_s), C.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            lib.gb_pv_fourier_destroy(self.h)
            self.h = None

    def __call__(self, op, src, dst):
        _check(lib.gb_pv_fourier_set_params(self.h, C.byref(self.cg.params())))
        rc = lib.gb_solver_pv_fourier(self.h, op.h, src.h, dst.h)
        r = CGResult()
        lib.gb_pv_fourier_result(self.h, C.byref(r))
        self.cg.result, self.cg.IterationsToComplete, self.cg.TrueResidual = r, r.iterations, r.true_residual
        _check(rc)


class FourierAcceleratedPV:
    """FourierAcceleratedPV(dwfPV, Umu, cg, group_in_s=2) (FourierAcceleratedPV.h:56-237):
    pvInv(src, dst) solves the Pauli-Villars (mass 1) system of a Moebius operator with
    constant real b, c by the library's gb_solver_pv_fourier: a twisted DFT along s makes
    it block diagonal, modes s and Ls-1-s pair into 5D twisted-mass Wilson systems solved
    group_in_s pairs at a time by the red-black Schur CG, and the recombined solutions are
    transformed back.  cg's IterationsToComplete is the sum over the pair solves."""

    def __init__(self, dwfPV, Umu, cg, group_in_s=2):
        self.dwfPV, self.Umu, self.cg, self.group_in_s = dwfPV, Umu, cg, int(group_in_s)
        if dwfPV.Ls % (2 * self.group_in_s) != 0:
            raise GridError(1, "Ls must be a multiple of 2 * group_in_s")
        self._pv = _PVFourierHandle(Umu, cg, self.group_in_s)

    def pvInv(self, src: FermionField, dst: FermionField):
        self._pv(self.dwfPV, src, dst)


class PauliVillarsSolverFourierAccel:
    """PauliVillarsSolverFourierAccel(Umu, CG) (PauliVillarsInverters.h:74-88): the
    Fourier-accelerated inverse of whatever Moebius operator it is called with."""

    def __init__(self, Umu, cg, group_in_s=2):
        self.Umu, self.CG, self.group_in_s = Umu, cg, int(group_in_s)
        self._pv = _PVFourierHandle(Umu, cg, self.group_in_s)

    def __call__(self, matrix, src, sol):
        if matrix.Ls % (2 * self.group_in_s) != 0:
            raise GridError(1, "Ls must be a multiple of 2 * group_in_s")
        self._pv(matrix, src, sol)


class MobiusFermion(_FermionOperator):
    """MobiusFermion<WilsonImplD/F>(U, FGrid, FrbGrid, UGrid, UrbGrid, mf, M5, b, c)."""

    def __init__(self, U, dims, Ls, mf, M5, b, c, phases=None, precision=F64, nrhs=1, stream=None, flags=0):
        self.dims = tuple(int(x) for x in dims)
        self.mass = float(mf)
        self.M5, self.b, self.c = float(M5), float(b), float(c)
        self.kind = 1
        ph = antiperiodic_t() if phases is None else np.ascontiguousarray(phases, dtype=np.float64)
        self.phases = ph
        h = _vp()
        _check(lib.gb_mobius_create(_dims(dims), int(Ls), float(mf), float(M5), float(b), float(c), _dptr(ph),
                                    int(precision), int(nrhs), _vp(stream or 0), int(flags), C.byref(h)))
        self._finish(h, U, stream)

    def cayley_coeffs(self) -> dict:
        out = np.empty(9 * self.Ls, dtype=np.float64)
        _check(lib.gb_op_cayley_coeffs(self.h, _dptr(out)))
        names = ["bs", "cs", "bee", "cee", "dee", "lee", "leem", "uee", "ueem"]
        return {n: out[k * self.Ls:(k + 1) * self.Ls].copy() for k, n in enumerate(names)}

    # CayleyFermion5D (CayleyFermion5DImplementation.h:57-153)
    def Dminus(self, i, o): _check(lib.gb_Dminus(self.h, i.h, o.h, 0))
    def DminusDag(self, i, o): _check(lib.gb_Dminus(self.h, i.h, o.h, 1))

    def _surface_in(self, fn, src4d, out5d):
        a = np.ascontiguousarray(src4d, dtype=np.complex128).reshape(-1)
        if a.size != self.vol4 * 12 * self.nrhs:
            raise GridError(1, "4D field has the wrong size")
        _check(fn(self.h, a.ctypes.data, 0, out5d.h))

    def _surface_out(self, fn, in5d):
        out = np.empty(self.vol4 * 12 * self.nrhs, dtype=np.complex128)
        _check(fn(self.h, in5d.h, out.ctypes.data, 0))
        return out

    # MADWF support (CayleyFermion5DImplementation.h:70-88)
    def P(self, i, o): _check(lib.gb_P(self.h, i.h, o.h, 0))
    def Pdag(self, i, o): _check(lib.gb_P(self.h, i.h, o.h, 1))

    def ImportPhysicalFermionSource(self, src4d, out5d):
        self._surface_in(lib.gb_import_physical_source, src4d, out5d)

    def ImportUnphysicalFermion(self, src4d, out5d):
        self._surface_in(lib.gb_import_unphysical_fermion, src4d, out5d)

    def ExportPhysicalFermionSolution(self, sol5d):
        return self._surface_out(lib.gb_export_physical_solution, sol5d)

    def ExportPhysicalFermionSource(self, src5d):
        return self._surface_out(lib.gb_export_physical_source, src5d)


class ZMobiusFermion(MobiusFermion):
    """ZMobiusFermion<WilsonImplD/F>(U, FGrid, FrbGrid, UGrid, UrbGrid, mf, M5, gamma, b, c)
    (Grid/qcd/action/fermion/ZMobiusFermion.h): complex omega_s = gamma[s]."""

    def __init__(self, U, dims, gamma, mf, M5, b, c, phases=None, precision=F64, nrhs=1, stream=None, flags=0):
        self.dims = tuple(int(x) for x in dims)
        self.mass = float(mf)
        self.M5, self.b, self.c = float(M5), float(b), float(c)
        self.gamma = [complex(z) for z in gamma]
        self.kind = 1
        ph = antiperiodic_t() if phases is None else np.ascontiguousarray(phases, dtype=np.float64)
        self.phases = ph
        gm = np.ascontiguousarray([v for z in self.gamma for v in (z.real, z.imag)], dtype=np.float64)
        h = _vp()
        _check(lib.gb_zmobius_create(_dims(dims), len(self.gamma), float(mf), float(M5), _dptr(gm), float(b), float(c),
                                     _dptr(ph), int(precision), int(nrhs), _vp(stream or 0), int(flags), C.byref(h)))
        self._finish(h, U, stream)


def zolotarev(epsilon, n, type=0):
    """Approx::zolotarev (Zolotarev.cc:296-417): (gamma, Delta) -- the Cayley-form zeros of
    the optimal rational approximation to sgn(x) on epsilon <= |x| <= 1 and its maximum
    error."""
    gamma = np.empty(int(n), dtype=np.float64)
    delta = C.c_double()
    _check(lib.gb_zolotarev(float(epsilon), int(n), int(type), _dptr(gamma), C.byref(delta)))
    return gamma, delta.value


def computeZmobiusGamma(mobius_param_out, Ls_out, mobius_param_in, Ls_in, lambda_bound):
    """Approx::computeZmobiusGamma (ZMobius.cc:149-175): (gamma, max_error) -- the Ls_out
    complex gamma_s of the ZMobius operator whose sign function best approximates, on
    0 <= x <= lambda_bound, that of the Moebius operator with Ls_in slices and b + c =
    mobius_param_in; gamma_s = mobius_param_out * omega_s."""
    gm = np.empty(2 * int(Ls_out), dtype=np.float64)
    err = C.c_double()
    _check(lib.gb_zmobius_gamma(int(Ls_out), float(mobius_param_out), int(Ls_in), float(mobius_param_in),
                                float(lambda_bound), _dptr(gm), C.byref(err)))
    return gm[0::2] + 1j * gm[1::2], err.value


def higham(epsilon, n):
    """Approx::higham (Zolotarev.cc:429-531): the tanh approximation; its Cayley zeros are
    all 1 (the Moebius operator)."""
    return np.ones(int(n), dtype=np.float64)


class MobiusZolotarevFermion(ZMobiusFermion):
    """MobiusZolotarevFermion(U, ..., mf, M5, b, c, lo, hi) (MobiusZolotarevFermion.h:45-70):
    the Cayley operator with omega_s = hi * gamma_s of zolotarev(lo / hi, Ls, 0)."""

    def __init__(self, U, dims, Ls, mf, M5, b, c, lo, hi, phases=None, precision=F64, nrhs=1, stream=None, flags=0):
        gamma, self.Delta = zolotarev(float(lo) / float(hi), Ls, 0)
        super().__init__(U, dims, list(float(hi) * gamma), mf, M5, b, c, phases, precision, nrhs, stream, flags)


class ShamirZolotarevFermion(MobiusZolotarevFermion):
    """ShamirZolotarevFermion(U, ..., mf, M5, lo, hi) (ShamirZolotarevFermion.h): b = 1, c = 0."""

    def __init__(self, U, dims, Ls, mf, M5, lo, hi, phases=None, precision=F64, nrhs=1, stream=None, flags=0):
        super().__init__(U, dims, Ls, mf, M5, 1.0, 0.0, lo, hi, phases, precision, nrhs, stream, flags)


class ScaledShamirFermion(MobiusFermion):
    """ScaledShamirFermion(U, ..., mf, M5, scale) (ScaledShamirFermion.h): Moebius with
    b + c = scale, b - c = 1."""

    def __init__(self, U, dims, Ls, mf, M5, scale, phases=None, precision=F64, nrhs=1, stream=None, flags=0):
        super().__init__(U, dims, Ls, mf, M5, 0.5 * (scale + 1.0), 0.5 * (scale - 1.0), phases, precision, nrhs, stream,
                         flags)


# ---- linear operators and solvers -----------------------------------------------------
class MdagMLinearOperator:
    kind = 0

    def __init__(self, op):
        self.op = op

    def HermOp(self, i, o):
        self.op.MdagM(i, o)

    def Op(self, i, o):
        self.op.M(i, o)

    def AdjOp(self, i, o):
        self.op.Mdag(i, o)


class SchurDiagMooeeOperator:
    kind = 1

    def __init__(self, op):
        self.op = op

    def Mpc(self, i, o):
        self.op.Mpc(i, o)

    def MpcDag(self, i, o):
        self.op.MpcDag(i, o)

    def HermOp(self, i, o):
        self.op.MpcDagMpc(i, o)

    Op = Mpc
    AdjOp = MpcDag


def _params(tol, maxit, err, **kw) -> CGParams:
    p = CGParams()
    lib.gb_cg_params_default(C.byref(p))
    p.tolerance = float(tol)
    p.max_iterations = int(maxit)
    p.err_on_no_conv = 1 if err else 0
    for k, v in kw.items():
        if v is not None:
            setattr(p, k, v)
    return p


class ConjugateGradient:
    def __init__(self, tol, maxit, err_on_no_conv=True, check_every=None, use_graphs=0):
        self.Tolerance, self.MaxIterations, self.ErrorOnNoConverge = tol, maxit, err_on_no_conv
        self.check_every = check_every
        self.use_graphs = int(use_graphs)
        self.IterationsToComplete = 0
        self.TrueResidual = 0.0
        self.result = None

    def params(self):
        return _params(self.Tolerance, self.MaxIterations, self.ErrorOnNoConverge, check_every=self.check_every,
                       use_graphs=self.use_graphs)

    def __call__(self, linop, src, psi):
        p, r = self.params(), CGResult()
        fn = lib.gb_cg_mdagm if linop.kind == 0 else lib.gb_cg_schur
        _check(fn(linop.op.h, src.h, psi.h, C.byref(p), C.byref(r)))
        self._store(r, linop.op)
        return r

    def _store(self, r, op):
        self.result = r
        self.IterationsToComplete = r.iterations
        self.TrueResidual = r.true_residual
        n = op.nrhs
        it = (C.c_int * n)()
        tr = (C.c_double * n)()
        lib.gb_cg_last_per_rhs(op.h, it, tr)
        self.per_rhs_iterations = list(it)
        self.per_rhs_true_residual = list(tr)


class ConjugateGradientReliableUpdate(ConjugateGradient):
    def __init__(self, tol, maxit, delta, linop_f, linop_d, err_on_no_conv=True, relup_every=0,
                 final_cleanup=True, check_every=None, use_graphs=0):
        super().__init__(tol, maxit, err_on_no_conv, check_every, use_graphs)
        self.Delta, self.linop_f, self.linop_d = delta, linop_f, linop_d
        self.relup_every, self.DoFinalCleanup = relup_every, final_cleanup
        self.ReliableUpdatesPerformed = 0
        self.IterationsToCleanup = 0

    def params(self):
        return _params(self.Tolerance, self.MaxIterations, self.ErrorOnNoConverge, delta=float(self.Delta),
                       relup_every=int(self.relup_every), final_cleanup=1 if self.DoFinalCleanup else 0,
                       check_every=self.check_every, use_graphs=self.use_graphs)

    def __call__(self, src, psi):
        p, r = self.params(), CGResult()
        _check(lib.gb_cg_reliable(self.linop_d.op.h, self.linop_f.op.h, self.linop_d.kind, src.h, psi.h,
                                  C.byref(p), C.byref(r)))
        self._store(r, self.linop_d.op)
        self.ReliableUpdatesPerformed = r.reliable_updates
        self.IterationsToCleanup = r.cleanup_iterations
        return r


class MixedParams(C.Structure):
    _fields_ = [("inner_tolerance", C.c_double), ("max_inner_iterations", C.c_int), ("max_outer_iterations", C.c_int),
                ("max_patchup_iterations", C.c_int), ("outer_loop_norm_mult", C.c_double)]


_proto("gb_mixed_params_default", [C.POINTER(MixedParams)], None)
_proto("gb_cg_mixed", [_vp, _vp, _i, _vp, _vp, C.POINTER(CGParams), C.POINTER(MixedParams), C.POINTER(CGResult)])


class MixedPrecisionConjugateGradient:
    """MixedPrecisionConjugateGradient(tol, maxinnerit, maxouterit, sp_grid, Linop_f, Linop_d)
    (ConjugateGradientMixedPrec.h:34-166): restarted FP32 inner CGs on Linop_f, FP64 outer
    residuals and a final FP64 patch-up CG on Linop_d.  With nrhs > 1 operators it is
    MixedPrecisionConjugateGradientBatched (every right-hand side in one inner solve)."""

    def __init__(self, tol, maxinnerit, maxouterit, sp_grid, linop_f, linop_d, maxpatchit=0, check_every=None,
                 use_graphs=0):
        self.Tolerance, self.InnerTolerance = float(tol), float(tol)
        self.MaxInnerIterations, self.MaxOuterIterations = int(maxinnerit), int(maxouterit)
        self.MaxPatchupIterations = int(maxpatchit)
        self.OuterLoopNormMult = 100.0
        self.linop_f, self.linop_d = linop_f, linop_d
        self.check_every, self.use_graphs = check_every, int(use_graphs)
        self.TotalInnerIterations = self.TotalOuterIterations = self.TotalFinalStepIterations = 0
        self.TrueResidual = 0.0

    def __call__(self, src, sol):
        if self.linop_f.kind != self.linop_d.kind:
            raise GridError(1, "Linop_f and Linop_d must be the same kind of operator")
        p, r = _params(self.Tolerance, 1, True, check_every=self.check_every, use_graphs=self.use_graphs), CGResult()
        m = MixedParams()
        lib.gb_mixed_params_default(C.byref(m))
        m.inner_tolerance = self.InnerTolerance
        m.max_inner_iterations, m.max_outer_iterations = self.MaxInnerIterations, self.MaxOuterIterations
        m.max_patchup_iterations = self.MaxPatchupIterations
        m.outer_loop_norm_mult = self.OuterLoopNormMult
        _check(lib.gb_cg_mixed(self.linop_d.op.h, self.linop_f.op.h, self.linop_d.kind, src.h, sol.h, C.byref(p),
                               C.byref(m), C.byref(r)))
        self.TotalInnerIterations, self.TotalOuterIterations = r.iterations, r.reliable_updates
        self.TotalFinalStepIterations, self.TrueResidual = r.cleanup_iterations, r.true_residual
        self.result = r
        return r


MixedPrecisionConjugateGradientBatched = MixedPrecisionConjugateGradient


MAX_SHIFTS = 32


class MultiShiftResult(C.Structure):
    _fields_ = [("nshift", C.c_int), ("iterations", C.c_int), ("converged", C.c_int),
                ("iterations_shift", C.c_int * MAX_SHIFTS), ("true_residual_shift", C.c_double * MAX_SHIFTS),
                ("seconds", C.c_double), ("flops", C.c_double)]


_proto("gb_cg_multishift", [_vp, _i, _vp, _i, _dp, _dp, C.POINTER(_vp), _i, _i, C.POINTER(MultiShiftResult)])


class MultiShiftFunction:
    """MultiShiftFunction (Grid/algorithms/approx/MultiShiftFunction.h:34-64): the poles
    (shifts, lightest first), residues, per-shift tolerances and norm of a partial-fraction
    rational function  f(x) = norm + sum_s residues[s] / (x + poles[s])."""

    def __init__(self, poles, residues=None, tolerances=1e-10, norm=0.0):
        self.order = len(poles)
        self.poles = [float(p) for p in poles]
        self.residues = [1.0] * self.order if residues is None else [float(r) for r in residues]
        self.tolerances = ([float(tolerances)] * self.order if np.isscalar(tolerances)
                           else [float(t) for t in tolerances])
        self.norm = float(norm)


class ConjugateGradientMultiShift:
    """ConjugateGradientMultiShift(maxit, shifts) (ConjugateGradientMultiShift.h:44-75):
    called with a list of output fields it solves (A + poles[s]) psi[s] = src for every
    shift; called with one output field it returns norm src + sum_s residues[s] psi[s]."""

    def __init__(self, maxit, shifts: MultiShiftFunction, check_every=10):
        self.MaxIterations = maxit
        self.shifts = shifts
        self.check_every = check_every
        self.IterationsToComplete = 0
        self.IterationsToCompleteShift = []
        self.TrueResidualShift = []

    def __call__(self, linop, src, psi):
        if isinstance(psi, FermionField):
            results = [FermionField(src.op, src.checkerboard, src.precision)
                       for _ in range(self.shifts.order)]
            self.solve(linop, src, results)
            axpby(psi, self.shifts.norm, 0.0, src, src)
            for res, r in zip(self.shifts.residues, results):
                axpby(psi, 1.0, res, psi, r)
            return psi
        return self.solve(linop, src, psi)

    def solve(self, linop, src, psi_list):
        ns = self.shifts.order
        if len(psi_list) != ns:
            raise GridError(1, "one output field per shift expected")
        m = np.ascontiguousarray(self.shifts.poles, dtype=np.float64)
        t = np.ascontiguousarray(self.shifts.tolerances, dtype=np.float64)
        ptrs = (_vp * ns)(*[f.h for f in psi_list])
        r = MultiShiftResult()
        _check(lib.gb_cg_multishift(linop.op.h, linop.kind, src.h, ns, _dptr(m), _dptr(t), ptrs,
                                    int(self.MaxIterations), int(self.check_every), C.byref(r)))
        self.IterationsToComplete = r.iterations
        self.IterationsToCompleteShift = list(r.iterations_shift[:ns])
        self.TrueResidualShift = list(r.true_residual_shift[:ns])
        self.result = r
        return r


class SchurRedBlackDiagMooeeSolve:
    """SchurRedBlackDiagMooeeSolve(solver)(op, src, sol).  `solver` is a ConjugateGradient
    (plain, in op's precision) or a ConjugateGradientReliableUpdate (mixed precision, whose
    linop_f.op supplies the inner operator)."""

    def __init__(self, solver):
        self.solver = solver
        self.unprec_residual = None

    def __call__(self, op, src, sol):
        s = self.solver
        p, r = s.params(), CGResult()
        res = np.zeros(op.nrhs, dtype=np.float64)
        _check(lib.gb_schur_solve(op.h, self._op_lo(), src.h, sol.h, C.byref(p), C.byref(r), _dptr(res)))
        self._take(r, op)
        self.unprec_residual = res
        return r

    def _op_lo(self):
        s = self.solver
        return s.linop_f.op.h if isinstance(s, ConjugateGradientReliableUpdate) else None

    def _state(self) -> CGSolver:
        """the gb_cg_solver of the library's solver functions for this solve"""
        st = CGSolver()
        st.cg = self.solver.params()
        st.op_lo = self._op_lo()
        return st

    def _take(self, r: CGResult, op):
        s = self.solver
        s._store(r, op)
        if isinstance(s, ConjugateGradientReliableUpdate):
            s.ReliableUpdatesPerformed = r.reliable_updates
            s.IterationsToCleanup = r.cleanup_iterations


class ZeroGuesser:
    """ZeroGuesser (Grid/algorithms/iterative/Guesser.h): a zero initial guess, which is
    what the Schur solve starts from."""

    def __call__(self, src, guess):
        guess.zero()


class PauliVillarsSolverUnprec:
    """PauliVillarsSolverUnprec(CG) (PauliVillarsInverters.h:32-52): M(m = 1) sol = src by
    CG on Mdag M at mass 1 (the library's gb_solver_pv_unprec, which restores the mass)."""

    def __init__(self, cg: ConjugateGradient):
        self.CG = cg

    def __call__(self, matrix, src, sol):
        st = CGSolver()
        st.cg = self.CG.params()
        rc = lib.gb_solver_pv_unprec(C.byref(st), matrix.h, src.h, sol.h)
        self.CG._store(st.result, matrix)
        _check(rc)


class PauliVillarsSolverRBprec:
    """PauliVillarsSolverRBprec(SchurSolver) (PauliVillarsInverters.h:54-72): the red-black
    Schur solve at mass 1 (the library's gb_solver_pv_rbprec)."""

    def __init__(self, schur: "SchurRedBlackDiagMooeeSolve"):
        self.SchurSolver = schur

    def __call__(self, matrix, src, sol):
        st = self.SchurSolver._state()
        rc = lib.gb_solver_pv_rbprec(C.byref(st), matrix.h, src.h, sol.h)
        self.SchurSolver._take(st.result, matrix)
        _check(rc)


class MADWFinnerIterCallbackBase:
    """Called with the outer residual at the end of every MADWF iteration."""

    def __call__(self, current_resid: float):
        pass


class MADWF:
    """MADWF(Mato, Mati, PauliVillarsSolvero, SchurSolveri, Guesseri, resid, maxiter,
    callback) (Grid/qcd/action/fermion/MADWF.h:47-209): the library's gb_madwf solves the
    outer (Moebius) system by defect correction, each step a Pauli-Villars solve of the
    outer operator and a Schur solve of the cheaper inner (e.g. ZMobius with smaller Ls)
    operator joined through the s = 0 slice of the P-rotated fields.  The two solvers (any
    callables solver(matrix, src, sol)) and the guesser are called back from it.  `src` is a
    4D field (canonical complex array, imported with ImportPhysicalFermionSource) or a full
    5D field of the outer operator; `sol5` receives the outer 5D solution.  Raises
    GridError (status NOT_CONVERGED) after maxiter steps, where Grid asserts."""

    def __init__(self, Mato, Mati, PauliVillarsSolvero, SchurSolveri, Guesseri, resid, maxiter, callback=None):
        self.Mato, self.Mati = Mato, Mati
        self.PauliVillarsSolvero, self.SchurSolveri, self.Guesseri = PauliVillarsSolvero, SchurSolveri, Guesseri
        self.target_resid, self.maxiter, self.callback = float(resid), int(maxiter), callback
        self.iterations = self.IterationsToComplete = 0
        self.FinalResidual = 0.0
        self.residuals = []

    def __call__(self, src, sol5):
        Mo, Mi = self.Mato, self.Mati
        if isinstance(src, FermionField):
            b = src
        else:
            b = Mo.FermionField()
            Mo.ImportPhysicalFermionSource(src, b)
        errors = []

        def guarded(body):
            # a Python exception cannot cross the C frames: keep it, end the solve, raise it
            def trampoline(*args):
                try:
                    body(*args)
                    return 0
                except GridError as e:
                    errors.append(e)
                    return e.status or 1
                except BaseException as e:  # noqa: BLE001 -- re-raised below
                    errors.append(e)
                    return 1
            return trampoline

        def pv(user, op, s, x):
            self.PauliVillarsSolvero(Mo, FermionField._view(Mo, s), FermionField._view(Mo, x))

        def inner(user, op, s, x):
            fs, fx = FermionField._view(Mi, s), FermionField._view(Mi, x)
            self.Guesseri(fs, fx)
            self.SchurSolveri(Mi, fs, fx)

        def step(user, it, resid):
            self.residuals.append(resid)
            self.iterations = self.IterationsToComplete = it
            self.FinalResidual = resid
            if self.callback is not None:
                self.callback(resid)

        self.residuals = []
        self.iterations = self.IterationsToComplete = 0
        pv_fn, inner_fn, cb_fn = _SOLVER_FN(guarded(pv)), _SOLVER_FN(guarded(inner)), _MADWF_CB(guarded(step))
        it, fr = C.c_int(), C.c_double()
        rc = lib.gb_madwf(Mo.h, Mi.h, pv_fn, None, inner_fn, None, b.h, sol5.h, self.target_resid, self.maxiter,
                          cb_fn, None, C.byref(it), C.byref(fr))
        self.iterations = self.IterationsToComplete = it.value
        self.FinalResidual = fr.value
        if errors:
            raise errors[0]
        _check(rc)


# ---- propagator-solve service ---------------------------------------------------------
class Request(C.Structure):
    _fields_ = [("dims", C.c_int * 4), ("Ls", C.c_int), ("mf", C.c_double), ("M5", C.c_double), ("b", C.c_double),
                ("c", C.c_double), ("eps", C.c_double), ("gauge_seed", C.c_uint64), ("nsrc", C.c_int),
                ("src_seed", C.c_uint64), ("tolerance", C.c_double), ("max_iterations", C.c_int),
                ("inner_precision", C.c_int), ("dry_seconds", C.c_double), ("t_submit", C.c_double),
                ("solution", C.POINTER(C.c_double))]


class RequestResult(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int), ("nsrc", C.c_int), ("chunk", C.c_int),
                ("iterations", C.c_int), ("reliable_updates", C.c_int), ("cleanup_iterations", C.c_int),
                ("true_residual", C.c_double), ("unprec_residual", C.c_double), ("solution_norm2", C.c_double),
                ("t_submit", C.c_double),
                ("t_start", C.c_double), ("t_end", C.c_double), ("dev_start", C.c_double), ("dev_end", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("budget_bytes", C.c_size_t), ("used_bytes", C.c_size_t), ("peak_used_bytes", C.c_size_t),
                ("running", C.c_int), ("max_running", C.c_int), ("queued", C.c_int), ("submitted", C.c_int64),
                ("finished", C.c_int64), ("now", C.c_double), ("cancelled", C.c_int64), ("rejected", C.c_int64),
                ("max_queued", C.c_int)]


_proto("gb_server_create", [C.c_size_t, _i, C.c_uint, C.POINTER(_vp)])
_proto("gb_server_submit", [_vp, C.POINTER(Request), C.POINTER(C.c_int64)])
_proto("gb_server_wait", [_vp, C.c_int64, _d])
_proto("gb_server_results", [_vp, C.POINTER(RequestResult), _i, _ip])
_proto("gb_server_stats", [_vp, C.POINTER(ServerStats)])
_proto("gb_server_destroy", [_vp])
_proto("gb_request_bytes", [C.POINTER(Request), C.POINTER(C.c_size_t)])
_proto("gb_server_set_age_limit", [_vp, _d])
_proto("gb_server_cancel_queued", [_vp, C.POINTER(C.c_int64)])
_proto("gb_server_trace", [_vp, _dp, _ip, _ip, _i, _ip])


def make_request(dims, Ls, mf, eps, gauge_seed, nsrc, src_seed, M5=1.8, b=1.5, c=0.5, tol=1e-10, maxit=20000,
                 inner=F32, dry_seconds=0.0, solution: np.ndarray | None = None) -> Request:
    r = Request()
    r.dims = (C.c_int * 4)(*[int(x) for x in dims])
    r.Ls, r.mf, r.M5, r.b, r.c, r.eps = int(Ls), float(mf), float(M5), float(b), float(c), float(eps)
    r.gauge_seed, r.nsrc, r.src_seed = int(gauge_seed), int(nsrc), int(src_seed)
    r.tolerance, r.max_iterations, r.inner_precision, r.dry_seconds = float(tol), int(maxit), int(inner), float(dry_seconds)
    r.solution = solution.ctypes.data_as(_dp) if solution is not None else C.POINTER(C.c_double)()
    r._keep = solution
    return r


def request_bytes(r: Request) -> int:
    n = C.c_size_t()
    _check(lib.gb_request_bytes(C.byref(r), C.byref(n)))
    return n.value


class Server:
    """Continuous-batching propagator-solve service (gb_server_*).  Admission: the first
    queued request that fits what is left of the HBM budget, in arrival order (or least
    work first with SHORTEST_FIRST); once the oldest has waited age_limit seconds nothing
    passes it (FIFO: only the oldest is ever admitted)."""

    DRY_RUN, GRAPHS, FIFO, SHORTEST_FIRST = 1, 2, 4, 8

    def __init__(self, hbm_budget_bytes: int, slots: int = 4, flags: int = 0):
        h = _vp()
        _check(lib.gb_server_create(int(hbm_budget_bytes), int(slots), int(flags), C.byref(h)))
        self.h = h
        self._keep = []

    def submit(self, r: Request) -> int:
        i = C.c_int64()
        self._keep.append(r)
        _check(lib.gb_server_submit(self.h, C.byref(r), C.byref(i)))
        return i.value

    def wait(self, count: int, timeout: float = 600.0) -> bool:
        return lib.gb_server_wait(self.h, int(count), float(timeout)) == 0

    def results(self, max_n: int = 4096):
        buf = (RequestResult * max_n)()
        n = C.c_int()
        _check(lib.gb_server_results(self.h, buf, max_n, C.byref(n)))
        return [buf[i] for i in range(n.value)]

    def stats(self) -> ServerStats:
        s = ServerStats()
        _check(lib.gb_server_stats(self.h, C.byref(s)))
        return s

    def set_age_limit(self, seconds: float):
        _check(lib.gb_server_set_age_limit(self.h, float(seconds)))

    def cancel_queued(self) -> int:
        """Shed every request not yet admitted (they finish with GB_ERR_CANCELLED)."""
        n = C.c_int64()
        _check(lib.gb_server_cancel_queued(self.h, C.byref(n)))
        return n.value

    def trace(self, max_n: int = 1 << 16):
        """(t, queued, running) samples at every submission, admission and completion."""
        t = np.empty(max_n, dtype=np.float64)
        q = np.empty(max_n, dtype=np.int32)
        r = np.empty(max_n, dtype=np.int32)
        n = C.c_int()
        _check(lib.gb_server_trace(self.h, t.ctypes.data_as(_dp), q.ctypes.data_as(_ip), r.ctypes.data_as(_ip),
                                   int(max_n), C.byref(n)))
        return t[:n.value], q[:n.value], r[:n.value]

    def close(self):
        if getattr(self, "h", None):
            lib.gb_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


# ---- NERSC gauge files (Grid/parallelIO/NerscIO.h) -------------------------------------
class NerscHeader(C.Structure):
    _fields_ = [("dims", C.c_int * 4), ("two_row", C.c_int), ("bits", C.c_int), ("big_endian", C.c_int),
                ("sequence_number", C.c_int), ("data_start", C.c_int64), ("link_trace", C.c_double),
                ("plaquette", C.c_double), ("checksum", C.c_uint32), ("checksum_computed", C.c_uint32),
                ("link_trace_computed", C.c_double), ("plaquette_computed", C.c_double),
                ("data_type", C.c_char * 64), ("floating_point", C.c_char * 32), ("ensemble_id", C.c_char * 64),
                ("ensemble_label", C.c_char * 64), ("boundary", (C.c_char * 32) * 4)]


_proto("gb_nersc_read_header", [C.c_char_p, C.POINTER(NerscHeader)])
_proto("gb_nersc_read", [C.c_char_p, _vp, _i, C.POINTER(NerscHeader), _i])
_proto("gb_nersc_write", [C.c_char_p, _vp, _i, _ip, _i, _i, _i, C.c_char_p, C.c_char_p, _i])
_proto("gb_gauge_stats", [_ip, _vp, _i, _dp, _dp])


def nersc_read_header(path) -> NerscHeader:
    h = NerscHeader()
    _check(lib.gb_nersc_read_header(str(path).encode(), C.byref(h)))
    return h


def nersc_read(path, check=True):
    """NerscIO::readConfiguration: (canonical FP64 gauge field, header).  The checksum,
    plaquette and link trace are verified when `check` (GridError otherwise)."""
    h = nersc_read_header(path)
    U = np.empty(int(np.prod(list(h.dims))) * 36, dtype=np.complex128)
    _check(lib.gb_nersc_read(str(path).encode(), U.ctypes.data, 0, C.byref(h), int(bool(check))))
    return U, h


def nersc_write(path, U, dims, two_row=False, bits=64, big_endian=True, ensemble_id="UKQCD", ensemble_label="DWF",
                sequence_number=1):
    """NerscIO::writeConfiguration of a canonical FP64 gauge field."""
    U = np.ascontiguousarray(U, dtype=np.complex128)
    _check(lib.gb_nersc_write(str(path).encode(), U.ctypes.data, 0, _dims(dims), int(bool(two_row)), int(bits),
                              int(bool(big_endian)), ensemble_id.encode(), ensemble_label.encode(),
                              int(sequence_number)))


class IldgHeader(C.Structure):
    _fields_ = [("dims", C.c_int * 4), ("precision", C.c_int), ("field", C.c_char * 32), ("lfn", C.c_char * 256),
                ("has_checksum", C.c_int), ("scidac_suma", C.c_uint32), ("scidac_sumb", C.c_uint32),
                ("scidac_suma_computed", C.c_uint32), ("scidac_sumb_computed", C.c_uint32),
                ("has_plaquette", C.c_int), ("plaquette", C.c_double), ("link_trace", C.c_double),
                ("plaquette_computed", C.c_double), ("link_trace_computed", C.c_double),
                ("data_offset", C.c_int64), ("data_bytes", C.c_int64)]


_proto("gb_ildg_read_header", [C.c_char_p, C.POINTER(IldgHeader)])
_proto("gb_ildg_read", [C.c_char_p, _vp, _i, C.POINTER(IldgHeader), _i])
_proto("gb_ildg_write", [C.c_char_p, _vp, _i, _ip, _i, C.c_char_p])


def ildg_read_header(path) -> IldgHeader:
    """The records of an ILDG file (no device work)."""
    h = IldgHeader()
    _check(lib.gb_ildg_read_header(str(path).encode(), C.byref(h)))
    return h


def ildg_read(path, check=True):
    """IldgReader::readConfiguration: (canonical FP64 gauge field, header); the SciDAC
    checksum, plaquette and link trace are verified when `check` (GridError otherwise)."""
    h = ildg_read_header(path)
    U = np.empty(int(np.prod(list(h.dims))) * 36, dtype=np.complex128)
    _check(lib.gb_ildg_read(str(path).encode(), U.ctypes.data, 0, C.byref(h), int(bool(check))))
    return U, h


def ildg_write(path, U, dims, precision=64, lfn=""):
    """IldgWriter::writeConfiguration of a canonical FP64 gauge field."""
    U = np.ascontiguousarray(U, dtype=np.complex128)
    _check(lib.gb_ildg_write(str(path).encode(), U.ctypes.data, 0, _dims(dims), int(precision), lfn.encode()))


_proto("gb_openqcd_read_header", [C.c_char_p, _ip, _dp])
_proto("gb_openqcd_read", [C.c_char_p, _vp, _i, _ip, _dp, _dp, _i])


def openqcd_read(path, check=True):
    """OpenQcdIO::readConfiguration: (canonical FP64 gauge field, dims (x, y, z, t),
    header plaquette, computed plaquette); the plaquettes must agree when `check`."""
    d = (C.c_int * 4)()
    p = C.c_double()
    _check(lib.gb_openqcd_read_header(str(path).encode(), d, C.byref(p)))
    U = np.empty(int(np.prod(list(d))) * 36, dtype=np.complex128)
    pc = C.c_double()
    _check(lib.gb_openqcd_read(str(path).encode(), U.ctypes.data, 0, d, C.byref(p), C.byref(pc), int(bool(check))))
    return U, tuple(d), p.value, pc.value


def gauge_stats(dims, U):
    """(avgPlaquette, linkTrace) of a canonical gauge field, computed on the device."""
    U = np.ascontiguousarray(U, dtype=np.complex128)
    p, t = C.c_double(), C.c_double()
    _check(lib.gb_gauge_stats(_dims(dims), U.ctypes.data, 0, C.byref(p), C.byref(t)))
    return p.value, t.value
