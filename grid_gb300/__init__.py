"""GB300-native Wilson / Moebius domain-wall fermion operators and CG solvers.

The compute path is the in-tree CUDA library ``libgbdwf.so`` (C ABI declared in
``include/gbdwf.h``); this package is a thin ctypes mirror of Grid's operator, linear
operator and solver classes over that ABI.  Importing the package loads the library and
raises if it has not been built: there is no CPU fallback.
"""
from .api import (  # noqa: F401
    GridError, lib, LIB_PATH, F64, F32, F16, RECON12, DF64, EVEN, ODD, FULL, DaggerNo, DaggerYes,
    FermionField, WilsonFermion, MobiusFermion, ZMobiusFermion, MobiusZolotarevFermion, ShamirZolotarevFermion,
    ScaledShamirFermion, zolotarev, higham, computeZmobiusGamma, WilsonTMFermion5D, FourierAcceleratedPV,
    PauliVillarsSolverFourierAccel, dft_s, copy_slice5, chiral_scale, MdagMLinearOperator, SchurDiagMooeeOperator,
    ConjugateGradient, ConjugateGradientReliableUpdate, SchurRedBlackDiagMooeeSolve, MixedPrecisionConjugateGradient,
    MixedPrecisionConjugateGradientBatched, MixedParams,
    ConjugateGradientMultiShift, MultiShiftFunction, MultiShiftResult,
    NerscHeader, nersc_read_header, nersc_read, nersc_write, gauge_stats,
    IldgHeader, ildg_read_header, ildg_read, ildg_write, openqcd_read,
    CGParams, random_gauge, unit_gauge, random_gaussian, random_z2, device_count,
    antiperiodic_t, periodic, set_device, PinnedArray, Stream, TransferQueue, norm2, innerProduct, axpy, axpby, axpy_norm,
    axpby_norm, innerProductNorm, rankInnerProduct,
    pickCheckerboard, setCheckerboard, InsertSlice, ExtractSlice, ZeroGuesser, PauliVillarsSolverUnprec,
    PauliVillarsSolverRBprec, MADWF, MADWFinnerIterCallbackBase, Server, Request, make_request, request_bytes,
)
