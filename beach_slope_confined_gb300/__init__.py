"""GB300-native ISPH step for the porous-beach solver Sinchanrc/Beach_Slope_Confined.

The product is ``libbsc.so`` (CUDA, sm_103a) behind the C ABI of
``include/bsc.h``.  This package builds it in-tree and binds it with ctypes;
``Solver`` exposes the reference's step routines by their Fortran names.
There is no CPU fallback: if the library is missing or no GPU is visible,
the calls raise.
"""
from __future__ import annotations

import ctypes
import os

from .binding import BscError, Context, csr_solve, setup_tank  # noqa: F401
from .scenario import Params, SolveInfo, Timing  # noqa: F401

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libbsc.so")

_lib = None


def lib() -> ctypes.CDLL:
    """The CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -m beach_slope_confined_gb300.build` (nvcc, sm_103a)")
        _lib = ctypes.CDLL(LIB_PATH)
        _lib.bsc_measure_peaks.argtypes = [ctypes.POINTER(ctypes.c_double)] * 3
        _lib.bsc_measure_peaks.restype = ctypes.c_int
        _lib.bsc_default_params.argtypes = [ctypes.POINTER(Params), ctypes.c_double]
        _lib.bsc_default_params.restype = ctypes.c_int
    return _lib


class Solver(Context):
    """A ``bsc_ctx`` on the current CUDA device."""

    def __init__(self, params: Params):
        super().__init__(lib(), "bsc_", params)


def solve_csr(params: Params, rowptr, col, val, b, x0):
    """bsc_csr_solve: standalone BiCGSTAB/FGMRES on a host CSR matrix."""
    return csr_solve(lib(), "bsc_", params, rowptr, col, val, b, x0)


def solve_csr_noalloc(params: Params, n: int, rowptr_ptr: int, col_ptr: int, val_ptr: int, b_ptr: int,
                      x_ptr: int, stream: int = 0):
    """bsc_csr_solve_noalloc: BiCGSTAB on a CSR matrix already in device
    memory, for hosts that may not allocate on the device.  The arguments are
    raw device addresses (int32 rowptr[n+1], int32 col, float64 val, b, x) and
    a cudaStream_t as an integer (0: the legacy default stream).  x is solved
    in place.  Returns (status, SolveInfo)."""
    f = lib().bsc_csr_solve_noalloc
    f.argtypes = [ctypes.POINTER(Params), ctypes.c_int32] + [ctypes.c_void_p] * 6 + [ctypes.POINTER(SolveInfo)]
    f.restype = ctypes.c_int
    info = SolveInfo()
    rc = f(ctypes.byref(params), int(n), rowptr_ptr, col_ptr, val_ptr, b_ptr, x_ptr, stream or None,
           ctypes.byref(info))
    return rc, info


def default_params(dl: float) -> Params:
    p = Params()
    rc = lib().bsc_default_params(ctypes.byref(p), dl)
    if rc:
        raise BscError(rc, "default_params", "")
    return p


def selftest(n: int = 1 << 22):
    """bsc_selftest: (FP32 rounding mismatches, largest FP32 ulp difference,
    largest relative errors of the Newton-Raphson reciprocal and of the
    Newton square root) over n inputs."""
    f = lib().bsc_selftest
    f.argtypes = [ctypes.c_int64, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                  ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    f.restype = ctypes.c_int
    a, b, c, d = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double(), ctypes.c_double()
    rc = f(int(n), ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d))
    if rc:
        raise BscError(rc, "selftest", "")
    return a.value, b.value, c.value, d.value


def measure_peaks():
    """(FP64 GFLOP/s, FP32 GFLOP/s, copy GB/s) measured on the current GPU."""
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    rc = lib().bsc_measure_peaks(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
    if rc:
        raise BscError(rc, "measure_peaks", "")
    return a.value, b.value, c.value
