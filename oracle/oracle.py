"""Python handle on the CPU oracle (TEST INFRASTRUCTURE).

Only the test-suite, the smoke check and the CPU-baseline leg of the benchmark
import this module; the product never does.  It builds ``oracle/liboracle.so``
from ``oracle/oracle.cpp`` on demand (g++, OpenMP, -ffp-contract=off) and
binds it with the same ``Context`` class as the CUDA library, under the
``orc_`` prefix.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.cpp")
LIB = os.path.join(HERE, "liboracle.so")
ROOT = os.path.dirname(HERE)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from beach_slope_confined_gb300.binding import Context, csr_solve  # noqa: E402

CXXFLAGS = ["-std=c++17", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]


def build(force: bool = False) -> str:
    """Compile the oracle if the library is missing or older than its source."""
    deps = [SRC, os.path.join(ROOT, "include", "bsc.h")]
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(d) for d in deps)):
        return LIB
    tmp = LIB + ".tmp"
    subprocess.run(["g++", *CXXFLAGS, "-o", tmp, SRC], check=True)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.orc_num_threads.restype = ctypes.c_int
        _lib.orc_set_threads.argtypes = [ctypes.c_int32]
        _lib.orc_set_threads.restype = None
    return _lib


def context(params) -> Context:
    return Context(lib(), "orc_", params)


def solve(params, rowptr, col, val, b, x0):
    return csr_solve(lib(), "orc_", params, rowptr, col, val, b, x0)


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def num_threads() -> int:
    return int(lib().orc_num_threads())
