"""The C ABI without a GPU: layout of the structs and the exported symbols.

* every struct of include/bsc.h has the same size and field offsets in C
  (compiled here with gcc) as in the ctypes mirror the Python host uses;
* libbsc.so loads and exports every function include/bsc.h declares
  (symbols are resolved, nothing is called);
* with no visible GPU, creating a context fails with BSC_E_NOT_BUILT rather
  than falling back to the CPU.
"""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from beach_slope_confined_gb300 import scenario as sc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "bsc.h")


def _declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(bsc_[a-z0-9_]+)\s*\(", src, re.M)))


def _c_layout(struct, fields):
    body = "\n".join(f'printf("%zu\\n", offsetof({struct}, {f}));' for f in fields)
    prog = f"""
#include <stdio.h>
#include <stddef.h>
#include "{HEADER}"
int main(void) {{ printf("%zu\\n", sizeof({struct})); {body} return 0; }}
"""
    with tempfile.TemporaryDirectory() as d:
        c, exe = os.path.join(d, "t.c"), os.path.join(d, "t")
        open(c, "w").write(prog)
        subprocess.run(["gcc", "-std=c99", "-o", exe, c], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    return [int(v) for v in out]


@pytest.mark.parametrize("struct,cls", [("bsc_params", sc.Params), ("bsc_state_view", sc.StateView),
                                        ("bsc_solve_info", sc.SolveInfo), ("bsc_timing", sc.Timing)])
def test_struct_layout_matches_ctypes(struct, cls):
    fields = [f[0] for f in cls._fields_]
    got = _c_layout(struct, fields)
    assert got[0] == ctypes.sizeof(cls)
    assert got[1:] == [getattr(cls, f).offset for f in fields]


def _lib_path():
    from beach_slope_confined_gb300 import LIB_PATH, build

    if not os.path.exists(LIB_PATH):
        build.build()
    return LIB_PATH


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(_lib_path())
    missing = [f for f in _declared_functions() if not hasattr(lib, f)]
    assert not missing, missing
    assert len(_declared_functions()) >= 30


def test_oracle_mirrors_the_step_routines():
    import oracle

    lib = oracle.lib()
    for f in _declared_functions():
        name = f.replace("bsc_", "orc_")
        if f in ("bsc_default_params", "bsc_measure_peaks", "bsc_get_timings", "bsc_reset_timings",
                 "bsc_synchronize", "bsc_csr_solve_noalloc", "bsc_selftest", "bsc_snapshot_begin",
                 "bsc_snapshot_wait"):
            continue
        assert hasattr(lib, name), name


def test_no_gpu_means_no_context():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    from beach_slope_confined_gb300 import BscError, Solver

    with pytest.raises(BscError) as e:
        Solver(sc.make_params(sc.TankSpec()))
    assert e.value.code == -8


@pytest.mark.parametrize("bad", [dict(mg_sweeps=0), dict(mg_omega=2.5), dict(mg_coarse_max=1000),
                                 dict(mg_scale=0.0)])
def test_multigrid_parameters_are_validated(bad):
    """bsc_create rejects out-of-range multigrid settings before touching a GPU."""
    from beach_slope_confined_gb300 import BscError, Solver

    with pytest.raises(BscError) as e:
        Solver(sc.make_params(sc.TankSpec(), precond="mg", **bad))
    assert e.value.code == -1
