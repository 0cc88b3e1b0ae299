"""The mixed path's PPE assembly against the FP64 one.

The mixed path assembles its FP64 system in one of two ways: by default in
double-float arithmetic (k_assemble_df, FP32 pairs of ~48 bits, dfloat.cuh),
or with BSC_ASSEMBLY=rcp in FP64 with Newton-Raphson reciprocals (rcp_nr in
bsc_internal.cuh, a relative error of about 2^-46 per quotient).  Each runs
here against the FP64 assembly with IEEE divisions (BSC_EXACT_DIV=1) on the
same state, and the assembled, Jacobi-scaled systems are compared entry by
entry: within 1e-12, the right-hand sides within 1e-11.
"""
import os

import numpy as np
import pytest

from beach_slope_confined_gb300 import Solver, scenario as sc, setup_tank
from pairrun import small_spec

pytestmark = pytest.mark.gpu


def _assembled(env):
    old = {k: os.environ.get(k) for k in ("BSC_EXACT_DIV", "BSC_ASSEMBLY")}
    os.environ.update(env)
    try:
        spec = small_spec(piston_ramp=0.0)
        scen = sc.build(spec)
        P = sc.make_params(spec, scen.bounds, precision="mixed", tol=1e-10, maxit=20000, precond="mg")
        g = Solver(P)
    finally:
        for k, v in old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    setup_tank(g, scen)
    for stage in (g.piston, g.projection, g.cellshift, g.resetid, g.neighbour, g.effpor, g.eddyvis, g.int_vel):
        stage()
    g.ppesolve()
    rp, col, val, rhs = g.export_csr()
    g.close()
    return rp, col, val, rhs


@pytest.mark.parametrize("variant", ["df", "rcp"])
def test_mixed_assembly_matches_fp64_division(variant):
    env = {"BSC_EXACT_DIV": "0", "BSC_ASSEMBLY": "rcp" if variant == "rcp" else "df"}
    rp_a, col_a, val_a, rhs_a = _assembled(env)
    rp_b, col_b, val_b, rhs_b = _assembled({"BSC_EXACT_DIV": "1", "BSC_ASSEMBLY": "df"})
    assert np.array_equal(rp_a, rp_b) and np.array_equal(col_a, col_b)
    rel = np.abs(val_a - val_b) / np.maximum(np.abs(val_b), 1e-300)
    rel[val_b == 0] = np.abs(val_a[val_b == 0])
    print(variant, "max entry rel diff", rel.max(), "rhs rel diff",
          np.linalg.norm(rhs_a - rhs_b) / np.linalg.norm(rhs_b))
    assert rel.max() < 1e-12
    assert np.linalg.norm(rhs_a - rhs_b) <= 1e-11 * np.linalg.norm(rhs_b)
    # the switch selects a different code path: some entries differ in the last bits
    assert not np.array_equal(val_a, val_b)


def test_device_arithmetic_selftest():
    """f32_of (FP64 -> FP32 rounding on the integer pipe) against the
    hardware conversion: at most one FP32 ulp apart, and apart only on exact
    ties (rounded away from zero, not to even); rcp_nr within 2^-44 and
    sqrt_nr within 2^-42 of CUDA's correctly rounded sqrt."""
    from beach_slope_confined_gb300 import selftest

    n = 1 << 22
    mism, max_ulp, rcp_rel, sqrt_rel = selftest(n)
    print("f32_of mismatches", mism, "max ulp", max_ulp, "rcp_nr max rel", rcp_rel, "sqrt_nr max rel", sqrt_rel)
    assert max_ulp <= 1
    assert mism <= n * 1e-4
    assert rcp_rel < 2.0 ** -44
    assert sqrt_rel < 2.0 ** -42
