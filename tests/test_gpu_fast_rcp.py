"""The mixed path's Newton-Raphson reciprocal (rcp_nr in bsc_internal.cuh).

The mixed path's FP64 PPE assembly divides by y0 (2 - x y0) refinement of an
FP32 reciprocal instead of the FP64 quotient; the bound is a relative error
of about 2^-46 per quotient.  Both variants run here on the same state (the
environment switch BSC_EXACT_DIV=1 selects the FP64 quotients) and the
assembled, Jacobi-scaled systems are compared entry by entry.
"""
import os

import numpy as np
import pytest

from beach_slope_confined_gb300 import Solver, scenario as sc, setup_tank
from pairrun import small_spec

pytestmark = pytest.mark.gpu


def _assembled(exact: bool):
    old = os.environ.get("BSC_EXACT_DIV")
    os.environ["BSC_EXACT_DIV"] = "1" if exact else "0"
    try:
        spec = small_spec()
        scen = sc.build(spec)
        P = sc.make_params(spec, scen.bounds, precision="mixed", tol=1e-10, maxit=20000, precond="mg")
        g = Solver(P)
    finally:
        if old is None:
            del os.environ["BSC_EXACT_DIV"]
        else:
            os.environ["BSC_EXACT_DIV"] = old
    setup_tank(g, scen)
    for stage in (g.piston, g.projection, g.cellshift, g.resetid, g.neighbour, g.effpor, g.eddyvis, g.int_vel):
        stage()
    g.ppesolve()
    rp, col, val, rhs = g.export_csr()
    g.close()
    return rp, col, val, rhs


def test_newton_reciprocal_assembly_matches_division():
    rp_a, col_a, val_a, rhs_a = _assembled(exact=False)
    rp_b, col_b, val_b, rhs_b = _assembled(exact=True)
    assert np.array_equal(rp_a, rp_b) and np.array_equal(col_a, col_b)
    # each entry: a handful of quotients, each within ~2^-46
    rel = np.abs(val_a - val_b) / np.maximum(np.abs(val_b), 1e-300)
    print("max entry rel diff", rel.max(), "rhs rel diff", np.linalg.norm(rhs_a - rhs_b) / np.linalg.norm(rhs_b))
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
