"""Salinity transport on the GPU (csrc/scalar.cu) against the oracle.

scalart's flux, scalarupdate and densityupdate are compared routine by
routine on the same state. Whole phase-3 steps (main.f90:198-260) are
compared over a few steps, on both solvers' stopping tolerances.
"""
import numpy as np
import pytest

from beach_slope_confined_gb300 import Solver, scenario as sc
from pairrun import make_pair, rel_l2, small_spec

pytestmark = pytest.mark.gpu


def pair(steps=2, **kw):
    spec = small_spec()
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, tol=1e-12, maxit=20000, salinity=True, **kw)
    g, c = make_pair(scen, P, Solver)
    for ctx in (g, c):
        ctx.step(steps)
    return g, c, scen


def test_scalart_flux_matches_oracle():
    g, c, scen = pair()
    fl = scen.tid == sc.TID_FLUID
    before = [ctx.download_state()["con"] for ctx in (g, c)]
    for ctx in (g, c):
        ctx.scalart()
        ctx.scalarupdate(1.0)  # con changes by exactly cdiff
    after = [ctx.download_state()["con"] for ctx in (g, c)]
    dg, dc = (after[0] - before[0])[fl], (after[1] - before[1])[fl]
    assert np.abs(dc).max() > 0
    assert rel_l2(before[0], before[1]) < 1e-11
    assert rel_l2(dg, dc) < 1e-9, rel_l2(dg, dc)


def test_densityupdate_matches_oracle():
    g, c, scen = pair(steps=1)
    for ctx in (g, c):
        ctx.densityupdate()
    a, b = g.download_state(), c.download_state()
    for f in ("oden", "mass", "rho"):
        assert rel_l2(a[f], b[f]) < 1e-12, f


@pytest.mark.parametrize("solver", ["bicgstab", "fgmres"])
def test_phase3_steps_match_oracle(solver):
    g, c, scen = pair(steps=4, solver=solver)
    a, b = g.download_state(), c.download_state()
    for f in ("x", "y", "con", "oden"):
        assert rel_l2(a[f], b[f]) < 1e-10, f
    for f in ("vx", "vy", "p"):
        assert rel_l2(a[f], b[f]) < 1e-7, f


def test_mixed_phase3_runs():
    spec = small_spec(dx=0.01)
    scen = sc.build(spec)
    out = {}
    for prec in ("fp64", "mixed"):
        P = sc.make_params(spec, scen.bounds, precision=prec, tol=1e-8, maxit=20000, precond="mg",
                           solver="fgmres", salinity=True)
        g, _ = make_pair(scen, P, Solver)
        info = g.step(3)
        assert info.converged
        out[prec] = g.download_state()
    assert rel_l2(out["mixed"]["con"], out["fp64"]["con"]) < 1e-8
