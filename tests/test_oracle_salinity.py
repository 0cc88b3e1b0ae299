"""Salinity transport in the oracle (scalar.f90), checked by invariants of
the reference's formulae (CPU):
  * a uniform concentration has no flux;
  * the flux is antisymmetric per pair once divided by ovol_i, so
    sum_i cdiff_i / ovol_i vanishes to roundoff on symmetric lists;
  * a short sub-step neither raises the maximum nor lowers the minimum;
  * densityupdate maps con to oden, mass and rho as scalar.f90:277-305.
"""
import numpy as np

import oracle
from beach_slope_confined_gb300 import scenario as sc
from beach_slope_confined_gb300.binding import setup_tank

from pairrun import small_spec


def salinity_ctx(spec=None, steps=1):
    spec = spec or small_spec()
    scen = sc.build(spec)
    c = oracle.context(sc.make_params(spec, scen.bounds, tol=1e-10, maxit=20000, salinity=True))
    setup_tank(c, scen)
    for _ in range(steps):  # a few phase-3 steps give velocities and nu_t
        c.step(1)
    return c, spec, scen


def test_uniform_concentration_has_no_flux():
    c, spec, scen = salinity_ctx(steps=0)
    s = c.download_state()
    s["con"][:] = 0.3
    c.upload_state(s)
    c.cellshift()
    c.neighbour()
    c.effpor()
    c.scalart()
    c.scalarupdate(1.0)
    assert np.array_equal(c.download_state()["con"], s["con"])


def test_flux_over_ovol_sums_to_zero():
    c, spec, scen = salinity_ctx(steps=2)
    before = c.download_state()
    c.scalart()
    c.scalarupdate(1.0)  # con changes by cdiff
    after = c.download_state()
    fl = scen.tid == sc.TID_FLUID
    q = (after["con"] - before["con"])[fl] / before["ovol"][fl]
    assert np.abs(q).max() > 0
    assert abs(q.sum()) <= 1e-11 * np.abs(q).sum()


def test_substep_keeps_bounds():
    c, spec, scen = salinity_ctx(steps=2)
    before = c.download_state()
    c.scalart()
    c.scalarupdate(spec.dt)
    after = c.download_state()
    fl = scen.tid == sc.TID_FLUID
    lo, hi = before["con"][fl].min(), before["con"][fl].max()
    assert after["con"][fl].min() >= lo - 1e-12
    assert after["con"][fl].max() <= hi + 1e-12
    assert not np.array_equal(after["con"], before["con"])


def test_densityupdate_formula():
    c, spec, scen = salinity_ctx(steps=1)
    c.densityupdate()
    s = c.download_state()
    fl = scen.tid == sc.TID_FLUID
    rmin, rmax = spec.rho0, spec.rho0 * 1.025
    od = 0.5 * (rmax + rmin) + s["con"][fl] * (rmax - rmin)
    assert np.allclose(s["oden"][fl], od, rtol=1e-15, atol=0)
    assert np.allclose(s["mass"][fl], od * s["ovol"][fl], rtol=1e-15, atol=0)
    assert np.allclose(s["rho"][fl], od * s["porosity"][fl], rtol=1e-15, atol=0)


def test_phase3_steps_move_salt():
    c, spec, scen = salinity_ctx(steps=0)
    s0 = c.download_state()
    c.step(3)
    s1 = c.download_state()
    fl = scen.tid == sc.TID_FLUID
    assert np.all(np.isfinite(s1["con"]))
    assert np.abs(s1["con"] - s0["con"])[fl].max() > 0
    # the density follows the salinity: con = -0.5 is fresh water, 0.5 sea water
    assert np.allclose(s1["oden"][fl], spec.rho0 * (1 + 0.025 * (0.5 + s1["con"][fl])), rtol=1e-14, atol=0)
    assert s1["oden"][fl].min() >= spec.rho0 * (1 - 1e-9)
    assert s1["oden"][fl].max() <= spec.rho0 * 1.025 * (1 + 1e-9)
