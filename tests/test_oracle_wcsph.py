"""The oracle's WCSPH forward map and its scatter-form adjoint (CPU).

The oracle restates the calibration workload in plain FP64 C++. Its adjoint
sends each pair term's derivatives to both particles. The CUDA adjoint
gathers instead: own sums plus the neighbours' sums. Here the oracle adjoint
is checked against central differences of the oracle's own forward run. The
GPU tests then hold the CUDA path to the oracle.
"""
import numpy as np
import pytest

import oracle
from beach_slope_confined_gb300 import scenario as sc
from beach_slope_confined_gb300.binding import setup_tank

NSTEPS = 40


def orc_case(dx=0.02, dt=2e-4, **kw):
    spec = sc.TankSpec(dx=dx, dt=dt, por_cells=(16, 4), **kw)
    scen = sc.build(spec)
    c = oracle.context(sc.make_params(spec, scen.bounds, precision="fp64"))
    setup_tank(c, scen)
    wp, grid = sc.wcsph_params(spec, scen)
    c.wcsph_setup(wp)
    return c, spec, scen, grid


def test_oracle_still_tank_stays_hydrostatic():
    c, spec, scen, _ = orc_case(piston_amp=(0.0,))
    eta = c.wcsph_forward(NSTEPS, NSTEPS)
    s = c.download_state()
    fl = scen.tid == sc.TID_FLUID
    assert np.all(np.isfinite(eta))
    assert np.abs(eta).max() < 0.05 * spec.depth
    assert np.hypot(s["vx"][fl], s["vy"][fl]).max() < 0.1
    assert s["rho"][fl].min() >= 0.99 * spec.rho0


def test_oracle_adjoint_matches_finite_differences():
    c, spec, scen, grid0 = orc_case()
    w = np.random.default_rng(11).standard_normal((NSTEPS, len(spec.probes)))
    a0, b0 = spec.darcy_alpha, spec.forch_beta

    def L(a, b, grid):
        c.wcsph_set_params(a, b, grid)
        return float(np.sum(w * c.wcsph_forward(NSTEPS, NSTEPS)))

    c.wcsph_set_params(a0, b0, grid0)
    c.wcsph_forward(NSTEPS, NSTEPS)
    grad = c.wcsph_adjoint(w)
    # the relative step of 1e-3 sits between truncation and roundoff
    for k, base in ((0, a0), (1, b0)):
        h = 1e-3 * base
        ab = [(a0 + h, b0), (a0 - h, b0)] if k == 0 else [(a0, b0 + h), (a0, b0 - h)]
        fd = (L(*ab[0], grid0) - L(*ab[1], grid0)) / (2 * h)
        assert abs(grad[k] - fd) <= 1e-4 * abs(fd), (k, grad[k], fd)
    gg = np.abs(grad[2:])
    for cell in np.argsort(gg)[-3:]:
        h = 1e-3 * grid0.reshape(-1)[cell]
        gp, gm = grid0.copy().reshape(-1), grid0.copy().reshape(-1)
        gp[cell] += h
        gm[cell] -= h
        fd = (L(a0, b0, gp) - L(a0, b0, gm)) / (2 * h)
        assert abs(grad[2 + cell] - fd) <= 1e-4 * abs(fd), (cell, grad[2 + cell], fd)


def test_oracle_wcsph_rejects_bad_parameters():
    c, spec, scen, grid0 = orc_case()
    wp, grid = sc.wcsph_params(spec, scen)
    wp.nprobe = 0
    with pytest.raises(Exception):
        c.wcsph_setup(wp)
