"""Particles leaving and entering the state on the GPU (csrc/buffers.cu)
against the oracle: the device compaction removes the same particles and
keeps the same order; insertion (including growth past the allocated
capacity) appends the same particles; whole steps afterwards agree within
the step tolerances."""
import numpy as np
import pytest

from beach_slope_confined_gb300 import Solver, scenario as sc
from beach_slope_confined_gb300.binding import REMOVE_BUFFER_LEFT, REMOVE_BUFFER_RIGHT, REMOVE_OUTFLOW
from pairrun import make_pair, rel_l2, small_spec
from test_oracle_buffers import BUFFER, new_block

pytestmark = pytest.mark.gpu


def pair():
    spec = small_spec()
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, tol=1e-12, maxit=20000)
    g, c = make_pair(scen, P, Solver)
    for ctx in (g, c):
        s = ctx.download_state()
        s["flags"][(s["tid"] == sc.TID_FLUID) & (s["x"] < 0.3)] |= BUFFER
        ctx.upload_state(s)
    return g, c, spec


MOVED = ("x", "y", "vx", "vy", "p", "oden", "mass", "con", "ovol")  # moved, never recomputed


def same(a, b):
    for f in MOVED:
        assert a[f].shape == b[f].shape, f
        assert np.array_equal(a[f], b[f]), f
    # porosity (and rho = n oden) come from effpor's sums, in different orders
    for f in ("porosity", "rho"):
        assert np.allclose(a[f], b[f], rtol=1e-13, atol=0), f


def test_removal_matches_oracle_and_steps():
    g, c, spec = pair()
    for rule, a, b in ((REMOVE_BUFFER_LEFT, 0.2, 0.0), (REMOVE_OUTFLOW, 1.0, 0.25), (REMOVE_BUFFER_RIGHT, 0.0, 0.0)):
        kg, kc = g.remove_particles(rule, a, b), c.remove_particles(rule, a, b)
        assert kg == kc > 0, (rule, kg, kc)
        same(g.download_state(), c.download_state())
    for ctx in (g, c):
        ctx.step(3)
    a, b = g.download_state(), c.download_state()
    for f in ("x", "y"):
        assert rel_l2(a[f], b[f]) < 1e-12, f
    for f in ("vx", "vy", "p"):
        assert rel_l2(a[f], b[f]) < 1e-7, f


def test_insertion_grows_and_matches_oracle():
    g, c, spec = pair()
    n0 = g.download_state()["x"].size
    # the first block exceeds the allocated rows (growth); the second fits the headroom
    for x0, nx in ((1.0, 6), (2.0, 4)):
        blk = new_block(spec, x0=x0, nx=nx)
        for ctx in (g, c):
            ctx.insert_particles(blk)
        a, b = g.download_state(), c.download_state()
        same(a, b)
        assert np.array_equal(a["x"][-blk["x"].size:], blk["x"])
    assert a["x"].size == n0 + 6 * 2 + 4 * 2
    for ctx in (g, c):
        ctx.step(3)
    a, b = g.download_state(), c.download_state()
    for f in ("x", "y"):
        assert rel_l2(a[f], b[f]) < 1e-12, f
    for f in ("vx", "vy", "p"):
        assert rel_l2(a[f], b[f]) < 1e-7, f


def test_outflow_inside_the_step_matches_oracle():
    spec = small_spec()
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, tol=1e-12, maxit=20000)
    P.outflow, P.outflow_xcut, P.outflow_ycut = 1, 0.5, 0.26  # drops the top rows near the piston
    g, c = make_pair(scen, P, Solver)
    n0 = g.download_state()["x"].size
    for ctx in (g, c):
        ctx.step(3)
    a, b = g.download_state(), c.download_state()
    assert a["x"].size == b["x"].size < n0
    for f in ("x", "y"):
        assert rel_l2(a[f], b[f]) < 1e-12, f
    for f in ("vx", "vy", "p"):
        assert rel_l2(a[f], b[f]) < 1e-7, f
