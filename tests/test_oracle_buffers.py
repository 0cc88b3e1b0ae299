"""Particles leaving and entering the state in the oracle: remove_buffer1/2
and the outflow cut-off of cellshiftalt remove exactly the particles their
rule selects and keep the rest in order; inserted particles follow the
existing ones; inserting and then removing restores the state exactly."""
import numpy as np

import oracle
from beach_slope_confined_gb300 import scenario as sc
from beach_slope_confined_gb300.binding import REMOVE_BUFFER_LEFT, REMOVE_BUFFER_RIGHT, REMOVE_OUTFLOW, setup_tank

from pairrun import small_spec

BUFFER = 0x04
FIELDS = ("x", "y", "vx", "vy", "p", "rho", "oden", "mass", "porosity", "con", "ovol")


def ctx_with_buffers():
    spec = small_spec()
    scen = sc.build(spec)
    c = oracle.context(sc.make_params(spec, scen.bounds, tol=1e-10, maxit=20000))
    setup_tank(c, scen)
    s = c.download_state()
    fl = (s["tid"] == sc.TID_FLUID) & (s["x"] < 0.3)
    s["flags"][fl] |= BUFFER
    c.upload_state(s)
    return c, spec, scen, s


def new_block(spec, x0=1.0, nx=5, ny=2):
    """A block of fluid particles above the still-water level."""
    dx = spec.dx
    xx, yy = np.meshgrid(x0 + dx * np.arange(nx), spec.depth + 2 * dx + dx * np.arange(ny), indexing="ij")
    m = xx.size
    return dict(x=xx.ravel().copy(), y=yy.ravel().copy(), vx=np.zeros(m), vy=np.zeros(m), p=np.zeros(m),
                rho=np.full(m, spec.rho0), oden=np.full(m, spec.rho0), mass=np.full(m, spec.rho0 * dx * dx),
                con=np.full(m, -0.5), tid=np.full(m, sc.TID_FLUID, np.int8), flags=np.zeros(m, np.uint8))


def test_remove_buffer_keeps_the_rest_in_order():
    c, spec, scen, s = ctx_with_buffers()
    for rule, a, sel in ((REMOVE_BUFFER_LEFT, 0.2, lambda t: ((t["flags"] & BUFFER) > 0) & (t["x"] <= 0.2)),
                         (REMOVE_BUFFER_RIGHT, 0.1, lambda t: ((t["flags"] & BUFFER) > 0) & (t["x"] >= 0.1))):
        before = c.download_state()
        gone = sel(before)
        assert gone.sum() > 0
        assert c.remove_particles(rule, a) == gone.sum()
        after = c.download_state()
        for f in FIELDS:
            assert np.array_equal(after[f], before[f][~gone]), f
        assert np.array_equal(after["tid"], before["tid"][~gone])


def test_outflow_cutoff():
    c, spec, scen, s = ctx_with_buffers()
    before = c.download_state()
    xl, yt = 1.5, 0.2
    gone = ((before["tid"] == sc.TID_FLUID) & ((before["flags"] & BUFFER) == 0) & (before["x"] <= xl)
            & (before["y"] > yt))
    assert c.remove_particles(REMOVE_OUTFLOW, xl, yt) == gone.sum() > 0
    after = c.download_state()
    assert np.array_equal(after["x"], before["x"][~gone])


def test_insert_then_remove_restores_the_state():
    c, spec, scen, s = ctx_with_buffers()
    c.remove_particles(REMOVE_BUFFER_RIGHT, -1e9)  # no buffers left
    before = c.download_state()
    blk = new_block(spec)
    blk["flags"][:] = BUFFER
    c.insert_particles(blk)
    mid = c.download_state()
    assert mid["x"].size == before["x"].size + blk["x"].size
    assert np.array_equal(mid["x"][before["x"].size:], blk["x"])
    assert np.allclose(mid["ovol"][before["x"].size:], blk["mass"] / blk["oden"], rtol=0, atol=0)
    c.remove_particles(REMOVE_BUFFER_RIGHT, -1e9)
    after = c.download_state()
    for f in FIELDS:
        assert np.array_equal(after[f], before[f]), f
