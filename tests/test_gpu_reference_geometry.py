"""The reference's own tank (init + gen_boundary + gen_fluid) stepped on the
GPU against the oracle: the step, the outflow cut-off and the buffer events
of the reference's time loop (main.f90:80-95, integrator.f90:55-110), on the
FP64 path within the step tolerances; the mixed path against the FP64 one."""
import numpy as np
import pytest

import oracle
from beach_slope_confined_gb300 import Solver, reference_geometry as rg, scenario as sc
from beach_slope_confined_gb300.binding import REMOVE_BUFFER_LEFT, REMOVE_BUFFER_RIGHT
from pairrun import rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tank():
    return rg.build()


def close(a, b):
    assert a["x"].size == b["x"].size
    assert np.array_equal(a["tid"], b["tid"]) and np.array_equal(a["flags"] & sc.FLAG_BUFFER, b["flags"] & sc.FLAG_BUFFER)
    for f in ("x", "y"):
        assert rel_l2(a[f], b[f]) < 1e-12, f
    for f in ("vx", "vy", "p"):
        assert rel_l2(a[f], b[f]) < 1e-7, f


def test_reference_tank_matches_oracle(tank):
    k = tank.constants
    P = rg.params(tank, solver="fgmres", tol=1e-12, maxit=20000)
    P.outflow = 1
    g, c = Solver(P), oracle.context(P)
    for ctx in (g, c):
        rg.setup(ctx, tank)
        ctx.step(2)
    close(g.download_state(), c.download_state())
    for ctx in (g, c):
        assert ctx.remove_particles(REMOVE_BUFFER_RIGHT, k.rv_buf_r) == 88
        ctx.insert_particles(rg.insertion(tank, 1))
        assert ctx.remove_particles(REMOVE_BUFFER_LEFT, k.rv_buf_l) == 86
        ctx.insert_particles(rg.insertion(tank, 2))
        ctx.step(2)
    close(g.download_state(), c.download_state())


def test_reference_tank_mixed_against_fp64(tank):
    out = {}
    for prec in ("fp64", "mixed"):
        g = Solver(rg.params(tank, precision=prec, solver="fgmres", precond="mg", tol=1e-8, maxit=2000))
        rg.setup(g, tank)
        g.step(3)
        out[prec] = g.download_state()
    a, b = out["mixed"], out["fp64"]
    for f in ("x", "y"):
        assert rel_l2(a[f], b[f]) < 1e-9, f
    for f in ("vx", "vy", "p"):
        assert rel_l2(a[f], b[f]) < 1e-5, f
