"""The reference's own tank (beach_slope_confined_gb300/reference_geometry.py,
after setup.f90 init, boundary.f90 gen_boundary and internal.f90 gen_fluid).

The reference ships no generated geometry, so the checks are: the lattice
sizes its integer formulas give for the default constants, worked by hand;
properties every block must have (counts, wall layers, dead rows, hydrostatic
pressure, the slope line, no overlapping particles, the cell memory order);
and the oracle stepping the tank and recycling its buffers as the reference's
time loop does (main.f90:80-95)."""
import math

import numpy as np
import pytest

import oracle
from beach_slope_confined_gb300 import reference_geometry as rg, scenario as sc
from beach_slope_confined_gb300.binding import REMOVE_BUFFER_LEFT, REMOVE_BUFFER_RIGHT


@pytest.fixture(scope="module")
def tank():
    return rg.build()


def blk(t, name):
    return t.block == t.block_names.index(name)


def test_lattice_sizes_by_hand(tank):
    k = tank.constants
    # fpx0 = floor(3.10 / 0.009) = 344, fpy0 = floor(0.65 / 0.009) + 1 = 73
    assert k.prrealx == (3.10 / 344) / 2.0 and k.prrealy == (0.65 / 72) / 2.0
    assert k.fmass == (0.65 * 3.10 * 1000.0) / (344 * 73)
    # bnx = floor(3.11 / 0.00882) = 352 and bny = floor(0.2 / (2 brrealy)) = 22, each + 2 bl
    assert (k.bnx, k.bny) == (358, 28)
    # the pore lattice at 2 prreal / sqrt(0.38): floor(3.10 / 0.014619) = 212, floor(0.65 / 0.014646) = 44
    assert (k.fpx, k.fpy) == (212, 44)
    assert (k.spx, k.spy) == (358, 92)
    assert k.h1 == (k.prrealy * 5.08) / (2.0 * math.sqrt(0.38))
    assert (k.cellx, k.celly) == (46, 14)        # ceil(3.11 / 4 h1) + 4, ceil(H / 4 h1) + 3
    assert k.dl == 2 * k.prrealx and k.dead_ht == 21
    assert k.line_grad == 15.0 * 22 / (180.0 * 7)


def test_block_counts_and_layers(tank):
    k, s, inp = tank.constants, tank.scenario, tank.inputs
    bn1 = math.floor((inp.wc - inp.lhs_btm - inp.open_lhs * 2 * k.prrealy) / (2 * k.brrealy)) - 2
    want = {"left_wall_low": 3 * k.bny, "left_wall_high": 3 * bn1, "bottom": 3 * (k.bnx - 6 + 7),
            "right_block": 60, "right_buffer": 5 * k.fpy, "left_buffer": 5 * inp.open_lhs}
    for name, n in want.items():
        assert blk(tank, name).sum() == n, name
    # the slope-clipped lattices, counted point by point
    sp = math.sqrt(inp.por)
    pore = sum(1 for j in range(1, k.fpx + 1) for i in range(1, k.fpy + 1)
               if not ((5 * k.brrealy + (k.fpy - i) * 2 * k.prrealy / sp + k.prrealy / sp - k.yl)
                       - k.line_grad * (5 * k.brrealx + (j - 1) * 2 * k.prrealx / sp + k.prrealx / sp
                                        + k.domain_shift - k.xl) > 0.0))
    assert blk(tank, "pore_fluid").sum() == pore
    # every wall block: one layer of wall particles facing the fluid, the rest ghosts
    low = blk(tank, "left_wall_low")
    assert np.all(s.x[low & (s.tid == sc.TID_WALL)] == s.x[low].max())
    assert (low & (s.tid == sc.TID_WALL)).sum() == k.bny - 3 + 1
    bot = blk(tank, "bottom")
    assert np.all(s.y[bot & (s.tid == sc.TID_WALL)] == s.y[bot].max())
    # fluid types
    fl = blk(tank, "pore_fluid") | blk(tank, "coastal_fluid") | blk(tank, "right_buffer") | blk(tank, "left_buffer")
    assert np.all(s.tid[fl] == sc.TID_FLUID) and np.all(s.tid[~fl] != sc.TID_FLUID)
    buf = blk(tank, "right_buffer") | blk(tank, "left_buffer")
    assert np.all((s.flags[buf] & sc.FLAG_BUFFER) > 0) and not np.any(s.flags[~buf] & sc.FLAG_BUFFER)


def test_slope_dead_rows_and_pressure(tank):
    k, s, inp = tank.constants, tank.scenario, tank.inputs
    above = lambda x, y: (y - k.yl) - k.line_grad * (x - k.xl)
    pore, coast = blk(tank, "pore_fluid"), blk(tank, "coastal_fluid")
    assert np.all(above(s.x[pore], s.y[pore]) <= 0.0)
    assert np.all(above(s.x[coast], s.y[coast] - 2 * k.dl) + k.prrealy >= 0.0)
    assert np.all(above(s.sx, s.sy) <= 0.0)
    # two dead rows, frozen, in the pore fluid and the right buffer
    for name in ("pore_fluid", "right_buffer"):
        b = blk(tank, name)
        dead = b & ((s.flags & sc.FLAG_DEAD) > 0)
        assert np.unique(np.round(s.y[dead], 12)).size == 2, name
        assert np.all(s.vx[dead] == 0.0) and np.all(s.vx[b & ~dead] != 0.0)
    # hydrostatic: p + rho g y constant within each lattice (coastal: before the 2 dl lift, top row 0)
    g = abs(inp.g) * inp.rho
    head = (s.p + g * s.y)[pore]
    assert np.ptp(head) < 1e-9 * head.max()
    c = coast & (s.p > 0)
    head = (s.p + g * (s.y - 2 * k.dl))[c]
    assert np.ptp(head) < 1e-9 * head.max()


def test_no_overlap_and_cell_order(tank):
    from scipy.spatial import cKDTree

    k, s = tank.constants, tank.scenario
    d, _ = cKDTree(np.c_[s.x, s.y]).query(np.c_[s.x, s.y], k=2)
    assert d[:, 1].min() > 0.4 * k.dl
    j, i = rg.cell_of(k, s.x, s.y)
    assert np.all(j >= 2) and np.all(i >= 2)
    key = j * 1000 + i
    assert np.all(np.diff(key) >= 0)          # x cells outer, y cells inner from the top
    j, i = rg.cell_of(k, s.sx, s.sy)
    assert np.all(j >= 2) and np.all(np.diff(j * 1000 + i) >= 0)
    assert np.allclose(s.smass, (3.23 * 0.8 * 1800.0) / (k.spx * k.spy), rtol=0, atol=0)


def test_oracle_steps_and_recycles_buffers(tank):
    k = tank.constants
    c = oracle.context(rg.params(tank, solver="fgmres", tol=1e-10, maxit=20000))
    rg.setup(c, tank)
    n0 = c.particle_count()
    c.step(2)
    s = c.download_state()
    assert (s["flags"] & sc.FLAG_BUFFER).astype(bool).sum() == 435   # no buffer crossed its release line
    assert np.isfinite(s["p"]).all() and np.hypot(s["vx"], s["vy"]).max() < 0.1
    # the buffer events of main.f90:80-95: columns 4-5 and 1-2 go and come back
    assert c.remove_particles(REMOVE_BUFFER_RIGHT, k.rv_buf_r) == tank.buffer1.x.size == 88
    c.insert_particles(rg.insertion(tank, 1))
    assert c.remove_particles(REMOVE_BUFFER_LEFT, k.rv_buf_l) == tank.buffer2.x.size == 86
    c.insert_particles(rg.insertion(tank, 2, relden=1.0))
    assert c.particle_count() == n0
    c.step(1)
    s = c.download_state()
    assert np.isfinite(s["x"]).all() and np.hypot(s["vx"], s["vy"]).max() < 0.1
    assert np.array_equal(s["con"][-86:], np.full(86, 0.5)) and np.array_equal(s["con"][-174:-86], np.full(88, -0.5))
