"""The reference's own scenario: the confined coastal aquifer with a beach
slope that ``init``, ``gen_boundary`` and ``gen_fluid`` build before the time
loop (setup.f90:9-151, boundary.f90:12-605, internal.f90:10-473, called at
main.f90:21-23).  With it the reference's geometry runs through this
library's step as it is, so the two can be compared on the same particles.

The geometry is nine rectangular lattices, each a 2-D array ``(row, column)``
walked column by column as the Fortran loops do:

- four wall blocks: the left wall below the inlet, the left wall above it, the
  bottom and the right-hand block (boundary.f90:24-33, 202-216, 300-309,
  393-404).  The innermost layer is wall (tid 1), the others ghost (tid 2);
- the soil lattice below the slope line (boundary.f90:528-549), returned as
  the porous solids;
- the fluid in the pores below the slope, at spacing 2 prreal/sqrt(por)
  (internal.f90:38-79);
- the right-hand inflow buffer, five columns (internal.f90:117-171);
- the coastal water above the slope, at spacing 2 prreal, lifted by 2 dl
  (internal.f90:262-304);
- the left-hand inflow buffer in the inlet opening, five columns
  (internal.f90:352-398).

Every particle is kept only when it falls in an interior cell of the
reference's cell grid (columns 2..cellx-1, rows 2..celly-1; setup.f90:126-137),
and the particles come out in the reference's memory order: cell by cell (x
cells outer, y cells inner from the top), in each cell in generation order.

Expressions keep the source's operand order; integer products stay integer
until they meet a real, as in Fortran.  The reference is built with -Ofast,
which may reassociate some of them, so positions agree with a given build of
the reference to a few ulps, not bit for bit.
"""
from __future__ import annotations

import dataclasses
import math
from typing import Dict, List, Optional

import numpy as np

from . import scenario as sc

TID_SOLID = 4  # boundary.f90:539


@dataclasses.dataclass
class RefInputs:
    """The module constants of initialize.f90:19-56 that the geometry reads."""

    wc: float = 0.650                   # water column over the slope toe
    L: float = 3.11
    H: float = 0.80
    pr: float = 0.0050 * 0.90           # nominal fluid half-spacing
    br: float = 0.00490 * 0.90          # nominal wall half-spacing
    wl: float = 3.10
    rho: float = 1000.0
    g: float = -9.810
    soill: float = 3.230
    soilh: float = 0.80
    set_ht: float = 0.10
    coastal_ht: float = 0.550
    por: float = 0.380
    bulkden: float = 1800.0
    entry_vel: float = -2.5 / (3600 * 24)
    lhs_btm: float = 0.20
    rel_den: float = 1.0250
    line_grad: float = 15.0             # slope angle in degrees, pi taken as 22/7
    hfac: float = 5.080
    distfac: float = 1.0
    bl: int = 3                         # wall layers
    open_lhs: int = 43                  # rows of the left-hand inlet
    incr: int = 4                       # cell side in units of h1


@dataclasses.dataclass
class RefConstants:
    """What ``init`` derives (setup.f90:47-151) and the two generators add."""

    prrealx: float
    prrealy: float
    brrealx: float
    brrealy: float
    solidx: float
    solidy: float
    fmass: float
    domain_shift: float
    h1: float
    dl: float
    lam: float
    cell: float                         # incr * h1
    cellx: int
    celly: int
    bnx: int
    bny: int
    fpx: int                            # the pore-fluid lattice (after setup.f90:88-89)
    fpy: int
    spx: int
    spy: int
    H: float
    xl: float
    yl: float
    line_grad: float                    # the slope as dy/dx
    xlcutoff: float
    ytcutoff: float                     # as gen_boundary leaves it (boundary.f90:204)
    xrcutoff: float                     # right end of comp_pos's buffer release window (setup.f90:94)
    release_xmin: float                 # left end of it (integrator.f90:886)
    ins_1: float                        # insertion periods (internal.f90:34-35)
    ins_2: float
    rv_buf_l: float                     # buffer removal lines (internal.f90:37-40)
    rv_buf_r: float
    dead_ht: int


def derive(inp: RefInputs) -> RefConstants:
    """setup.f90:47-151 (init)."""
    por = inp.por
    fpy = math.floor(inp.wc / (2 * inp.pr)) + 1
    fpx = math.floor(inp.wl / (2 * inp.pr))
    prrealx = (inp.wl / fpx) / 2.0
    prrealy = (inp.wc / (fpy - 1)) / 2.0
    fmass = ((inp.wc * inp.wl * 1.0) * inp.rho) / (fpx * fpy)
    spy = math.floor(inp.soilh / (2 * prrealy)) + 4
    spx = math.floor(inp.soill / (2 * prrealx))
    solidx = (inp.soill / spx) / 2.0
    solidy = (inp.soilh / (spy - 1)) / 2.0
    L = inp.L
    H = inp.H + 2 * prrealy
    bny = math.floor(H / (2 * inp.br))
    bnx = math.floor(L / (2 * inp.br))
    brrealx = (L / bnx) / 2.0
    brrealy = (H / bny) / 2.0
    h1 = (max(prrealx, prrealy) * inp.hfac) / (2.0 * math.sqrt(por))
    cell = inp.incr * h1
    cellx = math.ceil(L / cell) + 4
    celly = math.ceil(H / cell) + 3
    dl = min(2 * prrealx, 2 * prrealy)
    bny = math.floor(inp.lhs_btm / (2 * brrealy))
    domain_shift = 5 * prrealx
    bnx = bnx + 2 * inp.bl
    bny = bny + 2 * inp.bl
    bl = inp.bl
    xl = (2 * bl - 1) * brrealx + brrealx
    yl = (2 * bl - 1) * brrealy + solidy + inp.set_ht
    line_grad = (inp.line_grad * 22) / (180.0 * 7)
    sp = math.sqrt(por)
    fpy = math.floor(inp.wc / (2 * prrealy / sp))
    fpx = math.floor(inp.wl / (2 * prrealx / sp))
    xlcutoff = (brrealx * (2 * bl - 1)) + brrealx
    xrcutoff = (brrealx * (2 * bl - 1)) + (fpx - 1) * 2 * prrealx / sp + 3 * prrealx / sp + domain_shift - 0.001
    release_xmin = 8 * prrealx + brrealx + 0.001
    # gen_boundary's value (boundary.f90:200-204) replaces init's
    remain_len = inp.wc - inp.lhs_btm - inp.open_lhs * 2 * prrealy
    bn1 = math.floor(remain_len / (2 * brrealy)) - 2
    ytcutoff = (bny * 2 * brrealy) + (inp.open_lhs * 2 * prrealy) + bn1 * brrealy * 2 - brrealy
    # gen_fluid's event constants (internal.f90:30-40)
    bounlen = fpy * 2 * prrealy
    bounlen2 = inp.open_lhs * 2 * prrealy
    ins_1 = (4 * prrealx / sp) / abs(inp.entry_vel / 0.387)
    ins_2 = 4 * prrealx / ((bounlen / bounlen2) * abs(inp.entry_vel))
    rv_buf_r = ((brrealx * (2 * bl - 1)) + (fpx - 1) * 2 * prrealx / sp + prrealx / sp + domain_shift
                + 3 * 2 * prrealx / sp + 0.5 * prrealx / sp)
    rv_buf_l = 2 * prrealx + brrealx + 0.5 * prrealx
    dead_ht = math.ceil(0.3 / (2 * prrealy / sp))
    return RefConstants(prrealx, prrealy, brrealx, brrealy, solidx, solidy, fmass, domain_shift, h1, dl,
                        0.0010 * h1 ** 2, cell, cellx, celly, bnx, bny, fpx, fpy, spx, spy, H, xl, yl, line_grad,
                        xlcutoff, ytcutoff, xrcutoff, release_xmin, ins_1, ins_2, rv_buf_l, rv_buf_r, dead_ht)


@dataclasses.dataclass
class Block:
    """One generated lattice, flattened column by column."""

    name: str
    x: np.ndarray
    y: np.ndarray
    tid: np.ndarray
    vx: np.ndarray
    p: np.ndarray
    flags: np.ndarray
    mass: float
    density: float


def _grid(nrow: int, ncol: int):
    """Fortran indices (i, j) = (row, column), 1-based, in column-major order."""
    j, i = np.meshgrid(np.arange(1, ncol + 1), np.arange(1, nrow + 1))
    return i.ravel(order="F").astype(np.int64), j.ravel(order="F").astype(np.int64)


def _block(name, x, y, tid, mass, density, vx=None, p=None, flags=None) -> Block:
    n = x.size
    return Block(name, x, y, tid.astype(np.int8),
                 np.zeros(n) if vx is None else vx, np.zeros(n) if p is None else p,
                 np.zeros(n, np.uint8) if flags is None else flags.astype(np.uint8), mass, density)


def gen_boundary(inp: RefInputs, k: RefConstants) -> List[Block]:
    """boundary.f90:12-605: the four wall blocks and the soil lattice."""
    bl, brx, bry, ds = inp.bl, k.brrealx, k.brrealy, k.domain_shift
    sp = math.sqrt(inp.por)
    out = []
    # left wall below the inlet (boundary.f90:24-86)
    i, j = _grid(k.bny, bl)
    x = (j - 1) * brx * 2 + ds
    y = ((k.bny - i) * bry) * 2.0
    wall = (j == bl) & (i <= k.bny - bl + 1)
    out.append(_block("left_wall_low", x, y, np.where(wall, 1, 2), k.fmass, inp.rho))
    # left wall above the inlet (boundary.f90:200-232)
    remain_len = inp.wc - inp.lhs_btm - inp.open_lhs * 2 * k.prrealy
    bn1 = max(math.floor(remain_len / (2 * bry)) - 2, 0)
    i, j = _grid(bn1, bl)
    x = (j - 1) * brx * 2 + ds
    y = (k.bny * 2 * bry) + (inp.open_lhs * 2 * k.prrealy) + (bn1 - i) * bry * 2
    out.append(_block("left_wall_high", x, y, np.where(j == bl, 1, 2), k.fmass, inp.rho))
    # bottom (boundary.f90:300-330)
    nb = k.bnx - 2 * bl + 7
    i, j = _grid(bl, nb)
    x = (2 * bl - 1) * brx + brx + (j - 1) * brx * 2 + ds
    y = (bl - i) * 2 * bry
    out.append(_block("bottom", x, y, np.where(i == 1, 1, 2), k.fmass, inp.rho))
    # right-hand block behind the outflow buffer (boundary.f90:393-420)
    buy1 = k.fpy - 1
    i, j = _grid(20, bl)
    y = ((bry * (2 * bl - 1)) + buy1 * 2 * k.prrealy / sp + 2 * k.prrealy / sp) + bry + (20 - i) * 2 * bry
    x = ((brx * (2 * bl - 1)) + (k.fpx - 1) * 2 * k.prrealx / sp + 3 * k.prrealx / sp) + (j - 1) * 2 * brx + ds
    out.append(_block("right_block", x, y, np.where(j == 1, 1, 2), k.fmass, inp.rho))
    # soil lattice, dropped above the slope line (boundary.f90:528-549)
    i, j = _grid(k.spy, k.spx)
    y = (k.spy - i) * 2 * k.solidy + k.solidy + (bry * (2 * bl - 1)) - 6 * k.solidy
    x = (brx * (2 * bl - 1)) + (j - 1) * 2 * k.solidx + brx - 6 * k.solidx + ds
    below = ~(((y - k.yl) - k.line_grad * (x - k.xl)) > 0.0)
    smass = ((inp.soill * inp.soilh) * inp.bulkden) / (k.spx * k.spy)
    out.append(_block("soil", x[below], y[below], np.full(int(below.sum()), TID_SOLID), smass, inp.bulkden))
    return out


def gen_fluid(inp: RefInputs, k: RefConstants):
    """internal.f90:10-473: the two fluid lattices and the two inflow buffers,
    and the templates that insert_buffer1/2 put back (buffer1, buffer2)."""
    bl, brx, bry, ds, rho = inp.bl, k.brrealx, k.brrealy, k.domain_shift, inp.rho
    sp = math.sqrt(inp.por)
    prx, pry = k.prrealx, k.prrealy
    fpx, fpy = k.fpx, k.fpy
    g = abs(inp.g)
    x0 = bry * (2 * bl - 1)  # the bottom wall's top row, (2 bl - 1) brrealy
    head = (bry * inp.distfac) * (2 * bl - 1)

    def dead_rows(i, nrow):
        dcount = nrow - i + 1  # counted from the top row down
        return (dcount > k.dead_ht) & (dcount <= k.dead_ht + 2)

    blocks = []
    # pore fluid below the slope (internal.f90:38-79)
    i, j = _grid(fpy, fpx)
    y = x0 + (fpy - i) * 2 * pry / sp + pry / sp
    x = (brx * (2 * bl - 1)) + (j - 1) * 2 * prx / sp + prx / sp + ds
    vx = np.full(x.size, inp.entry_vel * fpy / fpy)
    p = (-y + head + inp.wc + pry / sp) * rho * g
    dead = dead_rows(i, fpy)
    vx[dead] = 0.0
    keep = ~(((y - k.yl) - k.line_grad * (x - k.xl)) > 0.0)
    fl = np.where(dead, sc.FLAG_DEAD, 0)
    blocks.append(_block("pore_fluid", x[keep], y[keep], np.full(int(keep.sum()), sc.TID_FLUID), k.fmass, rho,
                         vx[keep], p[keep], fl[keep]))
    # right-hand inflow buffer, five columns (internal.f90:117-171)
    i, j = _grid(fpy, 5)
    y = x0 + (fpy - i) * 2 * pry / sp + pry / sp
    x = (brx * (2 * bl - 1)) + (fpx - 1) * 2 * prx / sp + prx / sp + ds + j * 2 * prx / sp
    vx = np.full(x.size, inp.entry_vel * fpy / (fpy - 2))
    p = (-y + head + inp.wc + pry / sp) * rho * g
    dead = dead_rows(i, fpy)
    vx[dead] = 0.0
    fl = sc.FLAG_BUFFER | np.where(dead, sc.FLAG_DEAD, 0)
    blocks.append(_block("right_buffer", x, y, np.full(x.size, sc.TID_FLUID), k.fmass, rho, vx, p, fl))
    tpl = j > 3  # buffer1 = columns 4 and 5 (internal.f90:142-160)
    buffer1 = _block("buffer1", x[tpl], y[tpl], np.full(int(tpl.sum()), sc.TID_FLUID), k.fmass, rho, vx[tpl],
                     p[tpl], fl[tpl])
    # coastal water above the slope (internal.f90:262-304)
    cpy = math.floor(inp.coastal_ht / (2 * pry)) + 1
    cpx = math.floor(2.0 / (2 * prx))
    i, j = _grid(cpy, cpx)
    y = x0 + (cpy - i) * 2 * pry + pry + inp.set_ht
    x = (brx * (2 * bl - 1)) + (j - 1) * 2 * prx + prx + ds
    p = np.where(i == 1, 0.0, (-y + head + inp.coastal_ht + pry + inp.set_ht) * rho * g)
    keep = ~(((y - k.yl + pry) - k.line_grad * (x - k.xl)) < 0.0)
    y = y + 2 * k.dl  # the kept ones are lifted (internal.f90:290)
    blocks.append(_block("coastal_fluid", x[keep], y[keep], np.full(int(keep.sum()), sc.TID_FLUID), k.fmass * 1.0,
                         rho * 1.0, None, p[keep]))
    # left-hand inflow buffer in the inlet, five columns (internal.f90:352-398)
    bounlen = fpy * 2 * pry
    bounlen2 = inp.open_lhs * 2 * pry
    i, j = _grid(inp.open_lhs, 5)
    y = 2 * k.bny * bry - bry + pry + (inp.open_lhs - i) * 2 * pry
    x = (j - 1) * 2 * prx + brx
    vx = np.full(x.size, (-bounlen / bounlen2) * inp.entry_vel)
    p = (-y + head + inp.wc + pry) * rho * g
    fl = np.full(x.size, sc.FLAG_BUFFER)
    blocks.append(_block("left_buffer", x, y, np.full(x.size, sc.TID_FLUID), k.fmass * 1.0, rho * 1.0, vx, p, fl))
    tpl = j <= 2  # buffer2 = columns 1 and 2, pressure scaled by rel_den (internal.f90:376-388)
    buffer2 = _block("buffer2", x[tpl], y[tpl], np.full(int(tpl.sum()), sc.TID_FLUID), k.fmass, rho, vx[tpl],
                     p[tpl] * inp.rel_den, fl[tpl])
    return blocks, buffer1, buffer2


def cell_of(k: RefConstants, x: np.ndarray, y: np.ndarray):
    """The interior cell (column j, row i) holding each point, -1 outside:
    dpcell(i,j) spans [(j-2) c, (j-1) c) x [(celly-1-i) c, (celly-i) c)
    (setup.f90:130-133), over j = 2..cellx-1 and i = 2..celly-1."""
    xe = np.arange(0, k.cellx - 1) * k.cell  # left edges of columns 2.., then the right edge
    ye = np.arange(0, k.celly - 1) * k.cell  # bottom edges of rows celly-1, celly-2, ...
    cx = np.searchsorted(xe, x, side="right") - 1  # column j - 2
    cy = np.searchsorted(ye, y, side="right") - 1  # celly - 1 - row i
    inside = (cx >= 0) & (cx < k.cellx - 2) & (cy >= 0) & (cy < k.celly - 2)
    j = np.where(inside, cx + 2, -1)
    i = np.where(inside, k.celly - 1 - cy, -1)
    return j, i


def _binned(k: RefConstants, blocks: List[Block]):
    """Concatenate blocks in generation order, drop what no interior cell
    holds, and sort stably by the cell loop order (j outer, i inner)."""
    x = np.concatenate([b.x for b in blocks])
    y = np.concatenate([b.y for b in blocks])
    j, i = cell_of(k, x, y)
    inside = j >= 0
    key = j.astype(np.int64) * (k.celly + 1) + i
    order = np.nonzero(inside)[0]
    order = order[np.argsort(key[order], kind="stable")]
    cat = lambda f: np.concatenate([getattr(b, f) for b in blocks])[order]
    per = lambda v: np.concatenate([np.full(b.x.size, getattr(b, v)) for b in blocks])[order]
    src = np.concatenate([np.full(b.x.size, q) for q, b in enumerate(blocks)])[order]
    return dict(x=cat("x"), y=cat("y"), tid=cat("tid"), vx=cat("vx"), p=cat("p"), flags=cat("flags"),
                mass=per("mass"), rho=per("density"), block=src)


@dataclasses.dataclass
class ReferenceTank:
    inputs: RefInputs
    constants: RefConstants
    scenario: sc.Scenario
    block_names: List[str]
    block: np.ndarray            # which lattice each particle came from
    buffer1: Block               # insert_buffer1's template
    buffer2: Block               # insert_buffer2's template


def build(inp: Optional[RefInputs] = None) -> ReferenceTank:
    """init + gen_boundary + gen_fluid (main.f90:21-23)."""
    inp = inp or RefInputs()
    k = derive(inp)
    walls = gen_boundary(inp, k)
    soil = walls.pop()
    fluid, buffer1, buffer2 = gen_fluid(inp, k)
    blocks = walls + fluid
    P = _binned(k, blocks)
    S = _binned(k, [soil])
    spec = sc.TankSpec(dx=k.dl, length=inp.L, height=k.H, depth=inp.wc, kernel=0, h_factor=k.h1 / k.dl,
                       por=inp.por, d50=0.00102, darcy_alpha=450.0, forch_beta=1.75 * math.sqrt(450.0 / 150.0),
                       csh=0.5, dt=float(np.float32(0.001)), rho0=inp.rho, rho_solid=inp.bulkden, g=inp.g,
                       piston_amp=(), piston_period=(), piston_phase=(), jitter=0.0)
    n = P["x"].size
    # the reference's own cell grid with its ring of halo cells (setup.f90:126-137)
    bounds = (-k.cell, (k.cellx - 2) * k.cell, -k.cell, (k.celly - 2) * k.cell)
    scen = sc.Scenario(spec, P["x"], P["y"], P["vx"], np.zeros(n), P["p"], P["rho"], P["rho"].copy(), P["mass"],
                       P["tid"], P["flags"], P["x"].copy(), S["x"], S["y"], S["mass"], S["rho"],
                       np.full((1, 1), inp.por), (bounds[0], bounds[2]),
                       (bounds[1] - bounds[0], bounds[3] - bounds[2]), bounds)
    return ReferenceTank(inp, k, scen, [b.name for b in blocks], P["block"], buffer1, buffer2)


def state(tank: ReferenceTank) -> Dict[str, np.ndarray]:
    """The host arrays for bsc_upload_state.  con starts at 0 (the particle
    type's default, particle.f90:9); wall and ghost particles carry oden = rho
    where the reference leaves it 0 and never reads it."""
    d = sc.state_arrays(tank.scenario)
    d["con"] = np.zeros(tank.scenario.n)
    return d


def params(tank: ReferenceTank, **kw) -> sc.Params:
    """bsc_params with the reference's constants for this geometry: hybrid
    kernel, h1 and lam of setup.f90:47,99, dl = min(2 prrealx, 2 prrealy)
    (setup.f90:53), rel_den, the outflow cut-off lines of cellshiftalt and
    the window in which comp_pos turns buffer particles into fluid."""
    k, inp = tank.constants, tank.inputs
    kw.setdefault("max_neighbors", 96)
    p = sc.make_params(tank.scenario.spec, tank.scenario.bounds, **kw)
    p.kernel = 0
    p.h = k.h1
    p.lam = k.lam
    p.dl = k.dl
    p.rel_den = inp.rel_den
    p.outflow_xcut, p.outflow_ycut = k.xlcutoff, k.ytcutoff
    p.buffer_release_xmin, p.buffer_release_xmax = k.release_xmin, k.xrcutoff
    return p


def insertion(tank: ReferenceTank, which: int, relden: float = 1.0) -> Dict[str, np.ndarray]:
    """The particles insert_buffer1 (which=1) or insert_buffer2 (which=2)
    appends, as a bsc_insert_particles view: fluid, mass fmass (times relden
    for buffer2), oden = density, con -0.5 or 0.5 (internal.f90:475-542).
    Only template particles inside the entry cells go in; those are the
    interior cells that hold buffer particles at generation, which contain
    every template particle, so all of them are inserted."""
    b = tank.buffer1 if which == 1 else tank.buffer2
    k = tank.constants
    j, _ = cell_of(k, b.x, b.y)
    sel = j >= 0
    if which == 2:
        sel &= j <= k.cellx // 2  # entrycell2 lists columns 2..cellx/2 (internal.f90:450)
    m = int(sel.sum())
    scale = 1.0 if which == 1 else relden
    rho = np.full(m, b.density * scale)
    return dict(x=b.x[sel].copy(), y=b.y[sel].copy(), vx=b.vx[sel].copy(), vy=np.zeros(m), p=b.p[sel].copy(),
                rho=rho, oden=rho.copy(), mass=np.full(m, b.mass * scale), con=np.full(m, -0.5 if which == 1 else 0.5),
                ovol=np.full(m, b.mass / b.density), tid=np.full(m, sc.TID_FLUID, np.int8),
                flags=b.flags[sel].copy())


def setup(ctx, tank: ReferenceTank, *, initial_effpor: bool = True):
    """Upload the reference tank (porosity, state, soil) and run the initial
    effpor of main.f90:35-37."""
    s = tank.scenario
    ctx.upload_porosity(s.por_grid, s.por_origin, s.por_step)
    ctx.upload_state(state(tank))
    ctx.upload_solids(s.sx, s.sy, s.smass, s.srho)
    ctx.set_time(0.0, s.spec.dt)
    if initial_effpor:
        ctx.effpor()
