"""Seeded synthetic wave-tank scenarios for the ISPH step.

The reference builds its own confined-aquifer geometry in ``gen_boundary`` and
``gen_fluid`` (boundary.f90:12-605, internal.f90:10-473).  The workloads here
are the wave-tank cases of the benchmark instead: a 4.0 m x 0.6 m tank with
0.30 m still water, a piston wavemaker on the left, a porous 1:5 slope whose
toe is at x = 2.0 m, and three layers of wall particles.  Every input is
generated from a seed, so the CUDA path and the CPU oracle see the same bytes.

Particle conventions follow particle.f90:31-47:
  tid 1 = first wall layer (the "fixed" wall of ppesolve), tid 2 = the outer
  ("ghost") layers, tid 3 = fluid; porous solid particles (tid 4) are kept in
  a separate array, as the reference keeps them in ``porlist``.

Fluid sits on a square lattice of spacing dx.  Inside the slope the fluid
carries the superficial mass rho0 * n0 * dx^2 (n0 the matrix porosity), so
that its volume m/rho = dx^2 once ``effpor`` has set rho = n * rho0; the
reference gets the same consistency with a uniform mass on a lattice of
spacing dx/sqrt(por) (internal.f90:43-45, setup.f90:28).
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Dict, Optional

import numpy as np

MASK64 = np.uint64(0xFFFFFFFFFFFFFFFF)

TID_WALL, TID_GHOST, TID_FLUID = 1, 2, 3
FLAG_FREE, FLAG_VICINITY, FLAG_BUFFER, FLAG_DEAD, FLAG_PISTON = 1, 2, 4, 8, 16


def splitmix64_uniform(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """``count`` doubles in [0, 1) from the splitmix64 sequence of ``seed``.

    Element k is the (offset + k + 1)-th output of splitmix64 (Steele, Lea and
    Flood 2014), mapped to a double by its top 53 bits.
    """
    with np.errstate(over="ignore"):
        k = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


@dataclasses.dataclass
class TankSpec:
    """Geometry and physics of one wave-tank case."""

    dx: float = 0.01
    length: float = 4.0          # fluid between the piston (x=0) and the right wall
    height: float = 0.6          # wall height
    depth: float = 0.30          # still-water depth
    h_factor: float = 1.3        # h = h_factor * dx
    kernel: int = 1              # 1 = Wendland C2, 0 = the reference's hybrid kernel
    toe_x: float = 2.0
    slope: float = 0.2           # 1:5
    por: float = 0.4
    por_jitter: float = 0.0      # per-cell porosity = por +/- por_jitter (uniform)
    por_seed: int = 3
    por_cells: tuple = (40, 8)   # porosity grid over the slope bounding box
    d50: float = 5e-3
    darcy_alpha: float = 200.0
    forch_beta: float = 1.1
    wall_layers: int = 3
    jitter: float = 0.01         # +/- jitter * dx on the fluid lattice
    seed: int = 1
    piston_amp: tuple = (0.02,)
    piston_period: tuple = (1.2,)
    piston_phase: tuple = (0.0,)
    piston_ramp: float = 1.2     # half-cosine ramp of the stroke over this time
    rho0: float = 1000.0
    rho_solid: float = 2650.0
    g: float = -9.81
    csh: float = 0.2
    dt: float = 1e-4
    probes: tuple = (1.0, 1.5, 2.0, 2.5)
    salinity_front: float = 3.0  # initial salinity 0.5 tanh((x - front) / width)
    salinity_width: float = 0.1


def irregular_piston(total_amp: float = 0.03, modes: int = 8, tmin: float = 0.8,
                     tmax: float = 2.0, seed: int = 5):
    """Sum of ``modes`` sinusoids: equal amplitudes summing to ``total_amp``,
    periods evenly spread over [tmin, tmax], phases 2*pi*u from splitmix64."""
    amps = tuple([total_amp / modes] * modes)
    periods = tuple(np.linspace(tmin, tmax, modes).tolist())
    phases = tuple((2.0 * math.pi * splitmix64_uniform(seed, modes)).tolist())
    return amps, periods, phases


STARTUP_RAMP = 0.01  # s: the piston's start-up ramp at the c3 and c5 spacings


def config_spec(name: str) -> TankSpec:
    """The benchmark cases c1..c5 (dx, porosity field, piston, time step).

    c1 and c2 drive the piston with its plain stroke from t = 0: the wall
    starts at its rest position with the stroke's velocity.  At the finer c3
    and c5 spacings that impulsive start is unstable (at c3, dx = 1.2 mm, an
    interior particle reached 27 m/s in the second step and the state blew up
    in the fourth, on both precisions), so the stroke ramps in over 0.01 s
    (100 steps); ramps of 0.01, 0.02 and 0.05 s were all stable.  The c4
    calibration case and the small tanks of the unit tests keep the default
    1.2 s ramp."""
    if name == "c1":
        return TankSpec(dx=0.01, piston_ramp=0.0)
    if name == "c2":
        return TankSpec(dx=0.0025, piston_ramp=0.0)
    if name == "c3":
        return TankSpec(dx=0.0012, por_jitter=0.05, por_seed=3, piston_ramp=STARTUP_RAMP)
    if name == "c4":
        return TankSpec(dx=0.0035, dt=5e-5, por_cells=(16, 4))
    if name == "c5":
        a, t, p = irregular_piston()
        return TankSpec(dx=0.0006, piston_amp=a, piston_period=t, piston_phase=p,
                        piston_ramp=STARTUP_RAMP)
    raise KeyError(name)


@dataclasses.dataclass
class Scenario:
    spec: TankSpec
    # fluid + wall particles, id order
    x: np.ndarray
    y: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    p: np.ndarray
    rho: np.ndarray
    oden: np.ndarray
    mass: np.ndarray
    tid: np.ndarray
    flags: np.ndarray
    xrest: np.ndarray
    # porous solids
    sx: np.ndarray
    sy: np.ndarray
    smass: np.ndarray
    srho: np.ndarray
    # porosity grid over the slope
    por_grid: np.ndarray
    por_origin: tuple
    por_step: tuple
    bounds: tuple

    @property
    def n(self) -> int:
        return int(self.x.size)

    @property
    def n_fluid(self) -> int:
        return int(np.count_nonzero(self.tid == TID_FLUID))

    def porosity_at(self, x: np.ndarray, y: np.ndarray) -> np.ndarray:
        """Grid lookup with the same cell rule as the CUDA path."""
        nx, ny = self.por_grid.shape[1], self.por_grid.shape[0]
        ix = np.floor((x - self.por_origin[0]) / self.por_step[0]).astype(np.int64)
        iy = np.floor((y - self.por_origin[1]) / self.por_step[1]).astype(np.int64)
        inside = (ix >= 0) & (ix < nx) & (iy >= 0) & (iy < ny)
        out = np.full(x.shape, self.spec.por)
        out[inside] = self.por_grid[iy[inside], ix[inside]]
        return out


def piston_stroke(spec: TankSpec, t: float):
    """x_p(t) and v_p(t) of the wavemaker: s0 + r(t) (s(t) - s0), with
    s(t) = sum_k a_k sin(w_k t + phi_k), s0 = s(0) and the start-up ramp
    r(t) = (1 - cos(pi t / ramp)) / 2 for t < ramp (1 after it, or without a
    ramp).  The ramp takes the stroke from its starting value, so the wall
    starts at rest."""
    s = ds = s0 = 0.0
    for a, T, ph in zip(spec.piston_amp, spec.piston_period, spec.piston_phase):
        w = 2.0 * math.pi / T
        s += a * math.sin(w * t + ph)
        ds += a * w * math.cos(w * t + ph)
        s0 += a * math.sin(ph)
    r, dr = 1.0, 0.0
    if spec.piston_ramp > 0.0 and t < spec.piston_ramp:
        r = 0.5 * (1.0 - math.cos(math.pi * t / spec.piston_ramp))
        dr = 0.5 * math.pi / spec.piston_ramp * math.sin(math.pi * t / spec.piston_ramp)
    return s0 + r * (s - s0), dr * (s - s0) + r * ds


def kernel_w(spec: TankSpec, r: np.ndarray) -> np.ndarray:
    """W(r, h) of the selected kernel (kernel.f90:34-66 and its Wendland C2
    comment); r < 2h assumed."""
    h = spec.h_factor * spec.dx
    q = r / h
    if spec.kernel == 1:
        a = 1.0 - q / 2.0
        return (7.0 / (4 * 3.140 * h * h)) * (1.0 + 2.0 * q) * a ** 4
    c28 = float(np.float32(28.0) * np.float32(3.14))
    c3 = float(np.float32(3.0) * np.float32(3.14))
    t1 = np.where(q < 1.0, 4.0 - 6.0 * q * q + 3.0 * q ** 3, (2.0 - q) ** 3)
    t2 = np.where(q < 1.0, q ** 3 - 6.0 * q + 6.0, (2.0 - q) ** 3)
    return 0.1 * t1 * (10.0 / (c28 * h * h)) + 0.9 * t2 * (1.0 / (c3 * h * h))


def initial_porosity(spec, fx, fy, sx, sy, svol, spor, cap_por):
    """n = 1 - min(sum_s (1-por_s) W V_s, 1-por) (porous.f90:48-58,182-188)
    evaluated on the initial lattice, binned on cells of size 2h."""
    h = spec.h_factor * spec.dx
    n = np.ones(fx.size)
    if sx.size == 0:
        return n
    R = 2.0 * h
    x0, y0 = min(fx.min(), sx.min()) - R, min(fy.min(), sy.min()) - R
    sci = np.floor((sx - x0) / R).astype(np.int64)
    scj = np.floor((sy - y0) / R).astype(np.int64)
    ny = int(max(scj.max(), np.floor((fy.max() - y0) / R)) + 3)
    skey = sci * ny + scj
    order = np.argsort(skey, kind="stable")
    skey_s = skey[order]
    fci = np.floor((fx - x0) / R).astype(np.int64)
    fcj = np.floor((fy - y0) / R).astype(np.int64)
    frac = np.zeros(fx.size)
    for di in (-1, 0, 1):
        for dj in (-1, 0, 1):
            key = (fci + di) * ny + (fcj + dj)
            lo = np.searchsorted(skey_s, key, "left")
            hi = np.searchsorted(skey_s, key, "right")
            cnt = hi - lo
            maxc = int(cnt.max()) if cnt.size else 0
            for k in range(maxc):
                sel = np.nonzero(cnt > k)[0]
                s = order[lo[sel] + k]
                r = np.hypot(fx[sel] - sx[s], fy[sel] - sy[s])
                ok = r < R
                sel, s, r = sel[ok], s[ok], r[ok]
                frac[sel] += (1.0 - spor[s]) * kernel_w(spec, r) * svol[s]
    frac = np.minimum(frac, 1.0 - cap_por)
    return 1.0 - frac


def build(spec: TankSpec) -> Scenario:
    dx = spec.dx
    h = spec.h_factor * dx
    nl = spec.wall_layers
    nx = int(math.floor(spec.length / dx + 1e-9))
    ny = int(math.floor(spec.depth / dx + 1e-9))
    nyw = int(math.floor(spec.height / dx + 1e-9))
    stroke = sum(abs(a) for a in spec.piston_amp)
    # A stroke with nonzero phases starts away from zero; the piston's rest
    # coordinate is shifted by -x_p(0), so the wall starts on its lattice next
    # to the fluid and moves by x_p(t) - x_p(0).
    xp_start = piston_stroke(spec, 0.0)[0]

    # ---- fluid lattice with seeded jitter (column-major: x outer, y inner)
    ii, jj = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    fx = (ii.ravel() + 0.5) * dx
    fy = (jj.ravel() + 0.5) * dx
    u = splitmix64_uniform(spec.seed, 2 * fx.size)
    fx = fx + (2.0 * u[0::2] - 1.0) * spec.jitter * dx
    fy = fy + (2.0 * u[1::2] - 1.0) * spec.jitter * dx

    # ---- porosity grid over the slope bounding box
    top = max(spec.slope * (spec.length - spec.toe_x), 0.0)
    pnx, pny = spec.por_cells
    por_origin = (spec.toe_x, 0.0)
    por_step = (max(spec.length - spec.toe_x, spec.dx) / pnx, max(top, spec.dx) / pny)
    if spec.por_jitter > 0.0:
        pu = splitmix64_uniform(spec.por_seed, pnx * pny).reshape(pny, pnx)
        por_grid = spec.por + (2.0 * pu - 1.0) * spec.por_jitter
    else:
        por_grid = np.full((pny, pnx), spec.por)

    def below_slope(x, y):
        return (x >= spec.toe_x) & (y < spec.slope * (x - spec.toe_x))

    scen_stub = Scenario(spec, *([np.empty(0)] * 15), por_grid, por_origin, por_step, ())

    # ---- porous solid lattice below the slope line.  Like the soil lattice of
    # boundary.f90:532-533 (which starts three spacings inside the walls) it
    # runs under the bottom wall and behind the right wall for a full kernel
    # support, so the smoothed porosity of effpor has no wall deficit.
    ext = int(math.ceil(2.0 * h / dx))
    si, sj = np.meshgrid(np.arange(int(round(spec.toe_x / dx)), nx + ext),
                         np.arange(-ext, int(math.ceil(top / dx)) + 1), indexing="ij")
    sx = (si.ravel() + 0.5) * dx
    sy = (sj.ravel() + 0.5) * dx
    keep = below_slope(sx, sy)
    sx, sy = sx[keep], sy[keep]
    smass = np.full(sx.size, spec.rho_solid * dx * dx)
    srho = np.full(sx.size, spec.rho_solid)

    # fluid mass rho0 * n * dx^2 with n the kernel-smoothed porosity that
    # effpor will compute, so every fluid volume m/rho starts at dx^2
    n0 = initial_porosity(spec, fx, fy, sx, sy, smass / srho,
                          scen_stub.porosity_at(sx, sy), scen_stub.porosity_at(fx, fy))
    fmass = spec.rho0 * n0 * dx * dx

    # ---- walls: bottom (extends under the piston stroke), right wall, piston
    walls = []  # (x, y, tid, flags)
    i_left = -(nl + int(math.ceil((stroke + abs(xp_start)) / dx)) + nl + 2)
    i_right = nx + nl
    for k in range(nl):
        tid = TID_WALL if k == 0 else TID_GHOST
        xs = (np.arange(i_left, i_right) + 0.5) * dx
        walls.append((xs, np.full(xs.size, -(k + 0.5) * dx), tid, 0))
        ys = (np.arange(nyw) + 0.5) * dx
        # the right wall closes the fluid lattice at nx * dx, so the wall gap
        # stays one spacing when length / dx is not a whole number
        walls.append((np.full(ys.size, (nx + k + 0.5) * dx), ys, tid, 0))
        walls.append((np.full(ys.size, -(k + 0.5) * dx), ys, tid, FLAG_PISTON))
    wx = np.concatenate([w[0] for w in walls])
    wy = np.concatenate([w[1] for w in walls])
    wtid = np.concatenate([np.full(w[0].size, w[2], np.int8) for w in walls])
    wflags = np.concatenate([np.full(w[0].size, w[3], np.uint8) for w in walls])

    x = np.concatenate([fx, wx])
    y = np.concatenate([fy, wy])
    tid = np.concatenate([np.full(fx.size, TID_FLUID, np.int8), wtid])
    flags = np.concatenate([np.zeros(fx.size, np.uint8), wflags])
    mass = np.concatenate([fmass, np.full(wx.size, spec.rho0 * dx * dx)])
    rho = np.full(x.size, spec.rho0)
    oden = rho.copy()
    p = np.maximum(spec.rho0 * abs(spec.g) * (spec.depth - y), 0.0)
    vx = np.zeros(x.size)
    vy = np.zeros(x.size)
    xrest = x.copy()
    # the piston starts at x_rest + x_p(0): on its lattice, as x_rest carries
    # the -x_p(0) shift
    xp0, vp0 = piston_stroke(spec, 0.0)
    pist = (flags & FLAG_PISTON) != 0
    xrest[pist] -= xp0
    x[pist] = xrest[pist] + xp0
    vx[pist] = vp0

    margin = 4.0 * h
    bounds = (float(x.min() - stroke - abs(xp0) - margin), float(x.max() + stroke + abs(xp0) + margin),
              float(y.min() - margin), float(spec.height + margin))
    return Scenario(spec, x, y, vx, vy, p, rho, oden, mass, tid, flags, xrest,
                    sx, sy, smass, srho, por_grid, por_origin, por_step, bounds)


# ---------------------------------------------------------------------------
# ctypes mirror of bsc_params / bsc_state_view / bsc_solve_info (include/bsc.h)
# ---------------------------------------------------------------------------
_D = ctypes.c_double
_I = ctypes.c_int32
_PD = ctypes.POINTER(ctypes.c_double)


class Params(ctypes.Structure):
    _fields_ = [
        ("kernel", _I), ("precision", _I), ("h", _D), ("dl", _D), ("lam", _D),
        ("rho0", _D), ("rel_den", _D), ("g", _D), ("mu", _D), ("csh", _D),
        ("maxshift", _D), ("free_threshold", _D), ("por", _D),
        ("darcy_alpha", _D), ("forch_beta", _D), ("d50", _D), ("eddy_cs", _D),
        ("eddy_cv", _D), ("eddy_ce", _D), ("varts_ps", _D),
        ("buffer_release_xmin", _D), ("buffer_release_xmax", _D),
        ("dt_mode", _I), ("solver", _I), ("dt", _D), ("sig1", _D),
        ("tschmidt", _D), ("diffusivity", _D), ("restart", _I), ("maxit", _I),
        ("tol_mode", _I), ("max_outer", _I), ("tol", _D), ("inner_tol", _D),
        ("max_neighbors", _I), ("reorder_every", _I), ("piston_modes", _I),
        ("precond", _I), ("piston_amp", _D * 8), ("piston_period", _D * 8),
        ("piston_phase", _D * 8), ("piston_ramp", _D), ("xmin", _D), ("xmax", _D), ("ymin", _D),
        ("ymax", _D), ("mg_omega", _D), ("mg_scale", _D), ("mg_sweeps", _I), ("mg_coarse_max", _I),
        ("disp_long", _D), ("disp_trans", _D), ("buffer_con", _D), ("buffer_con_xmax", _D),
        ("salinity", _I), ("outflow", _I), ("outflow_xcut", _D), ("outflow_ycut", _D),
    ]


class StateView(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64)] + [
        (f, _PD) for f in ("x", "y", "vx", "vy", "xs", "ys", "vxs", "vys", "p",
                           "rho", "oden", "mass", "porosity", "gradvx", "nut",
                           "tke", "resist", "varts", "vel", "L", "xrest")
    ] + [("tid", ctypes.POINTER(ctypes.c_int8)), ("flags", ctypes.POINTER(ctypes.c_uint8)),
         ("con", _PD), ("ovol", _PD)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("iterations", _I), ("outer", _I), ("converged", _I), ("status", _I),
                ("rel_residual", _D), ("r0_norm", _D), ("b_norm", _D)]


class Timing(ctypes.Structure):
    _fields_ = [("ms", _D * 32), ("calls", ctypes.c_int64 * 32),
                ("kernel_launches", ctypes.c_int64)]


class WcsphParams(ctypes.Structure):
    """bsc_wcsph_params of include/bsc.h."""
    _fields_ = [("c0", _D), ("gamma", _D), ("delta", _D), ("surface_y", _D), ("nu", _D), ("alpha", _D),
                ("beta", _D), ("grid_x0", _D), ("grid_y0", _D), ("grid_dx", _D), ("grid_dy", _D),
                ("grid_nx", _I), ("grid_ny", _I), ("grid_por", _PD), ("nprobe", _I), ("probe_x", _D * 16),
                ("probe_depth", _D)]


def wcsph_params(spec: "TankSpec", scen: "Scenario", alpha: float = None, beta: float = None,
                 grid=None) -> "tuple":
    """The WCSPH model of the calibration case on a tank scenario: Tait EOS
    with c0 = 10 sqrt(g depth) and gamma = 7, delta-SPH coefficient 0.1, the
    still-water level as the hydrostatic reference, water's kinematic
    viscosity, the scenario's porosity grid and probes.  Returns (params,
    grid array) -- the array must stay alive while the params are used."""
    g = np.ascontiguousarray(scen.por_grid if grid is None else grid, dtype=np.float64)
    ny, nx = g.shape
    w = WcsphParams()
    w.c0 = 10.0 * np.sqrt(abs(spec.g) * spec.depth)
    w.gamma = 7.0
    w.delta = 0.1
    w.surface_y = spec.depth
    w.nu = 1.0e-6
    w.alpha = spec.darcy_alpha if alpha is None else alpha
    w.beta = spec.forch_beta if beta is None else beta
    w.grid_x0, w.grid_y0 = scen.por_origin
    w.grid_dx, w.grid_dy = scen.por_step
    w.grid_nx, w.grid_ny = nx, ny
    w.grid_por = g.ctypes.data_as(_PD)
    w.nprobe = len(spec.probes)
    for k, xp in enumerate(spec.probes):
        w.probe_x[k] = xp
    w.probe_depth = spec.depth
    return w, g


STATE_FIELDS = ("x", "y", "vx", "vy", "xs", "ys", "vxs", "vys", "p", "rho", "oden",
                "mass", "porosity", "gradvx", "nut", "tke", "resist", "varts", "vel",
                "xrest", "con", "ovol")

SOLVERS = {"bicgstab": 0, "fgmres": 1}
PRECONDS = {"none": 0, "mg": 1}
PRECISIONS = {"fp64": 0, "mixed": 1}


def make_params(spec: TankSpec, bounds=None, *, precision="fp64", solver="bicgstab",
                tol=1e-8, maxit=2000, restart=30, max_neighbors=48,
                reorder_every=20, tol_mode=0, dt_mode=0, inner_tol=1e-4,
                max_outer=20, precond="none", mg_omega=0.82, mg_scale=1.8, mg_sweeps=2,
                mg_coarse_max=128, salinity=False) -> Params:
    """bsc_params for a tank case (constants of initialize.f90:19-56 where the
    benchmark does not override them)."""
    p = Params()
    h = spec.h_factor * spec.dx
    p.kernel = spec.kernel
    p.precision = PRECISIONS[precision]
    p.h = h
    p.dl = spec.dx
    p.lam = 0.001 * h * h
    p.rho0 = spec.rho0
    p.rel_den = 1.025
    p.g = spec.g
    p.mu = 1e-3
    p.csh = spec.csh
    p.maxshift = 0.1
    p.free_threshold = 0.8 * 2.0
    p.por = spec.por
    p.darcy_alpha = spec.darcy_alpha
    p.forch_beta = spec.forch_beta
    p.d50 = spec.d50
    p.eddy_cs, p.eddy_cv, p.eddy_ce = 0.15, 0.08, 1.0
    p.varts_ps = 1.0
    p.buffer_release_xmin = -1e30
    p.buffer_release_xmax = 1e30
    p.dt_mode = dt_mode
    p.solver = SOLVERS[solver]
    p.dt = spec.dt
    p.sig1 = 0.2
    p.tschmidt = 1.0
    p.diffusivity = float(np.float32(1e-9))  # the reference's `Dm=1e-9` is a default-real literal
    p.restart = restart
    p.maxit = maxit
    p.tol_mode = tol_mode
    p.max_outer = max_outer
    p.tol = tol
    p.inner_tol = inner_tol
    p.max_neighbors = max_neighbors
    p.reorder_every = reorder_every
    p.piston_ramp = spec.piston_ramp
    p.piston_modes = len(spec.piston_amp)
    for k, (a, T, ph) in enumerate(zip(spec.piston_amp, spec.piston_period, spec.piston_phase)):
        p.piston_amp[k], p.piston_period[k], p.piston_phase[k] = a, T, ph
    p.precond = PRECONDS[precond]
    p.mg_omega, p.mg_scale = mg_omega, mg_scale
    p.mg_sweeps, p.mg_coarse_max = mg_sweeps, mg_coarse_max
    p.disp_long, p.disp_trans = 0.0025, 0.00025  # scalar.f90:118
    p.buffer_con, p.buffer_con_xmax = 0.5, 1.6
    p.salinity = 1 if salinity else 0
    if bounds is not None:
        p.xmin, p.xmax, p.ymin, p.ymax = bounds
    return p


def state_arrays(scen: Scenario) -> Dict[str, np.ndarray]:
    """Host SoA dictionary for bsc_upload_state."""
    n = scen.n
    d = dict(x=scen.x.copy(), y=scen.y.copy(), vx=scen.vx.copy(), vy=scen.vy.copy(),
             p=scen.p.copy(), rho=scen.rho.copy(), oden=scen.oden.copy(),
             mass=scen.mass.copy(), xrest=scen.xrest.copy(), tid=scen.tid.copy(),
             flags=scen.flags.copy())
    for f in ("xs", "ys", "vxs", "vys", "gradvx", "nut", "tke", "resist", "varts", "vel"):
        d[f] = np.zeros(n)
    d["porosity"] = np.ones(n)
    d["L"] = np.tile(np.array([1.0, 0.0, 0.0, 1.0]), n)
    # A saline wedge on the beach side (fluid only), in the reference's
    # convention: con runs from -0.5 (fresh, oden = rho0) to 0.5 (sea water,
    # oden = rho0 rel_den) through densityupdate (scalar.f90:293). ovol is
    # derived on upload as mass / oden.
    sp = scen.spec
    d["con"] = np.where(scen.tid == TID_FLUID,
                        0.5 * np.tanh((scen.x - sp.salinity_front) / sp.salinity_width), 0.0)
    return d


def empty_state(n: int) -> Dict[str, np.ndarray]:
    d = {f: np.zeros(n) for f in STATE_FIELDS}
    d["L"] = np.zeros(4 * n)
    d["tid"] = np.zeros(n, np.int8)
    d["flags"] = np.zeros(n, np.uint8)
    return d


def state_view(arrs: Dict[str, np.ndarray]) -> StateView:
    """A bsc_state_view pointing into numpy arrays (kept alive by the caller)."""
    v = StateView()
    v.n = int(arrs["x"].size)
    for f in STATE_FIELDS + ("L",):
        a = arrs.get(f)
        if a is not None:
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], f
            setattr(v, f, a.ctypes.data_as(_PD))
    v.tid = arrs["tid"].ctypes.data_as(ctypes.POINTER(ctypes.c_int8))
    v.flags = arrs["flags"].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    return v


def _as_dptr(a: Optional[np.ndarray]):
    if a is None:
        return None
    return a.ctypes.data_as(_PD)
