"""Pins of the CPU oracle (no GPU).

The reference has one known-answer test (solvertest.f90:10-19) and no golden
field outputs, so the SPH routines of the oracle are pinned by invariants the
reference's formulae imply:
  * kernel normalisation and W/grad-W consistency (kernel.f90:34-162);
  * exactness of the corrected gradient on linear fields (search.f90:77-85 +
    functions.f90:62-96, through eddyvis);
  * zero row sums of the PPE for non-free rows (isph.f90:181-296);
  * agreement of both Krylov solvers with a direct sparse solve;
  * a still tank stays close to hydrostatic rest.
"""
import ctypes
import json
import math
import os

import numpy as np
import pytest

import oracle
from beach_slope_confined_gb300 import scenario as sc
from beach_slope_confined_gb300.binding import setup_tank
from pairrun import advance_to_lists, small_spec

HERE = os.path.dirname(os.path.abspath(__file__))


def _kat():
    with open(os.path.join(HERE, "golden", "solvertest_kat.json")) as fh:
        return json.load(fh)


@pytest.mark.parametrize("solver", ["bicgstab", "fgmres"])
@pytest.mark.parametrize("restart", [4, 5])
def test_kat_solvertest(solver, restart):
    k = _kat()
    P = sc.make_params(small_spec(), solver=solver, tol=1e-12, maxit=200, restart=restart)
    rc, x, info = oracle.solve(P, k["rowptr"], k["col"], k["val"], k["b"], k["guess"])
    assert rc == 0 and info.converged
    assert np.allclose(x, k["solution"], rtol=0, atol=1e-10)


def _kernel(P, r):
    lib = oracle.lib()
    f = lib.orc_eval_kernel
    f.argtypes = [ctypes.POINTER(sc.Params), ctypes.c_double] + [ctypes.POINTER(ctypes.c_double)] * 3
    f.restype = ctypes.c_int
    w, g, w0 = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    assert f(ctypes.byref(P), r, ctypes.byref(w), ctypes.byref(g), ctypes.byref(w0)) == 0
    return w.value, g.value, w0.value


@pytest.mark.parametrize("kernel", [0, 1])
def test_kernel_normalisation_and_gradient(kernel):
    P = sc.make_params(small_spec(kernel=kernel))
    h = P.h
    r = np.linspace(0, 2 * h, 20001)[:-1] + h / 20000
    w = np.array([_kernel(P, x)[0] for x in r])
    # the reference writes pi as 3.14: the integral of W over the plane is pi/3.14
    integral = np.trapezoid(2 * math.pi * r * w, r)
    assert abs(integral - math.pi / 3.14) < 2e-5
    assert _kernel(P, 2 * h - 1e-12)[0] < 1e-9 / h ** 2
    # grad_i W = F (x_i - x_j) with F = W'(r)/r
    for x in (0.3 * h, 0.9 * h, 1.1 * h, 1.7 * h):
        e = 1e-6 * h
        dw = (_kernel(P, x + e)[0] - _kernel(P, x - e)[0]) / (2 * e)
        assert abs(_kernel(P, x)[1] * x - dw) < 1e-6 * abs(dw)
    assert _kernel(P, 0.5 * h)[2] == pytest.approx(_kernel(P, 1e-300)[0], rel=1e-12)


def _flat_tank(**kw):
    spec = small_spec(toe_x=10.0, slope=-1.0, piston_amp=(0.0,), **kw)
    return spec, sc.build(spec)


def test_corrected_gradient_exact_on_linear_field():
    spec, scen = _flat_tank()
    a, b, c, d = 0.3, -0.2, 0.5, 0.1
    scen.vx = a * scen.x + b * scen.y
    scen.vy = c * scen.x + d * scen.y
    fluid = scen.tid == sc.TID_FLUID
    scen.vx[~fluid] = 0.0
    scen.vy[~fluid] = 0.0
    P = sc.make_params(spec, scen.bounds)
    o = oracle.context(P)
    setup_tank(o, scen)
    o.cellshift()
    o.resetid()
    o.neighbour()
    o.eddyvis()
    s = o.download_state()
    h = P.h
    interior = fluid & (scen.x > 4 * h) & (scen.x < spec.length - 4 * h) & (scen.y > 4 * h) & (scen.y < spec.depth - 4 * h)
    assert interior.sum() > 100
    S = math.sqrt(2 * (a * a + d * d) + (b + c) ** 2)
    nut = (P.eddy_cs * P.dl) ** 2 * S
    assert np.allclose(s["nut"][interior], nut, rtol=1e-10, atol=0)
    # L M = I holds by construction; interior particles are not free
    assert not np.any(s["flags"][interior] & sc.FLAG_FREE)


def test_ppe_row_sums_and_direct_solve():
    scipy = pytest.importorskip("scipy.sparse.linalg")
    import scipy.sparse as sp

    spec = small_spec()
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, tol=1e-12, maxit=20000)
    o = oracle.context(P)
    setup_tank(o, scen)
    advance_to_lists((o,))
    o.effpor()
    o.eddyvis()
    o.int_vel()
    info = o.ppesolve()
    assert info.converged
    rp, col, val, rhs = o.export_csr()
    A = sp.csr_matrix((val, col, rp), shape=(o.n, o.n))
    s = o.download_state()
    free = (s["flags"] & sc.FLAG_FREE) != 0
    rowsum = np.asarray(A.sum(axis=1)).ravel()
    assert np.max(np.abs(rowsum[~free])) < 1e-12
    assert np.all(rowsum[free] > 0)
    assert np.allclose(A.diagonal(), 1.0)
    x = scipy.spsolve(A.tocsc(), rhs)
    assert np.linalg.norm(s["p"] - x) / np.linalg.norm(x) < 1e-9


@pytest.mark.parametrize("solver", ["bicgstab", "fgmres"])
def test_solvers_agree_with_direct(solver):
    scipy = pytest.importorskip("scipy.sparse.linalg")
    import scipy.sparse as sp

    spec = small_spec(dx=0.025)
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, solver=solver, tol=1e-11, maxit=50000)
    o = oracle.context(P)
    setup_tank(o, scen)
    advance_to_lists((o,))
    o.effpor(); o.eddyvis(); o.int_vel()
    assert o.ppesolve().converged
    rp, col, val, rhs = o.export_csr()
    A = sp.csr_matrix((val, col, rp), shape=(o.n, o.n))
    x = scipy.spsolve(A.tocsc(), rhs)
    p = o.download_state()["p"]
    assert np.linalg.norm(p - x) / np.linalg.norm(x) < 1e-8


def test_still_tank_stays_near_rest():
    spec, scen = _flat_tank()
    P = sc.make_params(spec, scen.bounds, tol=1e-9, maxit=20000)
    o = oracle.context(P)
    setup_tank(o, scen)
    mass0 = o.download_state()["mass"].sum()
    for _ in range(5):
        assert o.step(1).converged
    s = o.download_state()
    fluid = scen.tid == sc.TID_FLUID
    assert np.max(np.hypot(s["vx"], s["vy"])[fluid]) < 5e-3
    ph = spec.rho0 * abs(spec.g) * (spec.depth - s["y"])
    deep = fluid & (s["y"] < 0.5 * spec.depth) & (s["x"] > 0.1) & (s["x"] < spec.length - 0.1)
    assert np.max(np.abs(s["p"][deep] - ph[deep])) < 0.05 * spec.rho0 * abs(spec.g) * spec.depth
    assert s["mass"].sum() == mass0


def test_free_surface_flags_on_still_tank():
    spec, scen = _flat_tank()
    P = sc.make_params(spec, scen.bounds)
    o = oracle.context(P)
    setup_tank(o, scen)
    o.cellshift(); o.resetid(); o.neighbour(); o.freesurf()
    s = o.download_state()
    fluid = scen.tid == sc.TID_FLUID
    free = (s["flags"] & sc.FLAG_FREE) != 0
    top = fluid & (scen.y > spec.depth - spec.dx)
    assert np.all(free[top & (scen.x > 0.1) & (scen.x < spec.length - 0.1)])
    assert not np.any(free[fluid & (scen.y < spec.depth - 3 * spec.dx)])
    vic = (s["flags"] & sc.FLAG_VICINITY) != 0
    assert np.all(vic[top])


def test_timestep_rule_branches():
    spec = small_spec()
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, dt_mode=1)
    o = oracle.context(P)
    setup_tank(o, scen)
    s = sc.state_arrays(scen)
    s["vel"] = np.full(scen.n, 0.5)
    s["nut"] = np.full(scen.n, 1e-5)
    o.upload_state(s)
    for t, expect in ((0.5, min(0.2 * P.dl / 0.5, 0.2 * P.dl ** 2 / (1e-6 + 1e-5), 1e-3)),
                      (2.0, float(np.float32(min(np.float32(0.2 * P.dl / 0.5), np.float32(0.2 * P.dl ** 2 * 1e6), np.float32(0.002)))))):
        o.set_time(t, 1e-4)
        assert o.timestep() == pytest.approx(expect, rel=1e-15)
