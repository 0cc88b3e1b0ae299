"""Multigrid-preconditioned PPE solve (csrc/mg.cu) on the GPU.

The preconditioner changes how the Krylov method reaches the stopping test,
not the matrix or the test itself, so:
  * whole steps with FGMRES + V-cycle match the oracle's unpreconditioned
    BiCGSTAB to the tolerances of the other step tests (both solve to 1e-12);
  * the iteration count drops by a large factor;
  * the mixed path (FP32 V-cycle inside FP64 FGMRES) reaches the same
    relative residual and stays close to the FP64 path.
"""
import numpy as np
import pytest

from beach_slope_confined_gb300 import Solver, scenario as sc, setup_tank
from pairrun import make_pair, rel_l2, small_spec

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sweeps", [2, 1])
def test_mg_steps_match_oracle(sweeps):
    spec = small_spec()
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, tol=1e-12, maxit=20000, precond="mg", mg_sweeps=sweeps)
    g, c = make_pair(scen, P, Solver)
    for ctx in (g, c):
        ctx.step(5)
    a, b = g.download_state(), c.download_state()
    for f in ("x", "y"):
        assert rel_l2(a[f], b[f]) < 1e-12, f
    for f in ("vx", "vy", "p"):
        assert rel_l2(a[f], b[f]) < 1e-7, f


def test_mg_cuts_iterations():
    spec = small_spec(dx=0.01)
    scen = sc.build(spec)
    its = {}
    for pre in ("none", "mg"):
        P = sc.make_params(spec, scen.bounds, tol=1e-8, maxit=20000, precond=pre)
        g = Solver(P)
        setup_tank(g, scen)
        info = g.step(1)
        assert info.converged and info.rel_residual <= 1e-8
        its[pre] = info.iterations
        g.close()
    print("iterations:", its)
    assert its["mg"] * 5 < its["none"]


def test_mg_mixed_against_fp64():
    """The mixed path (FP32 V-cycle and inner FGMRES inside FP64 refinement)
    against the FP64 path, two steps of the moving c1 tank: the same residual,
    every field within 1e-6 (relative L2), the eddy viscosity included."""
    spec = small_spec(dx=0.01, piston_ramp=0.0)
    scen = sc.build(spec)
    out, infos = {}, {}
    for prec in ("fp64", "mixed"):
        P = sc.make_params(spec, scen.bounds, precision=prec, tol=1e-8, maxit=20000, precond="mg")
        g, _ = make_pair(scen, P, Solver)
        infos[prec] = g.step(2)
        out[prec] = g.download_state()
    assert infos["mixed"].converged and infos["mixed"].rel_residual <= 1e-8
    errs = {f: rel_l2(out["mixed"][f], out["fp64"][f])
            for f in ("x", "y", "vx", "vy", "p", "rho", "porosity", "nut", "tke", "vel")}
    print("mixed vs fp64 relative L2 (multigrid):", errs)
    for f, e in errs.items():
        assert e < 1e-6, (f, e)


def test_mg_deterministic():
    """Two runs of the same steps give the same bits: the hierarchy and every
    reduction are summed in a fixed order."""
    spec = small_spec(dx=0.01)
    scen = sc.build(spec)
    runs = []
    for _ in range(2):
        P = sc.make_params(spec, scen.bounds, tol=1e-8, maxit=20000, precond="mg")
        g = Solver(P)
        setup_tank(g, scen)
        g.step(2)
        runs.append(g.download_state())
        g.close()
    for f in ("x", "y", "vx", "vy", "p"):
        assert np.array_equal(runs[0][f], runs[1][f]), f


def test_mg_reorder_keeps_results():
    """A Morton reorder at every cell shift (which swaps the cell-map buffers
    under the cached per-iteration graphs) gives the same physics as every 20:
    to 1e-8 in FP64; to 1e-6 on the mixed path, whose FP32 pair sums change
    their order with the particles' (a stale cell map would be far off)."""
    spec = small_spec()
    scen = sc.build(spec)
    for prec in ("fp64", "mixed"):
        out = []
        for every in (1, 20):
            P = sc.make_params(spec, scen.bounds, precision=prec, tol=1e-10, maxit=20000, precond="mg",
                               reorder_every=every)
            g = Solver(P)
            setup_tank(g, scen)
            g.step(4)
            out.append(g.download_state())
            g.close()
        tol = 1e-8 if prec == "fp64" else 1e-6
        for f in ("x", "y", "vx", "vy", "p"):
            assert rel_l2(out[0][f], out[1][f]) < tol, (prec, f)


@pytest.mark.parametrize("env", [{"BSC_MG_POST_FUSED": "0"}, {"BSC_MG_POST": "2,1"}, {"BSC_MG_PRE": "1"},
                                 {"BSC_MG_CELL_SWEEPS": "4"}],
                         ids=["post-sweeps-unfused", "one-particle-post-sweep", "one-particle-pre-sweep",
                              "four-cell-level-sweeps"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_mg_sweep_variants_reach_the_same_solution(env, prec, monkeypatch):
    """The V-cycle's sweep variants only change how the solve gets there:
    two steps with each give the default's fields to the solve tolerance."""
    spec = small_spec(dx=0.01, piston_ramp=0.0)
    scen = sc.build(spec)
    out = []
    for e in ({}, env):
        for k, v in e.items():
            monkeypatch.setenv(k, v)
        P = sc.make_params(spec, scen.bounds, precision=prec, tol=1e-10, maxit=20000, precond="mg")
        g = Solver(P)
        setup_tank(g, scen)
        for _ in range(2):
            info = g.step(1)
            assert info.converged and info.rel_residual <= 1e-10
        out.append(g.download_state())
        g.close()
    a, b = out
    for f in ("x", "y"):
        assert rel_l2(b[f], a[f]) < 1e-12, f
    for f in ("vx", "vy", "p"):
        assert rel_l2(b[f], a[f]) < 1e-8, f
