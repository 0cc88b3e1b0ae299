"""The differentiable WCSPH step and its hand-written adjoint (csrc/wcsph.cu).

The calibration workload runs a weakly compressible SPH model of the porous
beach: Tait EOS, delta-SPH density diffusion, laminar viscosity, and
Darcy/Forchheimer drag in the porous layer. The reference has the same model
in wcsph.f90 and porous.f90 but never builds it. The workload returns
wave-probe elevations after every step. The adjoint returns the gradient of a
probe functional with respect to the Darcy coefficient alpha, the
Forchheimer coefficient beta and the porosity grid of the slope.

Checks:
  * The forward run of a still tank stays near hydrostatic equilibrium.
  * The adjoint gradient matches central finite differences of the same
    forward run for alpha, beta and every porosity cell the fluid sees, to
    1e-4 relative.
  * Checkpointing every K steps, with recomputation, gives the gradient of
    one whole segment.
  * A torch.autograd.Function built on the C ABI (this harness only)
    drives a few calibration steps that reduce a probe misfit.
"""
import time

import numpy as np
import pytest

import oracle
from beach_slope_confined_gb300 import Solver, scenario as sc, setup_tank

pytestmark = pytest.mark.gpu

NSTEPS = 200


def wc_case(dx=0.02, dt=2e-4, **kw):
    spec = sc.TankSpec(dx=dx, dt=dt, por_cells=(16, 4), **kw)
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, precision="fp64")
    g = Solver(P)
    setup_tank(g, scen)
    wp, grid = sc.wcsph_params(spec, scen)
    g.wcsph_setup(wp)
    return g, spec, scen, grid


def test_still_tank_stays_hydrostatic():
    g, spec, scen, grid = wc_case(piston_amp=(0.0,))
    eta = g.wcsph_forward(NSTEPS, 50)
    assert np.all(np.isfinite(eta))
    s = g.download_state()
    fl = scen.tid == sc.TID_FLUID
    v = np.hypot(s["vx"][fl], s["vy"][fl])
    print("max |eta|", np.abs(eta).max(), "max |v|", v.max(), "rho range", s["rho"][fl].min(), s["rho"][fl].max())
    # The lattice settles slightly under the kernel's truncation. No wave forms.
    assert np.abs(eta).max() < 0.05 * spec.depth
    assert v.max() < 0.1
    assert s["rho"][fl].min() >= spec.rho0 * 0.99
    assert s["rho"][fl].max() < spec.rho0 * 1.05
    g.close()


def test_forward_and_gradient_match_the_oracle():
    """The CUDA forward run and gather-form adjoint against the oracle's
    forward run and scatter-form adjoint. The two sum pair terms in different
    orders, so they agree to roundoff, amplified over the run."""
    g, spec, scen, grid0 = wc_case()
    c = oracle.context(sc.make_params(spec, scen.bounds, precision="fp64"))
    setup_tank(c, scen)
    wp, _ = sc.wcsph_params(spec, scen)
    c.wcsph_setup(wp)
    ns = 40
    eg, ec = g.wcsph_forward(ns, 10), c.wcsph_forward(ns, ns)
    a, b = g.download_state(), c.download_state()
    fl = scen.tid == sc.TID_FLUID
    errs = {f: float(np.max(np.abs(a[f][fl] - b[f][fl])) / np.max(np.abs(b[f][fl]))) for f in ("x", "y", "rho")}
    errs["v"] = float(np.max(np.hypot(a["vx"][fl] - b["vx"][fl], a["vy"][fl] - b["vy"][fl])) /
                      np.max(np.hypot(b["vx"][fl], b["vy"][fl])))
    errs["eta"] = float(np.max(np.abs(eg - ec)) / np.max(np.abs(ec)))
    w = np.random.default_rng(17).standard_normal((ns, len(spec.probes)))
    gg, gc = g.wcsph_adjoint(w), c.wcsph_adjoint(w)
    errs["grad_alpha_beta"] = float(np.max(np.abs(gg[:2] - gc[:2]) / np.abs(gc[:2])))
    errs["grad_grid"] = float(np.max(np.abs(gg[2:] - gc[2:])) / np.max(np.abs(gc[2:])))
    print("CUDA vs oracle (max relative):", errs)
    for f in ("x", "y", "rho"):
        assert errs[f] < 1e-12, f
    assert errs["v"] < 1e-9
    assert errs["eta"] < 1e-9
    assert errs["grad_alpha_beta"] < 1e-8
    assert errs["grad_grid"] < 1e-8
    g.close()
    c.close()


def _functional(g, w, alpha, beta, grid, every):
    g.wcsph_set_params(alpha, beta, grid)
    eta = g.wcsph_forward(NSTEPS, every)
    return float(np.sum(w * eta))


def test_adjoint_matches_finite_differences():
    g, spec, scen, grid0 = wc_case()
    rng = np.random.default_rng(7)
    w = rng.standard_normal((NSTEPS, len(spec.probes)))
    a0, b0 = spec.darcy_alpha, spec.forch_beta
    g.wcsph_set_params(a0, b0, grid0)
    g.wcsph_forward(NSTEPS, 25)
    grad = g.wcsph_adjoint(w)
    assert np.all(np.isfinite(grad))
    ng = grid0.size
    # Central differences with a relative step of 1e-3. The truncation error
    # is then under 1e-6 relative. At 1e-5 and below, roundoff in the
    # 200-step runs dominates the differences: the gap to the adjoint grows
    # from 1.5e-4 at 1e-5 to 1.4e-3 at 1e-7.
    fd = np.zeros(2 + ng)
    for k, (base, step) in enumerate(((a0, 1e-3 * a0), (b0, 1e-3 * b0))):
        vals = []
        for s in (+1, -1):
            a, b = (base + s * step, b0) if k == 0 else (a0, base + s * step)
            vals.append(_functional(g, w, a, b, grid0, 25))
        fd[k] = (vals[0] - vals[1]) / (2 * step)
    cells = np.nonzero(np.abs(grad[2:]) > 1e-6 * np.abs(grad[2:]).max())[0]
    for c in cells:
        vals = []
        step = 1e-3 * grid0.reshape(-1)[c]
        for s in (+1, -1):
            gr = grid0.copy().reshape(-1)
            gr[c] += s * step
            vals.append(_functional(g, w, a0, b0, gr, 25))
        fd[2 + c] = (vals[0] - vals[1]) / (2 * step)
    print("alpha: adjoint %.12e fd %.12e" % (grad[0], fd[0]))
    print("beta:  adjoint %.12e fd %.12e" % (grad[1], fd[1]))
    print("cells seen by the fluid:", len(cells), "of", ng)
    for k in (0, 1):
        assert abs(grad[k] - fd[k]) <= 1e-4 * abs(fd[k]), (k, grad[k], fd[k])
    gmax = np.abs(fd[2:]).max()
    assert gmax > 0
    worst = max(abs(grad[2 + c] - fd[2 + c]) / max(abs(fd[2 + c]), 1e-2 * gmax) for c in cells)
    print("porosity cells: worst relative difference %.2e" % worst)
    for c in cells:
        a_, f_ = grad[2 + c], fd[2 + c]
        assert abs(a_ - f_) <= 1e-4 * max(abs(f_), 1e-2 * gmax), (c, a_, f_)
    g.close()


def test_checkpoint_segments_give_the_same_gradient():
    g, spec, scen, grid0 = wc_case()
    w = np.random.default_rng(3).standard_normal((NSTEPS, len(spec.probes)))
    out = {}
    for every in (NSTEPS, 7, 1):
        eta = g.wcsph_forward(NSTEPS, every)
        out[every] = (eta, g.wcsph_adjoint(w))
    e0, g0 = out[NSTEPS]
    for every in (7, 1):
        e1, g1 = out[every]
        assert np.array_equal(e0, e1)
        assert np.max(np.abs(g1 - g0)) <= 1e-12 * np.max(np.abs(g0)), every
    g.close()


def test_autograd_calibration_reduces_misfit():
    torch = pytest.importorskip("torch")
    g, spec, scen, grid0 = wc_case()
    ng = grid0.size
    every = 25

    class ProbeElevations(torch.autograd.Function):
        """eta(alpha, beta, porosity grid) through bsc_wcsph_forward; the
        backward pass is bsc_wcsph_adjoint."""

        @staticmethod
        def forward(ctx, theta):
            t = theta.detach().cpu().double().numpy()
            g.wcsph_set_params(t[0], t[1], t[2:].reshape(grid0.shape))
            eta = g.wcsph_forward(NSTEPS, every)
            return torch.from_numpy(eta)

        @staticmethod
        def backward(ctx, d_eta):
            grad = g.wcsph_adjoint(d_eta.detach().cpu().double().numpy())
            return torch.from_numpy(grad)

    # The target comes from other coefficients and a uniform porosity of 0.45.
    target = np.concatenate([[260.0, 0.9], np.full(ng, 0.45)])
    with torch.no_grad():
        eta_hat = ProbeElevations.apply(torch.from_numpy(target))
    theta = torch.tensor(np.concatenate([[spec.darcy_alpha, spec.forch_beta], grid0.reshape(-1)]),
                         requires_grad=True)
    scale = torch.tensor([100.0, 1.0] + [0.05] * ng, dtype=torch.float64)

    def misfit(th):
        return ((ProbeElevations.apply(th) - eta_hat) ** 2).sum()

    J = misfit(theta)
    J.backward()
    J0 = J.item()
    # the autograd gradient is the adjoint's
    g.wcsph_set_params(spec.darcy_alpha, spec.forch_beta, grid0)
    eta = g.wcsph_forward(NSTEPS, every)
    direct = g.wcsph_adjoint(2.0 * (eta - eta_hat.numpy()))
    assert np.allclose(theta.grad.numpy(), direct, rtol=1e-12, atol=0)
    # normalised steepest descent with backtracking
    Js = [J0]
    step = 0.5
    th = theta.detach().clone()
    gr = theta.grad.detach().clone()
    for _ in range(4):
        d = -gr * scale * scale
        d = d / torch.sqrt(((d / scale) ** 2).sum())
        while step > 1e-4:
            cand = th + step * d
            cand[2:].clamp_(0.2, 0.8)
            with torch.no_grad():
                Jc = misfit(cand).item()
            if Jc < Js[-1]:
                break
            step *= 0.5
        th = cand.detach().clone().requires_grad_(True)
        Jt = misfit(th)
        Jt.backward()
        Js.append(Jt.item())
        gr = th.grad.detach().clone()
        step *= 2.0
    print("misfit:", Js)
    assert Js[-1] < 0.5 * Js[0]
    g.close()


def test_adjoint_costs_at_most_three_forwards():
    g, spec, scen, grid0 = wc_case(dx=0.01, dt=1e-4)
    w = np.random.default_rng(5).standard_normal((NSTEPS, len(spec.probes)))
    g.wcsph_forward(NSTEPS, 25)
    g.wcsph_adjoint(w)
    tf, ta = [], []
    for _ in range(3):
        t0 = time.perf_counter()
        g.wcsph_forward(NSTEPS, 25)
        t1 = time.perf_counter()
        g.wcsph_adjoint(w)
        t2 = time.perf_counter()
        tf.append(t1 - t0)
        ta.append(t2 - t1)
    ratio = min(ta) / min(tf)
    print("forward %.2f ms, adjoint %.2f ms, ratio %.2f" % (1e3 * min(tf), 1e3 * min(ta), ratio))
    assert ratio <= 3.0
    g.close()


def test_repeated_adjoint_after_one_forward():
    """The forward run keeps its last segment for the adjoint; a second
    adjoint of the same run (the segment buffers then hold the first
    segment) recomputes and gives the same gradient."""
    g, spec, scen, grid0 = wc_case()
    w = np.random.default_rng(9).standard_normal((NSTEPS, len(spec.probes)))
    g.wcsph_forward(NSTEPS, 30)
    g1 = g.wcsph_adjoint(w)
    g2 = g.wcsph_adjoint(w)
    assert np.max(np.abs(g1 - g2)) <= 1e-12 * np.max(np.abs(g1))
    g.close()
