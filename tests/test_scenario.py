"""Seeded scenario generator: counts, determinism, consistency of the inputs."""
import numpy as np
import pytest

from beach_slope_confined_gb300 import scenario as sc


def test_splitmix64_reference_values():
    # splitmix64 from state 0: first output 0xE220A8397B1DCDAF
    u = sc.splitmix64_uniform(0, 2)
    assert int(u[0] * 2 ** 53) == 0xE220A8397B1DCDAF >> 11


@pytest.mark.parametrize("name,fluid", [("c1", 12000), ("c2", 192000), ("c4", 1142 * 85)])
def test_fluid_counts(name, fluid):
    spec = sc.config_spec(name)
    assert int(spec.length / spec.dx + 1e-9) * int(spec.depth / spec.dx + 1e-9) == fluid
    if name == "c1":
        scen = sc.build(spec)
        assert scen.n_fluid == fluid
        assert scen.sx.size > 0


def test_deterministic_and_consistent():
    spec = sc.config_spec("c1")
    a, b = sc.build(spec), sc.build(spec)
    for f in ("x", "y", "mass", "sx", "sy"):
        assert np.array_equal(getattr(a, f), getattr(b, f))
    fluid = a.tid == sc.TID_FLUID
    # jitter is within +/- 0.01 dx of the lattice
    lat = (np.floor(a.x[fluid] / spec.dx) + 0.5) * spec.dx
    assert np.max(np.abs(a.x[fluid] - lat)) <= 0.01 * spec.dx + 1e-15
    # fluid mass = rho0 n dx^2, n in [por, 1]
    n = a.mass[fluid] / (spec.rho0 * spec.dx ** 2)
    assert n.min() >= spec.por - 1e-12 and n.max() <= 1.0
    # every solid lies below the slope line
    assert np.all(a.sy < spec.slope * (a.sx - spec.toe_x))
    # three wall layers with tid 1 innermost
    assert set(np.unique(a.tid)) == {1, 2, 3}


def test_porosity_field_per_cell():
    spec = sc.config_spec("c3")
    assert spec.por_jitter == 0.05
    spec.dx = 0.01  # the field does not depend on resolution
    scen = sc.build(spec)
    g = scen.por_grid
    assert g.shape == (8, 40)
    assert g.min() >= 0.35 and g.max() <= 0.45 and g.std() > 0.01


def test_irregular_piston_ramps_in_from_rest():
    """c5's eight-mode stroke has seeded phases, so it starts at s0 != 0; the
    0.01 s ramp takes it from s0 with zero velocity, and the wall's rest
    coordinate carries -s0, so the wall starts at rest on its lattice."""
    spec = sc.config_spec("c5")
    assert len(spec.piston_amp) == 8 and abs(sum(spec.piston_amp) - 0.03) < 1e-12
    assert min(spec.piston_period) == 0.8 and max(spec.piston_period) == 2.0
    assert spec.piston_ramp == sc.STARTUP_RAMP == 0.01
    s0 = sum(a * np.sin(p) for a, p in zip(spec.piston_amp, spec.piston_phase))
    x0, v0 = sc.piston_stroke(spec, 0.0)
    assert abs(x0 - s0) < 1e-15 and s0 != 0.0 and v0 == 0.0
    # the wall's speed stays that of the stroke over the ramp: no jump
    vmax = max(abs(sc.piston_stroke(spec, t)[1]) for t in np.linspace(0.0, 0.02, 201))
    assert vmax < 0.03 * 2 * np.pi / 0.8
    x1, v1 = sc.piston_stroke(spec, 10.0)
    assert abs(x1) <= 0.03
    spec.dx = 0.01
    scen = sc.build(spec)
    pist = (scen.flags & sc.FLAG_PISTON) != 0
    inner = pist & (scen.tid == sc.TID_WALL)
    assert np.allclose(scen.x[inner], -0.5 * spec.dx, rtol=0, atol=1e-15)
    assert np.all(scen.vx[pist] == 0.0)


def test_rampless_stroke_with_phases_starts_on_its_lattice():
    """Without a ramp a stroke with nonzero phases has x_p(0) != 0: the wall's
    rest coordinate absorbs -x_p(0), so the wall starts one spacing from the
    fluid and moves with the stroke's velocity."""
    spec = sc.config_spec("c5")
    spec.piston_ramp = 0.0
    spec.dx = 0.01  # the layout rule does not depend on resolution
    x0, v0 = sc.piston_stroke(spec, 0.0)
    assert x0 != 0.0 and v0 != 0.0
    scen = sc.build(spec)
    pist = (scen.flags & sc.FLAG_PISTON) != 0
    inner = pist & (scen.tid == sc.TID_WALL)
    assert np.allclose(scen.x[inner], -0.5 * spec.dx, rtol=0, atol=1e-15)
    assert np.allclose(scen.xrest[pist], scen.x[pist] - x0, rtol=0, atol=1e-15)
    assert np.all(scen.vx[pist] == v0)
    # the bottom wall reaches under the piston's leftmost excursion
    bottom = (scen.tid == sc.TID_WALL) & (scen.y < 0) & ~pist
    assert scen.x[bottom].min() < -0.5 * spec.dx - 2 * 0.03


def test_baseline_piston_starts():
    for name in ("c1", "c2"):
        spec = sc.config_spec(name)
        assert spec.piston_ramp == 0.0
        assert sc.piston_stroke(spec, 0.0) == (0.0, 0.02 * 2 * np.pi / 1.2)
    spec = sc.config_spec("c3")
    assert spec.piston_ramp == 0.01 and sc.piston_stroke(spec, 0.0) == (0.0, 0.0)
    assert sc.piston_stroke(spec, 0.01) == sc.piston_stroke(sc.config_spec("c1"), 0.01)
