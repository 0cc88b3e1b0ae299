"""Oracle fields of the benchmark tanks c1 and c2 after N steps (TEST FIXTURES).

    python tests/golden/make_config_fixtures.py [--config c1|c2|all] [--threads T]

Runs the CPU oracle (oracle/oracle.cpp, the C++ restatement of the reference's
step) on the seeded c1 and c2 wave tanks with both of the reference's PPE
solvers, BiCGSTAB (solver.f90:129-254) and FGMRES with restart 30
(solver.f90:306-347), each to a relative residual of 1e-8 at dt = 1e-4 s, and
writes what the GPU parity tests compare against:

  c1 (12000 fluid particles), 2000 steps:
      every fluid particle's x, y, vx, vy, p after step 2000, and a seeded
      sample of 2048 fluid ids after steps 500, 1000 and 1500;
  c2 (192000 fluid particles), 200 steps:
      a seeded sample of 16384 fluid ids after steps 100 and 200.

Each run also keeps its PPE iteration count and final relative residual per
step.  Files: tests/golden/<config>_<solver>.npz and
tests/golden/config_fixtures.json (the run lengths, thread count, wall time
and the two oracle solvers' difference at the last step: the spread that two
solves to 1e-8 leave after that many steps).

The fixtures are the oracle's output on the scenario generator's bytes, so
they change when either changes; rerun this script then.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import oracle  # noqa: E402  (the checker)
from beach_slope_confined_gb300 import scenario as sc  # noqa: E402
from beach_slope_confined_gb300.binding import setup_tank  # noqa: E402

FIELDS = ("x", "y", "vx", "vy", "p")
SOLVERS = ("bicgstab", "fgmres")
RESTART = 30
PLAN = {
    # config: (steps, {step: sample size or None for every fluid particle})
    "c1": (2000, {500: 2048, 1000: 2048, 1500: 2048, 2000: None}),
    "c2": (200, {100: 16384, 200: 16384}),
}
SAMPLE_SEED = 11


def sample_ids(scen, size):
    """Seeded sample of fluid ids (sorted), or every fluid id."""
    fluid = np.nonzero(scen.tid == sc.TID_FLUID)[0].astype(np.int32)
    if size is None or size >= fluid.size:
        return fluid
    u = sc.splitmix64_uniform(SAMPLE_SEED, fluid.size)
    return np.sort(fluid[np.argsort(u, kind="stable")[:size]])


def run(config, solver, threads):
    steps, snaps = PLAN[config]
    spec = sc.config_spec(config)
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, solver=solver, tol=1e-8, maxit=40000, restart=RESTART)
    oracle.set_threads(threads)
    o = oracle.context(P)
    setup_tank(o, scen)
    out = {"iterations": np.zeros(steps, np.int32), "rel_residual": np.zeros(steps)}
    t0 = time.perf_counter()
    for k in range(1, steps + 1):
        info = o.step(1)
        if not info.converged:
            raise RuntimeError(f"{config}/{solver}: step {k} did not converge ({info.rel_residual:.3e})")
        out["iterations"][k - 1] = info.iterations
        out["rel_residual"][k - 1] = info.rel_residual
        if k in snaps:
            s = o.download_state()
            ids = sample_ids(scen, snaps[k])
            out[f"ids_{k}"] = ids
            for f in FIELDS:
                out[f"{f}_{k}"] = s[f][ids]
        if k % 100 == 0:
            print(f"{config}/{solver}: step {k}/{steps}, {time.perf_counter() - t0:.0f} s", flush=True)
    wall = time.perf_counter() - t0
    o.close()
    np.savez_compressed(os.path.join(HERE, f"{config}_{solver}.npz"), **out)
    return out, wall


def spread(a, b, step):
    """Relative L2 difference of the two solvers' fields at `step`."""
    assert np.array_equal(a[f"ids_{step}"], b[f"ids_{step}"])
    return {f: float(np.linalg.norm(a[f"{f}_{step}"] - b[f"{f}_{step}"]) / np.linalg.norm(b[f"{f}_{step}"]))
            for f in FIELDS}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="all", choices=("c1", "c2", "all"))
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    args = ap.parse_args()
    meta_path = os.path.join(HERE, "config_fixtures.json")
    meta = {}
    if os.path.exists(meta_path):
        with open(meta_path) as fh:
            meta = json.load(fh)
    for config in (("c1", "c2") if args.config == "all" else (args.config,)):
        steps, snaps = PLAN[config]
        runs, walls = {}, {}
        for solver in SOLVERS:
            runs[solver], walls[solver] = run(config, solver, args.threads)
        scen = sc.build(sc.config_spec(config))
        meta[config] = {
            "steps": steps, "snapshots": sorted(snaps), "fluid_particles": scen.n_fluid,
            "particles": scen.n, "tol": 1e-8, "fgmres_restart": RESTART, "dt": sc.config_spec(config).dt,
            "oracle_threads": args.threads, "wall_s": walls,
            "mean_iterations": {s: float(runs[s]["iterations"].mean()) for s in SOLVERS},
            "solver_spread_last_step": spread(runs["fgmres"], runs["bicgstab"], steps),
        }
        with open(meta_path, "w") as fh:
            json.dump(meta, fh, indent=1, sort_keys=True)
        print(json.dumps(meta[config]), flush=True)


if __name__ == "__main__":
    main()
