"""A short, bounded run of the ISPH step for kernel profiling.

    python -m beach_slope_confined_gb300.profile_case c3 mixed 10

builds the named wave-tank case, uploads it and runs ``steps`` (default 1)
full steps with every PPE solve capped at ``maxit`` Krylov iterations, so a
profiler sees a few launches of each kernel of the step on the full-size
state.  A capped solve reports BSC_E_NOT_CONVERGED, which is expected here
and ignored; any other error raises.  Prints ``ok`` and the particle count.

    python -m beach_slope_confined_gb300.profile_case c4 fp64 --wcsph 20 --every 10

runs the WCSPH calibration workload instead: a forward run of 20 steps with
checkpoints every 10, then the adjoint of a probe functional.

    python -m beach_slope_confined_gb300.profile_case reference fp64 2000 --precond mg --steps 4

runs the reference's own tank (reference_geometry.build) instead of a wave
tank.
"""
from __future__ import annotations

import argparse

from . import BscError, Solver, scenario as sc, setup_tank

NOT_CONVERGED = -5


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("config", nargs="?", default="c3")
    ap.add_argument("precision", nargs="?", default="mixed", choices=("mixed", "fp64"))
    ap.add_argument("maxit", nargs="?", type=int, default=10)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--precond", default="none", choices=("none", "mg"))
    ap.add_argument("--wcsph", type=int, default=0, help="WCSPH forward + adjoint steps instead of ISPH steps")
    ap.add_argument("--every", type=int, default=10, help="WCSPH checkpoint interval")
    ap.add_argument("--salinity", action="store_true", help="the phase-3 step with salinity transport")
    args = ap.parse_args(argv)
    tank = None
    if args.config == "reference":
        from . import reference_geometry as rg

        tank = rg.build()
        scen = tank.scenario
    else:
        spec = sc.config_spec(args.config)
        scen = sc.build(spec)
    if args.wcsph > 0 and tank is None:
        import numpy as np

        g = Solver(sc.make_params(spec, scen.bounds, precision="fp64"))
        setup_tank(g, scen)
        wp, _grid = sc.wcsph_params(spec, scen)
        g.wcsph_setup(wp)
        g.wcsph_forward(args.wcsph, args.every)
        g.wcsph_adjoint(np.ones((args.wcsph, len(spec.probes))))
        g.synchronize()
        g.close()
        print("ok", scen.n)
        return
    # the inner-solve settings of bench.py for each preconditioner
    mg = args.precond == "mg"
    kw = dict(precision=args.precision, tol=1e-8, maxit=args.maxit, inner_tol=1e-5 if mg else 0.1,
              max_outer=40 if mg else 4, precond=args.precond, restart=40, salinity=args.salinity)
    if tank is None:
        g = Solver(sc.make_params(spec, scen.bounds, **kw))
        setup_tank(g, scen)
    else:
        g = Solver(rg.params(tank, solver="fgmres", **kw))
        rg.setup(g, tank)
    for _ in range(args.steps):
        try:
            g.step(1)
        except BscError as e:
            if e.code != NOT_CONVERGED:
                raise
    g.synchronize()
    g.close()
    print("ok", scen.n)


if __name__ == "__main__":
    main()
