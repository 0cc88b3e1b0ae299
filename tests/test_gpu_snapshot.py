"""Text snapshots (csrc/snapshot.cu) against output.f90:188-234 `combined`.

The library's files are compared line by line with the downloaded state,
formatted here by a plain restatement of the Fortran edit descriptors
F10.3, ES10.3 and F10.5 (1X between fields). The fluid, buffer and dead
particles go to their three files.
"""
import math
import os

import numpy as np
import pytest

from beach_slope_confined_gb300 import Solver, scenario as sc, setup_tank
from pairrun import small_spec

pytestmark = pytest.mark.gpu

BUFFER, DEAD = 0x04, 0x08


def f_fmt(v, w, d):
    """Fortran Fw.d: fixed point, right-justified, asterisks on overflow."""
    if math.isnan(v):
        return "NaN".rjust(w)
    s = f"{v:{w}.{d}f}"
    return "*" * w if len(s) > w else s


def es_fmt(v, w, d):
    """Fortran ESw.d: d.ddd and the exponent as E+dd (two digits) or +ddd."""
    m, e = f"{v:.{d}E}".split("E")
    ex = int(e)
    s = f"{m}E{'-' if ex < 0 else '+'}{abs(ex):02d}" if abs(ex) <= 99 else f"{m}{'-' if ex < 0 else '+'}{abs(ex):03d}"
    return "*" * w if len(s) > w else s.rjust(w)


def line(x, y, p, vx, vy, c):
    return " ".join([f_fmt(x, 10, 3), f_fmt(y, 10, 3), f_fmt(p, 10, 3), es_fmt(vx, 10, 3), es_fmt(vy, 10, 3),
                     f_fmt(c + 0.5, 10, 5)])


def test_formatter_edge_cases():
    assert es_fmt(0.0, 10, 3) == " 0.000E+00"
    assert es_fmt(-1.23456e-7, 10, 3) == "-1.235E-07"
    assert es_fmt(2.5e-120, 10, 3) == " 2.500-120"
    assert f_fmt(-1e-5, 10, 3) == "    -0.000"
    assert f_fmt(1.2345e7, 10, 3) == "**********"


def test_snapshot_matches_state(tmp_path):
    spec = small_spec()
    scen = sc.build(spec)
    g = Solver(sc.make_params(spec, scen.bounds, tol=1e-8, maxit=20000, salinity=True))
    setup_tank(g, scen)
    g.step(2)
    s = g.download_state()
    # route two fluid particles to the buffer and dead files
    fl = np.nonzero(scen.tid == sc.TID_FLUID)[0]
    s["flags"][fl[0]] |= BUFFER
    s["flags"][fl[1]] |= DEAD
    g.upload_state(s)
    g.snapshot(str(tmp_path), 7, wait=False)
    g.step(1)  # the next step runs while the files are written
    g.snapshot_wait()
    files = {k: tmp_path / sub / f"{k}_7.txt" for k, sub in (("fluid", "fluid"), ("buffer", "buffer"), ("dead", "fluid"))}
    for f in files.values():
        assert f.exists(), f
    want = {"fluid": [], "buffer": [], "dead": []}
    for i in range(s["x"].size):
        if s["tid"][i] != sc.TID_FLUID:
            continue
        b, d = bool(s["flags"][i] & BUFFER), bool(s["flags"][i] & DEAD)
        key = "fluid" if not (b or d) else "buffer" if b and not d else "dead" if d and not b else None
        if key:
            want[key].append(line(s["x"][i], s["y"][i], s["p"][i], s["vx"][i], s["vy"][i], s["con"][i]))
    for k, f in files.items():
        got = f.read_text().splitlines()
        assert got == want[k], (k, len(got), len(want[k]))
    assert len(want["buffer"]) == 1 and len(want["dead"]) == 1
    assert os.path.getsize(files["fluid"]) == 66 * (fl.size - 2)
    g.close()
