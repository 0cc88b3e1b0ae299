"""Regenerate tests/golden/solvertest_kat.json from the reference's only
known-answer test, solvertest.f90:10-19 (a 5x5 CSR system with unit values
whose exact solution is 1..5).  Reads the Fortran source as text; the
reference is never compiled or run.

    python tests/golden/make_golden.py /path/to/reference
"""
import json
import os
import re
import sys


def parse(src: str):
    def ints(name):
        m = re.search(name + r"\s*=\s*\(/([^/]*)/\)", src)
        return [int(v) for v in m.group(1).split(",")]

    def reals(name):
        m = re.search(name + r"\s*=\s*\(/([^/]*)/\)", src)
        return [float(v.replace("_dp", "")) for v in m.group(1).split(",")]

    row = ints(r"row")
    col = ints(r"col")
    b = reals(r"::b")
    tol = float(re.search(r"tls\s*=\s*([0-9.]+)_dp", src).group(1))
    n = len(row) - 1
    # unit values (val=1.0_dp, solvertest.f90:15); exact solution by substitution
    return {
        "source": "solvertest.f90:10-19",
        "n": n,
        "rowptr": [r - 1 for r in row],
        "col": [c - 1 for c in col],
        "val": [1.0] * len(col),
        "b": b,
        "guess": [1.0] * n,
        "reference_tol": tol,
        "solution": [1.0, 2.0, 3.0, 4.0, 5.0],
    }


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py /path/to/reference")
    ref = sys.argv[1]
    with open(os.path.join(ref, "solvertest.f90")) as fh:
        data = parse(fh.read())
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "solvertest_kat.json")
    with open(out, "w") as fh:
        json.dump(data, fh, indent=1)
    print(out)
