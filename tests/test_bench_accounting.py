"""The bench line's per-kernel accounting (bench.kernel_rooflines,
bench.kernel_traffic): algorithmic FP64 flops and bytes per launch from the
per-pair and per-row counts, both fractions, and `bound` the larger one.
Host arithmetic only: a fake timing record stands in for the library's."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


class FakeTiming:
    def __init__(self):
        self.ms = np.zeros(32)
        self.calls = np.zeros(32, dtype=np.int64)


def _timing(slot, ms_per_launch, launches):
    t = FakeTiming()
    t.ms[slot] = ms_per_launch * launches
    t.calls[slot] = launches
    return t


@pytest.mark.parametrize("prec,col", [("fp64", 0), ("mixed", 1)])
def test_neighbour_search_counts(prec, col):
    n, nnz, steps = 846333, 16836202, 20
    t = _timing(bench.T_K_NEIGHBOUR, 0.5, 2 * steps)
    (k,) = bench.kernel_rooflines(t, steps, nnz, 1, n, prec, 1000.0, 6800.0)
    assert k["kernel"] == bench.KERNEL_NAMES[bench.T_K_NEIGHBOUR][col]
    assert k["launches_per_step"] == 2 and k["ms_per_step"] == pytest.approx(1.0)
    flops = bench.FP64_FLOPS[bench.T_K_NEIGHBOUR][col] * nnz
    row_b, ent_b = bench.HBM_BYTES[bench.T_K_NEIGHBOUR][col]
    assert k["fp64_flops_per_launch"] == flops
    assert k["algorithmic_bytes_per_launch"] == row_b * n + ent_b * nnz
    assert k["achieved_gflops"] == pytest.approx(flops / 0.5e-3 / 1e9)
    assert k["achieved_gbs"] == pytest.approx((row_b * n + ent_b * nnz) / 0.5e-3 / 1e9)
    assert k["frac"] == pytest.approx(k["achieved_gflops"] / 1000.0)
    assert k["hbm_frac"] == pytest.approx(k["achieved_gbs"] / 6800.0)
    assert k["bound"] == ("fp64" if k["frac"] >= k["hbm_frac"] else "hbm")


def test_fp64_search_is_fp64_bound_and_mixed_search_hbm_bound():
    n, nnz = 846333, 16836202
    t = _timing(bench.T_K_NEIGHBOUR, 0.9, 2)
    (k,) = bench.kernel_rooflines(t, 1, nnz, 1, n, "fp64", 1056.0, 6784.0)
    assert k["bound"] == "fp64" and 0.3 < k["frac"] < 0.6
    t = _timing(bench.T_K_NEIGHBOUR, 0.36, 2)
    (k,) = bench.kernel_rooflines(t, 1, nnz, 1, n, "mixed", 1056.0, 6784.0)
    # the double-float search issues no FP64 operation per pair
    assert k["fp64_flops_per_launch"] == 0 and k["bound"] == "hbm"


def test_effpor_counts_solid_pairs():
    t = _timing(bench.T_K_EFFPOR, 0.5, 2)
    (k,) = bench.kernel_rooflines(t, 1, 10**7, 5467827, 846333, "fp64", 1000.0, 6800.0)
    assert k["pairs_per_launch"] == 5467827
    assert k["fp64_flops_per_launch"] == bench.FP64_FLOPS[bench.T_K_EFFPOR][0] * 5467827


def test_unlaunched_kernels_are_left_out():
    assert bench.kernel_rooflines(FakeTiming(), 1, 100, 1, 10, "mixed", 1.0, 1.0) == []


def test_traffic_scales_the_committed_bytes_per_row():
    tr = bench.kernel_traffic("k_neighbour<float>", 1000)
    assert tr is not None and 100 * 1000 < tr < 2000 * 1000
    assert bench.kernel_traffic("no such kernel", 1000) is None
