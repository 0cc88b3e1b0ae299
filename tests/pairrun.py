"""Helpers that drive the CUDA library and the CPU oracle side by side."""
from __future__ import annotations

import numpy as np

import oracle
from beach_slope_confined_gb300 import scenario as sc
from beach_slope_confined_gb300.binding import setup_tank


def small_spec(dx=0.02, kernel=1, **kw) -> sc.TankSpec:
    return sc.TankSpec(dx=dx, kernel=kernel, **kw)


def rel_err(a, b):
    """Normwise relative difference max|a-b| / max|b| (inf-norm)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.max(np.abs(b)) if b.size else 0.0
    return float(np.max(np.abs(a - b)) / den) if den > 0 else float(np.max(np.abs(a - b), initial=0.0))


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a - b))


def canonical_csr(rp, col, val, n):
    """The exported PPE as a canonical sparse matrix: duplicates summed and
    explicit zeros dropped.  The reference (and the oracle) leave the slots of
    a ghost row's fluid neighbours at column `pos` with value 0
    (isph.f90:125-128,274-296); the CUDA path stores them at the neighbour's
    column with value 0.  Both are the same matrix."""
    import scipy.sparse as sp

    A = sp.csr_matrix((val, col, rp), shape=(n, n))
    A.sum_duplicates()
    A.eliminate_zeros()
    A.sort_indices()
    return A


def make_pair(scen, params, gpu_factory):
    """(gpu, cpu) contexts with the same scenario uploaded and effpor run."""
    g = gpu_factory(params)
    c = oracle.context(params)
    for ctx in (g, c):
        setup_tank(ctx, scen)
    return g, c


def advance_to_lists(ctxs):
    """piston, projection, cellshift, resetid, neighbour (main.f90:46-49)."""
    for ctx in ctxs:
        ctx.piston()
        ctx.projection()
        ctx.cellshift()
        ctx.resetid()
        ctx.neighbour()


def sprinkle_flags(scen, frac_dead=0.01, frac_buffer=0.01, seed=7):
    """Mark a seeded random subset of fluid particles dead or buffer, to drive
    the branches of the reference that the wave tank never takes."""
    u = sc.splitmix64_uniform(seed, scen.n)
    fluid = scen.tid == sc.TID_FLUID
    dead = fluid & (u < frac_dead)
    buf = fluid & (u >= frac_dead) & (u < frac_dead + frac_buffer)
    scen.flags = scen.flags.copy()
    scen.flags[dead] |= sc.FLAG_DEAD
    scen.flags[buf] |= sc.FLAG_BUFFER
    # give the flagged particles some motion so the branches matter
    v = sc.splitmix64_uniform(seed + 1, 2 * scen.n)
    scen.vx = scen.vx.copy()
    scen.vy = scen.vy.copy()
    scen.vx[fluid] += 0.01 * (v[0::2][fluid] - 0.5)
    scen.vy[fluid] += 0.01 * (v[1::2][fluid] - 0.5)
    return scen
