"""bsc_csr_solve_noalloc against a direct solve of the same PPE systems.

The no-allocation entry point serves hosts that keep all device memory in
their own pool: the caller passes device pointers and the solver's work
vectors live in a fixed array inside the library.  The test takes the PPE
matrix the CUDA step assembled for a small tank, solves two different systems
with it one call after the other (the second call finds the first one's
leftovers in the shared array) and checks each solution against scipy's
sparse direct solve.  Both calls stop at a relative residual of 1e-12 (the true
residual, recomputed after the solve, is held to 1.5e-12) and the
Jacobi-scaled matrix has a condition number of about 600, so each solution is
within 600 * 1.5e-12 of the exact one: the test allows 1e-9.  The second call
must leave the device's free memory unchanged (the first one may commit the
library's array under lazy module loading).  It also checks the rejections:
too many rows, and host pointers.  This file runs last so that it sees a
device the other tests have already used; it passes as well in a fresh
process.
"""
import numpy as np
import pytest

from beach_slope_confined_gb300 import Solver, scenario as sc, setup_tank, solve_csr_noalloc
from pairrun import rel_err

pytestmark = pytest.mark.gpu

X_TOL = 1e-9          # condition number (~600) x RES_TOL, rounded up
RES_TOL = 1.5e-12     # the true residual after a stop at 1e-12, with room for the recurrence's drift
MAX_ROWS = 131072     # BSC_NOALLOC_MAX_ROWS of include/bsc.h
BSC_E_INVALID, BSC_E_CAPACITY = -1, -4


def _ppe_system():
    spec = sc.TankSpec(dx=0.02)
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, tol=1e-12, maxit=20000)
    g = Solver(P)
    setup_tank(g, scen)
    for stage in (g.piston, g.projection, g.cellshift, g.resetid, g.neighbour, g.effpor, g.eddyvis, g.int_vel):
        stage()
    g.ppesolve()
    rp, col, val, rhs = g.export_csr()
    g.close()
    return P, rp.astype(np.int32), col, val, rhs


def _device(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda:0")


def _noalloc(P, rp, col, val, b, x0):
    """One call on device copies of the arrays; also returns the change in the
    device's free memory across the call itself."""
    import torch

    d = [_device(a) for a in (rp, col, val, b, x0)]
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    free0 = torch.cuda.mem_get_info()[0]
    rc, info = solve_csr_noalloc(P, b.size, *(t.data_ptr() for t in d), stream=stream)
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    return rc, d[4].cpu().numpy(), info, free0 - free1


def test_noalloc_matches_direct_solve_on_two_calls_in_a_row():
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl

    P, rp, col, val, rhs = _ppe_system()
    n = rhs.size
    assert 0 < n <= MAX_ROWS
    A = sp.csr_matrix((val, col, rp), shape=(n, n)).tocsc()
    rng = np.random.default_rng(7)
    systems = [(rhs, np.zeros(n)),
               (0.5 * rhs + rng.standard_normal(n) * np.abs(rhs).max(), np.ones(n))]
    for k, (b, x0) in enumerate(systems):
        x_ref = spl.spsolve(A, b)
        rc, x, info, used = _noalloc(P, rp, col, val, b, x0)
        assert rc == 0 and info.converged, (rc, info.iterations, info.rel_residual)
        assert info.rel_residual <= RES_TOL
        assert rel_err(x, x_ref) <= X_TOL, rel_err(x, x_ref)
        if k == 1:
            assert used == 0, f"the second call changed the device's free memory by {used} bytes"


def test_noalloc_rejects_oversize_and_host_pointers():
    P, rp, col, val, rhs = _ppe_system()
    d = [_device(a) for a in (rp, col, val, rhs, np.zeros(rhs.size))]
    ptrs = [t.data_ptr() for t in d]
    rc, _ = solve_csr_noalloc(P, MAX_ROWS + 1, *ptrs)
    assert rc == BSC_E_CAPACITY
    host_x = np.zeros(rhs.size)
    rc, _ = solve_csr_noalloc(P, rhs.size, *ptrs[:4], host_x.ctypes.data)
    assert rc == BSC_E_INVALID
