"""ctypes mirror of the C ABI in include/bsc.h.

``Context`` exposes the reference's step routines by their Fortran names
(``projection``, ``cellshift``, ``resetid``, ``neighbour``, ``effpor``,
``eddyvis``, ``int_vel``, ``ppesolve``, ``comp_vel``, ``comp_pos``,
``freesurf``, ``opt2_shift``, ``timestep``; main.f90:46-64).  Each call raises
``BscError`` carrying the library's status code and message, the way the
Fortran shim would check the returned status.

The same class binds any shared library that exports the bsc.h entry points
under a different prefix, which is how the test-suite drives the CUDA library
and the CPU restatement side by side.
"""
from __future__ import annotations

import ctypes
import os
from typing import Dict, Optional, Tuple

import numpy as np

from .scenario import Params, SolveInfo, StateView, Timing, WcsphParams, empty_state, state_view

STATUS = {0: "BSC_OK", -1: "BSC_E_INVALID", -2: "BSC_E_CUDA", -3: "BSC_E_NOMEM",
          -4: "BSC_E_CAPACITY", -5: "BSC_E_NOT_CONVERGED", -6: "BSC_E_BREAKDOWN",
          -7: "BSC_E_NONFINITE", -8: "BSC_E_NOT_BUILT"}

# entry points shared by every library that implements bsc.h (minus prefix)
_PD = ctypes.POINTER(ctypes.c_double)
_P64 = ctypes.POINTER(ctypes.c_int64)
_P32 = ctypes.POINTER(ctypes.c_int32)
_VP = ctypes.c_void_p
COMMON_SIGNATURES = {
    "create": [ctypes.POINTER(Params), ctypes.POINTER(_VP)],
    "destroy": [_VP],
    "upload_state": [_VP, ctypes.POINTER(StateView)],
    "upload_solids": [_VP, ctypes.c_int64, _PD, _PD, _PD, _PD, _PD],
    "upload_porosity": [_VP, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                        ctypes.c_double, ctypes.c_double, _PD],
    "download_state": [_VP, ctypes.POINTER(StateView)],
    "set_time": [_VP, ctypes.c_double, ctypes.c_double],
    "get_time": [_VP, _PD, _PD],
    "piston": [_VP],
    "projection": [_VP],
    "cellshift": [_VP, ctypes.c_int32],
    "resetid": [_VP],
    "neighbour": [_VP],
    "freesurf": [_VP],
    "effpor": [_VP],
    "eddyvis": [_VP],
    "int_vel": [_VP],
    "ppesolve": [_VP, ctypes.POINTER(SolveInfo)],
    "comp_vel": [_VP],
    "comp_pos": [_VP],
    "opt2_shift": [_VP],
    "remove_particles": [_VP, ctypes.c_int32, ctypes.c_double, ctypes.c_double, _P64],
    "insert_particles": [_VP, ctypes.POINTER(StateView)],
    "particle_count": [_VP, _P64],
    "scalart": [_VP],
    "scalarupdate": [_VP, ctypes.c_double],
    "densityupdate": [_VP],
    "timestep": [_VP, _PD],
    "step": [_VP, ctypes.c_int32, ctypes.POINTER(SolveInfo)],
    "get_neighbors": [_VP, _P64, _P32],
    "export_csr": [_VP, _P64, _P32, _PD, _PD],
    "probe_eta": [_VP, ctypes.c_int32, _PD, ctypes.c_double, _PD],
    "csr_solve": [ctypes.POINTER(Params), ctypes.c_int32, _P32, _P32, _PD, _PD, _PD,
                  ctypes.POINTER(SolveInfo)],
}
OPTIONAL_SIGNATURES = {
    "get_timings": [_VP, ctypes.POINTER(Timing)],
    "reset_timings": [_VP],
    "synchronize": [_VP],
    "snapshot_begin": [_VP, ctypes.c_char_p, ctypes.c_int64],
    "snapshot_wait": [_VP],
    "wcsph_setup": [_VP, ctypes.POINTER(WcsphParams)],
    "wcsph_set_params": [_VP, ctypes.c_double, ctypes.c_double, _PD],
    "wcsph_forward": [_VP, ctypes.c_int32, ctypes.c_int32, _PD],
    "wcsph_adjoint": [_VP, _PD, _PD],
}


class BscError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS.get(code, code)} ({code}): {msg}")
        self.code = code


def bind(lib: ctypes.CDLL, prefix: str) -> Dict[str, ctypes._CFuncPtr]:
    fns = {}
    for name, argtypes in COMMON_SIGNATURES.items():
        f = getattr(lib, prefix + name)
        f.argtypes = argtypes
        f.restype = ctypes.c_int
        fns[name] = f
    for name, argtypes in OPTIONAL_SIGNATURES.items():
        f = getattr(lib, prefix + name, None)
        if f is not None:
            f.argtypes = argtypes
            f.restype = ctypes.c_int
            fns[name] = f
    le = getattr(lib, prefix + "last_error")
    le.argtypes = [_VP]
    le.restype = ctypes.c_char_p
    fns["last_error"] = le
    return fns


def _dp(a: np.ndarray):
    return a.ctypes.data_as(_PD)


REMOVE_BUFFER_RIGHT, REMOVE_BUFFER_LEFT, REMOVE_OUTFLOW = 1, 2, 3


class Context:
    """One solver context (a ``bsc_ctx*`` or its CPU counterpart)."""

    def __init__(self, lib: ctypes.CDLL, prefix: str, params: Params):
        self._lib = lib
        self._fn = bind(lib, prefix)
        self.params = params
        h = _VP()
        self._check(self._fn["create"](ctypes.byref(params), ctypes.byref(h)), "create")
        self._h = h
        self.n = 0

    # -- plumbing -----------------------------------------------------------
    def _check(self, rc: int, where: str):
        if rc != 0:
            msg = ""
            if getattr(self, "_h", None):
                raw = self._fn["last_error"](self._h)
                msg = raw.decode() if raw else ""
            raise BscError(rc, where, msg)

    def _call(self, name: str, *args):
        self._check(self._fn[name](self._h, *args), name)

    def close(self):
        if getattr(self, "_h", None):
            self._fn["destroy"](self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state --------------------------------------------------------------
    def upload_state(self, arrs: Dict[str, np.ndarray]):
        self._upload_keep = {k: np.ascontiguousarray(v) for k, v in arrs.items()}
        v = state_view(self._upload_keep)
        self.n = v.n
        self._call("upload_state", ctypes.byref(v))

    def upload_solids(self, x, y, m, rho, por=None):
        x, y, m, rho = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, m, rho))
        pp = None if por is None else _dp(np.ascontiguousarray(por, dtype=np.float64))
        self._call("upload_solids", int(x.size), _dp(x), _dp(y), _dp(m), _dp(rho), pp)

    def upload_porosity(self, grid: np.ndarray, origin, step):
        g = np.ascontiguousarray(grid, dtype=np.float64)
        ny, nx = g.shape
        self._call("upload_porosity", nx, ny, origin[0], origin[1], step[0], step[1], _dp(g))

    def download_state(self, out: Optional[Dict[str, np.ndarray]] = None) -> Dict[str, np.ndarray]:
        """The state in id order; into `out` (arrays shaped as empty_state's,
        e.g. in pinned host memory) when given, else into new arrays."""
        self.n = self.particle_count()
        if out is None:
            out = empty_state(self.n)
        v = state_view(out)
        self._call("download_state", ctypes.byref(v))
        out["L"] = out["L"].reshape(self.n, 4)
        return out

    def set_time(self, t: float, dt: float):
        self._call("set_time", t, dt)

    def get_time(self) -> Tuple[float, float]:
        t, dt = ctypes.c_double(), ctypes.c_double()
        self._call("get_time", ctypes.byref(t), ctypes.byref(dt))
        return t.value, dt.value

    # -- the reference's step routines (main.f90:46-64) ---------------------
    def piston(self): self._call("piston")
    def projection(self): self._call("projection")
    def cellshift(self, alt: bool = False): self._call("cellshift", int(alt))
    def resetid(self): self._call("resetid")
    def neighbour(self): self._call("neighbour")
    def freesurf(self): self._call("freesurf")
    def effpor(self): self._call("effpor")
    def eddyvis(self): self._call("eddyvis")
    def int_vel(self): self._call("int_vel")
    def comp_vel(self): self._call("comp_vel")
    def comp_pos(self): self._call("comp_pos")
    def opt2_shift(self): self._call("opt2_shift")
    def particle_count(self) -> int:
        k = ctypes.c_int64()
        self._call("particle_count", ctypes.byref(k))
        return int(k.value)

    def remove_particles(self, rule: int, a: float, b: float = 0.0) -> int:
        """bsc_remove_particles: REMOVE_BUFFER_RIGHT / _LEFT / REMOVE_OUTFLOW."""
        k = ctypes.c_int64()
        self._call("remove_particles", int(rule), float(a), float(b), ctypes.byref(k))
        self.n = self.particle_count()
        return int(k.value)

    def insert_particles(self, arrs: Dict[str, np.ndarray]):
        """bsc_insert_particles: append particles (host SoA dictionary)."""
        v = state_view(arrs)
        self._call("insert_particles", ctypes.byref(v))
        self.n = self.particle_count()

    def scalart(self): self._call("scalart")
    def scalarupdate(self, stime: float): self._call("scalarupdate", float(stime))
    def densityupdate(self): self._call("densityupdate")

    def ppesolve(self, check: bool = True) -> SolveInfo:
        info = SolveInfo()
        rc = self._fn["ppesolve"](self._h, ctypes.byref(info))
        if check:
            self._check(rc, "ppesolve")
        return info

    def timestep(self) -> float:
        dt = ctypes.c_double(0.0)
        self._call("timestep", ctypes.byref(dt))
        return dt.value

    def step(self, nsteps: int = 1) -> SolveInfo:
        info = SolveInfo()
        self._call("step", int(nsteps), ctypes.byref(info))
        return info

    # -- parity hooks -------------------------------------------------------
    def get_neighbors(self) -> Tuple[np.ndarray, np.ndarray]:
        self.n = self.particle_count()
        off = np.zeros(self.n + 1, np.int64)
        self._call("get_neighbors", off.ctypes.data_as(_P64), None)
        ids = np.zeros(int(off[-1]), np.int32)
        self._call("get_neighbors", off.ctypes.data_as(_P64), ids.ctypes.data_as(_P32))
        return off, ids

    def export_csr(self):
        self.n = self.particle_count()
        rp = np.zeros(self.n + 1, np.int64)
        self._call("export_csr", rp.ctypes.data_as(_P64), None, None, None)
        col = np.zeros(int(rp[-1]), np.int32)
        val = np.zeros(int(rp[-1]))
        rhs = np.zeros(self.n)
        self._call("export_csr", rp.ctypes.data_as(_P64), col.ctypes.data_as(_P32), _dp(val), _dp(rhs))
        return rp, col, val, rhs

    def probe_eta(self, xprobe, depth: float) -> np.ndarray:
        xp = np.ascontiguousarray(xprobe, dtype=np.float64)
        eta = np.zeros(xp.size)
        self._call("probe_eta", int(xp.size), _dp(xp), depth, _dp(eta))
        return eta

    def timings(self) -> Optional[Timing]:
        if "get_timings" not in self._fn:
            return None
        t = Timing()
        self._call("get_timings", ctypes.byref(t))
        return t

    def reset_timings(self):
        if "reset_timings" in self._fn:
            self._call("reset_timings")

    def synchronize(self):
        if "synchronize" in self._fn:
            self._call("synchronize")

    # -- text snapshots (output.f90 `combined`) ---------------------------------
    def snapshot(self, directory: str, index: int, wait: bool = True):
        """Write <directory>/fluid/fluid_<index>.txt, buffer/buffer_<index>.txt
        and fluid/dead_<index>.txt; with wait=False the files are written by a
        host thread while later calls run (snapshot_wait joins it)."""
        self._call("snapshot_begin", os.fsencode(directory), int(index))
        if wait:
            self.snapshot_wait()

    def snapshot_wait(self):
        self._call("snapshot_wait")

    # -- the differentiable WCSPH step (bsc_wcsph_*) ----------------------------
    def wcsph_setup(self, wp: WcsphParams):
        """Take the current state as the initial state of every WCSPH run."""
        self._call("wcsph_setup", ctypes.byref(wp))
        self._wc_np = int(wp.nprobe)
        self._wc_nx, self._wc_ny = int(wp.grid_nx), int(wp.grid_ny)

    def wcsph_set_params(self, alpha: float, beta: float, grid: np.ndarray):
        g = np.ascontiguousarray(grid, dtype=np.float64).reshape(-1)
        self._call("wcsph_set_params", float(alpha), float(beta), _dp(g))

    def wcsph_forward(self, nsteps: int, every: int) -> np.ndarray:
        """Probe elevations after each step, shape (nsteps, nprobe)."""
        eta = np.zeros((nsteps, self._wc_np))
        self._call("wcsph_forward", int(nsteps), int(every), _dp(eta))
        return eta

    def wcsph_adjoint(self, dJ_deta: np.ndarray) -> np.ndarray:
        """Gradient [dJ/dalpha, dJ/dbeta, dJ/dpor (grid, flattened)]."""
        d = np.ascontiguousarray(dJ_deta, dtype=np.float64)
        g = np.zeros(2 + self._wc_nx * self._wc_ny)
        self._call("wcsph_adjoint", _dp(d), _dp(g))
        return g


def csr_solve(lib: ctypes.CDLL, prefix: str, params: Params, rowptr, col, val, b, x0):
    """Standalone CSR solve (solver.f90:129 bicgstab(tls,guess,ls,val,row,col,bvecs,sl))."""
    f = getattr(lib, prefix + "csr_solve")
    f.argtypes = COMMON_SIGNATURES["csr_solve"]
    f.restype = ctypes.c_int
    rp = np.ascontiguousarray(rowptr, dtype=np.int32)
    cl = np.ascontiguousarray(col, dtype=np.int32)
    vl = np.ascontiguousarray(val, dtype=np.float64)
    bb = np.ascontiguousarray(b, dtype=np.float64)
    x = np.array(x0, dtype=np.float64, copy=True)
    info = SolveInfo()
    rc = f(ctypes.byref(params), int(bb.size), rp.ctypes.data_as(_P32), cl.ctypes.data_as(_P32),
           _dp(vl), _dp(bb), _dp(x), ctypes.byref(info))
    return rc, x, info


def setup_tank(ctx: Context, scen, *, initial_effpor: bool = True):
    """Upload a scenario (state, porosity field, solids) and run the initial
    ``effpor`` of main.f90:35-37."""
    from .scenario import state_arrays

    ctx.upload_porosity(scen.por_grid, scen.por_origin, scen.por_step)
    ctx.upload_state(state_arrays(scen))
    ctx.upload_solids(scen.sx, scen.sy, scen.smass, scen.srho)
    t0 = 0.0
    ctx.set_time(t0, scen.spec.dt)
    if initial_effpor:
        ctx.effpor()
