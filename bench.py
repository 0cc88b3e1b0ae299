"""Benchmark of the ISPH step: particle-steps/s on the ~1M-particle wave tank.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config c3]

Workload: the 4.0 m x 0.6 m tank at dx = 1.2 mm (833,250 fluid particles plus
walls; per-cell porosity 0.4 +/- 0.05 in the slope; the piston driven from
t = 0), Wendland C2 with h = 1.3 dx, PPE to relative residual 1e-8 (by
default FGMRES preconditioned by the cell-multigrid V-cycle; `--precond none`
runs the reference's unpreconditioned BiCGSTAB), fixed dt = 1e-4 s.  A step
is the whole main.f90:41-65 sequence (two neighbour searches, porosity, eddy
viscosity, predictor, PPE assembly + solve, projection, shifting).  The
headline `value` is the mixed-precision path (FP32 pair sums, FP32 inner
FGMRES and V-cycle, FP64 assembly and refinement); the plain FP64 path is
reported beside it.

`--impl reference` times the reference algorithm on the host cores instead:
the C++ OpenMP restatement of the Fortran routines (the Fortran itself needs
gfortran and Intel MKL, neither present on this machine), full steps of the same
tank with the reference's BiCGSTAB to the same residual, W untimed and K
timed.

Other modes (one JSON line each; no timing contract):
  --long N          N steps of the mixed and then the FP64 path from the same
                    start: ms and PPE iterations per step, and the mixed
                    path's relative L2 difference from the FP64 path for
                    every field after the run;
  --profile-case    a short bounded run for a profiler (see `profile_case`).

With `--gpus N` under torchrun every rank runs an independent replica of the
tank on its own GPU (the step does not shard across GPUs here); value = the
particle-steps of all ranks / the slowest rank's time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at 1M (mixed vs FP64, PPE res 1e-8); adjoint/forward time"
CONFIG = "c3"
T_STEP, T_PPE_SOLVE, T_SPMV, T_UPLOAD, T_DOWNLOAD, T_SCALAR = 15, 8, 16, 17, 18, 24
# single-kernel slots of bsc_timing (include/bsc.h)
T_K_NEIGHBOUR, T_K_ASSEMBLE, T_K_INT_VEL, T_K_EFFPOR, T_K_SHIFT = 25, 26, 27, 28, 29

# Algorithmic FP64 flops per pair of the pair kernels, counted from the
# formulas each kernel evaluates (an FMA is 2 flops; a division or a square
# root is 1): kernel slot -> (FP64 path, mixed path).  Per neighbour pair:
#   k_neighbour: offsets 2, d^2 3, root 1, grad W factor 6, grad W 2, the
#     moment sum M 10 (mixed: membership, root and grad W on FP32 pairs from
#     double-float offsets, grad W stored as a double-float; the FP64 test
#     only inside a 1e-10 band around the threshold, 0 per pair);
#   k_assemble: offsets 2, 1/(r^2+lam) 5, L grad W 6, the coefficient 6, the
#     diagonal 2, rho_ij 4, velocity differences 4, divergence 5, the Jacobi
#     scaling 1 (mixed: k_assemble_df runs that arithmetic on FP32 pairs; its
#     FP64 work is the two velocity differences and their splits and the
#     widening of the entry, 5);
#   k_int_vel: the two harmonic viscosity means and their sum 10, offsets
#     and r^2 5, 1/(r^2+lam) 2, L grad W 6, the coefficient 6, velocity
#     differences 2, viscous sums 6, SPS sums 6 (mixed: 0; offsets from the
#     FP32 cell offsets, velocity differences from FP32 roundings);
#   k_shift: 16 (mixed: 0; the position-shift sums run as double-floats,
#     the velocity-gradient sums in FP32).
# Per solid pair, k_effpor: offsets 2, d^2 3, root 1, W 9, the weighted sum
# 4 (mixed: FP32 terms summed as a double-float, 0).
FP64_FLOPS = {T_K_NEIGHBOUR: (24, 0), T_K_ASSEMBLE: (35, 5), T_K_INT_VEL: (43, 0), T_K_SHIFT: (16, 0),
              T_K_EFFPOR: (19, 0)}
# Algorithmic DRAM bytes: (per row, per neighbour entry) for each path, each
# input read and each output written once (neighbours' particle data counted
# once per row, as it is reused from cache):
#   k_neighbour: x, y, offsets, cell, flags (row) and the cell lists' share;
#     per entry the list index and grad W written (FP64, or the mixed path's
#     two FP32 halves); L, tr M, flags and the count written per row;
#   k_assemble: the row's and one neighbour's inputs (~100 B), the
#     right-hand side; per entry the list index and grad W read, the value
#     written (and the FP32 and FP16 copies on the mixed path);
#   k_int_vel: 175 B per row; per entry the list index and grad W (FP32 on
#     the mixed path);
#   k_shift: 150 B per row; per entry the list index and grad W (its two
#     FP32 halves on the mixed path);
#   k_effpor: 73 B per row (solids: a few MB per launch, not counted).
HBM_BYTES = {T_K_NEIGHBOUR: ((110, 20), (130, 20)), T_K_ASSEMBLE: ((108, 28), (148, 38)),
             T_K_INT_VEL: ((175, 20), (175, 12)), T_K_SHIFT: ((150, 20), (150, 20)),
             T_K_EFFPOR: ((73, 0), (73, 0))}
# what ncu shows limits a kernel that neither bound reaches (full captures of
# one launch each on the c2 tank)
KERNEL_LIMITER = {
    "k_neighbour<float>": "issue and latency of the double-float chains: 35 % warps active (64 registers), 10 cycles "
                          "between a warp's instructions; FP64 17 %, FMA 28.5 %, ALU 25 % of their pipes",
    "k_int_vel<float>": "latency of its per-neighbour gathers (long scoreboard 12.7 per issue), 34 % warps active",
    "k_assemble_df": "issue and latency: 58 % of issue slots, 29 % warps active (80 registers); FP64 35.5 %, "
                     "FMA 36.5 %, ALU 26 % of their pipes",
}
# the kernel each slot times: (FP64 path, mixed path)
KERNEL_NAMES = {T_K_NEIGHBOUR: ("k_neighbour<double>", "k_neighbour<float>"),
                T_K_ASSEMBLE: ("k_assemble<double>", "k_assemble_df"),
                T_K_INT_VEL: ("k_int_vel<double>", "k_int_vel<float>"),
                T_K_SHIFT: ("k_shift<double>", "k_shift<float>"),
                T_K_EFFPOR: ("k_effpor<double>", "k_effpor<float>")}


# --------------------------------------------------------------------------
# distributed plumbing (replicas only)
# --------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist

            backend = os.environ.get("BSC_DIST_BACKEND", "nccl")
            if backend == "nccl":
                import torch

                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch

        dev = "cuda" if os.environ.get("BSC_DIST_BACKEND", "nccl") == "nccl" else "cpu"
        t = torch.tensor([v], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def aggregate(per_rank_seconds: float, units_per_rank: float, dist: Dist):
    """Whole-job throughput: all ranks' units / the slowest rank's time."""
    tmax = dist.max(per_rank_seconds)
    return units_per_rank * dist.world / tmax, tmax


# --------------------------------------------------------------------------
# clocks during the timed region
# --------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
            return self
        # nvidia-smi takes a moment to start: the timed region begins once it
        # reports (bounded), so that its samples fall inside the region
        t0 = time.perf_counter()
        while not self.lines and self.proc.poll() is None and time.perf_counter() - t0 < 10.0:
            time.sleep(0.01)
        self.lines.clear()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = max(smax, float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


# --------------------------------------------------------------------------
# our arm
# --------------------------------------------------------------------------
def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def spmv_bytes(nnz: int, n: int, fp32: bool) -> int:
    """Algorithmic bytes of one SpMV launch (k_bicg_1): per stored entry the
    value and the column; per row the count, x_i, the result and the shadow
    residual of the fused dot.  Neighbour values x_j come from cache."""
    if fp32:
        return 8 * nnz + 16 * n
    return 12 * nnz + 28 * n


def spmv_mg_bytes(nnz: int, n: int, fp32: bool) -> int:
    """Algorithmic bytes of the SpMV w = A z of one multigrid-preconditioned
    FGMRES iteration: k_spmv_f (FP32 operator and vectors, the mixed path's
    inner solve) or k_spmv_z<double> (FP64).  Per stored entry the value and
    the column; per row the count, z_i and w_i.  Neighbour values z_j come
    from cache."""
    if fp32:
        return 8 * nnz + 12 * n
    return 12 * nnz + 20 * n


PINNED = False


def link_bandwidth(nbytes: int, reps: int = 3):
    """GB/s of one pinned host->device and one device->host copy of `nbytes`
    (torch copies timed with CUDA events): the host link the e2e copies run
    over, measured on this machine for comparison."""
    try:
        import torch

        h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
        d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        out = {}
        for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
            dst.copy_(src, non_blocking=True)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(reps):
                dst.copy_(src, non_blocking=True)
            e1.record()
            torch.cuda.synchronize()
            out[name] = reps * nbytes / (e0.elapsed_time(e1) * 1e-3) / 1e9
        return out
    except Exception as ex:  # no CUDA-capable torch
        return {"unavailable": repr(ex)[:80]}


def pinned_like(a: np.ndarray) -> np.ndarray:
    """A copy of `a` in page-locked host memory (torch's pinned allocator),
    so host<->device copies run at the interconnect's DMA rate."""
    global PINNED
    try:
        import torch

        t = torch.empty(a.shape, dtype=getattr(torch, str(a.dtype)), pin_memory=True)
        out = t.numpy()
        out[...] = a
        PINNED = True
        return out
    except Exception:  # no CUDA-capable torch: pageable copies
        return np.array(a, copy=True)


def fp64_bound_kernels():
    """The pair kernels whose time is set by the FP64 pipe (not HBM), from the
    committed ncu summary: name, FP64-pipe utilisation, DRAM throughput."""
    try:
        with open(os.path.join(ROOT, "profiles", "fp64_bound_kernels.json")) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return None


def traffic_per_row(kind: str):
    """DRAM bytes per row of one SpMV launch from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "spmv_dram_traffic.json")) as fh:
            return float(json.load(fh)[kind]["dram_bytes_per_row"])
    except (OSError, KeyError, ValueError):
        return None


def kernel_traffic(kernel: str, n: int):
    """DRAM bytes per launch of a pair kernel, from the committed ncu summary
    (bytes per row of a smaller capture, scaled to n rows)."""
    try:
        with open(os.path.join(ROOT, "profiles", "kernel_dram_traffic.json")) as fh:
            return float(json.load(fh)[kernel]["dram_bytes_per_row"]) * n
    except (OSError, KeyError, ValueError):
        return None


def solid_pairs(scen) -> int:
    """Fluid-solid pairs within the support 2h on the initial state: the
    pair count of effpor's porosity sum (the solids do not move, and the
    fluid near the bed barely does over a benchmark's steps)."""
    from scipy.spatial import cKDTree

    h = scen.spec.h_factor * scen.spec.dx
    fl = scen.tid == 3
    if scen.sx.size == 0:
        return 0
    tree = cKDTree(np.column_stack([scen.sx, scen.sy]))
    return int(tree.count_neighbors(cKDTree(np.column_stack([scen.x[fl], scen.y[fl]])), 2.0 * h * (1 - 1e-12)))


def kernel_rooflines(t, steps: int, nnz: int, spairs: int, n: int, prec: str, fp64_peak: float, hbm_peak: float):
    """Per pair kernel: event-timed ms per launch, launches per step, its
    algorithmic FP64 GFLOP/s against the measured FP64 FMA rate and its
    algorithmic GB/s against the measured HBM copy bandwidth; `bound` is the
    larger fraction."""
    out = []
    col = 0 if prec == "fp64" else 1
    for slot, name in KERNEL_NAMES.items():
        calls = int(t.calls[slot])
        if calls == 0:
            continue
        ms = t.ms[slot] / calls
        pairs = spairs if slot == T_K_EFFPOR else nnz
        flops = FP64_FLOPS[slot][col] * pairs
        gf = flops / (ms * 1e-3) / 1e9
        row_b, ent_b = HBM_BYTES[slot][col]
        byts = row_b * n + ent_b * nnz
        gbs = byts / (ms * 1e-3) / 1e9
        f64 = gf / fp64_peak if fp64_peak else 0.0
        fhbm = gbs / hbm_peak if hbm_peak else 0.0
        out.append({"kernel": name[col], "ms_per_launch": ms, "launches_per_step": calls / steps,
                    "ms_per_step": t.ms[slot] / steps, "fp64_flops_per_launch": flops, "pairs_per_launch": pairs,
                    "achieved_gflops": gf, "peak_gflops": fp64_peak, "frac": f64,
                    "algorithmic_bytes_per_launch": byts, "achieved_gbs": gbs, "hbm_frac": fhbm,
                    "bound": "fp64" if f64 >= fhbm else "hbm"})
    return out


def run_ours(args, dist: Dist):
    from beach_slope_confined_gb300 import Solver, measure_peaks, scenario as sc, setup_tank

    spec = sc.config_spec(args.config)
    scen = sc.build(spec)
    nf = scen.n_fluid
    results = {}
    states, times = {}, {}
    peaks = measure_peaks()
    spairs = solid_pairs(scen)
    for prec in ("mixed", "fp64"):
        if prec == "fp64" and args.no_fp64:
            continue
        P = sc.make_params(spec, scen.bounds, precision=prec, solver=args.solver, tol=1e-8, maxit=40000,
                           inner_tol=args.inner_tol, max_outer=60, precond=args.precond, restart=args.restart)
        g = Solver(P)
        setup_tank(g, scen)
        for _ in range(args.warmup):
            g.step(1)
        off, _ = g.get_neighbors()
        nnz = int(off[-1])
        g.synchronize()
        g.reset_timings()
        dist.barrier()
        iters = []
        with ClockSampler(dist.local) as clk:
            t0 = time.perf_counter()
            for _ in range(args.steps):
                info = g.step(1)
                iters.append((info.iterations, info.outer, info.rel_residual))
            g.synchronize()
            wall = time.perf_counter() - t0
        t = g.timings()
        dev_s = t.ms[T_STEP] / 1e3
        value, tmax = aggregate(dev_s, nf * args.steps, dist)
        spmv_ms = t.ms[T_SPMV] / max(1, t.calls[T_SPMV])
        results[prec] = dict(value=value, ms_per_step=tmax / args.steps * 1e3, wall_s=wall, nnz=nnz,
                             iters=iters, spmv_ms=spmv_ms, spmv_calls=int(t.calls[T_SPMV]),
                             solve_ms=t.ms[T_PPE_SOLVE] / args.steps, launches=int(t.kernel_launches),
                             clocks=clk.summary(), n=scen.n,
                             kernels=kernel_rooflines(t, args.steps, nnz, spairs, scen.n, prec, peaks[0],
                                                      measured_peak_hbm()[0]))
        states[prec] = g.download_state()
        times[prec] = g.get_time()
        # e2e through the C ABI with host buffers in pinned memory: every
        # iteration uploads the state and its time (t, dt), steps, and
        # downloads the state: the same step from the same inputs each time
        # (the time is an input too: without it each repeat would drive the
        # piston one step further from the uploaded particles)
        if prec == "mixed":
            host = g.download_state()
            t_in, dt_in = g.get_time()
            up = {k: pinned_like(v.reshape(-1)) for k, v in host.items()}
            out = {k: pinned_like(v) for k, v in host.items()}
            h2d = sum(a.nbytes for a in up.values())

            def e2e_iteration():
                g.upload_state(up)
                g.set_time(t_in, dt_in)
                info = g.step(1)
                g.download_state(out)
                return info.iterations

            # warm-up: an upload gathers the state into cell order, which
            # swaps the cell-map buffer that the solver's cached CUDA graphs
            # are keyed by, so successive iterations alternate between two
            # graph sets; both are built before the timed region
            for _ in range(max(3, args.warmup)):
                e2e_iteration()
            g.synchronize()
            g.reset_timings()
            dist.barrier()
            t0 = time.perf_counter()
            ke = max(1, min(args.steps, 5))
            e2e_its = [e2e_iteration() for _ in range(ke)]
            e2e_s = time.perf_counter() - t0
            te = g.timings()
            d2h = sum(np.asarray(a).nbytes for a in out.values())
            ev, _ = aggregate(e2e_s, nf * ke, dist)
            # where the time goes, per step: device-timed upload (copies,
            # derived fields, cell build), step and download (gathers to id
            # order, copies); the rest is host time between the calls
            up_ms, dn_ms, st_ms = (te.ms[k] / ke for k in (T_UPLOAD, T_DOWNLOAD, T_STEP))
            # after the measurement: the same iteration three more times, each
            # read back on its own (device ms of upload, step, download), and
            # the link's own copy rate for the same byte count
            per_it = []
            for _ in range(3):
                g.reset_timings()
                e2e_iteration()
                tt = g.timings()
                per_it.append([round(tt.ms[k], 3) for k in (T_UPLOAD, T_STEP, T_DOWNLOAD)])
            link = link_bandwidth(int(h2d))
            results[prec]["e2e"] = dict(value=ev, unit="particle-steps/s", h2d_bytes_per_step=int(h2d),
                                        d2h_bytes_per_step=int(d2h), steps=ke,
                                        host_memory="pinned" if PINNED else "pageable",
                                        ms_per_step=e2e_s / ke * 1e3, upload_ms=up_ms, step_ms=st_ms,
                                        download_ms=dn_ms, h2d_gbs=h2d / (up_ms * 1e-3) / 1e9 if up_ms else None,
                                        d2h_gbs=d2h / (dn_ms * 1e-3) / 1e9 if dn_ms else None,
                                        after_iterations_ms_upload_step_download=per_it, link=link,
                                        ppe_iterations=e2e_its)
        g.close()
    errs = None
    if "fp64" in states:
        errs = {"after_run": field_errors(states["mixed"], states["fp64"]),
                "one_step": one_step_errors(args, spec, scen, states["fp64"], times["fp64"])}
    return scen, results, errs, peaks


def one_step_errors(args, spec, scen, start, tdt):
    """One mixed step against one FP64 step from the same state (the FP64
    arm's state after its timed steps): the mixed path's error per step,
    which the runs' difference after many steps does not show (the tank's
    flow amplifies any perturbation, the FP64 path's own roundoff included,
    by about e every 100 steps)."""
    from beach_slope_confined_gb300 import Solver, setup_tank

    out = {}
    for prec in ("fp64", "mixed"):
        P = sc_params(args, spec, scen, prec)
        h = Solver(P)
        setup_tank(h, scen)
        h.upload_state(start)
        h.set_time(*tdt)
        h.effpor()
        h.step(1)
        out[prec] = h.download_state()
        h.close()
    e = field_errors(out["mixed"], out["fp64"])
    e["xy_per_spacing"] = float(np.max(np.hypot(out["mixed"]["x"] - out["fp64"]["x"],
                                                out["mixed"]["y"] - out["fp64"]["y"])) / spec.dx)
    return e


def sc_params(args, spec, scen, prec):
    from beach_slope_confined_gb300 import scenario as sc

    return sc.make_params(spec, scen.bounds, precision=prec, solver=args.solver, tol=1e-8, maxit=40000,
                          inner_tol=args.inner_tol, max_outer=60, precond=args.precond, restart=args.restart)


ERROR_FIELDS = ("x", "y", "vx", "vy", "p", "rho", "porosity", "nut", "tke", "vel", "gradvx", "resist", "varts")


def field_errors(a, b):
    """Relative L2 difference of every state field of `a` from `b`, plus
    the x displacement since the start (x - xrest): x itself is ~1 m, so its
    relative error says little about the motion."""
    out = {}
    for f in ERROR_FIELDS + ("x_displacement",):
        if f == "x_displacement":
            u, v = a["x"] - b["xrest"], b["x"] - b["xrest"]
        else:
            u, v = a[f], b[f]
        nv = np.linalg.norm(v)
        out[f] = float(np.linalg.norm(u - v) / nv) if nv > 0 else float(np.linalg.norm(u - v))
    # particles the two runs classify differently at the free surface (the
    # test tr M <= 1.6 of search.f90:300-306): each one switches its pressure
    # row, shift factor and artificial viscosity, and moves the fields far
    # more than the arithmetic does
    out["free_flag_mismatches"] = int(((a["flags"] ^ b["flags"]) & 1).sum())
    return out


def cpu_steps(scen, spec, threads: int, steps: int, warmup: int, solver: str = "bicgstab"):
    """Full steps of the reference algorithm on the host cores: the C++
    OpenMP restatement, PPE by the reference's BiCGSTAB (or FGMRES) to a
    relative residual of 1e-8, no iteration cap.  `warmup` untimed steps,
    then `steps` timed ones.  Returns (particle-steps/s, description, PPE
    iterations of the timed steps)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from beach_slope_confined_gb300 import scenario as sc
    from beach_slope_confined_gb300.binding import setup_tank

    oracle.set_threads(threads)
    P = sc.make_params(spec, scen.bounds, solver=solver, tol=1e-8, maxit=40000, restart=30)
    o = oracle.context(P)
    setup_tank(o, scen)
    for _ in range(warmup):
        o.step(1)
    iters = []
    t0 = time.perf_counter()
    for _ in range(steps):
        info = o.step(1)
        iters.append(int(info.iterations))
    wall = time.perf_counter() - t0
    o.close()
    desc = (f"steps {warmup + 1}-{warmup + steps} of the {scen.n_fluid}-fluid-particle tank, full steps of the "
            f"C++ OpenMP restatement on {threads} threads, PPE {solver} to rel-res 1e-8 "
            f"({statistics.mean(iters):.0f} iterations per step), {wall / steps:.2f} s per step")
    return scen.n_fluid * steps / wall, desc, iters


def run_wcsph(reps: int = 2):
    """The differentiable WCSPH workload (c4): a 500-step FP64 forward run with
    checkpoints every 50 steps, then the adjoint of the squared probe misfit
    against a target run (alpha=260, beta=0.9, porosity 0.45). Times both
    through the C ABI, with host timers around the synchronous calls. Checks
    the alpha and beta gradients against central differences of the same
    forward run."""
    from beach_slope_confined_gb300 import Solver, scenario as sc, setup_tank

    spec = sc.config_spec("c4")
    scen = sc.build(spec)
    nsteps, every = 500, 50
    g = Solver(sc.make_params(spec, scen.bounds, precision="fp64"))
    setup_tank(g, scen)
    wp, grid0 = sc.wcsph_params(spec, scen)
    g.wcsph_setup(wp)
    g.wcsph_set_params(260.0, 0.9, np.full_like(grid0, 0.45))
    eta_hat = g.wcsph_forward(nsteps, every)
    a0, b0 = spec.darcy_alpha, spec.forch_beta

    def misfit(a, b):
        g.wcsph_set_params(a, b, grid0)
        eta = g.wcsph_forward(nsteps, every)
        return float(np.sum((eta - eta_hat) ** 2)), eta

    J0, eta = misfit(a0, b0)
    dJ = 2.0 * (eta - eta_hat)
    grad = g.wcsph_adjoint(dJ)
    tf, ta = [], []
    for _ in range(max(1, reps)):
        t0 = time.perf_counter()
        g.wcsph_forward(nsteps, every)
        t1 = time.perf_counter()
        g.wcsph_adjoint(dJ)
        t2 = time.perf_counter()
        tf.append(t1 - t0)
        ta.append(t2 - t1)
    fwd, adj = min(tf), min(ta)
    # Central differences: the fourth-order stencil at a relative step of 3e-2,
    # and the two-point one at 1e-6. Roundoff, amplified over 500 steps,
    # limits the misfit's differences to about 1e-4 relative at steps of
    # 3e-3 and dominates them at 1e-6.
    fd = {}
    for rs, pts in ((3e-2, 4), (1e-6, 2)):
        out = {}
        for k, (name, base) in enumerate((("alpha", a0), ("beta", b0))):
            h = rs * base
            J = {}
            for m in ((-2, -1, 1, 2) if pts == 4 else (-1, 1)):
                J[m] = misfit(a0 + m * h, b0)[0] if k == 0 else misfit(a0, b0 + m * h)[0]
            if pts == 4:
                d = (8.0 * (J[1] - J[-1]) - (J[2] - J[-2])) / (12.0 * h)
            else:
                d = (J[1] - J[-1]) / (2.0 * h)
            out[name] = {"fd": d, "adjoint": float(grad[k]),
                         "rel_diff": abs(float(grad[k]) - d) / abs(d) if d != 0 else None}
        fd[f"{pts}-point, relative step {rs:g}"] = out
    g.close()
    return {"ratio": adj / fwd, "forward_ms": 1e3 * fwd, "adjoint_ms": 1e3 * adj,
            "workload": f"c4 tank, dx={spec.dx} m, {scen.n_fluid} fluid + {scen.n - scen.n_fluid} wall particles, "
                        f"{nsteps} FP64 WCSPH steps of dt={spec.dt} s, checkpoints every {every}",
            "forward_particle_steps_per_s": scen.n_fluid * nsteps / fwd,
            "misfit": J0, "gradient_alpha_beta": [float(grad[0]), float(grad[1])],
            "gradient_porosity_grid_norm": float(np.linalg.norm(grad[2:])),
            "finite_differences": fd}


def wcsph_check(args):
    """`--wcsph-check`: the c4 gradient checks.

    For the c4 case as configured (and, with `--wcsph-ramp R`, with the
    piston ramp set to R seconds): the misfit J of the squared probe
    elevations against the target run (alpha=260, beta=0.9, porosity 0.45),
    the adjoint gradient, and
      * central differences of alpha and beta at relative steps 1e-1 ..
        1e-7 (two-point) and at 3e-2 (four-point): where the differences
        agree with the adjoint, and where roundoff takes over;
      * central differences for every porosity cell the fluid sees, at
        relative steps 3e-2 .. 1e-6;
      * the oracle's FP64 adjoint (scatter form, every state kept) over the
        first `--wcsph-oracle-steps` steps of the same case, against the
        CUDA adjoint of the same shortened run.
    One JSON line."""
    from beach_slope_confined_gb300 import Solver, scenario as sc, setup_tank

    spec = sc.config_spec("c4")
    if args.wcsph_ramp is not None:
        spec.piston_ramp = args.wcsph_ramp
    scen = sc.build(spec)
    nsteps, every = 500, 50
    g = Solver(sc.make_params(spec, scen.bounds, precision="fp64"))
    setup_tank(g, scen)
    wp, grid0 = sc.wcsph_params(spec, scen)
    g.wcsph_setup(wp)
    g.wcsph_set_params(260.0, 0.9, np.full_like(grid0, 0.45))
    eta_hat = g.wcsph_forward(nsteps, every)
    a0, b0 = spec.darcy_alpha, spec.forch_beta

    def misfit(a, b, grid):
        g.wcsph_set_params(a, b, grid)
        eta = g.wcsph_forward(nsteps, every)
        return float(np.sum((eta - eta_hat) ** 2)), eta

    J0, eta = misfit(a0, b0, grid0)
    dJ = 2.0 * (eta - eta_hat)
    grad = g.wcsph_adjoint(dJ)
    out = {"mode": "wcsph-check", "piston_ramp": spec.piston_ramp, "steps": nsteps, "misfit": J0,
           "eta_rms": float(np.sqrt(np.mean(eta ** 2))), "eta_diff_rms": float(np.sqrt(np.mean((eta - eta_hat) ** 2))),
           "gradient_alpha_beta": [float(grad[0]), float(grad[1])]}

    def fd_param(k, rs, pts=2):
        base = (a0, b0)[k]
        h = rs * base
        J = {}
        for m in ((-2, -1, 1, 2) if pts == 4 else (-1, 1)):
            J[m] = misfit(a0 + m * h, b0, grid0)[0] if k == 0 else misfit(a0, b0 + m * h, grid0)[0]
        if pts == 4:
            return (8.0 * (J[1] - J[-1]) - (J[2] - J[-2])) / (12.0 * h)
        return (J[1] - J[-1]) / (2.0 * h)

    sweep = {}
    for rs in (1e-1, 3e-2, 1e-2, 3e-3, 1e-3, 1e-4, 1e-5, 1e-6, 1e-7):
        row = {}
        for k, name in enumerate(("alpha", "beta")):
            d = fd_param(k, rs)
            row[name] = abs(float(grad[k]) - d) / abs(d) if d != 0 else None
        sweep[f"{rs:g}"] = row
    out["alpha_beta_sweep_rel_diff"] = sweep
    four = {}
    for k, name in enumerate(("alpha", "beta")):
        d = fd_param(k, 3e-2, 4)
        four[name] = abs(float(grad[k]) - d) / abs(d) if d != 0 else None
    out["alpha_beta_4pt_3e-2_rel_diff"] = four
    # the plateau: the relative step whose worse alpha/beta difference is smallest
    plateau = min(sweep, key=lambda r: max(v for v in sweep[r].values() if v is not None))
    out["plateau_step"] = float(plateau)
    gp = grad[2:].reshape(grid0.shape)
    # the cells the fluid sees: adjoint gradient above 1e-6 of the largest
    # (the others carry ~1e-25 and their differences are exactly zero); each
    # difference is measured against max(|fd|, 1e-2 max|fd|), as the unit test
    # of the gradient does
    cells = [tuple(ix) for ix in np.argwhere(np.abs(gp) > 1e-6 * np.abs(gp).max())]
    por = {}
    for rs in (3e-2, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6):
        fds = []
        for (iy, ix) in cells:
            h = rs * grid0[iy, ix]
            gm, gpl = grid0.copy(), grid0.copy()
            gm[iy, ix] -= h
            gpl[iy, ix] += h
            fds.append((misfit(a0, b0, gpl)[0] - misfit(a0, b0, gm)[0]) / (2.0 * h))
        fds = np.asarray(fds)
        adj = np.asarray([gp[c] for c in cells])
        floor = 1e-2 * np.abs(fds).max() if fds.size else 0.0
        diffs = np.abs(adj - fds) / np.maximum(np.abs(fds), floor) if fds.size else np.zeros(0)
        top = np.argsort(-np.abs(adj))[:5]
        por[f"{rs:g}"] = {"cells": len(cells), "max_rel_diff": float(diffs.max()) if diffs.size else None,
                          "median_rel_diff": float(np.median(diffs)) if diffs.size else None,
                          "cells_within_1e-4": int((diffs < 1e-4).sum()),
                          "largest_five": [{"cell": [int(cells[k][0]), int(cells[k][1])], "adjoint": float(adj[k]),
                                            "fd": float(fds[k])} for k in top]}
    out["porosity_cells"] = por
    out["porosity_gradient_norm"] = float(np.linalg.norm(gp))
    g.close()
    # the oracle's FP64 adjoint on the first steps of the same case
    ns = args.wcsph_oracle_steps
    if ns > 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.set_threads(os.cpu_count() or 1)
        res = {}
        for side in ("cuda", "oracle"):
            P = sc.make_params(spec, scen.bounds, precision="fp64")
            h = Solver(P) if side == "cuda" else oracle.context(P)
            setup_tank(h, scen)
            h.wcsph_setup(wp)
            h.wcsph_set_params(260.0, 0.9, np.full_like(grid0, 0.45))
            target = h.wcsph_forward(ns, every if side == "cuda" else ns)
            h.wcsph_set_params(a0, b0, grid0)
            t0 = time.perf_counter()
            e = h.wcsph_forward(ns, every if side == "cuda" else ns)
            gr = h.wcsph_adjoint(2.0 * (e - target))
            res[side] = (e, gr, time.perf_counter() - t0)
            h.close()
        (ec, gc, tc), (eo, go, to) = res["cuda"], res["oracle"]
        out["oracle_comparison"] = {
            "steps": ns, "eta_max_rel_diff": float(np.max(np.abs(ec - eo)) / np.max(np.abs(eo))),
            "alpha_rel_diff": abs(float(gc[0] - go[0])) / abs(float(go[0])),
            "beta_rel_diff": abs(float(gc[1] - go[1])) / abs(float(go[1])),
            "porosity_grid_rel_diff": float(np.linalg.norm(gc[2:] - go[2:]) / np.linalg.norm(go[2:])),
            "cuda_s": tc, "oracle_s": to, "oracle_threads": os.cpu_count() or 1}
    print(json.dumps(out), flush=True)


def run_salinity(args):
    """The c3 tank with salinity transport: the phase-3 step of
    main.f90:198-260 (salinity sub-steps before the projection,
    densityupdate after the shift, eddyvis after the time step) on the mixed
    multigrid path. Stage events time the step and the salinity stages."""
    from beach_slope_confined_gb300 import Solver, scenario as sc, setup_tank

    spec = sc.config_spec(args.config)
    scen = sc.build(spec)
    P = sc.make_params(spec, scen.bounds, precision="mixed", solver=args.solver, tol=1e-8, maxit=40000,
                       inner_tol=args.inner_tol, max_outer=60, precond=args.precond, restart=args.restart,
                       salinity=True)
    g = Solver(P)
    setup_tank(g, scen)
    for _ in range(args.warmup):
        g.step(1)
    g.synchronize()
    g.reset_timings()
    for _ in range(args.steps):
        g.step(1)
    g.synchronize()
    t = g.timings()
    s = g.download_state()
    # an output.f90 `combined` snapshot, written by the library's host thread
    # while the next step runs
    import tempfile
    with tempfile.TemporaryDirectory() as tmp:
        g.synchronize()
        t0 = time.perf_counter()
        g.snapshot(tmp, 0, wait=False)
        t1 = time.perf_counter()
        g.step(1)
        g.synchronize()
        t2 = time.perf_counter()
        g.snapshot_wait()
        t3 = time.perf_counter()
        snap_bytes = sum(os.path.getsize(os.path.join(dp, f)) for dp, _, fs in os.walk(tmp) for f in fs)
    g.close()
    fl = scen.tid == sc.TID_FLUID
    step_ms = t.ms[T_STEP] / args.steps
    return {"workload": f"{args.config} tank with the saline wedge con = 0.5 tanh((x - {spec.salinity_front}) / "
                        f"{spec.salinity_width}), mixed multigrid path, phase-3 step",
            "ms_per_step": step_ms, "particle_steps_per_s": scen.n_fluid / (step_ms * 1e-3),
            "salinity_ms_per_step": t.ms[T_SCALAR] / args.steps,
            "salinity_launches_per_step": t.calls[T_SCALAR] / args.steps,
            "con_range": [float(s["con"][fl].min()), float(s["con"][fl].max())],
            "snapshot": {"bytes": snap_bytes, "queue_ms": 1e3 * (t1 - t0), "step_after_ms": 1e3 * (t2 - t1),
                         "written_after_ms": 1e3 * (t3 - t0)}}


def run_reference_tank(args, threads: int):
    """The reference's own tank (init + gen_boundary + gen_fluid of
    setup.f90, boundary.f90, internal.f90) on the FP64 and mixed paths, PPE by
    FGMRES with the cell-multigrid V-cycle to a relative residual of 1e-8,
    beside the oracle's step on the host cores (unpreconditioned FGMRES to
    the same residual).  The reference's own stop, 1e-3 of ||r0|| within 150
    iterations, needs its restart of 150; at this library's restart cap of 64
    the first step ends just above it."""
    from beach_slope_confined_gb300 import Solver, reference_geometry as rg

    tank = rg.build()
    s = tank.scenario
    nf = int(np.count_nonzero(s.tid == 3))
    out = {"workload": f"the reference's own tank: {s.n} particles ({nf} fluid) and {s.sx.size} soil solids, "
                       f"hybrid kernel h1={tank.constants.h1:.5f} m, FGMRES({args.restart}) + multigrid to 1e-8"}
    steps = 20
    for prec in ("fp64", "mixed"):
        g = Solver(rg.params(tank, precision=prec, solver="fgmres", precond="mg", tol=1e-8, maxit=2000,
                             restart=args.restart, inner_tol=1e-5, max_outer=60))
        rg.setup(g, tank)
        for _ in range(max(args.warmup, 3)):
            g.step(1)
        g.synchronize()
        g.reset_timings()
        for _ in range(steps):
            g.step(1)
        g.synchronize()
        out[prec + "_ms_per_step"] = g.timings().ms[T_STEP] / steps
        g.close()
    if not args.no_cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle

        oracle.set_threads(threads)
        o = oracle.context(rg.params(tank, solver="fgmres", tol=1e-8, maxit=20000, restart=args.restart))
        rg.setup(o, tank)
        o.step(1)
        t0 = time.perf_counter()
        o.step(3)
        cpu_ms = (time.perf_counter() - t0) / 3 * 1e3
        out.update(oracle_ms_per_step=cpu_ms, oracle_threads=threads,
                   oracle_over_mixed=cpu_ms / out["mixed_ms_per_step"])
    return out


def run_long(args):
    """`--long N`: N steps of the mixed path and then of the FP64 path from the
    same start, with per-step device ms and PPE iterations, and the mixed
    path's difference from the FP64 path for every field at the end."""
    from beach_slope_confined_gb300 import Solver, scenario as sc, setup_tank

    spec = sc.config_spec(args.config)
    scen = sc.build(spec)
    out = {"mode": "long", "config": args.config, "steps": args.long, "fluid_particles": scen.n_fluid,
           "precond": args.precond}
    states = {}
    for prec in ("mixed", "fp64"):
        P = sc.make_params(spec, scen.bounds, precision=prec, solver=args.solver, tol=1e-8, maxit=40000,
                           inner_tol=args.inner_tol, max_outer=60, precond=args.precond, restart=args.restart)
        g = Solver(P)
        setup_tank(g, scen)
        ms, its, res = [], [], []
        for _ in range(args.long):
            g.reset_timings()
            info = g.step(1)
            t = g.timings()
            ms.append(t.ms[T_STEP])
            its.append(int(info.iterations))
            res.append(float(info.rel_residual))
        states[prec] = g.download_state()
        g.close()
        ms, its = np.asarray(ms), np.asarray(its)
        win = slice(args.warmup, args.warmup + args.steps)
        blocks = [{"steps": f"{k + 1}-{min(k + 100, args.long)}", "ms_per_step": float(ms[k:k + 100].mean()),
                   "iterations": float(its[k:k + 100].mean())} for k in range(0, args.long, 100)]
        out[prec] = {"ms_per_step_mean": float(ms.mean()), "ms_per_step_min": float(ms.min()),
                     "ms_per_step_max": float(ms.max()), "iterations_mean": float(its.mean()),
                     "iterations_min": int(its.min()), "iterations_max": int(its.max()),
                     "max_rel_residual": float(max(res)),
                     "bench_window": {"steps": f"{args.warmup + 1}-{args.warmup + args.steps}",
                                      "ms_per_step": float(ms[win].mean()),
                                      "iterations": float(its[win].mean())},
                     "per_100_steps": blocks,
                     "particle_steps_per_s": scen.n_fluid / (ms.mean() * 1e-3)}
    out["mixed_over_fp64_speed"] = out["fp64"]["ms_per_step_mean"] / out["mixed"]["ms_per_step_mean"]
    out["mixed_vs_fp64_rel_l2"] = field_errors(states["mixed"], states["fp64"])
    fl = scen.tid == sc.TID_FLUID
    v = np.hypot(states["fp64"]["vx"][fl], states["fp64"]["vy"][fl])
    out["fp64_state"] = {"t": args.long * spec.dt, "max_speed": float(v.max()), "mean_speed": float(v.mean())}
    print(json.dumps(out), flush=True)


def profile_case(args):
    """`--profile-case`: a short, bounded run of the step for a profiler.

    Builds the `--config` tank (or the reference's own tank with
    `--config reference`), uploads it and runs `--steps` full steps of the
    `--precision` path with every PPE solve capped at `--maxit` Krylov
    iterations, so a profiler sees a few launches of each kernel on the
    full-size state.  A capped solve reports BSC_E_NOT_CONVERGED, which is
    expected here and ignored; any other error raises.  With `--wcsph K` it
    runs the WCSPH calibration workload instead: a forward run of K steps
    with checkpoints every `--every`, then the adjoint of a probe functional.
    Prints `ok` and the particle count."""
    from beach_slope_confined_gb300 import BscError, Solver, scenario as sc, setup_tank

    not_converged = -5
    tank = None
    if args.config == "reference":
        from beach_slope_confined_gb300 import reference_geometry as rg

        tank = rg.build()
        scen = tank.scenario
    else:
        spec = sc.config_spec(args.config)
        scen = sc.build(spec)
    if args.wcsph > 0 and tank is None:
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
    mg = args.precond == "mg"
    kw = dict(precision=args.precision, tol=1e-8, maxit=args.maxit, inner_tol=args.inner_tol,
              max_outer=40 if mg else 4, precond=args.precond, restart=args.restart, salinity=args.salinity)
    if tank is None:
        g = Solver(sc.make_params(spec, scen.bounds, solver=args.solver, **kw))
        setup_tank(g, scen)
    else:
        g = Solver(rg.params(tank, solver="fgmres", **kw))
        rg.setup(g, tank)
    for _ in range(args.steps):
        try:
            g.step(1)
        except BscError as e:
            if e.code != not_converged:
                raise
    g.synchronize()
    g.close()
    print("ok", scen.n)


def run_reference_arm(args, dist: Dist, threads: int):
    """`--impl reference`: the reference algorithm on the host cores (the
    oracle, a C++ OpenMP restatement of the Fortran), full uncapped steps of
    the same tank: W untimed, then K timed.  Rank 0 only."""
    from beach_slope_confined_gb300 import scenario as sc

    if dist.rank != 0:
        return
    spec = sc.config_spec(args.config)
    scen = sc.build(spec)
    value, desc, iters = cpu_steps(scen, spec, threads, max(1, args.steps), args.warmup, args.ref_solver)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * scen.n_fluid / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded wave tank, no dataset)",
            "config": {"workload": f"{args.config} wave tank, dx={spec.dx} m, {scen.n_fluid} fluid particles, "
                                   f"the reference's {args.ref_solver} PPE to rel-res 1e-8, dt={spec.dt} s",
                       "fluid_particles": scen.n_fluid},
            "ppe": {"iterations": iters},
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--config", default=CONFIG)
    ap.add_argument("--solver", default="bicgstab", choices=("bicgstab", "fgmres"))
    ap.add_argument("--ref-solver", default="bicgstab", choices=("bicgstab", "fgmres"),
                    help="the reference arm's PPE solver (FGMRES restarts at 30)")
    ap.add_argument("--inner-tol", type=float, default=None,
                    help="mixed path: relative tolerance of each FP32 inner solve (default 1e-5 with the "
                         "multigrid preconditioner, 0.1 for the BiCGSTAB sweeps without it)")
    ap.add_argument("--precond", default="mg", choices=("mg", "none"),
                    help="PPE preconditioner: cell multigrid inside FGMRES, or none (the reference's solvers)")
    ap.add_argument("--restart", type=int, default=40)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=2,
                    help="timed oracle steps of the cpu_baseline sample (after one untimed step)")
    ap.add_argument("--no-wcsph", action="store_true", help="skip the WCSPH forward/adjoint workload (c4)")
    ap.add_argument("--no-salinity", action="store_true", help="skip the salinity-transport step measurement")
    ap.add_argument("--no-reference-tank", action="store_true", help="skip the reference's own tank")
    ap.add_argument("--long", type=int, default=0, help="record N steps of both paths (see the module doc)")
    ap.add_argument("--profile-case", action="store_true", help="a bounded run for a profiler (see profile_case)")
    ap.add_argument("--precision", default="mixed", choices=("mixed", "fp64"), help="--profile-case path")
    ap.add_argument("--maxit", type=int, default=10, help="--profile-case: Krylov iterations per solve")
    ap.add_argument("--wcsph", type=int, default=0, help="--profile-case: WCSPH forward + adjoint steps")
    ap.add_argument("--every", type=int, default=10, help="--profile-case: WCSPH checkpoint interval")
    ap.add_argument("--salinity", action="store_true", help="--profile-case: the phase-3 step with salinity")
    ap.add_argument("--wcsph-check", action="store_true", help="the c4 gradient checks (see wcsph_check)")
    ap.add_argument("--wcsph-ramp", type=float, default=None, help="--wcsph-check: the piston ramp (s)")
    ap.add_argument("--wcsph-oracle-steps", type=int, default=20,
                    help="--wcsph-check: steps of the CUDA-vs-oracle adjoint comparison (0: skip)")
    args = ap.parse_args()
    if args.inner_tol is None:
        args.inner_tol = 1e-5 if args.precond == "mg" else 0.1
    if args.profile_case:
        profile_case(args)
        return
    if args.long:
        run_long(args)
        return
    if args.wcsph_check:
        wcsph_check(args)
        return
    dist = Dist()
    from beach_slope_confined_gb300 import scenario as sc

    threads = os.cpu_count() or 1
    if args.impl == "reference":
        run_reference_arm(args, dist, threads)
        dist.close()
        return

    scen, res, errs, peaks = run_ours(args, dist)
    if dist.rank != 0:
        dist.close()
        return
    spec = sc.config_spec(args.config)
    m = res["mixed"]
    hbm, peak_kind = measured_peak_hbm()
    mg = args.precond == "mg"
    if mg:
        byts = spmv_mg_bytes(m["nnz"], m["n"], fp32=True)
        kname = "k_spmv_f (FP32 ELL SpMV of the inner FGMRES)"
        tpr = traffic_per_row("spmv_f_fp32")
    else:
        byts = spmv_bytes(m["nnz"], m["n"], fp32=True)
        kname = "k_bicg_1<EllOp<float>,float> (FP32 ELL SpMV + dot)"
        tpr = traffic_per_row("fp32")
    achieved = byts / (m["spmv_ms"] * 1e-3) / 1e9 if m["spmv_ms"] > 0 else None
    spmv_roof = {"bound": "hbm", "kernel": kname,
                 "achieved": achieved, "peak": hbm, "unit": "GB/s",
                 "frac": (achieved / hbm) if achieved else None,
                 "traffic": (tpr * m["n"]) if tpr else None,
                 "algorithmic_bytes_per_launch": byts, "avg_launch_ms": m["spmv_ms"],
                 "launches_timed": m["spmv_calls"], "ms_per_step": m["spmv_ms"] * m["spmv_calls"] / args.steps,
                 "peak_source": f"{peak_kind} MEASURED_PEAKS.json hbm_gbs"}
    # the roofline of the timed kernel with the largest share of the step:
    # one of the FP64-pipe-bound pair kernels (against the measured FP64 FMA
    # rate), or the SpMV (against the measured HBM copy bandwidth)
    top = max(m["kernels"], key=lambda k: k["ms_per_step"]) if m["kernels"] else None
    if top and top["ms_per_step"] > spmv_roof["ms_per_step"]:
        common = {"kernel": top["kernel"] + " (mixed path)", "traffic": kernel_traffic(top["kernel"], m["n"]),
                  "avg_launch_ms": top["ms_per_launch"], "launches_per_step": top["launches_per_step"],
                  "share_of_step": top["ms_per_step"] / m["ms_per_step"],
                  "fp64": {"achieved_gflops": top["achieved_gflops"], "peak_gflops": top["peak_gflops"],
                           "frac": top["frac"], "algorithmic_fp64_flops_per_launch": top["fp64_flops_per_launch"],
                           "peak_source": "FP64 FMA rate measured by bsc_measure_peaks on this GPU (2 flops per FMA)"},
                  "limiter": KERNEL_LIMITER.get(top["kernel"])}
        if top["bound"] == "fp64":
            roofline = {"bound": "fp64", "achieved": top["achieved_gflops"], "peak": top["peak_gflops"],
                        "unit": "GFLOP/s", "frac": top["frac"], **common}
        else:
            roofline = {"bound": "hbm", "achieved": top["achieved_gbs"], "peak": hbm, "unit": "GB/s",
                        "frac": top["hbm_frac"], "algorithmic_bytes_per_launch": top["algorithmic_bytes_per_launch"],
                        "peak_source": f"{peak_kind} MEASURED_PEAKS.json hbm_gbs", **common}
    else:
        roofline = spmv_roof
    fp64 = None
    if "fp64" in res:
        f = res["fp64"]
        b64 = spmv_mg_bytes(f["nnz"], f["n"], fp32=False) if mg else spmv_bytes(f["nnz"], f["n"], fp32=False)
        a64 = b64 / (f["spmv_ms"] * 1e-3) / 1e9 if f["spmv_ms"] > 0 else None
        t64 = traffic_per_row("spmv_z_fp64" if mg else "fp64")
        fp64 = {"value": f["value"], "ms_per_step": f["ms_per_step"], "ppe_iterations": [i[0] for i in f["iters"]],
                "solve_ms_per_step": f["solve_ms"], "kernels": f["kernels"],
                "roofline_spmv": {"bound": "hbm",
                                  "kernel": "k_spmv_z<double>" if mg else "k_bicg_1<EllOp<double>,double>",
                                  "achieved": a64,
                                  "peak": hbm, "unit": "GB/s", "frac": (a64 / hbm) if a64 else None,
                                  "traffic": (t64 * f["n"]) if t64 else None}}
    wc = None if args.no_wcsph else run_wcsph()
    sal = None if args.no_salinity else run_salinity(args)
    rtank = None if args.no_reference_tank else run_reference_tank(args, threads)
    cpu = None
    if not args.no_cpu:
        v, desc, _ = cpu_steps(scen, spec, threads, args.cpu_steps, 1)
        cpu = {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": "port", "sample": desc}
    solver_desc = f"FGMRES({args.restart}) + cell-multigrid V-cycle" if mg else args.solver
    line = {
        "metric": METRIC, "value": m["value"], "unit": "particle-steps/s", "n_gpus": dist.world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": m["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32/f64 (mixed)",
        "data": "synthetic (seeded wave tank, no dataset)",
        "config": {"workload": f"{args.config} wave tank 4.0x0.6 m, depth 0.30 m, dx={spec.dx} m, "
                               f"{scen.n_fluid} fluid + {scen.n - scen.n_fluid} wall particles, Wendland C2 h=1.3dx, "
                               f"piston from t=0, {solver_desc} PPE to rel-res 1e-8, dt={spec.dt} s",
                   "fluid_particles": scen.n_fluid, "precond": args.precond,
                   "precision": ("mixed (FP32 pair sums and V-cycle, FP64 assembly and FGMRES)" if mg
                                 else "mixed (FP32 sweeps, FP64 refinement)"),
                   "l2": "inputs larger than L2 (particle state ~170 MB + neighbour lists ~0.9 GB)",
                   "parallelism": f"replicas x{dist.world}"},
        "ppe": {"iterations": [i[0] for i in m["iters"]], "refinement_sweeps": [i[1] for i in m["iters"]],
                "rel_residual": [i[2] for i in m["iters"]]},
        "fp64": fp64,
        "mixed_over_fp64_speed": (fp64["ms_per_step"] / m["ms_per_step"]) if fp64 else None,
        "mixed_vs_fp64_rel_l2": errs,
        "roofline": roofline,
        "roofline_spmv": spmv_roof,
        "kernels": m["kernels"],
        "cpu_baseline": cpu,
        "e2e": m.get("e2e"),
        "clocks": m["clocks"],
        "gpu_launches": m["launches"],
        "measured_peaks": {"fp64_gflops": peaks[0], "fp32_gflops": peaks[1], "copy_gbs": peaks[2]} if peaks else None,
        "fp64_bound_kernels": fp64_bound_kernels(),
        "wcsph_adjoint_forward_ratio": wc["ratio"] if wc else None,
        "wcsph": wc,
        "salinity": sal,
        "reference_tank": rtank,
    }
    print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
