/*
 * bsc.h -- C ABI of the GB300 ISPH step for the porous-beach solver
 * (Sinchanrc/Beach_Slope_Confined).
 *
 * The reference drives one ISPH step from its Fortran main program by calling
 * argument-less module subroutines in a fixed order (main.f90:44-65).  Those
 * routines communicate only through module globals (initialize.f90:19-79) and
 * the cell structure dpcell (domain.f90:28-46).  This header replaces each of
 * them with one entry point that takes an opaque context.  The context owns
 * all particle state, resident in GPU memory across steps, and one CUDA
 * stream.  Host buffers passed in are caller-owned and copied.
 *
 * Conventions
 *  - Every call returns BSC_OK (0) or a negative BSC_E_* code; the message of
 *    the last failure is available from bsc_last_error().  No exception ever
 *    crosses the ABI.
 *  - A context is single-host-thread: call it from one thread at a time.  In
 *    the reference the step routines run inside an OpenMP parallel region;
 *    the Fortran binding calls them from the master thread only.
 *  - Particle ids are the 0-based positions in the arrays given to
 *    bsc_upload_state().  Every array read back (download, neighbour sets,
 *    CSR export) is in that id order, whatever order the context keeps the
 *    particles in internally (it keeps them sorted by cell).
 *  - All indices crossing the ABI are 0-based.
 */
#ifndef BSC_H
#define BSC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define BSC_OK                0
#define BSC_E_INVALID        -1  /* bad argument or call order            */
#define BSC_E_CUDA           -2  /* CUDA runtime error                    */
#define BSC_E_NOMEM          -3  /* device or host allocation failed      */
#define BSC_E_CAPACITY       -4  /* neighbour list or cell capacity hit   */
#define BSC_E_NOT_CONVERGED  -5  /* Krylov solver hit maxit               */
#define BSC_E_BREAKDOWN      -6  /* Krylov breakdown (zero denominator)   */
#define BSC_E_NONFINITE      -7  /* NaN/Inf detected in the state         */
#define BSC_E_NOT_BUILT      -8  /* the CUDA library is missing/unusable  */

/* ---- enumerations ------------------------------------------------------- */
/* smoothing kernel: kernel.f90:34-162 (hybrid, live) and the Wendland C2
 * form kept as comments at kernel.f90:42-43,102-103 */
enum { BSC_KERNEL_HYBRID = 0, BSC_KERNEL_WENDLAND_C2 = 1 };
/* arithmetic of the step: plain FP64, or FP32 pair sums / SpMV / inner
 * Krylov with FP64 outer iterative refinement of the PPE */
enum { BSC_PREC_FP64 = 0, BSC_PREC_MIXED = 1 };
/* PPE solver: solver.f90:129-254 (BiCGSTAB) and :306-347 (FGMRES) */
enum { BSC_SOLVER_BICGSTAB = 0, BSC_SOLVER_FGMRES = 1 };
/* stopping test: ||r|| <= tol*||b|| (relative residual), or
 * ||r|| <= tol*||r0|| (the MKL dfgmres test used by solver.f90:321-324) */
enum { BSC_TOL_REL_B = 0, BSC_TOL_REL_R0 = 1 };
/* PPE preconditioner: none (the reference's solvers), or a V-cycle of
 * multigrid over the neighbour cells used by flexible GMRES(restart); the
 * V-cycle runs in FP64 on the FP64 path and in FP32 on the mixed path. */
enum { BSC_PRECOND_NONE = 0, BSC_PRECOND_MG = 1 };
/* time step: fixed dt, or the CFL/viscous rule of integrator.f90:908-976 */
enum { BSC_DT_FIXED = 0, BSC_DT_ADAPTIVE = 1 };

/* particle type ids, particle.f90:31-47 (tid) */
enum { BSC_TID_WALL = 1, BSC_TID_GHOST = 2, BSC_TID_FLUID = 3 };

/* particle flag bits (the logicals of particle.f90:40-41) */
#define BSC_FLAG_FREE      0x01u  /* free-surface particle              */
#define BSC_FLAG_VICINITY  0x02u  /* neighbour of a free-surface one    */
#define BSC_FLAG_BUFFER    0x04u  /* open-boundary buffer particle      */
#define BSC_FLAG_DEAD      0x08u  /* frozen ("dead") fluid particle     */
#define BSC_FLAG_PISTON    0x10u  /* wall particle moved by the piston  */

#define BSC_MAX_PISTON_MODES 8

/* ---- parameters (initialize.f90:19-56 and setup.f90:47-82) --------------- */
typedef struct bsc_params {
    int32_t kernel;              /* BSC_KERNEL_*                                   */
    int32_t precision;           /* BSC_PREC_*                                     */
    double  h;                   /* smoothing length h1; support radius is 2h      */
    double  dl;                  /* particle spacing dl (setup.f90:53)             */
    double  lam;                 /* lam = 0.001 h^2 (setup.f90:82)                 */
    double  rho0;                /* rho                                            */
    double  rel_den;             /* rel_den (seawater relative density)            */
    double  g;                   /* gravity, negative                              */
    double  mu;                  /* mu, used by the time-step rule                 */
    double  csh;                 /* shifting coefficient (times h^2)               */
    double  maxshift;            /* shift clamp, fraction of dl                    */
    double  free_threshold;      /* lamfs*maxdivr: free if tr(M) <= this           */
    double  por;                 /* porosity of the solid matrix (scalar/default)  */
    double  darcy_alpha;         /* Darcy coefficient (lamk in porous.f90:111)     */
    double  forch_beta;          /* Forchheimer coefficient (1.75 sqrt(lamk/150))  */
    double  d50;                 /* grain diameter                                 */
    double  eddy_cs;             /* Smagorinsky constant cs                        */
    double  eddy_cv;             /* cv                                             */
    double  eddy_ce;             /* ce                                             */
    double  varts_ps;            /* ps, free-surface artificial viscosity factor   */
    double  buffer_release_xmin; /* comp_pos buffer release window                 */
    double  buffer_release_xmax;
    int32_t dt_mode;             /* BSC_DT_*                                       */
    int32_t solver;              /* BSC_SOLVER_*                                   */
    double  dt;                  /* (initial) time step                            */
    double  sig1;                /* CFL factor                                     */
    double  tschmidt;            /* turbulent Schmidt number (scalar sub-steps)    */
    double  diffusivity;         /* molecular diffusivity Dm (scalar sub-steps)    */
    int32_t restart;             /* FGMRES restart length m                        */
    int32_t maxit;               /* max Krylov iterations per solve                */
    int32_t tol_mode;            /* BSC_TOL_*                                      */
    int32_t max_outer;           /* mixed: max FP64 refinement sweeps              */
    double  tol;                 /* PPE tolerance                                  */
    double  inner_tol;           /* mixed: FP32 inner solve relative tolerance     */
    int32_t max_neighbors;       /* neighbour-list capacity per particle           */
    int32_t reorder_every;       /* Morton reorder of the state every n cellshifts */
    int32_t piston_modes;        /* stroke s(t) = sum a_k sin(2 pi t/T_k + phi_k)  */
    int32_t precond;             /* BSC_PRECOND_* for the PPE solve                */
    double  piston_amp[BSC_MAX_PISTON_MODES];
    double  piston_period[BSC_MAX_PISTON_MODES];
    double  piston_phase[BSC_MAX_PISTON_MODES];
    double  piston_ramp;         /* x_p = s0 + r (s - s0), s0 = x_p(0), with       */
                                 /* r = (1-cos(pi t/ramp))/2 for t < ramp, else 1  */
    double  xmin, xmax, ymin, ymax; /* cell-grid bounds; all 0 = derive at upload */
    /* cell-aggregation multigrid (BSC_PRECOND_MG) */
    double  mg_omega;            /* smoother weight; with 2 sweeps the 2nd uses    *
                                  * 2.094x it (Chebyshev nodes of [a, 3a])         */
    double  mg_scale;            /* scaling of the coarse-grid correction          */
    int32_t mg_sweeps;           /* pre- and post-smoothing sweeps per level       */
    int32_t mg_coarse_max;       /* cells of the coarsest level (dense solve)      */
    /* salinity transport (scalar.f90:114-305) */
    double  disp_long, disp_trans;   /* dispersivities al, at (scalar.f90:118)     */
    double  buffer_con;          /* concentration held on inflow buffers ...       */
    double  buffer_con_xmax;     /* ... left of this x (scalar.f90:260-264)        */
    int32_t salinity;            /* 1: bsc_step runs the phase-3 step of           *
                                  * main.f90:198-260 with salinity sub-steps       */
    int32_t outflow;             /* 1: bsc_step drops fluid, non-buffer particles  *
                                  * with x <= outflow_xcut and y > outflow_ycut at  *
                                  * its second cell shift (cellshiftalt,           *
                                  * integrator.f90:55-110)                         */
    double  outflow_xcut, outflow_ycut;  /* xlcutoff, ytcutoff (setup.f90:77-78)   */
} bsc_params;

/* Host-side particle state, structure of arrays, n entries each, id order.
 * On upload, x..mass, tid and flags are required; NULL optional fields are
 * initialised as the reference does (porosity 1, L = identity, others 0).
 * On download every non-NULL pointer is filled. */
typedef struct bsc_state_view {
    int64_t  n;
    double  *x, *y, *vx, *vy;
    double  *xs, *ys, *vxs, *vys;
    double  *p, *rho, *oden, *mass;
    double  *porosity, *gradvx, *nut, *tke;
    double  *resist, *varts, *vel;
    double  *L;                  /* 4 per particle: coff(1..4), row-major 2x2    */
    double  *xrest;              /* piston particles: x at zero stroke           */
    int8_t  *tid;
    uint8_t *flags;
    double  *con;                /* salinity concentration (plist%con)            */
    double  *ovol;               /* original volume (plist%ovol); NULL on upload: *
                                  * mass / oden                                   */
} bsc_state_view;

typedef struct bsc_solve_info {
    int32_t iterations;          /* total inner Krylov iterations               */
    int32_t outer;               /* FP64 refinement sweeps (mixed), else 1      */
    int32_t converged;           /* 1 if the stopping test was met              */
    int32_t status;              /* BSC_OK / BSC_E_NOT_CONVERGED / _BREAKDOWN   */
    double  rel_residual;        /* final ||b-Ax|| / ||b|| (true residual)      */
    double  r0_norm;             /* ||b - A x0||                                */
    double  b_norm;              /* ||b||                                       */
} bsc_solve_info;

#define BSC_TIMING_SLOTS 32
typedef struct bsc_timing {
    /* cumulative device milliseconds per stage since the last reset, measured
     * with CUDA events on the context stream */
    double  ms[BSC_TIMING_SLOTS];
    int64_t calls[BSC_TIMING_SLOTS];
    int64_t kernel_launches;     /* kernels launched by the library since reset */
} bsc_timing;

/* stage slots of bsc_timing */
enum {
    BSC_T_PROJECTION = 0, BSC_T_CELLSHIFT, BSC_T_REORDER, BSC_T_NEIGHBOUR,
    BSC_T_EFFPOR, BSC_T_EDDYVIS, BSC_T_INT_VEL, BSC_T_PPE_ASSEMBLE,
    BSC_T_PPE_SOLVE, BSC_T_COMP_VEL, BSC_T_COMP_POS, BSC_T_FREESURF,
    BSC_T_SHIFT, BSC_T_TIMESTEP, BSC_T_PISTON, BSC_T_STEP,
    BSC_T_SPMV, BSC_T_UPLOAD, BSC_T_DOWNLOAD,
    /* with the BSC_PROFILE_ITER=1 environment variable: the five kernels of
     * one BiCGSTAB iteration per batch; with the multigrid preconditioner,
     * the phases of every FGMRES iteration instead: fine-level pre-smoothing
     * and restriction, coarse levels, fine-level post-smoothing, the SpMV,
     * and the orthogonalisation */
    BSC_T_BICG_1, BSC_T_BICG_2, BSC_T_BICG_3, BSC_T_BICG_4, BSC_T_BICG_5,
    /* salinity transport: scalart, scalarupdate and densityupdate */
    BSC_T_SCALAR,
    /* single kernels inside their stages, for the FP64-pipe rooflines: the
     * neighbour search, the PPE assembly, the int_vel pair sum, the porosity
     * sum and the shift's pair sum */
    BSC_T_K_NEIGHBOUR, BSC_T_K_ASSEMBLE, BSC_T_K_INT_VEL, BSC_T_K_EFFPOR, BSC_T_K_SHIFT
};

typedef struct bsc_ctx bsc_ctx;

/* ---- lifecycle ---------------------------------------------------------- */
/* Fill *p with the reference's constants (initialize.f90:19-56) for a
 * particle spacing dl; h follows setup.f90:47 with the hybrid kernel. */
int bsc_default_params(bsc_params* p, double dl);
/* Create a context on the current CUDA device (init, setup.f90:10). */
int bsc_create(const bsc_params* p, bsc_ctx** out);
int bsc_destroy(bsc_ctx* ctx);
const char* bsc_last_error(const bsc_ctx* ctx);
/* Copy particle state in (gen_fluid/gen_boundary output, memalloc and
 * matrixid, memory.f90:10-147).  Sizes the PPE at n rows (finmax). */
int bsc_upload_state(bsc_ctx* ctx, const bsc_state_view* host);
/* Porous solid particles (tid 4, the porlist of domain.f90:32);
 * por may be NULL (scalar params.por). */
int bsc_upload_solids(bsc_ctx* ctx, int64_t ns, const double* x, const double* y,
                      const double* mass, const double* rho, const double* por);
/* Per-cell porosity field: nx*ny values, row-major in y then x, cell (ix,iy)
 * covers [x0+ix*dx, x0+(ix+1)*dx) x [y0+iy*dy, ...).  Outside: params.por.
 * Used as the cap of the solid fraction (porous.f90:182-186).  Call before
 * bsc_upload_solids when solid porosities are to come from the field. */
int bsc_upload_porosity(bsc_ctx* ctx, int32_t nx, int32_t ny, double x0, double y0,
                        double dx, double dy, const double* values);
/* Copy the state back in id order (output.f90 writers / checkpoint). */
int bsc_download_state(bsc_ctx* ctx, bsc_state_view* host);
int bsc_set_time(bsc_ctx* ctx, double t, double dt);
int bsc_get_time(const bsc_ctx* ctx, double* t, double* dt);

/* ---- one entry per reference module routine (main.f90:46-64) ------------ */
int bsc_projection(bsc_ctx* ctx);                 /* isph.f90:16-47          */
int bsc_cellshift(bsc_ctx* ctx, int32_t alt);     /* integrator.f90:32-391   */
int bsc_resetid(bsc_ctx* ctx);                    /* isph.f90:88-113         */
int bsc_neighbour(bsc_ctx* ctx);                  /* search.f90:13-399       */
int bsc_freesurf(bsc_ctx* ctx);                   /* isph.f90:49-86          */
int bsc_effpor(bsc_ctx* ctx);                     /* porous.f90:107-224      */
int bsc_eddyvis(bsc_ctx* ctx);                    /* turbulence.f90:12-110   */
int bsc_int_vel(bsc_ctx* ctx);                    /* integrator.f90:458-713  */
int bsc_ppesolve(bsc_ctx* ctx, bsc_solve_info* out); /* isph.f90:115-485     */
int bsc_comp_vel(bsc_ctx* ctx);                   /* integrator.f90:715-865  */
int bsc_comp_pos(bsc_ctx* ctx);                   /* integrator.f90:867-906  */
int bsc_opt2_shift(bsc_ctx* ctx);                 /* part_shift.f90:12-192   */
int bsc_timestep(bsc_ctx* ctx, double* dt_inout); /* integrator.f90:908-976  */
/* Move the piston wall particles to x_p(t) at the context time (greenfield:
 * the reference has no wavemaker). */
int bsc_piston(bsc_ctx* ctx);
/* Salinity transport (scalar.f90; needs params.salinity = 1, which makes the
 * neighbour search keep each pair's distance for scalart). */
int bsc_scalart(bsc_ctx* ctx);                    /* scalar.f90:114-240      */
int bsc_scalarupdate(bsc_ctx* ctx, double stime); /* scalar.f90:242-275      */
int bsc_densityupdate(bsc_ctx* ctx);              /* scalar.f90:277-305      */
/* The whole main.f90:41-65 sequence, nsteps times (t += dt first).  With
 * params.salinity = 1, the phase-3 sequence of main.f90:198-260 instead:
 * solsteps x (scalart, scalarupdate(dtsol)) first, densityupdate after
 * opt2_shift, eddyvis after timestep (the open-boundary buffers of that
 * loop are not part of this library). */
int bsc_step(bsc_ctx* ctx, int32_t nsteps, bsc_solve_info* last);

/* ---- particles leaving and entering (internal.f90:475-614) -------------- */
enum {
    BSC_REMOVE_BUFFER_RIGHT = 1,  /* remove_buffer1: buffer particles with x >= a */
    BSC_REMOVE_BUFFER_LEFT = 2,   /* remove_buffer2: buffer particles with x <= a */
    BSC_REMOVE_OUTFLOW = 3        /* cellshiftalt (integrator.f90:55-110): fluid,
                                   * not buffer, x <= a (xlcutoff), y > b (ytcutoff) */
};
/* Remove the particles a rule selects, compacting the state on the device;
 * the survivors keep their order and are renumbered 0..n'-1 in it (a
 * download returns the host arrays minus the removed particles).  *removed
 * (optional) receives the count.  Neighbour lists are empty until the next
 * bsc_neighbour. */
int bsc_remove_particles(bsc_ctx* ctx, int32_t rule, double a, double b, int64_t* removed);
/* Append particles (insert_buffer1/2: the host picks the template particles
 * and sets tid, mass, density, oden, ovol, con and the buffer flag); they
 * take the ids after the last.  Fields left NULL default as in
 * bsc_upload_state. */
int bsc_insert_particles(bsc_ctx* ctx, const bsc_state_view* add);
/* The current particle count (it changes with removals, insertions and the
 * outflow cut-off of bsc_step). */
int bsc_particle_count(const bsc_ctx* ctx, int64_t* n);

/* ---- text snapshots (output.f90:188-234 `combined`) --------------------- */
/* Queue a snapshot of the current state: <dir>/fluid/fluid_<index>.txt,
 * <dir>/buffer/buffer_<index>.txt and <dir>/fluid/dead_<index>.txt, one line
 * per fluid particle in id order, x y p (F10.3) vx vy (ES10.3) con+0.5
 * (F10.5).  Returns once the device-side gather and copy are queued; a host
 * thread formats and writes the files while later calls run.  A second call
 * waits for the first. */
int bsc_snapshot_begin(bsc_ctx* ctx, const char* dir, int64_t index);
/* Wait for the queued snapshot; returns its write error, if any. */
int bsc_snapshot_wait(bsc_ctx* ctx);

/* ---- parity and diagnostics hooks --------------------------------------- */
/* Neighbour sets of the last bsc_neighbour call: offsets[n+1], ids sorted
 * ascending per particle.  ids may be NULL to query offsets[n] first. */
int bsc_get_neighbors(bsc_ctx* ctx, int64_t* offsets, int32_t* ids);
/* PPE of the last bsc_ppesolve (after Jacobi scaling) in id space, rows
 * column-sorted with the diagonal included: rowptr[n+1], col, val, rhs[n].
 * col/val may be NULL to query rowptr[n] first. */
int bsc_export_csr(bsc_ctx* ctx, int64_t* rowptr, int32_t* col, double* val, double* rhs);
/* Free-surface elevation at probe abscissae: eta = sum_i V_i w1(x_i - xp)
 * - depth over fluid particles, w1 the 1-D Wendland C2 kernel of radius 2h. */
int bsc_probe_eta(bsc_ctx* ctx, int32_t nprobe, const double* xprobe, double depth,
                  double* eta);
int bsc_get_timings(bsc_ctx* ctx, bsc_timing* out);
int bsc_reset_timings(bsc_ctx* ctx);
/* Block until all work queued on the context stream has finished. */
int bsc_synchronize(bsc_ctx* ctx);

/* ---- standalone sparse solve (solver.f90:129 bicgstab(tls,guess,ls,val,row,
 * col,bvecs,sl) / :306 fgmres) ------------------------------------------- */
/* Solve A x = b for a host CSR matrix (0-based rowptr[n+1], col, val) with
 * the solver/tolerance fields of *p; x holds the initial guess on entry.
 * Allocates and frees its own device buffers. */
int bsc_csr_solve(const bsc_params* p, int32_t n, const int32_t* rowptr,
                  const int32_t* col, const double* val, const double* b,
                  double* x, bsc_solve_info* info);

/* The same BiCGSTAB solve for callers that may not allocate device memory:
 * a program whose own pool or caching allocator holds the GPU's memory, where
 * a library's cudaMalloc could fail and its cudaFree would stall the device.
 * No counterpart in the reference: it exists for such hosts only.
 *  - rowptr, col, val, b, x are DEVICE pointers owned by the caller, all on
 *    the current device (or managed memory); x holds the initial guess on
 *    entry and the solution on return.  Work is queued on `stream` (NULL: the
 *    legacy default stream) and the call returns once it has finished.
 *  - Nothing is allocated: the work vectors live in a fixed device array of
 *    the library sized for n <= BSC_NOALLOC_MAX_ROWS rows (about 6.3 MB).
 *    Larger n returns BSC_E_CAPACITY; host pointers, pointers into another
 *    device's memory, a solver other than BSC_SOLVER_BICGSTAB, or n <= 0
 *    return BSC_E_INVALID.
 *  - Under CUDA's default lazy module loading the array's memory is
 *    committed by the first call on each device: make that call before the
 *    host reserves its pool (or set CUDA_MODULE_LOADING=EAGER, which commits
 *    it when the library's device code loads), and before any stream capture
 *    begins.  Each call looks up the array's address on the current device.
 *  - All calls share the array, and one process-wide host copy of the solver
 *    scalars: calls whose work overlaps on the GPU (other streams, other host
 *    threads) race and must be serialised by the caller. */
#define BSC_NOALLOC_MAX_ROWS 131072
int bsc_csr_solve_noalloc(const bsc_params* p, int32_t n, const int32_t* rowptr,
                          const int32_t* col, const double* val, const double* b,
                          double* x, void* stream, bsc_solve_info* info);

/* ---- differentiable WCSPH step and its adjoint ------------------------------ */
/* A weakly compressible step on the uploaded state (fluid, walls, piston and
 * porous solids of the ISPH context; FP64 context, Wendland C2 kernel):
 * Tait EOS clamped at zero pressure (dentopress, wcsph.f90:35-63),
 * continuity with delta-SPH diffusion and the hydrostatic correction
 * (calmasscons and updateden, wcsph.f90:65-154), symmetric pressure gradient,
 * Morris viscosity, gravity, implicit Darcy-Forchheimer drag (the Ergun form
 * of porous.f90:192-212) and the position update.  The reference's module
 * holds only those formulae and is not part of its build; these entry points
 * replace a WCSPH step loop built on them.  The calibrated parameters are the
 * drag coefficients and the porosity of a grid of cells over the slope (each
 * solid takes the porosity of the cell it lies in; solids outside the grid
 * keep por).  Grid cells must be at least 2h on a side, so that one kernel
 * support overlaps at most nine of them.  The adjoint returns the gradient of
 * any loss of the probe elevations, with the neighbour lists of every step
 * frozen, recomputing each segment of ckpt_every steps from a checkpoint; a
 * segment keeps about 4.5 kmax + 30 doubles per particle per step in device
 * memory. */
#define BSC_WCSPH_MAX_GRID 256
#define BSC_WCSPH_MAX_PROBES 16
typedef struct bsc_wcsph_params {
    double  c0;                  /* sound speed of the Tait EOS                    */
    double  gamma;               /* Tait exponent                                  */
    double  delta;               /* delta-SPH density-diffusion coefficient        */
    double  surface_y;           /* still-water level (hydrostatic density)        */
    double  nu;                  /* kinematic viscosity                            */
    double  alpha, beta;         /* Darcy and Forchheimer drag coefficients        */
    double  grid_x0, grid_y0, grid_dx, grid_dy;  /* porosity grid                  */
    int32_t grid_nx, grid_ny;    /* grid_nx * grid_ny <= BSC_WCSPH_MAX_GRID        */
    const double* grid_por;      /* porosities, index iy * grid_nx + ix            */
    int32_t nprobe;              /* <= BSC_WCSPH_MAX_PROBES                        */
    double  probe_x[BSC_WCSPH_MAX_PROBES];
    double  probe_depth;         /* eta = sum_i V_i w1(x_i - x_p) - probe_depth    */
} bsc_wcsph_params;
/* Takes the current state as the initial state of every later forward run
 * (densities set hydrostatic from surface_y) and sets the parameters. */
int bsc_wcsph_setup(bsc_ctx* ctx, const bsc_wcsph_params* w);
/* New values of the calibrated parameters (grid_por: grid_nx*grid_ny). */
int bsc_wcsph_set_params(bsc_ctx* ctx, double alpha, double beta, const double* grid_por);
/* nsteps steps from the initial state, a checkpoint every ckpt_every steps;
 * eta[nsteps * nprobe] receives the probe elevations after each step. */
int bsc_wcsph_forward(bsc_ctx* ctx, int32_t nsteps, int32_t ckpt_every, double* eta);
/* Reverse pass through the last forward run: given dJ/deta[nsteps * nprobe],
 * grad[0] = dJ/dalpha, grad[1] = dJ/dbeta, grad[2 + k] = dJ/dpor_k. */
int bsc_wcsph_adjoint(bsc_ctx* ctx, const double* dJ_deta, double* grad);

/* ---- hardware probes ---------------------------------------------------- */
/* Measured FP64 and FP32 FMA throughput (GFLOP/s, 2 flops per FMA) and a
 * device-to-device copy bandwidth (GB/s, read+write) on the current device. */
int bsc_measure_peaks(double* fp64_gflops, double* fp32_gflops, double* copy_gbs);
/* Self-test of the device arithmetic the mixed path uses in place of FP64
 * instructions, over n hashed inputs (|x| in 2^[-100,101]): the integer-pipe
 * FP64->FP32 rounding against the hardware conversion (inputs that differ,
 * largest difference in FP32 ulps) and the Newton-Raphson reciprocal (largest
 * |x r(x) - 1|). */
int bsc_selftest(int64_t n, int64_t* f32_mismatches, int64_t* f32_max_ulp, double* rcp_max_rel,
                 double* sqrt_max_rel);

#ifdef __cplusplus
}
#endif
#endif /* BSC_H */
