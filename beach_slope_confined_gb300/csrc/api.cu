// api.cu -- the extern "C" entry points of include/bsc.h.
//
// Each entry point replaces one argument-less module routine of the reference
// (main.f90:46-64).  The context owns every device buffer; all of them are
// sized at the first bsc_upload_state (memalloc/matrixid, memory.f90:10-147)
// and reused by later uploads of the same particle count, so a step never
// allocates.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <numeric>
#include <vector>

#include "bsc_internal.cuh"

struct bsc_ctx : bsc::Ctx {};

namespace bsc {

int set_err(Ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

int cuda_err(Ctx* c, cudaError_t e, const char* where) {
    char buf[256];
    std::snprintf(buf, sizeof buf, "%s: %s (%s)", where, cudaGetErrorName(e), cudaGetErrorString(e));
    return set_err(c, e == cudaErrorMemoryAllocation ? BSC_E_NOMEM : BSC_E_CUDA, buf);
}

void timing_flush(Ctx* c) {
    if (c->ev_used == 0) return;
    cudaEventSynchronize(c->evs[2 * (c->ev_used - 1) + 1]);
    for (int k = 0; k < c->ev_used; ++k) {
        float f = 0.f;
        if (cudaEventElapsedTime(&f, c->evs[2 * k], c->evs[2 * k + 1]) == cudaSuccess) {
            c->ms[c->ev_slot[k]] += f;
            c->calls[c->ev_slot[k]]++;
        }
    }
    c->ev_used = 0;
}

static void derive_kparams(Ctx* c) {
    const bsc_params& P = c->P;
    KParams& K = c->K;
    const double h = P.h;
    K.kernel = P.kernel;
    K.h = h;
    K.H = 2 * h;
    K.H2 = K.H * K.H;
    // the neighbour test sqrt((xi-xj)^2+(yi-yj)^2) < 2h (search.f90:59) as a
    // test on d2: the correctly rounded square root is monotone, so the test
    // holds exactly for d2 below the smallest double whose root reaches 2h
    double t = K.H2;
    while (t > 0.0 && std::sqrt(t) >= K.H) t = std::nextafter(t, 0.0);
    while (std::sqrt(t) < K.H) t = std::nextafter(t, INFINITY);
    K.H2x = t;
    K.lam = P.lam;
    K.dl = P.dl;
    K.rho0 = P.rho0;
    K.rel_den = P.rel_den;
    K.g = P.g;
    K.csh = P.csh;
    K.maxshift = P.maxshift;
    K.free_thr = P.free_threshold;
    K.por = P.por;
    K.alpha = P.darcy_alpha;
    K.beta = P.forch_beta;
    K.d50 = P.d50;
    K.eddy_cs = P.eddy_cs;
    K.eddy_cv = P.eddy_cv;
    K.eddy_ce = P.eddy_ce;
    K.varts_ps = P.varts_ps;
    K.bxmin = P.buffer_release_xmin;
    K.bxmax = P.buffer_release_xmax;
    // kernel.f90:52-53: 10/(28*3.14 h^2) and 1/(3*3.14 h^2), 28.0*3.14 and
    // 3.0*3.14 evaluated in single precision as the reference does
    K.hyb_A = 0.1 * (10.0 / ((double)(28.0f * 3.14f) * (h * h)));
    K.hyb_B = (1.0 - 0.1) * (1.0 / ((double)(3.0f * 3.14f) * (h * h)));
    K.wend_F = 35.0 / (4.0 * 3.140 * ((h * h) * (h * h)));
    K.wend_W = 7.0 / (4 * 3.140 * (h * h));
    K.w0 = (P.kernel == BSC_KERNEL_WENDLAND_C2) ? K.wend_W : 4.0 * K.hyb_A + 6.0 * K.hyb_B;
    K.inv_w0 = 1.0 / K.w0;
    K.inv_h = 1.0 / h;
    K.half_inv_h = 0.5 * K.inv_h;
    K.hyb_n1 = (9.0 * K.hyb_A + 3.0 * K.hyb_B) / (h * h * h);  // r < h: n1 r - n0 - n2/(r h)
    K.hyb_n0 = 12.0 * K.hyb_A / (h * h);
    K.hyb_n2 = 6.0 * K.hyb_B;
    K.hyb_f = 3.0 * (K.hyb_A + K.hyb_B);                        // r >= h: -f (2-q)^2/(r h)
    K.kmax = P.max_neighbors;
}

static uint64_t spread_bits(uint32_t v) {
    uint64_t x = v;
    x = (x | (x << 16)) & 0x0000FFFF0000FFFFull;
    x = (x | (x << 8)) & 0x00FF00FF00FF00FFull;
    x = (x | (x << 4)) & 0x0F0F0F0F0F0F0F0Full;
    x = (x | (x << 2)) & 0x3333333333333333ull;
    x = (x | (x << 1)) & 0x5555555555555555ull;
    return x;
}

static void free_all(Ctx* c) {
    if (c->stream) cudaStreamSynchronize(c->stream);
    wc_free(c);
    snap_free(c);
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
    for (void* p : c->allocs) cudaFree(p);
    c->allocs.clear();
    mg_free(c);
    if (c->h_sc) cudaFreeHost(c->h_sc);
    if (c->h_flag) cudaFreeHost(c->h_flag);
    c->h_sc = nullptr;
    c->h_it = nullptr;
    c->h_flag = nullptr;
    c->cap = 0;
}

static int alloc_state(Ctx* c, State& S, int64_t n) {
    double** f[N_DBL_FIELDS] = {&S.x, &S.y, &S.vx, &S.vy, &S.xs, &S.ys, &S.vxs, &S.vys, &S.p, &S.rho, &S.oden,
                                &S.mass, &S.por, &S.gradvx, &S.nut, &S.tke, &S.resist, &S.varts, &S.vel, &S.xrest,
                                &S.vol, &S.L0, &S.L1, &S.L2, &S.L3, &S.con, &S.ovol, &S.cdiff};
    for (int k = 0; k < N_DBL_FIELDS; ++k)
        if (int rc = dalloc(c, f[k], n)) return rc;
    if (int rc = dalloc(c, &S.tid, n)) return rc;
    if (int rc = dalloc(c, &S.flags, n)) return rc;
    return dalloc(c, &S.id, n);
}

// Krylov and reduction work shared by the PPE and the standalone solve
static int alloc_solver_work(Ctx* c, int64_t n, bool fp64, bool fp32) {
    const int m = c->P.solver == BSC_SOLVER_FGMRES ? std::max(1, std::min(c->P.restart, 64)) : 1;
    c->fg_m = m;
    int rc;
    if ((rc = dalloc(c, &c->r, 6 * n))) return rc;  // r rh pd v s tv contiguous (csr_solve relies on it)
    c->rh = c->r + n; c->pd = c->r + 2 * n; c->v = c->r + 3 * n; c->s = c->r + 4 * n; c->tv = c->r + 5 * n;
    if (c->P.solver == BSC_SOLVER_FGMRES && fp64)
        if ((rc = dalloc(c, &c->V, (int64_t)(m + 1) * n))) return rc;
    if (fp32) {
        // FGMRES-IR: FP64 outer basis V, FP32 preconditioned vectors Z, and
        // the FP32 BiCGSTAB sweep vectors
        c->ir_m = std::max(1, std::min(c->P.max_outer, 40));
        if ((rc = dalloc(c, &c->V, (int64_t)(c->ir_m + 1) * n))) return rc;
        if ((rc = dalloc(c, &c->Zf, (int64_t)c->ir_m * n))) return rc;
        if ((rc = dalloc(c, &c->xf, 9 * n))) return rc;
        c->rf = c->xf + n; c->sf = c->xf + 2 * n; c->rhf = c->xf + 3 * n; c->pf = c->xf + 4 * n;
        c->vf = c->xf + 5 * n; c->tf = c->xf + 6 * n; c->bf = c->xf + 7 * n; c->xbf = c->xf + 8 * n;
    }
    if ((rc = dalloc(c, &c->Hd, fg_layout_size(64)))) return rc;
    if ((rc = dalloc(c, &c->part, (int64_t)RED_GRID * 64))) return rc;
    if ((rc = dalloc(c, &c->sc, 1)) || (rc = dalloc(c, &c->sc2, 1))) return rc;
    if ((rc = dalloc(c, &c->ticket, 1))) return rc;
    BSC_CUDA(c, cudaMemsetAsync(c->ticket, 0, sizeof(unsigned), c->stream));
    if (!c->h_sc) BSC_CUDA(c, cudaMallocHost((void**)&c->h_sc, 4 * sizeof(Scalars)));
    std::memset(c->h_sc, 0, 4 * sizeof(Scalars));
    c->h_it = c->h_sc + 2;
    return BSC_OK;
}

static int alloc_for(Ctx* c, int64_t n) {
    free_all(c);
    int rc;
    if ((rc = alloc_state(c, c->S, n)) || (rc = alloc_state(c, c->S2, n))) return rc;
    if ((rc = dalloc(c, &c->pcell, n)) || (rc = dalloc(c, &c->pslot, n)) || (rc = dalloc(c, &c->sorted, n))) return rc;
    if ((rc = dalloc(c, &c->posf, n)) || (rc = dalloc(c, &c->lstage, 4 * n))) return rc;
    const int64_t slots = ((n + 31) / 32) * 32 * (int64_t)c->K.kmax;
    if ((rc = dalloc(c, &c->nbr, slots)) || (rc = dalloc(c, &c->cnt, n)) || (rc = dalloc(c, &c->cand_nc, n))) return rc;
    // FP64 grad W and PPE values in both precisions; the mixed path adds FP32
    // copies for its FP32 pair sums and inner Krylov sweeps
    if ((rc = dalloc(c, &c->gw, slots)) || (rc = dalloc(c, &c->aval, slots))) return rc;
    if (c->P.salinity && ((rc = dalloc(c, &c->ndist, slots)) || (rc = dalloc(c, &c->sdisp, 4 * n)))) return rc;
    if (c->mixed) {
        float* tw = nullptr;
        if ((rc = dalloc(c, &tw, 7 * n))) return rc;
        c->f_vol = tw; c->f_nu = tw + n; c->f_nut = tw + 2 * n; c->f_tke = tw + 3 * n; c->f_varts = tw + 4 * n;
        c->f_q = tw + 5 * n;
        c->f_vol_lo = tw + 6 * n;
        if ((rc = dalloc(c, &c->gwf, slots)) || (rc = dalloc(c, &c->gwl, slots)) || (rc = dalloc(c, &c->ellf, slots)) ||
            (rc = dalloc(c, &c->avalh, slots)) || (rc = dalloc(c, &c->ellh, slots)) ||
            (rc = dalloc(c, &c->ellh_ok, (n + 31) / 32)) || (rc = dalloc(c, &c->asm_df, 5 * n)) ||
            (rc = dalloc(c, &c->posd, n)) || (rc = dalloc(c, &c->udf, n)))
            return rc;
    }
    if ((rc = dalloc(c, &c->b, n))) return rc;
    if ((rc = alloc_solver_work(c, n, !c->mixed, c->mixed))) return rc;
    if ((rc = dalloc(c, &c->d_flag, 4))) return rc;
    BSC_CUDA(c, cudaMallocHost((void**)&c->h_flag, 4 * sizeof(int32_t)));
    if ((rc = dalloc(c, &c->stepsc, 4))) return rc;
    BSC_CUDA(c, cudaMemsetAsync(c->stepsc, 0, 4 * sizeof(double), c->stream));
    BSC_CUDA(c, cudaMemsetAsync(c->d_flag, 0, 4 * sizeof(int32_t), c->stream));
    c->cap = n;
    return BSC_OK;
}

// cell grid from the bounds (or the particle extents) and its Morton ranks
static int setup_grid(Ctx* c, const double* hx, const double* hy, int64_t n) {
    const bsc_params& P = c->P;
    double xmin = P.xmin, xmax = P.xmax, ymin = P.ymin, ymax = P.ymax;
    if (!(xmax > xmin && ymax > ymin)) {
        xmin = *std::min_element(hx, hx + n) - 4 * P.h;
        xmax = *std::max_element(hx, hx + n) + 4 * P.h;
        ymin = *std::min_element(hy, hy + n) - 4 * P.h;
        ymax = *std::max_element(hy, hy + n) + 4 * P.h;
    }
    KParams& K = c->K;
    K.cs = 2.0 * P.h * (1.0 + 1e-9);  // >= 2h so the 3x3 stencil holds the support
    K.gx0 = xmin - K.cs;
    K.gy0 = ymin - K.cs;
    const double nxd = std::ceil((xmax - K.gx0) / K.cs) + 1, nyd = std::ceil((ymax - K.gy0) / K.cs) + 1;
    if (!(nxd * nyd < 16.0e6)) return set_err(c, BSC_E_CAPACITY, "cell grid larger than 16M cells");
    const bool same = c->ncell > 0 && K.nx == (int)nxd && K.ny == (int)nyd && c->grid_x0 == K.gx0 &&
                      c->grid_y0 == K.gy0;
    if (same) return BSC_OK;  // re-upload on the same grid: ranks and solid lists stay valid
    c->grid_x0 = K.gx0;
    c->grid_y0 = K.gy0;
    c->solids_dirty = true;
    K.nx = (int)nxd;
    K.ny = (int)nyd;
    const int ncell = K.nx * K.ny;
    if (ncell != c->ncell) {
        int rc;
        if ((rc = dalloc(c, &c->cell_start, ncell)) || (rc = dalloc(c, &c->cell_count, ncell)) ||
            (rc = dalloc(c, &c->cell_rank, ncell)) || (rc = dalloc(c, &c->cell_tmp, ncell)) ||
            (rc = dalloc(c, &c->scan_part, 4096)) || (rc = dalloc(c, &c->scell_start, ncell)) ||
            (rc = dalloc(c, &c->scell_count, ncell)))
            return rc;
        c->ncell = ncell;
    }
    // Morton (Z-order) rank of every cell
    std::vector<uint64_t> code(ncell);
    std::vector<int32_t> ord(ncell), rank(ncell);
    for (int cx = 0; cx < K.nx; ++cx)
        for (int cy = 0; cy < K.ny; ++cy) code[cx * K.ny + cy] = spread_bits(cx) | (spread_bits(cy) << 1);
    std::iota(ord.begin(), ord.end(), 0);
    std::sort(ord.begin(), ord.end(), [&](int a, int b) { return code[a] < code[b]; });
    for (int q = 0; q < ncell; ++q) rank[ord[q]] = q;
    BSC_H2D(c, c->cell_rank, rank.data(), sizeof(int32_t) * ncell);
    BSC_MEMSET(c, c->scell_start, 0, sizeof(int32_t) * ncell);
    BSC_MEMSET(c, c->scell_count, 0, sizeof(int32_t) * ncell);
    return BSC_OK;
}

__global__ void k_derive_after_upload(int64_t n, State S, int ovol_given) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    S.vol[i] = S.mass[i] / S.rho[i];
    if (!ovol_given) S.ovol[i] = S.mass[i] / S.oden[i];  // internal.f90:103: ovol = fmass / rho
    S.cdiff[i] = 0.0;
    S.id[i] = (int32_t)i;
}

__global__ void k_to_id_order(int64_t n, const double* __restrict__ src, double* __restrict__ dst,
                              const int32_t* __restrict__ id) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) dst[id[k]] = src[k];
}

// L of the state view is n x 4 interleaved; the device keeps four arrays
__global__ void k_split_L(int64_t n, const double* __restrict__ L4, State S) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double4 l = reinterpret_cast<const double4*>(L4)[i];
    S.L0[i] = l.x; S.L1[i] = l.y; S.L2[i] = l.z; S.L3[i] = l.w;
}

__global__ void k_join_L_to_id_order(int64_t n, State S, double* __restrict__ L4) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    reinterpret_cast<double4*>(L4)[S.id[k]] = make_double4(S.L0[k], S.L1[k], S.L2[k], S.L3[k]);
}

__global__ void k_fill(int64_t n, double* __restrict__ d, double v) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) d[i] = v;
}

__global__ void k_to_id_order_u8(int64_t n, const uint8_t* __restrict__ src, uint8_t* __restrict__ dst,
                                 const int32_t* __restrict__ id) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) dst[id[k]] = src[k];
}

static int check_flags(Ctx* c) {
    BSC_CUDA(c, cudaMemcpyAsync(c->h_flag, c->d_flag, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    const int f = c->h_flag[0];
    if (f) {
        BSC_CUDA(c, cudaMemsetAsync(c->d_flag, 0, 4 * sizeof(int32_t), c->stream));
        if (f & 1) return set_err(c, BSC_E_CAPACITY, "a particle has more neighbours than max_neighbors");
        if (f & 2) return set_err(c, BSC_E_NONFINITE, "non-finite particle position");
    }
    return BSC_OK;
}

// the integrator.f90:949-972 time-step rule, on the host
static void dt_rule(Ctx* c, double umax, double numax) {
    const bsc_params& P = c->P;
    const double sig1 = P.sig1, dl = P.dl, mu = P.mu, rho = P.rho0, t = c->t;
    double dt;
    if (t <= 1.0)
        dt = std::min(std::min(sig1 * dl / umax, sig1 * (dl * dl) / ((mu / rho) + numax)), 0.0010);
    else if (t > 1.0 && t <= 2.50)
        dt = (double)std::min(std::min((float)(sig1 * dl / umax), (float)(sig1 * (dl * dl) * rho / mu)), 0.002f);
    else if (t > 3.0 && t <= 4.0)
        dt = (double)std::min(std::min((float)(sig1 * dl / umax), (float)(sig1 * (dl * dl) * rho / mu)), 0.004f);
    else
        dt = std::min(std::min(sig1 * dl / umax, sig1 * (dl * dl) / ((mu / rho) + numax)), 0.0050);
    if (!std::isfinite(numax)) numax = 0.0;
    // salinity sub-steps cover the next step's dt: the rule's dt, or the
    // fixed dt of the benchmark mode
    const double dtn = P.dt_mode == BSC_DT_ADAPTIVE ? dt : c->dt;
    double dtsol = sig1 * (dl * dl) / (P.diffusivity + numax / P.tschmidt);
    int solsteps = 1;
    if (dtsol < dtn) {
        solsteps = (int)std::ceil(dtn / dtsol);
        dtsol = dtn / solsteps;
    }
    c->dtsol = dtsol < dtn ? dtsol : dtn;
    c->solsteps = solsteps;
    c->umax = umax;
    c->numax = numax;
    if (P.dt_mode == BSC_DT_ADAPTIVE) c->dt = dt;
}

static int timestep_host(Ctx* c) {
    int rc = op_timestep_reduce(c);
    if (rc) return rc;
    double h[2];
    BSC_CUDA(c, cudaMemcpyAsync(h, c->stepsc, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    dt_rule(c, h[0], h[1]);
    return BSC_OK;
}

}  // namespace bsc

using namespace bsc;

#define CTX_GUARD(ctx)                                  \
    do {                                                \
        if (!(ctx)) return BSC_E_INVALID;               \
    } while (0)
#define STATE_GUARD(ctx)                                                           \
    do {                                                                           \
        if (!(ctx)) return BSC_E_INVALID;                                          \
        if (!(ctx)->have_state) return set_err(ctx, BSC_E_INVALID, "no state uploaded"); \
    } while (0)

extern "C" {

int bsc_default_params(bsc_params* p, double dl) {
    if (!p || !(dl > 0)) return BSC_E_INVALID;
    std::memset(p, 0, sizeof *p);
    const double por = 0.38;
    p->kernel = BSC_KERNEL_HYBRID;
    p->precision = BSC_PREC_FP64;
    p->h = dl * 5.08 / 4.0;  // setup.f90:47 with the fluid spacing 2 prrealx/sqrt(por)
    p->dl = dl;
    p->lam = 0.001 * p->h * p->h;
    p->rho0 = 1000.0;
    p->rel_den = 1.025;
    p->g = -9.81;
    p->mu = 0.001;
    p->csh = 0.5;
    p->maxshift = 0.1;
    p->free_threshold = 0.8 * 2.0;
    p->por = por;
    p->darcy_alpha = 450.0;
    p->forch_beta = 1.75 * std::sqrt(450.0 / 150.0);
    p->d50 = 0.001020;
    p->eddy_cs = 0.15;
    p->eddy_cv = 0.08;
    p->eddy_ce = 1.0;
    p->varts_ps = 1.0;
    p->buffer_release_xmin = -1e30;
    p->buffer_release_xmax = 1e30;
    p->dt_mode = BSC_DT_ADAPTIVE;
    p->solver = BSC_SOLVER_FGMRES;
    p->dt = (double)0.001f;
    p->sig1 = 0.2;
    p->tschmidt = 1.0;
    p->diffusivity = (double)1e-9f;  // `Dm=1e-9`, a default-real literal (integrator.f90:915, scalar.f90:118)
    p->restart = 150 > 64 ? 64 : 150;
    p->maxit = 150;
    p->tol_mode = BSC_TOL_REL_R0;
    p->max_outer = 20;
    p->tol = (double)0.001f;
    p->inner_tol = 1e-4;
    p->max_neighbors = 64;
    p->reorder_every = 20;
    p->precond = BSC_PRECOND_NONE;
    p->mg_omega = 0.82;
    p->mg_scale = 1.8;
    p->mg_sweeps = 2;
    p->mg_coarse_max = MG_COARSE_MAX;
    p->disp_long = 0.0025;     // scalar.f90:118
    p->disp_trans = 0.00025;
    p->buffer_con = 0.5;       // scalar.f90:260-264
    p->buffer_con_xmax = 1.6;
    p->salinity = 0;
    p->outflow = 0;
    p->outflow_xcut = p->outflow_ycut = 0.0;
    return BSC_OK;
}

int bsc_create(const bsc_params* p, bsc_ctx** out) {
    if (!p || !out) return BSC_E_INVALID;
    *out = nullptr;
    if (!(p->h > 0) || !(p->dl > 0) || p->max_neighbors <= 0 || p->max_neighbors > 1024 || p->maxit < 0 ||
        !(p->tol > 0) || (p->solver != BSC_SOLVER_BICGSTAB && p->solver != BSC_SOLVER_FGMRES) ||
        (p->precision != BSC_PREC_FP64 && p->precision != BSC_PREC_MIXED) ||
        (p->kernel != BSC_KERNEL_HYBRID && p->kernel != BSC_KERNEL_WENDLAND_C2) || p->piston_modes < 0 ||
        p->piston_modes > BSC_MAX_PISTON_MODES || (p->precond != BSC_PRECOND_NONE && p->precond != BSC_PRECOND_MG))
        return BSC_E_INVALID;
    if (p->precond == BSC_PRECOND_MG &&
        (!(p->mg_omega > 0 && p->mg_omega < 2) || !(p->mg_scale > 0) || p->mg_sweeps < 1 || p->mg_sweeps > 8 ||
         p->mg_coarse_max < 4 || p->mg_coarse_max > MG_COARSE_MAX))
        return BSC_E_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return BSC_E_NOT_BUILT;
    bsc_ctx* c = new (std::nothrow) bsc_ctx();
    if (!c) return BSC_E_NOMEM;
    c->P = *p;
    c->mixed = p->precision == BSC_PREC_MIXED;
    c->dt = p->dt;
    derive_kparams(c);
    cudaGetDevice(&c->device);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete c;
        return BSC_E_CUDA;
    }
    for (int k = 0; k < 2 * Ctx::EVPOOL; ++k) cudaEventCreate(&c->evs[k]);
    for (int k = 0; k < 6; ++k) cudaEventCreate(&c->ev_spmv[k]);
    if (const char* e = std::getenv("BSC_GRAPHS")) c->use_graphs = e[0] != '0';
    if (const char* e = std::getenv("BSC_DEBUG")) c->debug = e[0] == '1';
    if (const char* e = std::getenv("BSC_SPMV_UNROLL")) c->spmv_unroll = e[0] == '1';
    if (const char* e = std::getenv("BSC_PROFILE_ITER")) c->prof_iter = e[0] == '1';
    if (const char* e = std::getenv("BSC_MG_TAIL")) c->mg_tail_cells = std::atoi(e);
    // two sweeps: the weights are the reciprocal degree-2 Chebyshev nodes of
    // an interval [a, 3a] (measured best on the c3 tank: [0.45, 1.35]), i.e.
    // mg_omega and (2 + 1/sqrt2)/(2 - 1/sqrt2) times it; otherwise plain
    // damped Jacobi with mg_omega
    c->mg_w[0] = c->P.mg_omega;
    c->mg_w[1] = c->P.mg_sweeps == 2 ? c->P.mg_omega * ((2.0 + M_SQRT1_2) / (2.0 - M_SQRT1_2)) : c->P.mg_omega;
    if (const char* e = std::getenv("BSC_MG_W")) std::sscanf(e, "%lf,%lf", &c->mg_w[0], &c->mg_w[1]);
    if (const char* e = std::getenv("BSC_MG_POST")) {
        std::sscanf(e, "%d,%d,%lf", &c->mg_post[0], &c->mg_post[1], &c->mg_wpost);
        for (int k = 0; k < 2; ++k) c->mg_post[k] = std::max(0, std::min(c->mg_post[k], 8));
    }
    if (const char* e = std::getenv("BSC_MG_PRE")) c->mg_pre_fine = std::max(0, std::min(std::atoi(e), 8));
    if (const char* e = std::getenv("BSC_MG_POST_FUSED")) c->mg_post_fused = e[0] != '0';
    if (const char* e = std::getenv("BSC_MG_CELL_SWEEPS")) c->mg_cell4 = std::atoi(e) == 4;
    if (const char* e = std::getenv("BSC_EXACT_DIV")) c->exact_div = e[0] == '1';
    if (const char* e = std::getenv("BSC_ASSEMBLY")) c->asm_rcp = std::string(e) == "rcp";
    if (const char* e = std::getenv("BSC_NEIGHBOUR")) c->nb_warpcell = std::string(e) == "warpcell";
    for (int k = 0; k < 6; ++k) cudaEventCreate(&c->ev_it[k]);
    for (int k = 0; k < 2; ++k) cudaEventCreateWithFlags(&c->ev_lag[k], cudaEventDisableTiming);
    for (int k = 0; k < Ctx::NCOPY; ++k) cudaStreamCreateWithFlags(&c->copy_stream[k], cudaStreamNonBlocking);
    for (int k = 0; k <= Ctx::NCOPY; ++k) cudaEventCreateWithFlags(&c->copy_ev[k], cudaEventDisableTiming);
    *out = c;
    return BSC_OK;
}

int bsc_destroy(bsc_ctx* c) {
    if (!c) return BSC_OK;
    free_all(c);
    for (void* p : c->pallocs)
        if (p) cudaFree(p);
    c->pallocs.clear();
    for (int k = 0; k < 2 * Ctx::EVPOOL; ++k)
        if (c->evs[k]) cudaEventDestroy(c->evs[k]);
    for (int k = 0; k < 6; ++k)
        if (c->ev_spmv[k]) cudaEventDestroy(c->ev_spmv[k]);
    for (int k = 0; k < 2; ++k)
        if (c->ev_lag[k]) cudaEventDestroy(c->ev_lag[k]);
    for (int k = 0; k < Ctx::NCOPY; ++k)
        if (c->copy_stream[k]) cudaStreamDestroy(c->copy_stream[k]);
    for (int k = 0; k <= Ctx::NCOPY; ++k)
        if (c->copy_ev[k]) cudaEventDestroy(c->copy_ev[k]);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return BSC_OK;
}

const char* bsc_last_error(const bsc_ctx* c) { return c ? c->err.c_str() : "null context"; }

int bsc_set_time(bsc_ctx* c, double t, double dt) {
    CTX_GUARD(c);
    if (!(dt > 0)) return set_err(c, BSC_E_INVALID, "set_time: dt must be > 0");
    c->t = t;
    c->dt = dt;
    return BSC_OK;
}

int bsc_get_time(const bsc_ctx* c, double* t, double* dt) {
    if (!c) return BSC_E_INVALID;
    if (t) *t = c->t;
    if (dt) *dt = c->dt;
    return BSC_OK;
}

// the copy streams wait for everything queued on c->stream so far
static int copy_fork(Ctx* c) {
    BSC_CUDA(c, cudaEventRecord(c->copy_ev[Ctx::NCOPY], c->stream));
    for (int k = 0; k < Ctx::NCOPY; ++k) BSC_CUDA(c, cudaStreamWaitEvent(c->copy_stream[k], c->copy_ev[Ctx::NCOPY], 0));
    return BSC_OK;
}
// c->stream waits for every copy stream
static int copy_join(Ctx* c) {
    for (int k = 0; k < Ctx::NCOPY; ++k) {
        BSC_CUDA(c, cudaEventRecord(c->copy_ev[k], c->copy_stream[k]));
        BSC_CUDA(c, cudaStreamWaitEvent(c->stream, c->copy_ev[k], 0));
    }
    return BSC_OK;
}

int bsc_upload_state(bsc_ctx* c, const bsc_state_view* s) {
    CTX_GUARD(c);
    if (!s || s->n <= 0 || s->n > (1ll << 30) || !s->x || !s->y || !s->vx || !s->vy || !s->p || !s->rho ||
        !s->oden || !s->mass || !s->tid || !s->flags)
        return set_err(c, BSC_E_INVALID, "upload_state: missing required field or bad n");
    StageTimer tm(c, BSC_T_UPLOAD);
    const int64_t n = s->n;
    int rc;
    if (c->cap < n || c->cap > 2 * n) {
        c->ncell = 0;
        if ((rc = alloc_for(c, std::max(n, c->cap_hint)))) return rc;
        c->cap_hint = 0;
    } else if (c->n != n) {  // the arrays have room: drop what was sized for the old count
        drop_graphs(c);
        wc_free(c);
    }
    c->n = n;
    if ((rc = setup_grid(c, s->x, s->y, n))) return rc;
    State& S = c->S;
    if ((rc = copy_fork(c))) return rc;
    int nq = 0;  // copies round-robin over the copy streams
    auto up = [&](double* d, const double* h, double dflt) -> int {
        if (h) {
            BSC_CUDA(c, cudaMemcpyAsync(d, h, sizeof(double) * n, cudaMemcpyHostToDevice,
                                        c->copy_stream[nq++ % Ctx::NCOPY]));
        } else if (dflt == 0.0) {
            BSC_CUDA(c, cudaMemsetAsync(d, 0, sizeof(double) * n, c->stream));
        } else {
            k_fill<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, d, dflt);
            BSC_LAUNCH(c);
        }
        return BSC_OK;
    };
    if ((rc = up(S.x, s->x, 0)) || (rc = up(S.y, s->y, 0)) || (rc = up(S.vx, s->vx, 0)) || (rc = up(S.vy, s->vy, 0)) ||
        (rc = up(S.xs, s->xs, 0)) || (rc = up(S.ys, s->ys, 0)) || (rc = up(S.vxs, s->vxs, 0)) ||
        (rc = up(S.vys, s->vys, 0)) || (rc = up(S.p, s->p, 0)) || (rc = up(S.rho, s->rho, 0)) ||
        (rc = up(S.oden, s->oden, 0)) || (rc = up(S.mass, s->mass, 0)) || (rc = up(S.por, s->porosity, 1.0)) ||
        (rc = up(S.gradvx, s->gradvx, 0)) || (rc = up(S.nut, s->nut, 0)) || (rc = up(S.tke, s->tke, 0)) ||
        (rc = up(S.resist, s->resist, 0)) || (rc = up(S.varts, s->varts, 0)) || (rc = up(S.vel, s->vel, 0)) ||
        (rc = up(S.xrest, s->xrest ? s->xrest : s->x, 0)) || (rc = up(S.con, s->con, 0)) ||
        (s->ovol && (rc = up(S.ovol, s->ovol, 0))))
        return rc;
    if (s->L) {
        cudaStream_t cs = c->copy_stream[nq++ % Ctx::NCOPY];
        BSC_CUDA(c, cudaMemcpyAsync(c->lstage, s->L, 4 * sizeof(double) * n, cudaMemcpyHostToDevice, cs));
        k_split_L<<<blocks_for(n, 256), 256, 0, cs>>>(n, c->lstage, S);
        BSC_LAUNCH(c);
    } else {
        if ((rc = up(S.L0, nullptr, 1.0)) || (rc = up(S.L1, nullptr, 0)) || (rc = up(S.L2, nullptr, 0)) ||
            (rc = up(S.L3, nullptr, 1.0)))
            return rc;
    }
    BSC_CUDA(c, cudaMemcpyAsync(S.tid, s->tid, n, cudaMemcpyHostToDevice, c->copy_stream[nq++ % Ctx::NCOPY]));
    BSC_CUDA(c, cudaMemcpyAsync(S.flags, s->flags, n, cudaMemcpyHostToDevice, c->copy_stream[nq++ % Ctx::NCOPY]));
    if ((rc = copy_join(c))) return rc;
    k_derive_after_upload<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, S, s->ovol != nullptr);
    BSC_LAUNCH(c);
    c->have_state = true;
    c->have_lists = c->have_csr = false;
    c->cellshifts = 0;  // the first build gathers the state into cell order
    if ((rc = cells_build(c, true))) return rc;
    if (c->ns > 0 && (rc = solids_build(c))) return rc;
    return check_flags(c);
}

int bsc_upload_porosity(bsc_ctx* c, int32_t nx, int32_t ny, double x0, double y0, double dx, double dy,
                        const double* v) {
    CTX_GUARD(c);
    if (nx <= 0 || ny <= 0 || !v || !(dx > 0) || !(dy > 0)) return set_err(c, BSC_E_INVALID, "upload_porosity");
    int rc;
    if ((rc = palloc(c, &c->pgrid, (int64_t)nx * ny))) return rc;
    BSC_H2D(c, c->pgrid, v, sizeof(double) * nx * ny);
    c->hpgrid.assign(v, v + (int64_t)nx * ny);
    c->K.pnx = nx; c->K.pny = ny; c->K.px0 = x0; c->K.py0 = y0; c->K.pdx = dx; c->K.pdy = dy;
    c->K.pgrid = c->pgrid;
    return BSC_OK;
}

int bsc_upload_solids(bsc_ctx* c, int64_t ns, const double* x, const double* y, const double* m,
                      const double* rho, const double* por) {
    CTX_GUARD(c);
    if (ns < 0 || (ns > 0 && (!x || !y || !m || !rho))) return set_err(c, BSC_E_INVALID, "upload_solids");
    c->ns = ns;
    if (ns == 0) return BSC_OK;
    int rc;
    if ((rc = palloc(c, &c->sx, ns)) || (rc = palloc(c, &c->sy, ns)) || (rc = palloc(c, &c->svol, ns)) ||
        (rc = palloc(c, &c->spor, ns)) || (rc = palloc(c, &c->sposf, ns)) || (rc = palloc(c, &c->swf, ns)))
        return rc;
    std::vector<double> vol(ns), sp(ns);
    const KParams& K = c->K;
    for (int64_t k = 0; k < ns; ++k) {
        vol[k] = m[k] / rho[k];
        if (por) {
            sp[k] = por[k];
        } else if (K.pnx > 0) {
            // same lookup as the fluid-side cap (porosity_at in pairs.cu)
            double fx = std::floor((x[k] - K.px0) / K.pdx), fy = std::floor((y[k] - K.py0) / K.pdy);
            bool in = fx >= 0 && fx < K.pnx && fy >= 0 && fy < K.pny;
            sp[k] = in ? c->hpgrid[(int64_t)fy * K.pnx + (int64_t)fx] : K.por;
        } else {
            sp[k] = K.por;
        }
    }
    BSC_H2D(c, c->sx, x, sizeof(double) * ns);
    BSC_H2D(c, c->sy, y, sizeof(double) * ns);
    BSC_H2D(c, c->svol, vol.data(), sizeof(double) * ns);
    BSC_H2D(c, c->spor, sp.data(), sizeof(double) * ns);
    c->solids_dirty = true;
    if (c->ncell > 0) return solids_build(c);
    return BSC_OK;
}

int bsc_download_state(bsc_ctx* c, bsc_state_view* s) {
    STATE_GUARD(c);
    if (!s || s->n != c->n) return set_err(c, BSC_E_INVALID, "download_state: size mismatch");
    StageTimer tm(c, BSC_T_DOWNLOAD);
    const int64_t n = c->n;
    const State& S = c->S;
    const State& T = c->S2;  // free outside a reorder: per-field staging in id order
    const unsigned g = blocks_for(n, 256);
    // every gather and copy is queued on the copy streams (each field's
    // gather, then its copy); one wait at the end
    int rc;
    if ((rc = copy_fork(c))) return rc;
    int nq = 0;
    auto dn = [&](const double* src, double* stage, double* host) -> int {
        if (!host) return BSC_OK;
        cudaStream_t cs = c->copy_stream[nq++ % Ctx::NCOPY];
        k_to_id_order<<<g, 256, 0, cs>>>(n, src, stage, S.id);
        BSC_LAUNCH(c);
        BSC_CUDA(c, cudaMemcpyAsync(host, stage, sizeof(double) * n, cudaMemcpyDeviceToHost, cs));
        return BSC_OK;
    };
    auto dn8 = [&](const uint8_t* src, uint8_t* stage, uint8_t* host) -> int {
        if (!host) return BSC_OK;
        cudaStream_t cs = c->copy_stream[nq++ % Ctx::NCOPY];
        k_to_id_order_u8<<<g, 256, 0, cs>>>(n, src, stage, S.id);
        BSC_LAUNCH(c);
        BSC_CUDA(c, cudaMemcpyAsync(host, stage, n, cudaMemcpyDeviceToHost, cs));
        return BSC_OK;
    };
    if ((rc = dn(S.x, T.x, s->x)) || (rc = dn(S.y, T.y, s->y)) || (rc = dn(S.vx, T.vx, s->vx)) ||
        (rc = dn(S.vy, T.vy, s->vy)) || (rc = dn(S.xs, T.xs, s->xs)) || (rc = dn(S.ys, T.ys, s->ys)) ||
        (rc = dn(S.vxs, T.vxs, s->vxs)) || (rc = dn(S.vys, T.vys, s->vys)) || (rc = dn(S.p, T.p, s->p)) ||
        (rc = dn(S.rho, T.rho, s->rho)) || (rc = dn(S.oden, T.oden, s->oden)) || (rc = dn(S.mass, T.mass, s->mass)) ||
        (rc = dn(S.por, T.por, s->porosity)) || (rc = dn(S.gradvx, T.gradvx, s->gradvx)) ||
        (rc = dn(S.nut, T.nut, s->nut)) || (rc = dn(S.tke, T.tke, s->tke)) ||
        (rc = dn(S.resist, T.resist, s->resist)) || (rc = dn(S.varts, T.varts, s->varts)) ||
        (rc = dn(S.vel, T.vel, s->vel)) || (rc = dn(S.xrest, T.xrest, s->xrest)) || (rc = dn(S.con, T.con, s->con)) ||
        (rc = dn(S.ovol, T.ovol, s->ovol)))
        return rc;
    if (s->L) {
        cudaStream_t cs = c->copy_stream[nq++ % Ctx::NCOPY];
        k_join_L_to_id_order<<<g, 256, 0, cs>>>(n, S, c->lstage);
        BSC_LAUNCH(c);
        BSC_CUDA(c, cudaMemcpyAsync(s->L, c->lstage, 4 * sizeof(double) * n, cudaMemcpyDeviceToHost, cs));
    }
    if ((rc = dn8((const uint8_t*)S.tid, (uint8_t*)T.tid, (uint8_t*)s->tid)) || (rc = dn8(S.flags, T.flags, s->flags)))
        return rc;
    if ((rc = copy_join(c))) return rc;
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    return BSC_OK;
}

#define OP(name, slot, body)                 \
    int name(bsc_ctx* c) {                   \
        STATE_GUARD(c);                      \
        StageTimer tm(c, slot);              \
        return (body);                       \
    }

OP(bsc_projection, BSC_T_PROJECTION, op_projection(c))
OP(bsc_piston, BSC_T_PISTON, op_piston(c))
OP(bsc_comp_pos, BSC_T_COMP_POS, op_comp_pos(c))
OP(bsc_freesurf, BSC_T_FREESURF, (c->have_lists ? op_freesurf(c) : set_err(c, BSC_E_INVALID, "freesurf before neighbour")))
OP(bsc_eddyvis, BSC_T_EDDYVIS, op_eddyvis(c))
OP(bsc_int_vel, BSC_T_INT_VEL, op_int_vel(c, c->stepsc))
OP(bsc_comp_vel, BSC_T_COMP_VEL, op_comp_vel(c))
OP(bsc_opt2_shift, BSC_T_SHIFT, op_opt2_shift(c))

int bsc_effpor(bsc_ctx* c) {
    STATE_GUARD(c);
    StageTimer tm(c, BSC_T_EFFPOR);
    return op_effpor(c);
}

int bsc_cellshift(bsc_ctx* c, int32_t alt) {
    (void)alt;  // the outflow cut-offs of cellshiftalt belong to open-boundary runs
    STATE_GUARD(c);
    StageTimer tm(c, BSC_T_CELLSHIFT);
    return cells_build(c, true);
}

// resetid: the slot order of the cell list is the row numbering of the PPE
int bsc_resetid(bsc_ctx* c) {
    STATE_GUARD(c);
    return BSC_OK;
}

int bsc_neighbour(bsc_ctx* c) {
    STATE_GUARD(c);
    int rc;
    {
        StageTimer tm(c, BSC_T_NEIGHBOUR);
        rc = op_neighbour(c);
    }
    if (rc) return rc;
    return check_flags(c);
}

int bsc_ppesolve(bsc_ctx* c, bsc_solve_info* out) {
    STATE_GUARD(c);
    int rc;
    {
        StageTimer tm(c, BSC_T_PPE_ASSEMBLE);
        rc = op_ppe_assemble(c);
    }
    if (rc) return rc;
    StageTimer tm(c, BSC_T_PPE_SOLVE);
    rc = op_ppe_solve(c, out);
    if (rc == BSC_E_NOT_CONVERGED || rc == BSC_E_BREAKDOWN) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "ppesolve: %s after %d iterations, rel residual %.3e",
                      rc == BSC_E_BREAKDOWN ? "breakdown" : "not converged", out ? out->iterations : -1,
                      out ? out->rel_residual : -1.0);
        c->err = buf;
    }
    return rc;
}

int bsc_timestep(bsc_ctx* c, double* dt_inout) {
    STATE_GUARD(c);
    StageTimer tm(c, BSC_T_TIMESTEP);
    int rc = timestep_host(c);
    if (rc) return rc;
    if (dt_inout) *dt_inout = c->dt;
    return BSC_OK;
}

int bsc_step(bsc_ctx* c, int32_t nsteps, bsc_solve_info* last) {
    STATE_GUARD(c);
    if (nsteps < 0) return set_err(c, BSC_E_INVALID, "step: nsteps < 0");
    bsc_solve_info loc{};
    bsc_solve_info* info = last ? last : &loc;
    for (int s = 0; s < nsteps; ++s) {
        StageTimer whole(c, BSC_T_STEP);
        int rc;
        c->t = c->t + c->dt;
#define RUN(slot, expr)                  \
    do {                                 \
        StageTimer tm_(c, slot);         \
        if ((rc = (expr))) return rc;    \
    } while (0)
        if (c->P.salinity) {
            // phase 3 of main.f90:198-260: solsteps salinity sub-steps on the
            // lists of the previous step (built here on the first step)
            if (!c->have_lists) {
                RUN(BSC_T_CELLSHIFT, cells_build(c, true));
                RUN(BSC_T_NEIGHBOUR, op_neighbour(c));
            }
            if (!(c->dtsol > 0.0)) RUN(BSC_T_TIMESTEP, timestep_host(c));
            for (int k = 0; k < c->solsteps; ++k) {
                RUN(BSC_T_SCALAR, op_scalart(c));
                RUN(BSC_T_SCALAR, op_scalarupdate(c, c->dtsol));
            }
        }
        RUN(BSC_T_PISTON, op_piston(c));
        RUN(BSC_T_PROJECTION, op_projection(c));
        RUN(BSC_T_CELLSHIFT, cells_build(c, true));
        RUN(BSC_T_NEIGHBOUR, op_neighbour(c));
        RUN(BSC_T_EFFPOR, op_effpor(c));
        RUN(BSC_T_EDDYVIS, op_eddyvis(c));
        RUN(BSC_T_INT_VEL, op_int_vel(c, c->stepsc));
        RUN(BSC_T_PPE_ASSEMBLE, op_ppe_assemble(c));
        {
            StageTimer tm_(c, BSC_T_PPE_SOLVE);
            rc = op_ppe_solve(c, info);
            if (rc) {
                char buf[160];
                std::snprintf(buf, sizeof buf, "step %d: PPE %s after %d iterations, rel residual %.3e", s,
                              rc == BSC_E_BREAKDOWN ? "breakdown" : "not converged", info->iterations,
                              info->rel_residual);
                if (rc == BSC_E_NOT_CONVERGED || rc == BSC_E_BREAKDOWN) c->err = buf;
                return rc;
            }
        }
        RUN(BSC_T_COMP_VEL, op_comp_vel(c));
        RUN(BSC_T_COMP_POS, op_comp_pos(c));
        RUN(BSC_T_CELLSHIFT, cells_build(c, true));
        if (c->P.outflow) {  // cellshiftalt's outflow cut-off (integrator.f90:60-61)
            int64_t gone = 0;
            RUN(BSC_T_CELLSHIFT, bsc_remove_particles(c, BSC_REMOVE_OUTFLOW, c->P.outflow_xcut, c->P.outflow_ycut,
                                                      &gone));
        }
        RUN(BSC_T_NEIGHBOUR, op_neighbour(c));
        RUN(BSC_T_FREESURF, op_freesurf(c));
        RUN(BSC_T_EFFPOR, op_effpor(c));
        RUN(BSC_T_SHIFT, op_opt2_shift(c));
        if (c->P.salinity) RUN(BSC_T_SCALAR, op_densityupdate(c));
        // the host needs umax and numax for an adaptive dt, and numax for
        // the salinity sub-steps; otherwise the reduction stays on the device
        if (c->P.dt_mode == BSC_DT_ADAPTIVE || c->P.salinity) {
            RUN(BSC_T_TIMESTEP, timestep_host(c));
        } else {
            RUN(BSC_T_TIMESTEP, op_timestep_reduce(c));
        }
        if (c->P.salinity) RUN(BSC_T_EDDYVIS, op_eddyvis(c));
#undef RUN
    }
    int rc = check_flags(c);
    if (c->timing) timing_flush(c);
    return rc;
}

int bsc_get_neighbors(bsc_ctx* c, int64_t* offsets, int32_t* ids) {
    STATE_GUARD(c);
    if (!c->have_lists) return set_err(c, BSC_E_INVALID, "get_neighbors before neighbour");
    if (!offsets) return set_err(c, BSC_E_INVALID, "get_neighbors: offsets required");
    const int64_t n = c->n, kmax = c->K.kmax, slots = ((n + 31) / 32) * 32 * kmax;
    std::vector<int32_t> cnt(n), id(n), nb;
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    BSC_D2H(c, cnt.data(), c->cnt, sizeof(int32_t) * n);
    BSC_D2H(c, id.data(), c->S.id, sizeof(int32_t) * n);
    std::vector<int64_t> slot_of(n);
    for (int64_t k = 0; k < n; ++k) slot_of[id[k]] = k;
    offsets[0] = 0;
    for (int64_t q = 0; q < n; ++q) offsets[q + 1] = offsets[q] + cnt[slot_of[q]];
    if (!ids) return BSC_OK;
    nb.resize(slots);
    BSC_D2H(c, nb.data(), c->nbr, sizeof(int32_t) * slots);
    for (int64_t q = 0; q < n; ++q) {
        const int64_t k = slot_of[q];
        int32_t* dst = ids + offsets[q];
        for (int e = 0; e < cnt[k]; ++e) dst[e] = id[nb[ell(k, e, (int)kmax)]];
        std::sort(dst, dst + cnt[k]);
    }
    return BSC_OK;
}

int bsc_export_csr(bsc_ctx* c, int64_t* rowptr, int32_t* col, double* val, double* rhs) {
    STATE_GUARD(c);
    if (!c->have_csr) return set_err(c, BSC_E_INVALID, "export_csr before ppesolve");
    if (!rowptr) return set_err(c, BSC_E_INVALID, "export_csr: rowptr required");
    const int64_t n = c->n, kmax = c->K.kmax, slots = ((n + 31) / 32) * 32 * kmax;
    std::vector<int32_t> cnt(n), id(n);
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    BSC_D2H(c, cnt.data(), c->cnt, sizeof(int32_t) * n);
    BSC_D2H(c, id.data(), c->S.id, sizeof(int32_t) * n);
    std::vector<int64_t> slot_of(n);
    for (int64_t k = 0; k < n; ++k) slot_of[id[k]] = k;
    rowptr[0] = 0;
    for (int64_t q = 0; q < n; ++q) rowptr[q + 1] = rowptr[q] + cnt[slot_of[q]] + 1;
    if (rhs) {
        std::vector<double> b(n);
        BSC_D2H(c, b.data(), c->b, sizeof(double) * n);
        for (int64_t q = 0; q < n; ++q) rhs[q] = b[slot_of[q]];
    }
    if (!col && !val) return BSC_OK;
    std::vector<int32_t> nb(slots);
    std::vector<double> v(slots);
    BSC_D2H(c, nb.data(), c->nbr, sizeof(int32_t) * slots);
    // the FP64 system on both paths (the mixed path's outer refinement
    // solves it; its FP32 and FP16 copies only serve the inner sweeps)
    BSC_D2H(c, v.data(), c->aval, sizeof(double) * slots);
    std::vector<std::pair<int32_t, double>> row;
    for (int64_t q = 0; q < n; ++q) {
        const int64_t k = slot_of[q];
        row.clear();
        row.push_back({(int32_t)q, 1.0});
        for (int e = 0; e < cnt[k]; ++e) {
            const int64_t x = ell(k, e, (int)kmax);
            row.push_back({id[nb[x]], v[x]});
        }
        std::stable_sort(row.begin(), row.end(), [](auto& a, auto& b) { return a.first < b.first; });
        for (size_t e = 0; e < row.size(); ++e) {
            if (col) col[rowptr[q] + e] = row[e].first;
            if (val) val[rowptr[q] + e] = row[e].second;
        }
    }
    return BSC_OK;
}

int bsc_probe_eta(bsc_ctx* c, int32_t np, const double* xp, double depth, double* eta) {
    STATE_GUARD(c);
    if (!xp || !eta) return set_err(c, BSC_E_INVALID, "probe_eta: null pointer");
    return op_probe_eta(c, np, xp, depth, eta);
}

int bsc_get_timings(bsc_ctx* c, bsc_timing* out) {
    CTX_GUARD(c);
    if (!out) return BSC_E_INVALID;
    timing_flush(c);
    for (int k = 0; k < BSC_TIMING_SLOTS; ++k) {
        out->ms[k] = c->ms[k];
        out->calls[k] = c->calls[k];
    }
    out->kernel_launches = c->launches;
    return BSC_OK;
}

int bsc_reset_timings(bsc_ctx* c) {
    CTX_GUARD(c);
    timing_flush(c);
    for (int k = 0; k < BSC_TIMING_SLOTS; ++k) {
        c->ms[k] = 0;
        c->calls[k] = 0;
    }
    c->launches = 0;
    return BSC_OK;
}

int bsc_synchronize(bsc_ctx* c) {
    CTX_GUARD(c);
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    return BSC_OK;
}

int bsc_csr_solve(const bsc_params* p, int32_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                  const double* b, double* x, bsc_solve_info* info) {
    if (!p || n <= 0 || !rowptr || !col || !val || !b || !x || !info) return BSC_E_INVALID;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return BSC_E_NOT_BUILT;
    Ctx c;
    c.P = *p;
    c.timing = false;  // no event pool on this temporary context
    if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess) return BSC_E_CUDA;
    const int64_t nnz = rowptr[n];
    int rc = alloc_solver_work(&c, n, true, false);
    int32_t *drp = nullptr, *dcol = nullptr;
    double *dval = nullptr, *db = nullptr, *dx = nullptr;
    if (!rc) rc = dalloc(&c, &drp, n + 1);
    if (!rc) rc = dalloc(&c, &dcol, nnz);
    if (!rc) rc = dalloc(&c, &dval, nnz);
    if (!rc) rc = dalloc(&c, &db, n);
    if (!rc) rc = dalloc(&c, &dx, n);
    if (!rc) {
        auto up = [&](void* d, const void* h, size_t bytes) {
            if (!rc && cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c.stream) != cudaSuccess) rc = BSC_E_CUDA;
        };
        up(drp, rowptr, sizeof(int32_t) * (n + 1));
        up(dcol, col, sizeof(int32_t) * nnz);
        up(dval, val, sizeof(double) * nnz);
        up(db, b, sizeof(double) * n);
        up(dx, x, sizeof(double) * n);
        if (!rc) rc = csr_solve_device(&c, n, drp, dcol, dval, db, dx, info);
        if (rc == BSC_OK || rc == BSC_E_NOT_CONVERGED || rc == BSC_E_BREAKDOWN) {
            cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream);
            cudaStreamSynchronize(c.stream);
        }
    }
    free_all(&c);
    cudaStreamDestroy(c.stream);
    return rc;
}

}  // extern "C"
