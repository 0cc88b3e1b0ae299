// bsc_internal.cuh -- device state layout and shared helpers of libbsc.
//
// Layout in HBM (one context = one GPU, state resident across steps):
//  * particle state: structure of arrays, FP64, one slot per particle, slots
//    kept sorted by cell (Morton order of the 2h cells) and re-sorted every
//    `reorder_every` cell shifts; `id[slot]` maps back to the caller's order;
//  * cell list: cells of side >= 2h (3x3 stencil covers the 2h support),
//    cell_start/cell_count over cells, `sorted[]` = slots in cell order;
//  * neighbour lists: ELL with 32-slot slices stored column-major
//    (entry k of slot i at ((i/32)*kmax + k)*32 + i%32), holding the
//    neighbour slot and grad_i W, so each column read by a warp is one
//    coalesced transaction;
//  * PPE: the Jacobi-scaled matrix has a unit diagonal; its off-diagonal
//    values share the neighbour-list layout (no extra column indices).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/bsc.h"

namespace bsc {

constexpr int WARP = 32;
constexpr int NB_BLOCK = 128;     // threads per block for particle kernels
constexpr int RED_BLOCK = 256;    // threads per block for reductions
constexpr int RED_GRID = 912;     // fixed reduction grid (6 x 152 SMs): deterministic sums

// ---- particle state (SoA) --------------------------------------------------
struct State {
    double *x, *y, *vx, *vy, *xs, *ys, *vxs, *vys, *p, *rho, *oden, *mass;
    double *por, *gradvx, *nut, *tke, *resist, *varts, *vel, *xrest, *vol;
    double *L0, *L1, *L2, *L3;
    double *con, *ovol, *cdiff;  // salinity, original volume, salinity rate
    int8_t* tid;
    uint8_t* flags;
    int32_t* id;
};
constexpr int N_DBL_FIELDS = 28;

// ---- neighbour list (ELL, 32-slot slices) ----------------------------------
__host__ __device__ inline int64_t ell(int64_t i, int k, int kmax) {
    return ((i >> 5) * (int64_t)kmax + k) * 32 + (i & 31);
}

// ---- solver scalars kept on the device -------------------------------------
struct Scalars {
    double rhob[2];            // rho of the current iteration, by iteration parity
    double bestb[2];           // smallest residual norm so far, by iteration parity
    double rho, alpha, omega, beta;
    double rr, bnorm, r0norm, target;
    double tmp[8];
    int32_t done, breakdown, it, k5;  // k5: work of the last kernel of a BiCGSTAB iteration
};

// FP64 -> FP32 on the integer pipe: round to nearest (ties away from zero)
// by adding half an FP32 ulp to the bit pattern, then repacking exponent and
// mantissa.  For finite |v| below 2^127; magnitudes below FP32's normal
// range become signed zeros.  The hardware conversion issues on the FP64
// pipe, this GPU's scarce resource; this is a dozen integer operations.
__device__ __forceinline__ float f32_of(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v) + (1ull << 28);
    const unsigned hi = (unsigned)(b >> 32), lo = (unsigned)b;
    const int e = (int)((hi >> 20) & 0x7ffu) - 896;  // FP64 bias 1023 -> FP32 bias 127
    const unsigned sign = hi & 0x80000000u;
    const unsigned m = ((hi & 0xfffffu) << 3) | (lo >> 29);
    return __uint_as_float(e > 0 ? (sign | ((unsigned)e << 23) | m) : sign);
}

// FP32 -> FP64 on the integer pipe (exact), for normal FP32 values
__device__ __forceinline__ double f64_of(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned hi = (u & 0x80000000u) | ((((u >> 23) & 0xffu) + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    return __hiloint2double((int)hi, (int)(u << 29));
}

// an FP64 value in the pair arithmetic's type R: the integer-pipe rounding
// for R = float, unchanged for R = double
template <typename R>
__device__ __forceinline__ R to_r(double v) {
    if constexpr (sizeof(R) == 4)
        return f32_of(v);
    else
        return v;
}

// 1/x by one Newton-Raphson step for the reciprocal, y1 = y0 (2 - x y0), from
// y0 = the FP32 reciprocal of x rounded to FP32.  y0 is within 2^-23 of 1/x
// (two FP32 roundings), so y1 is within about 2^-46 (the step squares the
// relative error) plus FP64 rounding.  The conversions run on the integer
// pipe (f32_of, f64_of): two FMAs on the FP64 pipe instead of a full FP64
// division.  For |x| outside [2^-125, 2^126) (and NaN, infinities) it
// returns the FP64 quotient.
__device__ __forceinline__ double rcp_nr(double x) {
    const int ex = (int)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff;
    if (ex < 1023 - 125 || ex > 1023 + 125) return 1.0 / x;
    const double y0 = f64_of(__frcp_rn(f32_of(x)));
    return fma(y0, fma(-x, y0, 1.0), y0);
}

// sqrt(x) for x > 0 in FP32's normal range: an FP32 seed of 1/sqrt(x) (the
// rounding on the integer pipe, the reciprocal root on the special-function
// unit) and one coupled Newton step in FP64, Goldschmidt's iteration as set
// out by Markstein (IA-64 and Elementary Functions, 2000):
//   r0 = x y0, h0 = y0 / 2, e = 1/2 - r0 h0, r = r0 + r0 e.
// The relative error is about 3/2 e0^2 for a seed error e0 (~2^-22): within
// 2^-42.  Four FP64 operations.
// Three FP64 operations: h0 = y0 / 2 is formed in FP32 (exact there) and
// widened on the integer pipe like y0.
__device__ __forceinline__ double sqrt_nr(double x) {
    const float yf = rsqrtf(f32_of(x));
    const double y0 = f64_of(yf), h0 = f64_of(0.5f * yf);
    const double r0 = x * y0;
    const double e = fma(-r0, h0, 0.5);
    return fma(r0, e, r0);
}

// a < b for non-negative doubles a and b (b finite), on the integer pipe:
// the bit patterns of non-negative IEEE doubles order like their values, and
// any a with the sign bit set (only a NaN can have it here) compares as not
// below.  The pair searches take their exact d^2 < T test this way, off the
// FP64 pipe that bounds them.
__device__ __forceinline__ bool nonneg_below(double a, double b) {
    return (unsigned long long)__double_as_longlong(a) < (unsigned long long)__double_as_longlong(b);
}

// an FGMRES cycle has stopped (converged, broken down or at its restart
// length): the kernels of iterations queued past that point return at once
__device__ __forceinline__ bool fg_skip(const Scalars* sc) { return sc->done || sc->tmp[2] != 0.0; }
__device__ __forceinline__ bool mg_skip(const Scalars* sk) { return sk && fg_skip(sk); }

// ---- kernel constants --------------------------------------------------------
struct KParams {
    int kernel;
    double h, H, H2, lam, dl, rho0, rel_den, g, csh, maxshift, free_thr;
    double H2x;  // sqrt_rn(d2) < H exactly when d2 < H2x (the reference's neighbour test)
    double por, alpha, beta, d50;
    double eddy_cs, eddy_cv, eddy_ce, varts_ps;
    double bxmin, bxmax;
    // kernel coefficients: grad_i W = F(r) (x_i - x_j)
    double hyb_A, hyb_B, wend_F, wend_W, w0, inv_w0;
    double inv_h, half_inv_h, hyb_n0, hyb_n1, hyb_n2, hyb_f;  // 1/h, 1/(2h), folded hybrid-gradient constants
    // cell grid
    double gx0, gy0, cs;
    int nx, ny;
    int kmax;
    // porosity field
    int pnx, pny;
    double px0, py0, pdx, pdy;
    const double* pgrid;
};

struct Ctx;

// ---- error handling ----------------------------------------------------------
int set_err(Ctx* c, int code, const std::string& msg);
int cuda_err(Ctx* c, cudaError_t e, const char* where);
#define BSC_CUDA(c, call)                                  \
    do {                                                   \
        cudaError_t e_ = (call);                           \
        if (e_ != cudaSuccess) return cuda_err((c), e_, #call); \
    } while (0)
#define BSC_LAUNCH(c)                                      \
    do {                                                   \
        (c)->launches++;                                   \
        cudaError_t e_ = cudaGetLastError();               \
        if (e_ != cudaSuccess) return cuda_err((c), e_, __func__); \
    } while (0)

// every transfer is ordered on the context stream (a non-blocking stream does
// not synchronise with the legacy default stream); host buffers may be
// temporaries, so host-side copies complete before the macro returns
#define BSC_H2D(c, dst, src, bytes)                                                                 \
    do {                                                                                            \
        BSC_CUDA(c, cudaMemcpyAsync((dst), (src), (bytes), cudaMemcpyHostToDevice, (c)->stream));   \
        BSC_CUDA(c, cudaStreamSynchronize((c)->stream));                                            \
    } while (0)
#define BSC_D2H(c, dst, src, bytes)                                                                 \
    do {                                                                                            \
        BSC_CUDA(c, cudaMemcpyAsync((dst), (src), (bytes), cudaMemcpyDeviceToHost, (c)->stream));   \
        BSC_CUDA(c, cudaStreamSynchronize((c)->stream));                                            \
    } while (0)
#define BSC_MEMSET(c, dst, v, bytes) BSC_CUDA(c, cudaMemsetAsync((dst), (v), (bytes), (c)->stream))

template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };

inline unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// ---- the context ---------------------------------------------------------------
// ---- cell-aggregation multigrid (mg.cu) -------------------------------------
// Level 0 is the PPE in the neighbour-list layout; level 1 aggregates the
// particles of each neighbour-search cell; every further level merges 2x2
// cells.  Levels >= 1 are structured grids with 9-point stencils.
constexpr int MG_MAX_LEVELS = 24;
constexpr int MG_COARSE_MAX = 128;  // cells of the coarsest level (dense inverse)
struct MgLevel {
    int nx = 0, ny = 0;            // cells; index cx * ny + cy
    int64_t nc = 0;
    double* A = nullptr;           // 9 x nc, stencil-major: A[s * nc + c], s = (dx+1)*3 + (dy+1)
    double* dinv = nullptr;        // 1 / centre coefficient, 0 on empty cells
    float* Af = nullptr;           // FP32 copies (mixed path)
    float* dinvf = nullptr;
    void *b = nullptr, *x = nullptr, *y = nullptr, *t = nullptr;  // V-cycle vectors (FP64 or FP32)
    // the restriction of the pre-smoothed residual as an operator on b: per
    // cell of level l+1, 36 weights over the 6x6 patch of this level's cells
    // around its 2x2 children (36 x nc of level l+1, in the V-cycle's type)
    void* R = nullptr;
};
struct Mg {
    int nlev = 0;                  // levels 1..nlev are structured; nlev is solved densely
    int tail_l0 = 0;               // levels tail_l0..nlev run in one single-CTA kernel
    MgLevel L[MG_MAX_LEVELS + 1];
    double* cinv = nullptr;        // inverse of the coarsest level, FP64, row-major
    float* cinvf = nullptr;        // its FP32 copy (mixed path)
    int tail_smem = 0;             // bytes of shared memory the tail stages its levels in; 0: none
    double* rowslots = nullptr;    // 9 x n: each row's sums over the 3x3 neighbour cells
    float* rowslotsf = nullptr;    // their FP32 copy (mixed path)
    int64_t n = 0;                 // rows the buffers are sized for
    int gx = 0, gy = 0;            // level-1 grid they are sized for
    int m = 0;                     // FGMRES restart length
    bool f32 = false;
    void *r0 = nullptr, *y0 = nullptr, *t0 = nullptr;  // fine-level V-cycle vectors
    double* V = nullptr;           // FGMRES basis (m+1) x n (FP64 path)
    double* Z = nullptr;           // preconditioned vectors m x n (FP64 path)
    float *Vf = nullptr, *Zf = nullptr;  // the same in FP32 (mixed path's inner solve)
    float *wf = nullptr, *rf = nullptr;  // FP32 work vectors
    const Scalars* skip = nullptr;  // the calling FGMRES's scalars: V-cycles queued past its stop return at once
    std::vector<void*> allocs;
};

struct WcState;    // the differentiable WCSPH step (wcsph.cu)
struct SnapState;  // text snapshots in flight (snapshot.cu)

struct Ctx {
    bsc_params P{};
    KParams K{};
    cudaStream_t stream = nullptr;
    int device = 0;
    std::string err;
    double t = 0.0, dt = 0.0, umax = 0.0, numax = 0.0, dtsol = 0.0;
    int solsteps = 1;
    int64_t n = 0, cap = 0, ns = 0;
    int64_t launches = 0;
    int64_t cellshifts = 0;
    bool have_lists = false, have_csr = false, have_state = false;
    bool mixed = false;

    State S{}, S2{};           // S2: gather target of the Morton reorder
    std::vector<void*> allocs; // buffers sized by the particle count
    std::vector<void*> pallocs; // porosity field and solids

    // cell list
    int ncell = 0;
    int32_t *cell_start = nullptr, *cell_count = nullptr, *cell_rank = nullptr, *cell_tmp = nullptr;
    int32_t *pcell = nullptr, *pslot = nullptr, *sorted = nullptr;
    int32_t *scan_part = nullptr;
    // positions as float offsets from the origin of their own cell (the FP32
    // pre-test of the pair searches); fluid/wall particles and solids
    float2* posf = nullptr;
    double* lstage = nullptr;  // 4n: the interleaved L of the host state view, on the device
    float2* sposf = nullptr;
    float* swf = nullptr;         // solids' (1 - n_s) V_s in FP32 (the mixed path's porosity sum)
    // mixed path: FP32 twins of per-particle fields read per pair by the FP32
    // pair sums, written once per particle by each stage's prologue kernel
    // (an FP64 -> FP32 conversion runs on GB300's FP64 pipe: per pair it costs
    // as much as an FP64 add)
    float *f_vol = nullptr, *f_nu = nullptr, *f_nut = nullptr, *f_tke = nullptr, *f_varts = nullptr,
          *f_q = nullptr;
    // the low part of V as a double-float {f_vol, f_vol_lo}, beside f_vol
    float* f_vol_lo = nullptr;
    // u = v/n as double-floats (hi x, lo x, hi y, lo y): eddyvis and varts
    // take their velocity differences from them on the FP32 pipe
    float4* udf = nullptr;
    // solids: their own cell list, static after upload
    double *sx = nullptr, *sy = nullptr, *svol = nullptr, *spor = nullptr;
    int32_t *scell_start = nullptr, *scell_count = nullptr;
    double* pgrid = nullptr;
    std::vector<double> hpgrid;   // host copy of the porosity field
    bool solids_dirty = true;     // solid cell list needs a rebuild
    double grid_x0 = 0.0, grid_y0 = 0.0;

    // neighbour lists
    int32_t* nbr = nullptr;
    double2* gw = nullptr;        // FP64 grad W (the FP64 path; the mixed path's FP64 assembly variants)
    double* ndist = nullptr;      // pair distance per slot (salinity: scalart's radial)
    double* sdisp = nullptr;      // salinity: D_x, D_y, Dm + nu_t/Sc, 1/n per particle (4n)
    // mixed path: grad W as a double-float, {gwf, gwl} (gwf alone is its FP32
    // rounding, which the FP32 pair sums read)
    float2* gwf = nullptr;
    float2* gwl = nullptr;
    float2* asm_df = nullptr;     // mixed assembly: five per-particle double-float inputs
    float4* posd = nullptr;       // mixed search: offsets to the cell origin as double-floats
    bool asm_rcp = false;         // mixed assembly in FP64 with Newton reciprocals (BSC_ASSEMBLY=rcp)
    bool nb_warpcell = false;     // BSC_NEIGHBOUR=warpcell: warp-per-cell candidate phase
    int32_t* cand_nc = nullptr;   // its survivors per row (-1: one-pass loop)
    int32_t* cnt = nullptr;
    int32_t* d_flag = nullptr;    // device error flags (capacity, nonfinite)
    int32_t* h_flag = nullptr;    // pinned mirror

    // PPE
    double* aval = nullptr;       // FP64 off-diagonals (ELL layout)
    int2* ellf = nullptr;         // FP32 off-diagonals with their columns, packed (mixed)
    uint32_t* ellh = nullptr;     // FP16 off-diagonals with 16-bit column offsets (mixed V-cycle)
    uint8_t* ellh_ok = nullptr;   // per 32-row slice: every offset fits 16 bits
    __half* avalh = nullptr;      // FP16 off-diagonals (mixed): the V-cycle's fine-level sweeps
    double* b = nullptr;
    float* bf = nullptr;
    // Krylov work (FP64) and (FP32)
    double *r = nullptr, *rh = nullptr, *pd = nullptr, *v = nullptr, *s = nullptr, *tv = nullptr, *xw = nullptr;
    float *rf = nullptr, *rhf = nullptr, *pf = nullptr, *vf = nullptr, *sf = nullptr, *tf = nullptr, *xf = nullptr;
    float* xbf = nullptr;         // best inner iterate (mixed)
    float* Zf = nullptr;          // FGMRES-IR preconditioned vectors, ir_m x cap (mixed)
    Scalars* sc2 = nullptr;       // FGMRES-IR outer scalars (h_sc[1] mirrors them)
    unsigned* ticket = nullptr;   // last-block counter of the Krylov reductions (kept at 0 between launches)
    int ir_m = 0;
    // instantiated CUDA graphs of one batch of Krylov iterations, keyed by
    // the operator and vectors they were captured with
    struct GraphEntry {
        const void* k0;
        const void* k1;
        const void* k2;
        int64_t n;
        cudaGraphExec_t exec;
        int64_t kernels = 0;      // kernels in the graph (counted at capture)
    };
    std::vector<GraphEntry> graphs;
    bool use_graphs = true;
    bool capturing = false;       // a graph capture of the context stream is open
    bool debug = false;           // BSC_DEBUG=1: per-sweep solver trace on stderr
    int spmv_unroll = 1;          // four ELL entries per round (BSC_SPMV_UNROLL=0: one)
    bool prof_iter = false;       // BSC_PROFILE_ITER=1: events around each Krylov kernel
    int mg_tail_cells = -1;       // BSC_MG_TAIL=<cells>: largest level in the single-CTA tail
    double mg_w[2] = {0.82, 0.82};  // smoother weights: the first sweep of a pre/post pair, the later ones
    // post-sweeps on the cell levels and on the particle level (0:
    // mg_sweeps) and the first post-sweep's weight (0: mg_w[0]); pre-sweeps
    // on the particle level (0: mg_sweeps).  BSC_MG_POST=<coarse>,<fine>[,<w>]
    // and BSC_MG_PRE=<n> set them (one sweep fewer on the particle level
    // speeds up 20-step windows but costs as much in iterations over a
    // 2000-step run, so the default keeps mg_sweeps everywhere)
    int mg_post[2] = {0, 0};
    int mg_pre_fine = 0;
    double mg_wpost = 0.0;
    bool mg_post_fused = true;  // a cell level's two post-sweeps in one launch (BSC_MG_POST_FUSED=0: two)
    bool mg_cell4 = false;      // BSC_MG_CELL_SWEEPS=4: four sweeps each way on the per-level cell levels
    bool exact_div = false;       // BSC_EXACT_DIV=1: IEEE divisions in the mixed path's FP64 assembly
    cudaEvent_t ev_it[6] = {};
    double* V = nullptr;          // FGMRES basis (m+1) x cap, FP64
    float* Vf = nullptr;          // FGMRES basis FP32 (mixed)
    double* Hd = nullptr;         // Hessenberg + Givens + y on device
    double* part = nullptr;       // reduction partials RED_GRID x 64
    Scalars* sc = nullptr;
    Scalars* h_sc = nullptr;      // pinned mirror
    Scalars* h_it = nullptr;      // pinned: scalars after the last two queued FGMRES iterations, by parity
    cudaEvent_t ev_lag[2] = {};   // end of the last two queued FGMRES iterations, by parity
    // host<->device state copies spread over several streams (several copy
    // engines at once), forked from and joined back into `stream`
    WcState* wc = nullptr;        // WCSPH forward/adjoint state, after bsc_wcsph_setup
    SnapState* snap = nullptr;    // snapshot staging and its writer thread
    int64_t cap_hint = 0;         // the next allocation's capacity (particle insertion headroom)
    static constexpr int NCOPY = 4;
    cudaStream_t copy_stream[NCOPY] = {};
    cudaEvent_t copy_ev[NCOPY + 1] = {};
    int fg_m = 0;

    // timing: stage events recorded on the stream, resolved lazily
    static constexpr int EVPOOL = 256;
    cudaEvent_t evs[2 * EVPOOL] = {};
    int ev_slot[EVPOOL] = {};
    int ev_used = 0;
    double ms[BSC_TIMING_SLOTS] = {0};
    int64_t calls[BSC_TIMING_SLOTS] = {0};
    bool timing = true;
    // around one SpMV per Krylov batch (pair 0); pairs 1 and 2: the SpMV of
    // the multigrid FGMRES iterations, by iteration parity
    cudaEvent_t ev_spmv[6] = {};
    double* stepsc = nullptr;     // device: umax, numax (timestep reductions)
    Mg mg;                        // multigrid preconditioner of the PPE (mg.cu)
};

void timing_flush(Ctx* c);

// an event on the context stream; inside a graph capture it becomes an
// external event node, so it is recorded on every replay and stays timeable
inline void record_event(Ctx* c, cudaEvent_t e) {
    if (c->capturing)
        cudaEventRecordWithFlags(e, c->stream, cudaEventRecordExternal);
    else
        cudaEventRecord(e, c->stream);
}

// destroy the cached graphs (their kernels hold pointers that are about to change)
void drop_graphs(Ctx* c);


// ---- stage timer: a pair of CUDA events on the context stream -----------------
struct StageTimer {
    Ctx* c;
    int k = -1;
    StageTimer(Ctx* c_, int slot) : c(c_) {
        if (!c->timing) return;
        if (c->ev_used == Ctx::EVPOOL) timing_flush(c);
        k = c->ev_used++;
        c->ev_slot[k] = slot;
        cudaEventRecord(c->evs[2 * k], c->stream);
    }
    ~StageTimer() {
        if (k >= 0) cudaEventRecord(c->evs[2 * k + 1], c->stream);
    }
};

// ---- module entry points (implemented in the .cu files) -----------------------
// cells.cu
int cells_build(Ctx* c, bool allow_reorder);
int scan_exclusive(Ctx* c, const int32_t* in, int32_t* out, int n);
// every FP64 field of a State, for kernels that move whole particles
struct FieldPtrs {
    double* d[N_DBL_FIELDS];
};
FieldPtrs fields_of(State& s);
int solids_build(Ctx* c);
int op_projection(Ctx* c);
int op_piston(Ctx* c);
int op_comp_pos(Ctx* c);
// pairs.cu
int op_neighbour(Ctx* c);
int op_freesurf(Ctx* c);
int op_effpor(Ctx* c);
int op_eddyvis(Ctx* c);
int op_int_vel(Ctx* c, const double* d_umax);
int op_comp_vel(Ctx* c);
int op_opt2_shift(Ctx* c);
int op_scalart(Ctx* c);
int op_scalarupdate(Ctx* c, double stime);
int op_densityupdate(Ctx* c);
int op_timestep_reduce(Ctx* c);
int op_probe_eta(Ctx* c, int np, const double* xp, double depth, double* eta);
// ppe.cu
int op_ppe_assemble(Ctx* c);
int op_ppe_solve(Ctx* c, bsc_solve_info* info);
// multigrid: build the hierarchy for the assembled PPE; apply one V-cycle
// z = M v to an FP64 vector (FP64 or FP32 arithmetic); release the buffers
int mg_setup(Ctx* c);
void wc_free(Ctx* c);
void snap_free(Ctx* c);
int mg_vcycle_f64(Ctx* c, const double* v, double* z);
int mg_vcycle_f32(Ctx* c, const float* v, float* z);
void mg_free(Ctx* c);
int fg_layout_size(int m);
int csr_solve_device(Ctx* c, int32_t n, const int32_t* rp, const int32_t* col, const double* val,
                     const double* b, double* x, bsc_solve_info* info);

// per-particle-count buffers: freed and re-made when the count changes
template <typename T>
int dalloc(Ctx* c, T** p, int64_t count) {
    void* q = nullptr;
    size_t bytes = (size_t)(count > 0 ? count : 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaMalloc");
    c->allocs.push_back(q);
    *p = (T*)q;
    return BSC_OK;
}

// buffers that outlive a state re-upload (porosity field, solids): replaced
// in place when uploaded again, freed at destroy
template <typename T>
int palloc(Ctx* c, T** p, int64_t count) {
    if (*p) {
        cudaStreamSynchronize(c->stream);
        cudaFree(*p);
        for (auto& q : c->pallocs)
            if (q == (void*)*p) q = nullptr;
        *p = nullptr;
    }
    void* q = nullptr;
    size_t bytes = (size_t)(count > 0 ? count : 1) * sizeof(T);
    cudaError_t e = cudaMalloc(&q, bytes);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaMalloc");
    c->pallocs.push_back(q);
    *p = (T*)q;
    return BSC_OK;
}

}  // namespace bsc
