// cells.cu -- cell list (cellshift/resetid), Morton reorder, O(N) updates.
//
// The reference keeps particles in per-cell slot lists and migrates them one
// cell at a time through eight transfer queues (integrator.f90:32-391), then
// renumbers them serially (resetid, isph.f90:88-113).  Here the whole list is
// rebuilt by a counting sort every cell shift: one key per particle, an
// atomic histogram, an exclusive scan over cells taken in Morton order, a
// scatter, and a per-cell sort of the slots so the order inside a cell is
// deterministic.  Every `reorder_every` shifts the state itself is gathered
// into that order (the "Morton reorder"), so neighbours sit close in memory.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>

#include "bsc_internal.cuh"

namespace bsc {

__host__ __device__ inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// cell of a point: floor((x - x0) / cs) clamped to the grid; NaN -> cell 0
__host__ __device__ inline int cell_coord(double v, double v0, double inv, int nmax) {
    double f = floor((v - v0) * inv);
    if (!(f == f)) return 0;
    if (f < 0.0) return 0;
    if (f > (double)(nmax - 1)) return nmax - 1;
    return (int)f;
}

__global__ void k_bin(int64_t n, const double* __restrict__ x, const double* __restrict__ y, double gx0,
                      double gy0, double inv_cs, int nx, int ny, int32_t* __restrict__ pcell,
                      int32_t* __restrict__ pslot, int32_t* __restrict__ cell_count, int32_t* __restrict__ flag) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double xi = x[i], yi = y[i];
    if (!(isfinite(xi) && isfinite(yi))) atomicOr(flag, 2);
    int cx = cell_coord(xi, gx0, inv_cs, nx);
    int cy = cell_coord(yi, gy0, inv_cs, ny);
    int c = cx * ny + cy;
    pcell[i] = c;
    pslot[i] = atomicAdd(&cell_count[c], 1);
}

// ---- exclusive scan of int32 (4096 elements per block) -----------------------
constexpr int SCAN_T = 1024, SCAN_PER = 4, SCAN_TILE = SCAN_T * SCAN_PER;

__device__ inline int block_exclusive_scan(int v, int* total) {
    __shared__ int wsum[SCAN_T / 32];
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int inc = v;
    for (int o = 1; o < 32; o <<= 1) {
        int t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        int s = (lane < SCAN_T / 32) ? wsum[lane] : 0;
        int si = s;
        for (int o = 1; o < 32; o <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, si, o);
            if (lane >= o) si += t;
        }
        if (lane < SCAN_T / 32) wsum[lane] = si - s;
        if (lane == 31) wsum[0] = wsum[0];  // keep
        if (lane == SCAN_T / 32 - 1) *total = si;
    }
    __syncthreads();
    return inc - v + wsum[w];
}

__global__ void k_scan_tile(const int32_t* __restrict__ in, int32_t* __restrict__ out, int32_t* __restrict__ part,
                            int n) {
    __shared__ int tot;
    int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_PER;
    int v[SCAN_PER], s = 0;
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        v[k] = (base + k < n) ? in[base + k] : 0;
        s += v[k];
    }
    int ex = block_exclusive_scan(s, &tot);
#pragma unroll
    for (int k = 0; k < SCAN_PER; ++k) {
        if (base + k < n) out[base + k] = ex;
        ex += v[k];
    }
    if (threadIdx.x == 0 && part) part[blockIdx.x] = tot;
}

__global__ void k_scan_add(int32_t* __restrict__ out, const int32_t* __restrict__ part, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += part[i / SCAN_TILE];
}

int scan_exclusive(Ctx* c, const int32_t* in, int32_t* out, int n) {
    int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb > SCAN_TILE) return set_err(c, BSC_E_CAPACITY, "scan: too many cells");
    k_scan_tile<<<nb, SCAN_T, 0, c->stream>>>(in, out, c->scan_part, n);
    BSC_LAUNCH(c);
    if (nb > 1) {
        k_scan_tile<<<1, SCAN_T, 0, c->stream>>>(c->scan_part, c->scan_part, nullptr, nb);
        BSC_LAUNCH(c);
        k_scan_add<<<blocks_for(n, 256), 256, 0, c->stream>>>(out, c->scan_part, n);
        BSC_LAUNCH(c);
    }
    return BSC_OK;
}

__global__ void k_to_rank(int ncell, const int32_t* __restrict__ rank, const int32_t* __restrict__ cnt,
                          int32_t* __restrict__ tmp) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncell) tmp[rank[c]] = cnt[c];
}

__global__ void k_from_rank(int ncell, const int32_t* __restrict__ rank, const int32_t* __restrict__ tmp,
                            int32_t* __restrict__ start) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c < ncell) start[c] = tmp[rank[c]];
}

__global__ void k_place(int64_t n, const int32_t* __restrict__ pcell, const int32_t* __restrict__ pslot,
                        const int32_t* __restrict__ start, int32_t* __restrict__ sorted) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < n) sorted[start[pcell[i]] + pslot[i]] = (int32_t)i;
}

// insertion sort of each cell's slots: in-cell order = ascending slot index
__global__ void k_sort_cells(int ncell, const int32_t* __restrict__ start, const int32_t* __restrict__ cnt,
                             int32_t* __restrict__ sorted) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    int s = start[c], m = cnt[c];
    for (int a = 1; a < m; ++a) {
        int v = sorted[s + a], b = a - 1;
        while (b >= 0 && sorted[s + b] > v) {
            sorted[s + b + 1] = sorted[s + b];
            --b;
        }
        sorted[s + b + 1] = v;
    }
}


__global__ void k_gather_state(int64_t n, const int32_t* __restrict__ perm, FieldPtrs src, FieldPtrs dst,
                               const int8_t* __restrict__ tid_s, int8_t* __restrict__ tid_d,
                               const uint8_t* __restrict__ fl_s, uint8_t* __restrict__ fl_d,
                               const int32_t* __restrict__ id_s, int32_t* __restrict__ id_d,
                               const int32_t* __restrict__ pc_s, int32_t* __restrict__ pc_d) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    int j = perm[k];
#pragma unroll
    for (int f = 0; f < N_DBL_FIELDS; ++f) dst.d[f][k] = src.d[f][j];
    tid_d[k] = tid_s[j];
    fl_d[k] = fl_s[j];
    id_d[k] = id_s[j];
    pc_d[k] = pc_s[j];
}

__global__ void k_iota(int64_t n, int32_t* __restrict__ a) {
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k < n) a[k] = (int32_t)k;
}

FieldPtrs fields_of(State& s) {
    FieldPtrs f;
    double* a[N_DBL_FIELDS] = {s.x, s.y, s.vx, s.vy, s.xs, s.ys, s.vxs, s.vys, s.p, s.rho, s.oden, s.mass, s.por,
                               s.gradvx, s.nut, s.tke, s.resist, s.varts, s.vel, s.xrest, s.vol, s.L0, s.L1, s.L2,
                               s.L3, s.con, s.ovol, s.cdiff};
    for (int k = 0; k < N_DBL_FIELDS; ++k) f.d[k] = a[k];
    return f;
}

// Rebuild the cell list; with `allow_reorder` the state is gathered into
// cell order when the reorder period is due (always on the first build).
int cells_build(Ctx* c, bool allow_reorder) {
    const int64_t n = c->n;
    const KParams& K = c->K;
    BSC_CUDA(c, cudaMemsetAsync(c->cell_count, 0, sizeof(int32_t) * c->ncell, c->stream));
    k_bin<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, c->S.x, c->S.y, K.gx0, K.gy0, 1.0 / K.cs, K.nx, K.ny,
                                                    c->pcell, c->pslot, c->cell_count, c->d_flag);
    BSC_LAUNCH(c);
    k_to_rank<<<blocks_for(c->ncell, 256), 256, 0, c->stream>>>(c->ncell, c->cell_rank, c->cell_count, c->cell_tmp);
    BSC_LAUNCH(c);
    int rc = scan_exclusive(c, c->cell_tmp, c->cell_tmp, c->ncell);
    if (rc) return rc;
    k_from_rank<<<blocks_for(c->ncell, 256), 256, 0, c->stream>>>(c->ncell, c->cell_rank, c->cell_tmp, c->cell_start);
    BSC_LAUNCH(c);
    k_place<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, c->pcell, c->pslot, c->cell_start, c->sorted);
    BSC_LAUNCH(c);
    k_sort_cells<<<blocks_for(c->ncell, 128), 128, 0, c->stream>>>(c->ncell, c->cell_start, c->cell_count, c->sorted);
    BSC_LAUNCH(c);
    c->cellshifts++;
    const int every = c->P.reorder_every > 0 ? c->P.reorder_every : 1;
    if (allow_reorder && (c->cellshifts == 1 || (c->cellshifts - 1) % every == 0)) {
        StageTimer tm(c, BSC_T_REORDER);
        k_gather_state<<<blocks_for(n, 256), 256, 0, c->stream>>>(
            n, c->sorted, fields_of(c->S), fields_of(c->S2), c->S.tid, c->S2.tid, c->S.flags, c->S2.flags, c->S.id,
            c->S2.id, c->pcell, c->pslot);
        BSC_LAUNCH(c);
        std::swap(c->S, c->S2);
        std::swap(c->pcell, c->pslot);  // pslot now holds the gathered cells
        k_iota<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, c->sorted);
        BSC_LAUNCH(c);
    }
    c->have_lists = false;
    return BSC_OK;
}

// solids: static, sorted by cell on the host once
int solids_build(Ctx* c) {
    if (!c->solids_dirty) return BSC_OK;
    c->solids_dirty = false;
    const KParams& K = c->K;
    const int64_t ns = c->ns;
    std::vector<double> hx(ns), hy(ns), hv(ns), hp(ns);
    BSC_D2H(c, hx.data(), c->sx, sizeof(double) * ns);
    BSC_D2H(c, hy.data(), c->sy, sizeof(double) * ns);
    BSC_D2H(c, hv.data(), c->svol, sizeof(double) * ns);
    BSC_D2H(c, hp.data(), c->spor, sizeof(double) * ns);
    std::vector<int32_t> key(ns), ord(ns);
    const double inv = 1.0 / K.cs;
    for (int64_t k = 0; k < ns; ++k)
        key[k] = cell_coord(hx[k], K.gx0, inv, K.nx) * K.ny + cell_coord(hy[k], K.gy0, inv, K.ny);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return key[a] < key[b]; });
    std::vector<int32_t> start(c->ncell, 0), count(c->ncell, 0);
    for (int64_t k = 0; k < ns; ++k) count[key[k]]++;
    for (int q = 1; q < c->ncell; ++q) start[q] = start[q - 1] + count[q - 1];
    std::vector<double> sx2(ns), sy2(ns), sv2(ns), sp2(ns);
    std::vector<float2> so(ns);
    std::vector<float> sw(ns);
    for (int64_t k = 0; k < ns; ++k) {
        sx2[k] = hx[ord[k]]; sy2[k] = hy[ord[k]]; sv2[k] = hv[ord[k]]; sp2[k] = hp[ord[k]];
        sw[k] = (float)((1.0 - sp2[k]) * sv2[k]);
        const int cxk = key[ord[k]] / K.ny, cyk = key[ord[k]] % K.ny;
        so[k] = make_float2((float)(sx2[k] - (K.gx0 + cxk * K.cs)), (float)(sy2[k] - (K.gy0 + cyk * K.cs)));
    }
    BSC_H2D(c, c->sposf, so.data(), sizeof(float2) * ns);
    BSC_H2D(c, c->swf, sw.data(), sizeof(float) * ns);
    BSC_H2D(c, c->sx, sx2.data(), sizeof(double) * ns);
    BSC_H2D(c, c->sy, sy2.data(), sizeof(double) * ns);
    BSC_H2D(c, c->svol, sv2.data(), sizeof(double) * ns);
    BSC_H2D(c, c->spor, sp2.data(), sizeof(double) * ns);
    BSC_H2D(c, c->scell_start, start.data(), sizeof(int32_t) * c->ncell);
    BSC_H2D(c, c->scell_count, count.data(), sizeof(int32_t) * c->ncell);
    return BSC_OK;
}

// ---- isph.f90:16-47 projection ------------------------------------------------
__global__ void k_projection(int64_t n, State S, double dt) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (S.tid[i] == BSC_TID_FLUID && !(S.flags[i] & BSC_FLAG_DEAD)) {
        double n_ = S.por[i];
        double x = S.x[i], y = S.y[i];
        S.xs[i] = x;
        S.x[i] = x + (dt * S.vx[i] / n_);
        S.ys[i] = y;
        S.y[i] = y + (dt * S.vy[i] / n_);
    }
}

int op_projection(Ctx* c) {
    k_projection<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, c->dt);
    BSC_LAUNCH(c);
    return BSC_OK;
}

// ---- wavemaker (greenfield) -----------------------------------------------------
__global__ void k_piston(int64_t n, State S, double xp, double vp) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (S.flags[i] & BSC_FLAG_PISTON) {
        S.x[i] = S.xrest[i] + xp;
        S.vx[i] = vp;
        S.vxs[i] = vp;
        S.vy[i] = 0.0;
        S.vys[i] = 0.0;
    }
}

// x_p(t) = s0 + r(t) (s(t) - s0) with s(t) = sum_k a_k sin(w_k t + phi_k),
// s0 = s(0) and the ramp r(t) = (1 - cos(pi t / ramp)) / 2 (1 after it): the
// ramp takes the stroke from its starting value, so a stroke whose phases
// put it away from zero at t = 0 starts at rest too (the wall's rest
// coordinate carries -s0)
int op_piston(Ctx* c) {
    const bsc_params& P = c->P;
    double s = 0, ds = 0, s0 = 0;
    for (int k = 0; k < P.piston_modes && k < BSC_MAX_PISTON_MODES; ++k) {
        double w = 2.0 * M_PI / P.piston_period[k];
        s += P.piston_amp[k] * std::sin(w * c->t + P.piston_phase[k]);
        ds += P.piston_amp[k] * w * std::cos(w * c->t + P.piston_phase[k]);
        s0 += P.piston_amp[k] * std::sin(P.piston_phase[k]);
    }
    double r = 1.0, dr = 0.0;
    if (P.piston_ramp > 0.0 && c->t < P.piston_ramp) {
        r = 0.5 * (1.0 - std::cos(M_PI * c->t / P.piston_ramp));
        dr = 0.5 * M_PI / P.piston_ramp * std::sin(M_PI * c->t / P.piston_ramp);
    }
    k_piston<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, s0 + r * (s - s0), dr * (s - s0) + r * ds);
    BSC_LAUNCH(c);
    return BSC_OK;
}

// ---- integrator.f90:867-906 comp_pos ---------------------------------------------
__global__ void k_comp_pos(int64_t n, State S, double dt, double bxmin, double bxmax) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint8_t f = S.flags[i];
    if (S.tid[i] == BSC_TID_FLUID && !(f & BSC_FLAG_DEAD)) {
        double n_ = S.por[i];
        double x = (S.x[i] + S.xs[i] + dt * S.vx[i] / n_) / 2.0;
        S.x[i] = x;
        S.y[i] = (S.y[i] + S.ys[i] + dt * S.vy[i] / n_) / 2.0;
        if ((f & BSC_FLAG_BUFFER) && x > bxmin && x < bxmax) S.flags[i] = f & (uint8_t)~BSC_FLAG_BUFFER;
    }
}

int op_comp_pos(Ctx* c) {
    k_comp_pos<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, c->dt, c->K.bxmin, c->K.bxmax);
    BSC_LAUNCH(c);
    return BSC_OK;
}

}  // namespace bsc
