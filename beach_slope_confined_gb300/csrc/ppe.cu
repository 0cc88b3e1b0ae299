// ppe.cu -- pressure Poisson equation: assembly, SpMV, Krylov solvers.
//
// Assembly follows isph.f90:115-456 row by row: fluid rows use the row
// particle's corrected gradient, ghost (tid 2) rows couple to walls only with
// the raw gradient, fixed-wall (tid 1) rows use each fluid neighbour's
// correction matrix and the row particle's m/rho; free-surface rows weight the
// diagonal contributions of fluid neighbours by 1 + oden_j/(rho0*rel_den).
// Each row is divided by its diagonal (the Jacobi scaling of :434-442), so the
// stored matrix is I + N with N's values in the neighbour-list layout.
//
// Solvers: BiCGSTAB (the update order of solver.f90:163-213) and restarted
// FGMRES(m) (the public algorithm behind the MKL call of solver.f90:319-343)
// with classical Gram-Schmidt and one re-orthogonalisation pass.  All scalars
// live on the device; each kernel starts by checking the `done` flag so the
// host can queue a batch of iterations and test convergence once per batch.
// Reductions are two-stage with a fixed grid, hence deterministic.
//
// Mixed precision: the matrix is assembled in FP64 in both paths and the
// mixed path keeps an FP32 copy of it.  Its solve is FGMRES-IR: a flexible
// GMRES outer loop in FP64 (true residual b - A x in FP64) whose
// preconditioner is a short FP32 BiCGSTAB sweep with FP64 dot products; a
// breakdown of BiCGSTAB restarts it from the current iterate.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "bsc_internal.cuh"
#include "dfloat.cuh"
#include "ellop.cuh"

namespace bsc {

// ============================================================================
// assembly
// ============================================================================
// FAST (the mixed path): the per-pair and per-row quotients by rcp_nr, a
// Newton-Raphson reciprocal within ~2^-46 of the FP64 quotient.  The FP64
// path divides (correctly rounded, as the reference).
template <typename R, bool FAST>
__global__ void __launch_bounds__(NB_BLOCK) k_assemble(int64_t n, State S, KParams K, const int32_t* __restrict__ nbr,
                                                        const typename Vec2<R>::type* __restrict__ gw,
                                                        const int32_t* __restrict__ cnt, R* __restrict__ aval,
                                                        int2* __restrict__ ellf, __half* __restrict__ avalh,
                                                        double* __restrict__ b, const double* __restrict__ q,
                                                        const double* __restrict__ usx, const double* __restrict__ usy,
                                                        double dt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int tid_i = S.tid[i];
    const bool free_i = S.flags[i] & BSC_FLAG_FREE;
    const double xi = S.x[i], yi = S.y[i];
    const R ni = (R)S.por[i], qi = (R)q[i];
    const R L0 = (R)S.L0[i], L1 = (R)S.L1[i], L2 = (R)S.L2[i], L3 = (R)S.L3[i];
    const double usxi = usx[i], usyi = usy[i];
    auto quot = [](double a, double d) -> double { return FAST ? a * rcp_nr(d) : a / d; };
    const R mi_over_rhoi = (R)quot(S.mass[i], S.rho[i]);
    const R lamp_f = (R)(1.0 / (K.rho0 * K.rel_den));
    // per-row quotients hoisted out of the pair loop (FP64 divisions are
    // expensive on this GPU): 1/n_i, and v*_i/n_i for the fixed-wall rows
    const R inv_ni = (R)quot(1.0, ni);
    const double vxi_n = quot(S.vxs[i], (double)ni), vyi_n = quot(S.vys[i], (double)ni);
    const int m = cnt[i];
    R dia = 0, fv = 0;
    for (int k = 0; k < m; ++k) {
        const int64_t e = ell(i, k, K.kmax);
        const int j = nbr[e];
        const auto g = gw[e];
        const int tid_j = S.tid[j];
        const double dx = xi - S.x[j], dy = yi - S.y[j];
        const R p_dist = (R)quot(1.0, (R)(dx * dx + dy * dy) + (R)K.lam);
        const R pvol = (R)S.vol[j];
        R val = 0;
        if (tid_i == BSC_TID_FLUID) {
            const R lamp = (free_i && tid_j == BSC_TID_FLUID) ? (R)1 + (R)S.oden[j] * lamp_f : (R)1;
            const R gx = L0 * g.x + L1 * g.y, gy = L2 * g.x + L3 * g.y;
            const R t = (R)2 * pvol * ((R)dx * gx + (R)dy * gy) * p_dist;
            val = -t;
            dia += t * lamp;
            // divergence of the porous-weighted predicted velocity (:241-270)
            R ddx, ddy;
            if (tid_j == BSC_TID_FLUID) {
                // 2 rho_i rho_j / (n_i n_j (rho_i/n_i + rho_j/n_j)) = 2 q_i q_j / (q_i + q_j)
                const R qj = (R)q[j];
                const R rho_ij = (R)quot((R)2 * qi * qj, qi + qj);
                ddx = rho_ij * (R)(usx[j] - usxi);
                ddy = rho_ij * (R)(usy[j] - usyi);
            } else {
                ddx = qi * ((R)(S.vxs[j] - S.vxs[i]) * inv_ni);
                ddy = qi * ((R)(S.vys[j] - S.vys[i]) * inv_ni);
            }
            fv += pvol * (ddx * gx + ddy * gy);
        } else if (tid_i == BSC_TID_GHOST) {
            if (tid_j <= 2) {
                const R t = (R)2 * pvol * ((R)dx * g.x + (R)dy * g.y) * p_dist;
                val = -t;
                dia += t;
            }
        } else if (tid_i == BSC_TID_WALL) {
            if (tid_j == BSC_TID_FLUID) {
                const R Lj0 = (R)S.L0[j], Lj1 = (R)S.L1[j], Lj2 = (R)S.L2[j], Lj3 = (R)S.L3[j];
                const R gx = Lj0 * g.x + Lj1 * g.y, gy = Lj2 * g.x + Lj3 * g.y;
                const R t = (R)2 * mi_over_rhoi * ((R)dx * gx + (R)dy * gy) * p_dist;
                val = -t;
                dia += t;
                const R qj = (R)q[j];
                const R ddx = qj * (R)(usx[j] - vxi_n);
                const R ddy = qj * (R)(usy[j] - vyi_n);
                fv += mi_over_rhoi * (ddx * gx + ddy * gy);
            } else {
                const R t = (R)2 * pvol * ((R)dx * g.x + (R)dy * g.y) * p_dist;
                val = -t;
                dia += t;
            }
        }
        aval[e] = val;
    }
    const double d = (double)dia;
    if (d == 0.0 || !isfinite(d)) {
        // zero-neighbour guard: identity row, b = 0 (the reference divides by 0)
        for (int k = 0; k < m; ++k) {
            aval[ell(i, k, K.kmax)] = 0;
            if (ellf) ellf[ell(i, k, K.kmax)] = make_int2(nbr[ell(i, k, K.kmax)], 0);
            if (avalh) avalh[ell(i, k, K.kmax)] = __float2half_rn(0.f);
        }
        b[i] = 0.0;
        return;
    }
    const R inv = (R)(1.0 / d);
    for (int k = 0; k < m; ++k) {
        const int64_t e = ell(i, k, K.kmax);
        const R v = aval[e] * inv;
        aval[e] = v;
        if (ellf) {  // the mixed path's inner-sweep copy (rounded on the integer pipe) and V-cycle copy
            const float vf = f32_of(v);
            ellf[e] = make_int2(nbr[e], __float_as_int(vf));
            avalh[e] = __float2half_rn(vf);
        }
    }
    b[i] = ((double)fv / dt) / d;
}

// ---- the mixed path's assembly in double-float arithmetic (dfloat.cuh) -------------
// The same coefficients as k_assemble (isph.f90:115-456, every row type),
// with the pair arithmetic on FP32 pairs of ~48 bits instead of FP64: the
// FP64 pipe, this kernel's bound on this GPU, is left with the two velocity
// differences (formed exactly in FP64, then split), the split of grad W and
// the widening of each entry, seven operations a pair instead of about
// thirty-four.  Positions enter as offsets from the particle's own cell
// origin, split once per particle: a coordinate of ~1 m split into two
// floats keeps ~2^-48 m, which would cost the pair offset (~1e-3 m) about
// 1e-12 of its accuracy; the offset keeps ~2^-48 of a cell.
//
// Per particle (k_asm_df_pre): offsets ox, oy from the cell origin, V = m/rho,
// q = rho/n and the free-surface factor 1 + oden/(rho0 rel_den), as
// double-floats, array by array.
__global__ void k_asm_df_pre(int64_t n, State S, KParams K, const int32_t* __restrict__ pcell,
                             const double* __restrict__ q, float2* __restrict__ pre) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = pcell[i], cx = c / K.ny, cy = c - cx * K.ny;
    pre[i] = df_pack(df_of(S.x[i] - (K.gx0 + cx * K.cs)));
    pre[n + i] = df_pack(df_of(S.y[i] - (K.gy0 + cy * K.cs)));
    pre[2 * n + i] = df_pack(df_of(S.vol[i]));
    pre[3 * n + i] = df_pack(df_of(q[i]));
    pre[4 * n + i] = df_pack(df_of(1.0 + S.oden[i] * (1.0 / (K.rho0 * K.rel_den))));
}

__global__ void __launch_bounds__(NB_BLOCK) k_assemble_df(int64_t n, State S, KParams K,
                                                           const int32_t* __restrict__ nbr,
                                                           const float2* __restrict__ gwf,
                                                           const float2* __restrict__ gwl,
                                                           const int32_t* __restrict__ cnt,
                                                           const int32_t* __restrict__ pcell,
                                                           const float2* __restrict__ pre, double* __restrict__ aval,
                                                           int2* __restrict__ ellf, __half* __restrict__ avalh,
                                                           double* __restrict__ b, const double* __restrict__ q,
                                                           const double* __restrict__ usx,
                                                           const double* __restrict__ usy, double dt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2* __restrict__ pox = pre;
    const float2* __restrict__ poy = pre + n;
    const float2* __restrict__ pvl = pre + 2 * n;
    const float2* __restrict__ pq = pre + 3 * n;
    const float2* __restrict__ plamp = pre + 4 * n;
    float2* __restrict__ vdf = reinterpret_cast<float2*>(aval);  // entries between the two passes
    const int tid_i = S.tid[i];
    const bool free_i = S.flags[i] & BSC_FLAG_FREE;
    const int ci = pcell[i], cxi = ci / K.ny, cyi = ci - cxi * K.ny;
    const df2 oxi = df_unpack(pox[i]), oyi = df_unpack(poy[i]);
    const df2 cs = df_of(K.cs), lam = df_of(K.lam);
    const double ni64 = S.por[i];
    const df2 qi = df_unpack(pq[i]);
    const df2 L0 = df_of(S.L0[i]), L1 = df_of(S.L1[i]), L2 = df_of(S.L2[i]), L3 = df_of(S.L3[i]);
    const double usxi = usx[i], usyi = usy[i];
    // fixed-wall rows: m_i/rho_i and v*_i/n_i; wall neighbours of fluid rows: 1/n_i
    const df2 mi_over_rhoi = df_mul(df_of(S.mass[i]), df_rcp(df_of(S.rho[i])));
    const df2 inv_ni = df_rcp(df_of(ni64));
    const double vxsi = S.vxs[i], vysi = S.vys[i];
    const double vxi_n = vxsi / ni64, vyi_n = vysi / ni64;
    const int m = cnt[i];
    df2 dia{0.0f, 0.0f}, fv{0.0f, 0.0f};
    for (int k = 0; k < m; ++k) {
        const int64_t e = ell(i, k, K.kmax);
        const int j = nbr[e];
        // grad W as the neighbour search left it, a double-float
        const float2 gh = gwf[e], gl = gwl[e];
        const df2 gxr{gh.x, gl.x}, gyr{gh.y, gl.y};
        const int tid_j = S.tid[j];
        const int cj = pcell[j], cxj = cj / K.ny, cyj = cj - cxj * K.ny;
        const df2 dx = df_pair_offset(oxi, pox[j], cxi - cxj, cs);
        const df2 dy = df_pair_offset(oyi, poy[j], cyi - cyj, cs);
        const df2 p_dist = df_rcp(df_add(df_add(df_sqr(dx), df_sqr(dy)), lam));
        const df2 pvol = df_unpack(pvl[j]);
        df2 val{0.0f, 0.0f};
        if (tid_i == BSC_TID_FLUID) {
            const df2 gx = df_add(df_mul(L0, gxr), df_mul(L1, gyr));
            const df2 gy = df_add(df_mul(L2, gxr), df_mul(L3, gyr));
            const df2 t = df_mul(df_mul(df_twice(pvol), df_add(df_mul(dx, gx), df_mul(dy, gy))), p_dist);
            val = df_neg(t);
            dia = df_add(dia, (free_i && tid_j == BSC_TID_FLUID) ? df_mul(t, df_unpack(plamp[j])) : t);
            // divergence of the porous-weighted predicted velocity (:241-270)
            df2 ddx, ddy;
            if (tid_j == BSC_TID_FLUID) {
                // 2 q_i q_j / (q_i + q_j), q = rho / n
                const df2 qj = df_unpack(pq[j]);
                const df2 rho_ij = df_mul(df_twice(df_mul(qi, qj)), df_rcp(df_add(qi, qj)));
                ddx = df_mul(rho_ij, df_of(usx[j] - usxi));
                ddy = df_mul(rho_ij, df_of(usy[j] - usyi));
            } else {
                ddx = df_mul(qi, df_mul(df_of(S.vxs[j] - vxsi), inv_ni));
                ddy = df_mul(qi, df_mul(df_of(S.vys[j] - vysi), inv_ni));
            }
            fv = df_add(fv, df_mul(pvol, df_add(df_mul(ddx, gx), df_mul(ddy, gy))));
        } else if (tid_i == BSC_TID_GHOST) {
            if (tid_j <= 2) {
                const df2 t = df_mul(df_mul(df_twice(pvol), df_add(df_mul(dx, gxr), df_mul(dy, gyr))), p_dist);
                val = df_neg(t);
                dia = df_add(dia, t);
            }
        } else if (tid_i == BSC_TID_WALL) {
            if (tid_j == BSC_TID_FLUID) {
                const df2 Lj0 = df_of(S.L0[j]), Lj1 = df_of(S.L1[j]), Lj2 = df_of(S.L2[j]), Lj3 = df_of(S.L3[j]);
                const df2 gx = df_add(df_mul(Lj0, gxr), df_mul(Lj1, gyr));
                const df2 gy = df_add(df_mul(Lj2, gxr), df_mul(Lj3, gyr));
                const df2 t =
                    df_mul(df_mul(df_twice(mi_over_rhoi), df_add(df_mul(dx, gx), df_mul(dy, gy))), p_dist);
                val = df_neg(t);
                dia = df_add(dia, t);
                // q_j (v*_j/n_j - v*_i/n_i), the wall row's v*_i/n_i in FP64
                const df2 qj = df_unpack(pq[j]);
                const df2 ddx = df_mul(qj, df_of(usx[j] - vxi_n));
                const df2 ddy = df_mul(qj, df_of(usy[j] - vyi_n));
                fv = df_add(fv, df_mul(mi_over_rhoi, df_add(df_mul(ddx, gx), df_mul(ddy, gy))));
            } else {
                const df2 t = df_mul(df_mul(df_twice(pvol), df_add(df_mul(dx, gxr), df_mul(dy, gyr))), p_dist);
                val = df_neg(t);
                dia = df_add(dia, t);
            }
        }
        vdf[e] = df_pack(val);
    }
    const double d = df_to_double(dia);
    if (d == 0.0 || !isfinite(d)) {
        // zero-neighbour guard: identity row, b = 0 (the reference divides by 0)
        for (int k = 0; k < m; ++k) {
            const int64_t e = ell(i, k, K.kmax);
            aval[e] = 0.0;
            ellf[e] = make_int2(nbr[e], 0);
            avalh[e] = __float2half_rn(0.f);
        }
        b[i] = 0.0;
        return;
    }
    const df2 inv = df_rcp(dia);
    for (int k = 0; k < m; ++k) {
        const int64_t e = ell(i, k, K.kmax);
        const df2 v = df_mul(df_unpack(vdf[e]), inv);
        aval[e] = df_to_double(v);
        // the inner sweeps' FP32 copy is the high half (the FP32 rounding of
        // the value); the V-cycle's FP16 copy is rounded from it
        ellf[e] = make_int2(nbr[e], __float_as_int(v.hi));
        avalh[e] = __float2half_rn(v.hi);
    }
    b[i] = df_to_double(df_mul(df_mul(fv, df_rcp(df_of(dt))), inv));
}

__global__ void k_vs_over_por(int64_t n, State S, double* __restrict__ q, double* __restrict__ ux,
                              double* __restrict__ uy) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double nn = S.por[i];
    q[i] = S.rho[i] / nn;
    ux[i] = S.vxs[i] / nn;
    uy[i] = S.vys[i] / nn;
}

// the V-cycle's packed FP16 entries (EllPack16) of the assembled rows: one
// thread per row over whole warps (the rows of the last slice past n count as
// fitting), each warp one 32-row slice
__global__ void k_pack16(int64_t n, int64_t npad, const int32_t* __restrict__ nbr, const __half* __restrict__ avalh,
                         const int32_t* __restrict__ cnt, int kmax, uint32_t* __restrict__ ent,
                         uint8_t* __restrict__ ok) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= npad) return;  // npad and the block size are multiples of 32: whole warps
    bool fits = true;
    if (i < n) {
        const int64_t b = i & ~(int64_t)31;
        const int m = cnt[i];
        for (int k = 0; k < m; ++k) {
            const int64_t e = ell(i, k, kmax);
            const int64_t d = (int64_t)nbr[e] - b;
            fits = fits && d >= -32768 && d <= 32767;
            ent[e] = (uint32_t)(uint16_t)(int16_t)d | ((uint32_t)__half_as_ushort(avalh[e]) << 16);
        }
    }
    const unsigned all = __all_sync(0xffffffffu, fits);
    if ((threadIdx.x & 31) == 0) ok[i >> 5] = all ? 1 : 0;
}

int op_ppe_assemble(Ctx* c) {
    if (!c->have_lists) return set_err(c, BSC_E_INVALID, "ppesolve before neighbour");
    double *q = c->s, *ux = c->tv, *uy = c->v;
    k_vs_over_por<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, q, ux, uy);
    BSC_LAUNCH(c);
    const unsigned g = blocks_for(c->n, NB_BLOCK);
    // FP64 assembly in both paths: the PPE coefficients are sums whose FP32
    // rounding moves the pressure by ~5e-6 (relative) at 1e-8 residual; the
    // mixed path keeps an FP32 copy for its inner sweeps
    if (c->mixed && !c->exact_div && !c->asm_rcp) {
        // mixed path: double-float pair arithmetic (k_assemble_df)
        k_asm_df_pre<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, c->K, c->pcell, q, c->asm_df);
        BSC_LAUNCH(c);
        StageTimer tk(c, BSC_T_K_ASSEMBLE);
        k_assemble_df<<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gwf, c->gwl, c->cnt, c->pcell,
                                                      c->asm_df, c->aval, c->ellf, c->avalh, c->b, q, ux, uy, c->dt);
        BSC_LAUNCH(c);
    } else {
        StageTimer tk(c, BSC_T_K_ASSEMBLE);
        if (c->mixed && !c->exact_div)
            k_assemble<double, true><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gw, c->cnt, c->aval,
                                                                    c->ellf, c->avalh, c->b, q, ux, uy, c->dt);
        else
            k_assemble<double, false><<<g, NB_BLOCK, 0, c->stream>>>(
                c->n, c->S, c->K, c->nbr, c->gw, c->cnt, c->aval, c->mixed ? c->ellf : nullptr,
                c->mixed ? c->avalh : nullptr, c->b, q, ux, uy, c->dt);
        BSC_LAUNCH(c);
    }
    if (c->mixed) {
        const int64_t npad = ((c->n + 31) / 32) * 32;
        k_pack16<<<blocks_for(npad, 256), 256, 0, c->stream>>>(c->n, npad, c->nbr, c->avalh, c->cnt, c->K.kmax,
                                                                c->ellh, c->ellh_ok);
        BSC_LAUNCH(c);
    }
    c->have_csr = true;
    return BSC_OK;
}

// ============================================================================
// operators: unit-diagonal ELL (the PPE) and general CSR (standalone solve)
// ============================================================================
struct CsrOp {
    const int32_t* rp;
    const int32_t* col;
    const double* val;
    const void* key() const { return val; }
    template <typename X, typename A>
    __device__ __forceinline__ A row(int64_t i, const X* __restrict__ x) const {
        A s = 0;
        for (int k = rp[i]; k < rp[i + 1]; ++k) s += (A)val[k] * (A)x[col[k]];
        return s;
    }
};

// ============================================================================
// reductions: RED_GRID blocks write partials; consumers reduce them in a
// fixed order (deterministic for a given n)
// ============================================================================
// Warp sum into lane 0.  Only the lanes that feed lane 0 add (16, 8, 4, 2, 1
// of them): lane 0 does the same additions in the same order as a full
// butterfly, with a fifth of the FP64 work, which is what GB300's FP64 pipe
// is short of.
__device__ __forceinline__ double warp_sum_to_lane0(double x) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double y = __shfl_down_sync(0xffffffffu, x, o);
        if (lane < o) x += y;
    }
    return x;
}
__device__ __forceinline__ float warp_sum_to_lane0(float x) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    return x;
}

// per-block partial sums of D values into part[d * RED_GRID + block]; the
// values may be float (warp sums in FP32, block sum in FP64) or double
template <int D, typename V>
__device__ __forceinline__ void block_partials(V (&v)[D], double* __restrict__ part) {
    __shared__ double sh[D][RED_BLOCK / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        const V x = warp_sum_to_lane0(v[d]);
        if (lane == 0) sh[d][w] = (double)x;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            double x = (lane < RED_BLOCK / 32) ? sh[d][lane] : 0.0;
            x = warp_sum_to_lane0(x);
            if (lane == 0) part[d * RED_GRID + blockIdx.x] = x;
        }
    }
}

// every block reduces the partials itself (fixed order): no finalize launch
template <int D>
__device__ __forceinline__ void reduce_partials(const double* __restrict__ part, double (&out)[D]) {
    __shared__ double sh[D][RED_BLOCK / 32];
    __shared__ double res[D];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int d = 0; d < D; ++d) {
        double x = 0.0;
        for (int k = threadIdx.x; k < RED_GRID; k += blockDim.x) x += __ldcg(part + d * RED_GRID + k);
        x = warp_sum_to_lane0(x);
        if (lane == 0) sh[d][w] = x;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
#pragma unroll
        for (int d = 0; d < D; ++d) {
            double x = (lane < RED_BLOCK / 32) ? sh[d][lane] : 0.0;
            x = warp_sum_to_lane0(x);
            if (lane == 0) res[d] = x;
        }
    }
    __syncthreads();
#pragma unroll
    for (int d = 0; d < D; ++d) out[d] = res[d];
}


// ============================================================================
// BiCGSTAB, value type T (double or float), dots accumulated in double
// ============================================================================
// r = b - A x; rhat = r; p = r; partials (r.r, b.b)
template <typename Op, typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_bicg_init(int64_t n, Op A, const T* __restrict__ x,
                                                          const T* __restrict__ b, T* __restrict__ r,
                                                          T* __restrict__ rh, T* __restrict__ p,
                                                          double* __restrict__ part) {
    double acc[2] = {0.0, 0.0};
    GRID_LOOP(i, n) {
        const double ri = (double)b[i] - A.template row<T, double>(i, x);
        const T rt = (T)ri;
        r[i] = rt; rh[i] = rt; p[i] = rt;
        acc[0] += (double)rt * (double)rt;
        acc[1] += (double)b[i] * (double)b[i];
    }
    block_partials<2>(acc, part);
}

__global__ void k_bicg_setup(const double* __restrict__ part, Scalars* sc, double tol, int rel_r0) {
    double v[2];
    reduce_partials<2>(part, v);
    if (threadIdx.x == 0) {
        sc->rr = v[0];
        sc->rho = v[0];
        sc->bestb[0] = sqrt(v[0]);
        sc->k5 = 0;
        sc->bnorm = sqrt(v[1]);
        sc->r0norm = sqrt(v[0]);
        sc->target = tol * (rel_r0 ? sc->r0norm : sc->bnorm);
        sc->done = (sc->r0norm <= sc->target) ? 1 : 0;
        sc->breakdown = 0;
        sc->it = 0;
        sc->alpha = sc->omega = 1.0;
    }
}

// restart after a breakdown: k_bicg_init has set r = rhat = p = b - A x from
// the current iterate; the target, iteration count and best residual carry on
__global__ void k_bicg_restart(const double* __restrict__ part, Scalars* sc) {
    double v[2];
    reduce_partials<2>(part, v);
    if (threadIdx.x == 0) {
        sc->rr = v[0];
        sc->rho = v[0];
        sc->k5 = 0;
        sc->done = (sqrt(v[0]) <= sc->target) ? 1 : 0;
        sc->breakdown = (v[0] == 0.0 && !sc->done) ? 1 : 0;
    }
}

// Every block writes its partial sums; the block that finishes last (ticket
// taken after a fence) reduces them in block order and returns true, so one
// block publishes each scalar and the consumer kernels stream without any
// reduction of their own.  The ticket is reset by that block.
template <int D>
__device__ __forceinline__ bool finish_partials(double (&v)[D], double* __restrict__ part,
                                                unsigned* __restrict__ ticket, double (&tot)[D]) {
    block_partials<D>(v, part);
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    reduce_partials<D>(part, tot);
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// v = A p; alpha = rho / (rhat . v)
template <typename Op, typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_bicg_1(int64_t n, Op A, const T* __restrict__ p, T* __restrict__ v,
                                                       const T* __restrict__ rh, double* __restrict__ part,
                                                       Scalars* sc, unsigned* __restrict__ ticket) {
    if (sc->done | sc->breakdown) return;
    double acc[1] = {0.0}, d[1];
    GRID_LOOP(i, n) {
        const T vi = (T)A.template row<T, T>(i, p);
        v[i] = vi;
        acc[0] += (double)rh[i] * (double)vi;
    }
    if (finish_partials<1>(acc, part, ticket, d) && threadIdx.x == 0) {
        const double rho = sc->rho;
        if (d[0] == 0.0 || rho == 0.0) sc->breakdown = 1;
        else sc->tmp[0] = rho / d[0];
    }
}

// s = r - alpha v
template <typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_bicg_2(int64_t n, const T* __restrict__ r, const T* __restrict__ v,
                                                       T* __restrict__ s, const Scalars* __restrict__ sc) {
    if (sc->done | sc->breakdown) return;
    const T a = (T)sc->tmp[0];
    GRID_LOOP(i, n) s[i] = r[i] - a * v[i];
}

// t = A s; omega = (t.s)/(t.t)
template <typename Op, typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_bicg_3(int64_t n, Op A, const T* __restrict__ s, T* __restrict__ t,
                                                       double* __restrict__ part, Scalars* sc,
                                                       unsigned* __restrict__ ticket) {
    if (sc->done | sc->breakdown) return;
    double acc[2] = {0.0, 0.0}, d[2];
    GRID_LOOP(i, n) {
        const T ti = (T)A.template row<T, T>(i, s);
        t[i] = ti;
        acc[0] += (double)ti * (double)s[i];
        acc[1] += (double)ti * (double)ti;
    }
    if (finish_partials<2>(acc, part + 2 * RED_GRID, ticket, d) && threadIdx.x == 0)
        sc->tmp[1] = (d[1] == 0.0) ? 0.0 : d[0] / d[1];
}

// x += alpha p + omega s; r = s - omega t; then (last block) the residual
// test, rho, beta and what k_bicg_5 has to do.  With `track` (the FP32 sweeps
// of the mixed path) the minimum-residual iterate is kept and a sweep whose
// residual grows past `blowup` times that minimum stops: BiCGSTAB's residual
// is not monotone, and in FP32 on this operator it can diverge.
template <typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_bicg_4(int64_t n, T* __restrict__ x, const T* __restrict__ p,
                                                       const T* __restrict__ s, const T* __restrict__ t,
                                                       T* __restrict__ r, const T* __restrict__ rh,
                                                       double* __restrict__ part, Scalars* sc,
                                                       unsigned* __restrict__ ticket, int track, double blowup) {
    if (sc->done | sc->breakdown) return;
    const double alpha = sc->tmp[0], omega = sc->tmp[1];
    const T a = (T)alpha, w = (T)omega;
    double acc[2] = {0.0, 0.0}, d[2];
    GRID_LOOP(i, n) {
        const T si = s[i];
        x[i] = x[i] + a * p[i] + w * si;
        const T ri = si - w * t[i];
        r[i] = ri;
        acc[0] += (double)ri * (double)ri;
        acc[1] += (double)rh[i] * (double)ri;
    }
    if (finish_partials<2>(acc, part + 4 * RED_GRID, ticket, d) && threadIdx.x == 0) {
        const double rn = sqrt(d[0]), best = sc->bestb[0], rho = sc->rho;
        const bool conv = rn <= sc->target;
        const bool improved = rn < best;
        const bool stop = track && !conv && (!(rn == rn) || rn > blowup * best);
        const bool brk = !conv && !stop && (omega == 0.0 || d[1] == 0.0);
        sc->tmp[2] = (conv || stop || brk) ? 0.0 : (d[1] / rho) * (alpha / omega);
        sc->rr = d[0];
        sc->rho = d[1];
        if (improved) sc->bestb[0] = rn;
        sc->it += 1;
        sc->done = (conv || stop) ? 1 : 0;
        sc->breakdown = brk ? 1 : 0;
        sc->k5 = ((track && improved) ? 1 : 0) | ((conv || stop || brk) ? 0 : 2);
    }
}

// bit 1: keep x as the best iterate; bit 2: p = r + beta (p - omega v)
template <typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_bicg_5(int64_t n, T* __restrict__ p, const T* __restrict__ r,
                                                       const T* __restrict__ v, Scalars* sc, const T* __restrict__ x,
                                                       T* __restrict__ xbest, unsigned* __restrict__ ticket) {
    const int mode = sc->k5;
    if (mode == 0) return;
    if ((mode & 1) && xbest) {
        GRID_LOOP(i, n) xbest[i] = x[i];
    }
    if (mode & 2) {
        const T bt = (T)sc->tmp[2], w = (T)sc->tmp[1];
        GRID_LOOP(i, n) p[i] = r[i] + bt * (p[i] - w * v[i]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(ticket, 1u) == gridDim.x - 1) {  // every block has read `mode`
            sc->k5 = 0;
            *ticket = 0u;
        }
    }
}

// ============================================================================
// FGMRES(m) with CGS2, value type T, basis V[(m+1) x n], Hessenberg on device
// ============================================================================
// layout of Hd: H[(m+1)*m] | cs[m] | sn[m] | g[m+1] | y[m] | hcol[m+1] | ctl[4]
struct FgLayout {
    int m;
    __host__ __device__ int H(int i, int j) const { return i * m + j; }
    __host__ __device__ int cs(int k) const { return (m + 1) * m + k; }
    __host__ __device__ int sn(int k) const { return (m + 1) * m + m + k; }
    __host__ __device__ int g(int k) const { return (m + 1) * m + 2 * m + k; }
    __host__ __device__ int y(int k) const { return (m + 1) * m + 3 * m + 1 + k; }
    __host__ __device__ int hc(int k) const { return (m + 1) * m + 4 * m + 1 + k; }
    __host__ __device__ int size() const { return (m + 1) * m + 5 * m + 2; }
};

// r = b - A x; partials (r.r, b.b)
template <typename Op, typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_resid(int64_t n, Op A, const T* __restrict__ x,
                                                      const T* __restrict__ b, T* __restrict__ r,
                                                      double* __restrict__ part) {
    double acc[2] = {0.0, 0.0};
    GRID_LOOP(i, n) {
        const double ri = (double)b[i] - A.template row<T, double>(i, x);
        const T rt = (T)ri;
        r[i] = rt;
        acc[0] += ri * ri;
        acc[1] += (double)b[i] * (double)b[i];
    }
    block_partials<2>(acc, part);
}

// cycle start: beta = ||r||; v0 = r/beta; g = beta e1; ctl: j = 0, cycle_done
__global__ void k_fg_start(const double* __restrict__ part, Scalars* sc, double* Hd, FgLayout F, int first,
                           double tol, int rel_r0) {
    double v[2];
    reduce_partials<2>(part, v);
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double beta = sqrt(v[0]);
        if (first) {
            sc->bnorm = sqrt(v[1]);
            sc->r0norm = beta;
            sc->target = tol * (rel_r0 ? beta : sc->bnorm);
            sc->it = 0;
            sc->breakdown = 0;
        }
        sc->rr = v[0];
        sc->done = (beta <= sc->target) ? 1 : 0;
        sc->tmp[0] = beta;  // scale for v0
        sc->tmp[1] = 0.0;   // j (columns completed in this cycle)
        sc->tmp[2] = 0.0;   // cycle finished flag
        for (int k = 0; k <= F.m; ++k) Hd[F.g(k)] = 0.0;
        Hd[F.g(0)] = beta;
    }
}

template <typename T>
__global__ void k_fg_v0(int64_t n, const T* __restrict__ r, T* __restrict__ V0, const Scalars* __restrict__ sc) {
    if (sc->done) return;
    const double inv = 1.0 / sc->tmp[0];
    GRID_LOOP(i, n) V0[i] = (T)((double)r[i] * inv);
}

// w = A v_j
template <typename Op, typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_fg_spmv(int64_t n, Op A, const T* __restrict__ V, T* __restrict__ w,
                                                        int j, const Scalars* __restrict__ sc) {
    if (fg_skip(sc)) return;
    const T* vj = V + (int64_t)j * n;
    GRID_LOOP(i, n) w[i] = (T)A.template row<T, T>(i, vj);
}

constexpr int FG_MAXM = 64;

// partials of V_i . w for i = 0..j
template <typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_fg_mdot(int64_t n, const T* __restrict__ V, const T* __restrict__ w,
                                                        int j, double* __restrict__ part,
                                                        const Scalars* __restrict__ sc) {
    if (fg_skip(sc)) return;
    // up to j+1 <= FG_MAXM dots, 8 at a time to bound registers
    for (int i0 = 0; i0 <= j; i0 += 8) {
        double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const int cntv = min(8, j + 1 - i0);
        GRID_LOOP(k, n) {
            const double wk = (double)w[k];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (q < cntv) acc[q] += (double)V[(int64_t)(i0 + q) * n + k] * wk;
        }
        block_partials<8>(acc, part + (int64_t)i0 * RED_GRID);
        __syncthreads();
    }
}

// h(0..j) = reduced dots (added to column j of H on the second pass)
__global__ void k_fg_hcol(const double* __restrict__ part, double* Hd, FgLayout F, int j, int accumulate,
                          const Scalars* __restrict__ sc) {
    if (fg_skip(sc)) return;
    // one warp per dot, fixed order
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = w; i <= j; i += nw) {
        double x = 0.0;
        for (int k = lane; k < RED_GRID; k += 32) x += part[(int64_t)i * RED_GRID + k];
        x = warp_sum_to_lane0(x);
        if (lane == 0) {
            Hd[F.hc(i)] = x;
            Hd[F.H(i, j)] = accumulate ? Hd[F.H(i, j)] + x : x;
        }
    }
}

// w -= sum_i h_i V_i; partial (w.w) when `norm`
template <typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_fg_maxpy(int64_t n, const T* __restrict__ V, T* __restrict__ w, int j,
                                                         const double* __restrict__ Hd, FgLayout F, int norm,
                                                         double* __restrict__ part, const Scalars* __restrict__ sc) {
    if (fg_skip(sc)) return;
    __shared__ double h[FG_MAXM];
    for (int i = threadIdx.x; i <= j; i += blockDim.x) h[i] = Hd[F.hc(i)];
    __syncthreads();
    double acc[1] = {0.0};
    GRID_LOOP(k, n) {
        double s = (double)w[k];
        for (int i = 0; i <= j; ++i) s -= h[i] * (double)V[(int64_t)i * n + k];
        const T st = (T)s;
        w[k] = st;
        acc[0] += (double)st * (double)st;
    }
    if (norm) block_partials<1>(acc, part);
}

// h(j+1,j) = ||w||; Givens; residual estimate; cycle/convergence control
__device__ void fg_givens(const double* __restrict__ part, Scalars* sc, double* Hd, FgLayout F, int j) {
    // the column and the earlier rotations are staged in shared memory by
    // all threads; one thread then applies the rotations (a serial chain
    // that would otherwise wait on global memory at every step)
    __shared__ double hcol[FG_MAXM + 1], csv[FG_MAXM], snv[FG_MAXM];
    double v[1];
    reduce_partials<1>(part, v);
    const int t = threadIdx.x;
    for (int i = t; i <= j; i += blockDim.x) hcol[i] = Hd[F.H(i, j)];
    for (int i = t; i < j; i += blockDim.x) {
        csv[i] = Hd[F.cs(i)];
        snv[i] = Hd[F.sn(i)];
    }
    __syncthreads();
    if (t == 0) {
        const double hn = sqrt(v[0]);
        hcol[j + 1] = hn;
        for (int i = 0; i < j; ++i) {
            const double a = hcol[i], c = hcol[i + 1];
            hcol[i] = csv[i] * a + snv[i] * c;
            hcol[i + 1] = -snv[i] * a + csv[i] * c;
        }
        const double a = hcol[j], c = hcol[j + 1];
        const double den = sqrt(a * a + c * c);
        sc->it += 1;
        sc->tmp[1] = (double)(j + 1);
        if (den == 0.0) {
            sc->breakdown = 1;
            sc->tmp[1] = (double)j;
            sc->tmp[2] = 1.0;
        } else {
            const double cs = a / den, sn = c / den;
            Hd[F.cs(j)] = cs;
            Hd[F.sn(j)] = sn;
            hcol[j] = den;
            hcol[j + 1] = 0.0;
            const double gj = Hd[F.g(j)];
            const double gn = -sn * gj;
            Hd[F.g(j + 1)] = gn;
            Hd[F.g(j)] = cs * gj;
            sc->tmp[3] = hn;  // scale of v_{j+1}
            if (fabs(gn) <= sc->target || hn == 0.0 || j + 1 == F.m) sc->tmp[2] = 1.0;
        }
    }
    __syncthreads();
    for (int i = t; i <= j + 1; i += blockDim.x) Hd[F.H(i, j)] = hcol[i];
}

// `mirror` (pinned host memory, optional) receives the scalars after this
// iteration, whether it ran or was skipped
__global__ void k_fg_givens(const double* __restrict__ part, Scalars* sc, double* Hd, FgLayout F, int j,
                            Scalars* mirror) {
    if (!fg_skip(sc)) fg_givens(part, sc, Hd, F, j);
    if (mirror && threadIdx.x == 0) *mirror = *sc;
}

// v_{j+1} = w / h(j+1,j)
template <typename T>
__global__ void k_fg_next(int64_t n, const T* __restrict__ w, T* __restrict__ V, int j, const Scalars* __restrict__ sc) {
    if (sc->done || sc->tmp[2] != 0.0) return;
    const double inv = 1.0 / sc->tmp[3];
    T* vn = V + (int64_t)(j + 1) * n;
    GRID_LOOP(i, n) vn[i] = (T)((double)w[i] * inv);
}

// y = H^-1 g over the completed columns
// the triangle and g staged in shared memory by the block; one thread then
// substitutes (a serial chain that would otherwise wait on global memory)
__global__ void k_fg_backsolve(Scalars* sc, double* Hd, FgLayout F) {
    __shared__ double Hs[FG_MAXM][FG_MAXM + 1], gs[FG_MAXM], ys[FG_MAXM];
    if (sc->done) return;
    const int k = (int)sc->tmp[1];
    for (int e = threadIdx.x; e < k * k; e += blockDim.x) {
        const int i = e / k, q = e - i * k;
        if (q >= i) Hs[i][q] = Hd[F.H(i, q)];
    }
    for (int i = threadIdx.x; i < k; i += blockDim.x) gs[i] = Hd[F.g(i)];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int i = k - 1; i >= 0; --i) {
            double s = gs[i];
            for (int q = i + 1; q < k; ++q) s -= Hs[i][q] * ys[q];
            ys[i] = s / Hs[i][i];
        }
    __syncthreads();
    for (int i = threadIdx.x; i < F.m; i += blockDim.x) Hd[F.y(i)] = i < k ? ys[i] : 0.0;
}

// x += sum_i y_i V_i
template <typename T>
__global__ void k_fg_update(int64_t n, T* __restrict__ x, const T* __restrict__ V, const double* __restrict__ Hd,
                            FgLayout F, const Scalars* __restrict__ sc) {
    if (sc->done) return;
    __shared__ double y[FG_MAXM];
    const int k = (int)sc->tmp[1];
    for (int i = threadIdx.x; i < k; i += blockDim.x) y[i] = Hd[F.y(i)];
    __syncthreads();
    GRID_LOOP(q, n) {
        double s = (double)x[q];
        for (int i = 0; i < k; ++i) s += y[i] * (double)V[(int64_t)i * n + q];
        x[q] = (T)s;
    }
}

// ============================================================================
// host drivers
// ============================================================================
template <typename T>
struct Work {
    T *x, *b, *r, *rh, *p, *v, *s, *t, *V;
};

int fetch_scalars(Ctx* c) {
    BSC_CUDA(c, cudaMemcpyAsync(c->h_sc, c->sc, sizeof(Scalars), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    return BSC_OK;
}

// Iterations queued between two convergence checks.  A batch is captured
// once as a CUDA graph and replayed; kernels of iterations past convergence
// return at their first instruction.
inline int batch_for(int64_t n) { return n > 200000 ? 16 : 8; }

// a cached graph for `body`, captured on the context stream
template <typename F>
int batch_graph(Ctx* c, const void* k0, const void* k1, const void* k2, int64_t n, F body, cudaGraphExec_t* out) {
    for (auto& g : c->graphs)
        if (g.k0 == k0 && g.k1 == k1 && g.k2 == k2 && g.n == n) {
            *out = g.exec;
            return BSC_OK;
        }
    cudaGraph_t graph = nullptr;
    BSC_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    body();
    BSC_CUDA(c, cudaStreamEndCapture(c->stream, &graph));
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaGraphInstantiate");
    c->graphs.push_back({k0, k1, k2, n, exec});
    *out = exec;
    return BSC_OK;
}

void drop_graphs(Ctx* c) {
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (auto& g : c->graphs) cudaGraphExecDestroy(g.exec);
    c->graphs.clear();
}

// Run `body` (which returns a status) as a CUDA graph cached under the key
// (k0, k1, k2, n): captured on first use, replayed after.  A failure inside
// the capture ends it and returns the failure.
template <typename F>
int graph_run(Ctx* c, const void* k0, const void* k1, const void* k2, int64_t n, F body) {
    if (!c->use_graphs) return body();
    for (auto& g : c->graphs)
        if (g.k0 == k0 && g.k1 == k1 && g.k2 == k2 && g.n == n) {
            BSC_CUDA(c, cudaGraphLaunch(g.exec, c->stream));
            c->launches += g.kernels;
            return BSC_OK;
        }
    BSC_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int64_t l0 = c->launches;
    c->capturing = true;
    const int rc = body();
    c->capturing = false;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
    if (rc || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        (void)cudaGetLastError();
        return rc ? rc : cuda_err(c, e, "cudaStreamEndCapture");
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_err(c, e, "cudaGraphInstantiate");
    c->graphs.push_back({k0, k1, k2, n, exec, c->launches - l0});
    BSC_CUDA(c, cudaGraphLaunch(exec, c->stream));
    return BSC_OK;
}

// `xbest` (optional): keep the minimum-residual iterate there and stop a
// diverging solve; *rr_out is then the squared best residual
template <typename Op, typename T>
int run_bicgstab(Ctx* c, int64_t n, const Op& A, Work<T> w, double tol, int rel_r0, int maxit, int* iters,
                 double* rr_out, T* xbest = nullptr) {
    const int G = RED_GRID, B = RED_BLOCK;
    k_bicg_init<Op, T><<<G, B, 0, c->stream>>>(n, A, w.x, w.b, w.r, w.rh, w.p, c->part);
    BSC_LAUNCH(c);
    k_bicg_setup<<<1, B, 0, c->stream>>>(c->part, c->sc, tol, rel_r0);
    BSC_LAUNCH(c);
    if (xbest) BSC_CUDA(c, cudaMemcpyAsync(xbest, w.x, sizeof(T) * n, cudaMemcpyDeviceToDevice, c->stream));
    // the first SpMV of every batch is bracketed by events (recorded into the
    // graph too) so the dominant kernel's duration is measured in place
    bool first = true;
    // external event nodes when captured into a graph, so they stay
    // timeable; a plain record on the uncaptured tail batch
    bool capturing = false;
    auto rec = [&](cudaEvent_t e) {
        if (capturing) cudaEventRecordWithFlags(e, c->stream, cudaEventRecordExternal);
        else cudaEventRecord(e, c->stream);
    };
    auto one = [&]() {
        const bool pr = first && c->prof_iter;
        if (first && c->timing) rec(c->ev_spmv[0]);
        k_bicg_1<Op, T><<<G, B, 0, c->stream>>>(n, A, w.p, w.v, w.rh, c->part, c->sc, c->ticket);
        if (first && c->timing) rec(c->ev_spmv[1]);
        first = false;
        k_bicg_2<T><<<G, B, 0, c->stream>>>(n, w.r, w.v, w.s, c->sc);
        if (pr) rec(c->ev_it[2]);
        k_bicg_3<Op, T><<<G, B, 0, c->stream>>>(n, A, w.s, w.t, c->part, c->sc, c->ticket);
        if (pr) rec(c->ev_it[3]);
        k_bicg_4<T><<<G, B, 0, c->stream>>>(n, w.x, w.p, w.s, w.t, w.r, w.rh, c->part, c->sc, c->ticket,
                                            xbest != nullptr, 1e3);
        if (pr) rec(c->ev_it[4]);
        k_bicg_5<T><<<G, B, 0, c->stream>>>(n, w.p, w.r, w.v, c->sc, w.x, xbest, c->ticket);
        if (pr) rec(c->ev_it[5]);
    };
    const int batch = batch_for(n);
    constexpr int kMaxRestarts = 8;
    int launched = 0, restarts = 0;
    for (;;) {
        int rc = fetch_scalars(c);
        if (rc) return rc;
        const Scalars& h = *c->h_sc;
        if (h.breakdown && !h.done && h.it < maxit && restarts < kMaxRestarts) {
            // rho or omega vanished: restart from x with a fresh shadow residual
            ++restarts;
            k_bicg_init<Op, T><<<G, B, 0, c->stream>>>(n, A, w.x, w.b, w.r, w.rh, w.p, c->part);
            BSC_LAUNCH(c);
            k_bicg_restart<<<1, B, 0, c->stream>>>(c->part, c->sc);
            BSC_LAUNCH(c);
            c->launches += 2;
            continue;
        }
        if (h.done || h.breakdown || h.it >= maxit || launched >= maxit) break;
        const int nb = std::min(batch, maxit - h.it);
        if (launched > 0 && c->timing) {  // the previous batch has completed (fetch_scalars synced)
            float ms = 0.f;
            if (cudaEventElapsedTime(&ms, c->ev_spmv[0], c->ev_spmv[1]) == cudaSuccess) {
                c->ms[BSC_T_SPMV] += ms;
                c->calls[BSC_T_SPMV]++;
            }
            if (c->prof_iter) {
                const cudaEvent_t ev[6] = {c->ev_spmv[0], c->ev_spmv[1], c->ev_it[2], c->ev_it[3], c->ev_it[4],
                                           c->ev_it[5]};
                for (int k = 0; k < 5; ++k)
                    if (cudaEventElapsedTime(&ms, ev[k], ev[k + 1]) == cudaSuccess) {
                        c->ms[BSC_T_BICG_1 + k] += ms;
                        c->calls[BSC_T_BICG_1 + k]++;
                    }
            }
            (void)cudaGetLastError();  // a failed diagnostic query must not fail the solve
        }
        first = true;
        if (c->use_graphs && nb == batch) {
            cudaGraphExec_t ge = nullptr;
            rc = batch_graph(c, A.key(), (const void*)w.x, (const void*)xbest, n, [&]() {
                capturing = true;
                for (int q = 0; q < batch; ++q) one();
                capturing = false;
            }, &ge);
            if (rc) return rc;
            BSC_CUDA(c, cudaGraphLaunch(ge, c->stream));
        } else {
            for (int q = 0; q < nb; ++q) one();
        }
        c->launches += 5 * nb;
        launched += nb;
        BSC_CUDA(c, cudaGetLastError());
    }
    *iters = c->h_sc->it;
    if (xbest) {
        const double b = c->h_sc->bestb[0];
        *rr_out = b * b;
    } else {
        *rr_out = c->h_sc->rr;
    }
    return c->h_sc->breakdown && !c->h_sc->done ? BSC_E_BREAKDOWN : BSC_OK;
}

template <typename Op, typename T>
int run_fgmres(Ctx* c, int64_t n, const Op& A, Work<T> w, double tol, int rel_r0, int maxit, int m, int* iters,
               double* rr_out) {
    const int G = RED_GRID, B = RED_BLOCK;
    FgLayout F{m};
    int first = 1;
    T* wv = w.t;
    for (;;) {
        k_resid<Op, T><<<G, B, 0, c->stream>>>(n, A, w.x, w.b, w.r, c->part);
        BSC_LAUNCH(c);
        k_fg_start<<<1, B, 0, c->stream>>>(c->part, c->sc, c->Hd, F, first, tol, rel_r0);
        BSC_LAUNCH(c);
        first = 0;
        int rc = fetch_scalars(c);
        if (rc) return rc;
        if (c->h_sc->done || c->h_sc->it >= maxit) break;
        k_fg_v0<T><<<G, B, 0, c->stream>>>(n, w.r, w.V, c->sc);
        BSC_LAUNCH(c);
        const int mm = std::min(m, maxit - c->h_sc->it);
        for (int j = 0; j < mm; ++j) {
            k_fg_spmv<Op, T><<<G, B, 0, c->stream>>>(n, A, w.V, wv, j, c->sc);
            for (int pass = 0; pass < 2; ++pass) {
                k_fg_mdot<T><<<G, B, 0, c->stream>>>(n, w.V, wv, j, c->part, c->sc);
                k_fg_hcol<<<1, 1024, 0, c->stream>>>(c->part, c->Hd, F, j, pass, c->sc);
                k_fg_maxpy<T><<<G, B, 0, c->stream>>>(n, w.V, wv, j, c->Hd, F, pass, c->part, c->sc);
                c->launches += 3;
            }
            k_fg_givens<<<1, B, 0, c->stream>>>(c->part, c->sc, c->Hd, F, j, nullptr);
            k_fg_next<T><<<G, B, 0, c->stream>>>(n, wv, w.V, j, c->sc);
            c->launches += 3;
        }
        BSC_LAUNCH(c);
        k_fg_backsolve<<<1, 256, 0, c->stream>>>(c->sc, c->Hd, F);
        k_fg_update<T><<<G, B, 0, c->stream>>>(n, w.x, w.V, c->Hd, F, c->sc);
        c->launches += 2;
        BSC_LAUNCH(c);
        rc = fetch_scalars(c);
        if (rc) return rc;
        if (c->h_sc->breakdown && c->h_sc->tmp[1] == 0.0) break;
    }
    *iters = c->h_sc->it;
    *rr_out = c->h_sc->rr;
    return BSC_OK;
}

// FP64 true residual of the FP32-valued unit-diagonal matrix: r = b - A x
__global__ void __launch_bounds__(RED_BLOCK) k_ir_resid(int64_t n, EllOp<double> A, const double* __restrict__ x,
                                                         const double* __restrict__ b, double* __restrict__ r,
                                                         float* __restrict__ rf, double* __restrict__ part) {
    double acc[2] = {0.0, 0.0};
    GRID_LOOP(i, n) {
        const double ri = b[i] - A.template row<double, double>(i, x);
        r[i] = ri;
        rf[i] = (float)ri;
        acc[0] += ri * ri;
        acc[1] += b[i] * b[i];
    }
    block_partials<2>(acc, part);
}

__global__ void k_ir_norms(const double* __restrict__ part, double* out) {
    double v[2];
    reduce_partials<2>(part, v);
    if (threadIdx.x == 0) {
        out[0] = sqrt(v[0]);
        out[1] = sqrt(v[1]);
    }
}

__global__ void k_ir_add(int64_t n, double* __restrict__ x, const float* __restrict__ d) {
    GRID_LOOP(i, n) x[i] += (double)d[i];
}

__global__ void k_copy_f64(int64_t n, const double* __restrict__ a, double* __restrict__ b) {
    GRID_LOOP(i, n) b[i] = a[i];
}

// ---- FGMRES-IR pieces (mixed path) ----------------------------------------------
__global__ void k_d2f(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
    GRID_LOOP(i, n) b[i] = (float)a[i];
}

// w = A z with the FP64 operator and a preconditioned vector (FP32 or FP64)
template <typename ZT>
__global__ void __launch_bounds__(RED_BLOCK) k_spmv_z(int64_t n, EllOp<double> A, const ZT* __restrict__ z,
                                                       double* __restrict__ w, const Scalars* __restrict__ sc) {
    if (fg_skip(sc)) return;
    GRID_LOOP(i, n) w[i] = A.template row<ZT, double>(i, z);
}

// x += sum_i y_i z_i, z_i the preconditioned vectors of the cycle
template <typename ZT>
__global__ void k_fg_update_z(int64_t n, double* __restrict__ x, const ZT* __restrict__ Z,
                              const double* __restrict__ Hd, FgLayout F, const Scalars* __restrict__ sc) {
    if (sc->done) return;
    __shared__ double y[FG_MAXM];
    const int k = (int)sc->tmp[1];
    for (int i = threadIdx.x; i < k; i += blockDim.x) y[i] = Hd[F.y(i)];
    __syncthreads();
    GRID_LOOP(q, n) {
        double s = x[q];
        for (int i = 0; i < k; ++i) s += y[i] * (double)Z[(int64_t)i * n + q];
        x[q] = s;
    }
}

int fetch_outer(Ctx* c) {
    BSC_CUDA(c, cudaMemcpyAsync(c->h_sc + 1, c->sc2, sizeof(Scalars), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    return BSC_OK;
}

// Flexible GMRES in FP64 on the FP64 operator (outer), right-preconditioned
// by an FP32 BiCGSTAB sweep on the FP32 copy of the operator (inner, minimum-
// residual iterate, FP64 dot products).  The outer iteration minimises the
// true FP64 residual over all corrections found so far, so a poor sweep only
// costs its iterations; x converges to the FP64 system's solution.
int run_fgmres_ir(Ctx* c, int64_t n, bsc_solve_info* si) {
    const bsc_params& P = c->P;
    const int G = RED_GRID, B = RED_BLOCK;
    const int rel_r0 = P.tol_mode == BSC_TOL_REL_R0;
    const int m = c->ir_m;
    const FgLayout F{m};
    const EllOp<double> A{c->aval, c->nbr, c->cnt, c->K.kmax, c->spmv_unroll};
    const EllPackF Af{c->ellf, c->cnt, c->K.kmax};
    double* x = c->S.p;
    double* w = c->tv;
    const int budget = std::max(50, std::min(1000, P.maxit / std::max(1, P.max_outer)));
    int first = 1, outer = 0, inner = 0;
    for (;;) {
        k_resid<EllOp<double>, double><<<G, B, 0, c->stream>>>(n, A, x, c->b, c->r, c->part);
        BSC_LAUNCH(c);
        k_fg_start<<<1, B, 0, c->stream>>>(c->part, c->sc2, c->Hd, F, first, P.tol, rel_r0);
        BSC_LAUNCH(c);
        first = 0;
        int rc = fetch_outer(c);
        if (rc) return rc;
        if (c->h_sc[1].done || outer >= P.max_outer || inner >= P.maxit) break;
        k_fg_v0<double><<<G, B, 0, c->stream>>>(n, c->r, c->V, c->sc2);
        BSC_LAUNCH(c);
        for (int j = 0; j < m && outer < P.max_outer && inner < P.maxit; ++j) {
            float* zj = c->Zf + (int64_t)j * n;
            k_d2f<<<G, B, 0, c->stream>>>(n, c->V + (int64_t)j * n, c->rf);
            BSC_CUDA(c, cudaMemsetAsync(c->xf, 0, sizeof(float) * n, c->stream));
            Work<float> wk{c->xf, c->rf, c->sf, c->rhf, c->pf, c->vf, c->tf, c->bf, nullptr};
            int it = 0;
            double rri = 0.0;
            rc = run_bicgstab<EllPackF, float>(c, n, Af, wk, P.inner_tol, 0, std::min(budget, P.maxit - inner),
                                                   &it, &rri, zj);
            if (rc && rc != BSC_E_BREAKDOWN) return rc;
            inner += it;
            ++outer;
            // |v_j| = 1: a sweep that did not reduce it falls back to z_j = v_j
            if (!(rri < 1.0) || !std::isfinite(rri)) k_d2f<<<G, B, 0, c->stream>>>(n, c->V + (int64_t)j * n, zj);
            if (c->debug) std::fprintf(stderr, "[bsc] FGMRES-IR outer %d: sweep %d iterations, |r_inner|/|v| %.3e\n",
                                       outer, it, std::sqrt(rri));
            k_spmv_z<<<G, B, 0, c->stream>>>(n, A, zj, w, c->sc2);
            for (int pass = 0; pass < 2; ++pass) {
                k_fg_mdot<double><<<G, B, 0, c->stream>>>(n, c->V, w, j, c->part, c->sc2);
                k_fg_hcol<<<1, 1024, 0, c->stream>>>(c->part, c->Hd, F, j, pass, c->sc2);
                k_fg_maxpy<double><<<G, B, 0, c->stream>>>(n, c->V, w, j, c->Hd, F, pass, c->part, c->sc2);
            }
            k_fg_givens<<<1, B, 0, c->stream>>>(c->part, c->sc2, c->Hd, F, j, nullptr);
            k_fg_next<double><<<G, B, 0, c->stream>>>(n, w, c->V, j, c->sc2);
            c->launches += 11;
            BSC_CUDA(c, cudaGetLastError());
            if ((rc = fetch_outer(c))) return rc;
            if (c->h_sc[1].tmp[2] != 0.0) break;
        }
        k_fg_backsolve<<<1, 256, 0, c->stream>>>(c->sc2, c->Hd, F);
        k_fg_update_z<<<G, B, 0, c->stream>>>(n, x, c->Zf, c->Hd, F, c->sc2);
        c->launches += 2;
        BSC_CUDA(c, cudaGetLastError());
        if (c->h_sc[1].breakdown && c->h_sc[1].tmp[1] == 0.0) break;
    }
    // true residual of the returned pressure
    double* norms = c->Hd + F.size();
    k_resid<EllOp<double>, double><<<G, B, 0, c->stream>>>(n, A, x, c->b, c->r, c->part);
    BSC_LAUNCH(c);
    k_ir_norms<<<1, B, 0, c->stream>>>(c->part, norms);
    BSC_LAUNCH(c);
    double nrm[2];
    BSC_CUDA(c, cudaMemcpyAsync(nrm, norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    si->iterations = inner;
    si->outer = outer;
    si->b_norm = c->h_sc[1].bnorm;
    si->r0_norm = c->h_sc[1].r0norm;
    si->rel_residual = nrm[1] > 0 ? nrm[0] / nrm[1] : nrm[0];
    const double ref = rel_r0 ? si->r0_norm : si->b_norm;
    si->converged = nrm[0] <= P.tol * ref ? 1 : 0;
    si->status = si->converged ? BSC_OK : BSC_E_NOT_CONVERGED;
    return si->status;
}

// with BSC_PROFILE_ITER: the phases of the last multigrid-FGMRES iteration
// (events ev_it[0..5], the stream idle) into timing slots BICG_1..5
void mg_iter_profile(Ctx* c) {
    if (!c->prof_iter) return;
    for (int k = 0; k < 5; ++k) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, c->ev_it[k], c->ev_it[k + 1]) == cudaSuccess) {
            c->ms[BSC_T_BICG_1 + k] += ms;
            c->calls[BSC_T_BICG_1 + k]++;
        }
    }
    (void)cudaGetLastError();
}

// the SpMV bracketed by ev_spmv (the stream idle) into the SPMV slot
void spmv_time(Ctx* c, int pair = 0) {
    if (!c->timing) return;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev_spmv[2 * pair], c->ev_spmv[2 * pair + 1]) == cudaSuccess) {
        c->ms[BSC_T_SPMV] += ms;
        c->calls[BSC_T_SPMV]++;
    }
    (void)cudaGetLastError();
}

// One FGMRES restart cycle of multigrid-preconditioned iterations.
// Orthogonalisation is one classical Gram-Schmidt pass (one fused dot
// kernel, one fused update): with the V-cycle the cycles are short (about
// 25 columns), and a second pass changed no iteration count at 846k rows in
// either precision while costing a third of the Krylov work per iteration.
// queue(j, mirror) queues iteration j, whose last kernel copies the scalars
// `dsc` into the pinned `mirror`.  Iteration j+1 is queued before iteration
// j's scalars are read, so the GPU never waits for the host between
// iterations; an iteration queued past the cycle's stop returns at every
// kernel.  With per-iteration profiling on (events shared by all
// iterations), each iteration is read before the next one is queued.
// `h` receives the scalars of the last iteration that ran; *iters counts them.
template <typename Q>
int fg_cycle(Ctx* c, int m, int budget, Scalars* h, int* iters, Q queue) {
    if (!c->h_it) return set_err(c, BSC_E_INVALID, "multigrid FGMRES without its pinned scalar mirror");
    const bool lag = !c->prof_iter;
    int last = -1;  // queued, not yet read
    for (int j = 0;; ++j) {
        const bool more = j < m && *iters + (lag && last >= 0 ? 1 : 0) < budget;
        if (more) {
            if (int rc = queue(j, c->h_it + (j & 1))) return rc;
            BSC_CUDA(c, cudaEventRecord(c->ev_lag[j & 1], c->stream));
        }
        const int chk = lag ? last : (more ? j : -1);
        if (chk >= 0) {
            BSC_CUDA(c, cudaEventSynchronize(c->ev_lag[chk & 1]));
            *h = c->h_it[chk & 1];
            ++*iters;
            mg_iter_profile(c);
            spmv_time(c, 1 + (chk & 1));
            if (h->tmp[2] != 0.0) return BSC_OK;  // iteration j, if queued, skips
        }
        if (!more) return BSC_OK;
        last = j;
    }
}

// Flexible GMRES(m) in FP64 on the FP64 operator, right-preconditioned by
// one FP64 multigrid V-cycle per iteration (mg.cu).  Each iteration runs as a
// cached CUDA graph, one per Krylov column.  Stops on the Arnoldi residual
// estimate and reports the true residual of the returned pressure.
int run_fgmres_mg(Ctx* c, int64_t n, bsc_solve_info* si) {
    const bsc_params& P = c->P;
    const int G = RED_GRID, B = RED_BLOCK;
    const int rel_r0 = P.tol_mode == BSC_TOL_REL_R0;
    Mg& mg = c->mg;
    const int m = mg.m;
    const FgLayout F{m};
    const EllOp<double> A{c->aval, c->nbr, c->cnt, c->K.kmax, c->spmv_unroll};
    double* x = c->S.p;
    double* w = c->tv;
    double* V = mg.V;
    double* Z = mg.Z;
    int first = 1, iters = 0, rc;
    for (;;) {
        k_resid<EllOp<double>, double><<<G, B, 0, c->stream>>>(n, A, x, c->b, c->r, c->part);
        BSC_LAUNCH(c);
        k_fg_start<<<1, B, 0, c->stream>>>(c->part, c->sc2, c->Hd, F, first, P.tol, rel_r0);
        BSC_LAUNCH(c);
        first = 0;
        if ((rc = fetch_outer(c))) return rc;
        if (c->h_sc[1].done || iters >= P.maxit) break;
        k_fg_v0<double><<<G, B, 0, c->stream>>>(n, c->r, V, c->sc2);
        BSC_LAUNCH(c);
        mg.skip = c->sc2;
        rc = fg_cycle(c, m, P.maxit, c->h_sc + 1, &iters, [&](int j, Scalars* mirror) -> int {
            double* zj = Z + (int64_t)j * n;
            const double* vj = V + (int64_t)j * n;
            // one iteration (V-cycle, SpMV, Gram-Schmidt, Givens) as a cached graph per
            // column j, keyed by the cell map too, whose buffer a Morton
            // reorder swaps
            return graph_run(c, c->pcell, vj, zj, n, [&]() -> int {
                if (int r = mg_vcycle_f64(c, vj, zj)) return r;
                // the SpMV w = A z_j is bracketed by events: the dominant
                // HBM-bound kernel, timed in place
                if (c->timing) record_event(c, c->ev_spmv[2 + 2 * (j & 1)]);
                k_spmv_z<double><<<blocks_for(n, B), B, 0, c->stream>>>(n, A, zj, w, c->sc2);
                if (c->timing) record_event(c, c->ev_spmv[3 + 2 * (j & 1)]);
                if (c->prof_iter) record_event(c, c->ev_it[4]);
                // separate single-block kernels for the column of H and the
                // Givens step: in FP64 the fused last-block forms (as on the
                // mixed path) measured slower, 122 against 107 us per
                // iteration at 846k rows (their last block has a quarter of
                // k_fg_hcol's warps)
                k_fg_mdot<double><<<G, B, 0, c->stream>>>(n, V, w, j, c->part, c->sc2);
                k_fg_hcol<<<1, 1024, 0, c->stream>>>(c->part, c->Hd, F, j, 0, c->sc2);
                k_fg_maxpy<double><<<G, B, 0, c->stream>>>(n, V, w, j, c->Hd, F, 1, c->part, c->sc2);
                k_fg_givens<<<1, B, 0, c->stream>>>(c->part, c->sc2, c->Hd, F, j, mirror);
                k_fg_next<double><<<G, B, 0, c->stream>>>(n, w, V, j, c->sc2);
                if (c->prof_iter) record_event(c, c->ev_it[5]);
                c->launches += 6;
                BSC_CUDA(c, cudaGetLastError());
                return BSC_OK;
            });
        });
        mg.skip = nullptr;
        if (rc) return rc;
        k_fg_backsolve<<<1, 256, 0, c->stream>>>(c->sc2, c->Hd, F);
        k_fg_update_z<double><<<G, B, 0, c->stream>>>(n, x, Z, c->Hd, F, c->sc2);
        c->launches += 2;
        BSC_CUDA(c, cudaGetLastError());
        if (c->h_sc[1].breakdown && c->h_sc[1].tmp[1] == 0.0) break;
    }
    double* norms = c->Hd + F.size();
    k_resid<EllOp<double>, double><<<G, B, 0, c->stream>>>(n, A, x, c->b, c->r, c->part);
    BSC_LAUNCH(c);
    k_ir_norms<<<1, B, 0, c->stream>>>(c->part, norms);
    BSC_LAUNCH(c);
    double nrm[2];
    BSC_CUDA(c, cudaMemcpyAsync(nrm, norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    si->iterations = iters;
    si->outer = 1;
    si->b_norm = c->h_sc[1].bnorm;
    si->r0_norm = c->h_sc[1].r0norm;
    si->rel_residual = nrm[1] > 0 ? nrm[0] / nrm[1] : nrm[0];
    const double ref = rel_r0 ? si->r0_norm : si->b_norm;
    si->converged = nrm[0] <= P.tol * ref ? 1 : 0;
    si->status = si->converged ? BSC_OK : BSC_E_NOT_CONVERGED;
    return si->status;
}

// ---- mixed path: FGMRES-IR with an FP32 inner FGMRES + FP32 V-cycle -------------
// The inner Krylov method runs entirely in FP32 (basis, Gram-Schmidt, SpMV,
// V-cycle); dot products are summed per thread in FP32 and across threads in
// FP64.  The outer iteration recomputes the true residual in FP64 and adds
// each FP32 correction to the FP64 pressure (iterative refinement).
__global__ void __launch_bounds__(RED_BLOCK) k_norm2f(int64_t n, const float* __restrict__ r,
                                                       double* __restrict__ part) {
    float acc = 0.f;
    GRID_LOOP(i, n) acc += r[i] * r[i];
    float a[2] = {acc, acc};
    block_partials<2>(a, part);
}

__global__ void k_fgf_v0(int64_t n, const float* __restrict__ r, float* __restrict__ V0,
                         const Scalars* __restrict__ sc) {
    if (sc->done) return;
    const float inv = (float)(1.0 / sc->tmp[0]);
    GRID_LOOP(i, n) V0[i] = r[i] * inv;
}

__global__ void k_fgf_next(int64_t n, const float* __restrict__ w, float* __restrict__ V, int j,
                           const Scalars* __restrict__ sc) {
    if (fg_skip(sc)) return;
    const float inv = (float)(1.0 / sc->tmp[3]);
    float* vn = V + (int64_t)(j + 1) * n;
    GRID_LOOP(i, n) vn[i] = w[i] * inv;
}

__global__ void __launch_bounds__(RED_BLOCK) k_spmv_f(int64_t n, EllPackF A, const float* __restrict__ z,
                                                       float* __restrict__ w, const Scalars* __restrict__ sc) {
    if (fg_skip(sc)) return;
    GRID_LOOP(i, n) w[i] = A.template row<float, float>(i, z);
}

// h_i = V_i . w for i <= j, 8 columns per pass, summed per thread in T; the
// block that finishes last (ticket taken after a fence) sums the partials
// into column j of H, one warp per dot in lane order as k_fg_hcol does
template <typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_fgf_mdot(int64_t n, const T* __restrict__ V,
                                                         const T* __restrict__ w, int j,
                                                         double* __restrict__ part, const Scalars* __restrict__ sc,
                                                         unsigned* __restrict__ ticket, double* Hd, FgLayout F) {
    if (fg_skip(sc)) return;
    for (int i0 = 0; i0 <= j; i0 += 8) {
        T acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        const int cntv = min(8, j + 1 - i0);
        GRID_LOOP(k, n) {
            const T wk = w[k];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (q < cntv) acc[q] += V[(int64_t)(i0 + q) * n + k] * wk;
        }
        block_partials<8>(acc, part + (int64_t)i0 * RED_GRID);
        __syncthreads();
    }
    __shared__ bool last;
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int i = wp; i <= j; i += nw) {
        double x = 0.0;
        for (int k = lane; k < RED_GRID; k += 32) x += __ldcg(part + (int64_t)i * RED_GRID + k);
        x = warp_sum_to_lane0(x);
        if (lane == 0) {
            Hd[F.hc(i)] = x;
            Hd[F.H(i, j)] = x;
        }
    }
    if (threadIdx.x == 0) *ticket = 0u;
}

// w -= sum_i h_i V_i and the partials of w.w; the block that finishes last
// runs the Givens step of k_fg_givens (h(j+1,j) = ||w||, rotations,
// residual estimate) and copies the scalars to the host mirror
template <typename T>
__global__ void __launch_bounds__(RED_BLOCK) k_fgf_maxpy_givens(int64_t n, const T* __restrict__ V,
                                                                 T* __restrict__ w, int j, double* Hd, FgLayout F,
                                                                 double* __restrict__ part, Scalars* sc,
                                                                 unsigned* __restrict__ ticket, Scalars* mirror) {
    if (fg_skip(sc)) {  // the cycle has stopped: publish the scalars as k_fg_givens does
        if (mirror && blockIdx.x == 0 && threadIdx.x == 0) *mirror = *sc;
        return;
    }
    __shared__ T h[FG_MAXM];
    for (int i = threadIdx.x; i <= j; i += blockDim.x) h[i] = (T)Hd[F.hc(i)];
    __syncthreads();
    T acc = 0;
    GRID_LOOP(k, n) {
        T s = w[k];
        for (int i = 0; i <= j; ++i) s -= h[i] * V[(int64_t)i * n + k];
        w[k] = s;
        acc += s * s;
    }
    T a[1] = {acc};
    block_partials<1>(a, part);
    __shared__ bool last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    fg_givens(part, sc, Hd, F, j);
    __syncthreads();
    if (threadIdx.x == 0) {
        *ticket = 0u;
        if (mirror) *mirror = *sc;
    }
}

// w -= sum_i h_i V_i; partial (w.w) when `norm`
__global__ void __launch_bounds__(RED_BLOCK) k_fgf_maxpy(int64_t n, const float* __restrict__ V, float* __restrict__ w,
                                                          int j, const double* __restrict__ Hd, FgLayout F, int norm,
                                                          double* __restrict__ part, const Scalars* __restrict__ sc) {
    if (fg_skip(sc)) return;
    __shared__ float h[FG_MAXM];
    for (int i = threadIdx.x; i <= j; i += blockDim.x) h[i] = (float)Hd[F.hc(i)];
    __syncthreads();
    float acc = 0.f;
    GRID_LOOP(k, n) {
        float s = w[k];
        for (int i = 0; i <= j; ++i) s -= h[i] * V[(int64_t)i * n + k];
        w[k] = s;
        acc += s * s;
    }
    float a[1] = {acc};
    if (norm) block_partials<1>(a, part);
}

// x += sum_i y_i z_i (FP64 pressure, FP32 preconditioned vectors)
__global__ void k_ir_addz(int64_t n, double* __restrict__ x, const float* __restrict__ Z,
                          const double* __restrict__ Hd, FgLayout F, const Scalars* __restrict__ sc) {
    if (sc->done) return;
    __shared__ double y[FG_MAXM];
    const int k = (int)sc->tmp[1];
    for (int i = threadIdx.x; i < k; i += blockDim.x) y[i] = Hd[F.y(i)];
    __syncthreads();
    GRID_LOOP(q, n) {
        double s = x[q];
        for (int i = 0; i < k; ++i) s += y[i] * (double)Z[(int64_t)i * n + q];
        x[q] = s;
    }
}

int run_fgmres_ir_mg(Ctx* c, int64_t n, bsc_solve_info* si) {
    const bsc_params& P = c->P;
    const int G = RED_GRID, B = RED_BLOCK;
    const int rel_r0 = P.tol_mode == BSC_TOL_REL_R0;
    Mg& mg = c->mg;
    const int m = mg.m;
    const FgLayout F{m};
    const EllOp<double> A{c->aval, c->nbr, c->cnt, c->K.kmax, c->spmv_unroll};
    const EllPackF Af{c->ellf, c->cnt, c->K.kmax};
    double* x = c->S.p;
    float *V = mg.Vf, *Z = mg.Zf, *w = mg.wf, *rf = mg.rf;
    // each inner solve asks for the reduction still needed (with a margin),
    // but for no more than inner_tol, the most the FP32 arithmetic is trusted
    // to deliver; the FP64 outer loop compounds the reductions
    const double floor_tol = std::min(std::max(P.inner_tol, 1e-7), 0.5);
    int first = 1, outer = 0, inner = 0, rc;
    for (;;) {
        k_resid<EllOp<double>, double><<<G, B, 0, c->stream>>>(n, A, x, c->b, c->r, c->part);
        BSC_LAUNCH(c);
        k_fg_start<<<1, B, 0, c->stream>>>(c->part, c->sc2, c->Hd, F, first, P.tol, rel_r0);
        BSC_LAUNCH(c);
        first = 0;
        if ((rc = fetch_outer(c))) return rc;
        if (c->h_sc[1].done || outer >= P.max_outer || inner >= P.maxit) break;
        ++outer;
        const double beta = c->h_sc[1].tmp[0], need = c->h_sc[1].target / beta;
        const double inner_tol = std::min(std::max(floor_tol, 0.3 * need), 0.5);
        // inner: A d = r in FP32 from d = 0, one FGMRES(m) cycle
        k_d2f<<<G, B, 0, c->stream>>>(n, c->r, rf);
        k_norm2f<<<G, B, 0, c->stream>>>(n, rf, c->part);
        k_fg_start<<<1, B, 0, c->stream>>>(c->part, c->sc, c->Hd, F, 1, inner_tol, 1);
        k_fgf_v0<<<G, B, 0, c->stream>>>(n, rf, V, c->sc);
        c->launches += 4;
        mg.skip = c->sc;
        rc = fg_cycle(c, m, P.maxit, c->h_sc, &inner, [&](int j, Scalars* mirror) -> int {
            float* zj = Z + (int64_t)j * n;
            const float* vj = V + (int64_t)j * n;
            // one inner iteration as a cached graph per column j (and cell map)
            return graph_run(c, c->pcell, vj, zj, n, [&]() -> int {
                if (int r = mg_vcycle_f32(c, vj, zj)) return r;
                // the FP32 SpMV w = A z_j is bracketed by events (the
                // dominant HBM-bound kernel, timed in place)
                if (c->timing) record_event(c, c->ev_spmv[2 + 2 * (j & 1)]);
                k_spmv_f<<<blocks_for(n, B), B, 0, c->stream>>>(n, Af, zj, w, c->sc);
                if (c->timing) record_event(c, c->ev_spmv[3 + 2 * (j & 1)]);
                if (c->prof_iter) record_event(c, c->ev_it[4]);
                // the column of H and the Givens step finish in the last
                // block of the dot and update kernels (no single-block launches)
                k_fgf_mdot<float><<<G, B, 0, c->stream>>>(n, V, w, j, c->part, c->sc, c->ticket, c->Hd, F);
                k_fgf_maxpy_givens<float><<<G, B, 0, c->stream>>>(n, V, w, j, c->Hd, F, c->part, c->sc, c->ticket,
                                                                  mirror);
                k_fgf_next<<<G, B, 0, c->stream>>>(n, w, V, j, c->sc);
                if (c->prof_iter) record_event(c, c->ev_it[5]);
                c->launches += 4;
                BSC_CUDA(c, cudaGetLastError());
                return BSC_OK;
            });
        });
        mg.skip = nullptr;
        if (rc) return rc;
        k_fg_backsolve<<<1, 256, 0, c->stream>>>(c->sc, c->Hd, F);
        k_ir_addz<<<G, B, 0, c->stream>>>(n, x, Z, c->Hd, F, c->sc);
        c->launches += 2;
        BSC_CUDA(c, cudaGetLastError());
        if (c->debug)
            std::fprintf(stderr, "[bsc] FGMRES-IR outer %d: |r|/target %.3e, inner tol %.1e, %d inner iterations\n",
                         outer, beta / c->h_sc[1].target, inner_tol, inner);
    }
    double* norms = c->Hd + F.size();
    k_resid<EllOp<double>, double><<<G, B, 0, c->stream>>>(n, A, x, c->b, c->r, c->part);
    BSC_LAUNCH(c);
    k_ir_norms<<<1, B, 0, c->stream>>>(c->part, norms);
    BSC_LAUNCH(c);
    double nrm[2];
    BSC_CUDA(c, cudaMemcpyAsync(nrm, norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    si->iterations = inner;
    si->outer = outer;
    si->b_norm = c->h_sc[1].bnorm;
    si->r0_norm = c->h_sc[1].r0norm;
    si->rel_residual = nrm[1] > 0 ? nrm[0] / nrm[1] : nrm[0];
    const double ref = rel_r0 ? si->r0_norm : si->b_norm;
    si->converged = nrm[0] <= P.tol * ref ? 1 : 0;
    si->status = si->converged ? BSC_OK : BSC_E_NOT_CONVERGED;
    return si->status;
}

int solve_status(bsc_solve_info* info, int rc) {
    if (rc != BSC_OK) return rc;
    return info->converged ? BSC_OK : BSC_E_NOT_CONVERGED;
}

// x <- solution of the PPE, warm-started from the current pressure
int op_ppe_solve(Ctx* c, bsc_solve_info* info) {
    if (!c->have_csr) return set_err(c, BSC_E_INVALID, "ppe solve before assembly");
    const int64_t n = c->n;
    const bsc_params& P = c->P;
    const int rel_r0 = P.tol_mode == BSC_TOL_REL_R0;
    bsc_solve_info loc{};
    bsc_solve_info* si = info ? info : &loc;
    *si = bsc_solve_info{};
    int rc = BSC_OK, iters = 0;
    double rr = 0.0;
    if (P.precond == BSC_PRECOND_MG) {
        if ((rc = mg_setup(c))) return rc;
        return c->mixed ? run_fgmres_ir_mg(c, n, si) : run_fgmres_mg(c, n, si);
    }
    if (!c->mixed) {
        EllOp<double> A{c->aval, c->nbr, c->cnt, c->K.kmax, c->spmv_unroll};
        Work<double> w{c->S.p, c->b, c->r, c->rh, c->pd, c->v, c->s, c->tv, c->V};
        if (P.solver == BSC_SOLVER_FGMRES)
            rc = run_fgmres<EllOp<double>, double>(c, n, A, w, P.tol, rel_r0, P.maxit, c->fg_m, &iters, &rr);
        else
            rc = run_bicgstab<EllOp<double>, double>(c, n, A, w, P.tol, rel_r0, P.maxit, &iters, &rr);
        if (rc && rc != BSC_E_BREAKDOWN) return rc;
        // true residual of the returned pressure
        k_resid<EllOp<double>, double><<<RED_GRID, RED_BLOCK, 0, c->stream>>>(n, A, c->S.p, c->b, c->r, c->part);
        BSC_LAUNCH(c);
        k_ir_norms<<<1, RED_BLOCK, 0, c->stream>>>(c->part, c->Hd + FgLayout{c->fg_m}.size());
        BSC_LAUNCH(c);
        double nrm[2];
        BSC_CUDA(c, cudaMemcpyAsync(nrm, c->Hd + FgLayout{c->fg_m}.size(), 2 * sizeof(double), cudaMemcpyDeviceToHost,
                                    c->stream));
        BSC_CUDA(c, cudaStreamSynchronize(c->stream));
        si->iterations = iters;
        si->outer = 1;
        si->b_norm = c->h_sc->bnorm;
        si->r0_norm = c->h_sc->r0norm;
        si->rel_residual = nrm[1] > 0 ? nrm[0] / nrm[1] : nrm[0];
        const double ref = rel_r0 ? si->r0_norm : si->b_norm;
        si->converged = (c->h_sc->done != 0) || (nrm[0] <= P.tol * ref);
        si->status = c->h_sc->breakdown && !si->converged ? BSC_E_BREAKDOWN
                     : (si->converged ? BSC_OK : BSC_E_NOT_CONVERGED);
        return si->status;
    }
    // ---- mixed: FGMRES-IR (FP64 outer, FP32 BiCGSTAB sweeps)
    return run_fgmres_ir(c, n, si);
}

// ---- standalone CSR solve (device buffers allocated by the caller context) ----
int csr_solve_device(Ctx* c, int32_t n, const int32_t* rp, const int32_t* col, const double* val, const double* b,
                     double* x, bsc_solve_info* info) {
    CsrOp A{rp, col, val};
    double* work = c->r;  // [r rh p v s t] laid out by the caller
    Work<double> w{x, const_cast<double*>(b), work, work + n, work + 2 * n, work + 3 * n, work + 4 * n, work + 5 * n,
                   c->V};
    const bsc_params& P = c->P;
    const int rel_r0 = P.tol_mode == BSC_TOL_REL_R0;
    int iters = 0;
    double rr = 0;
    int rc = (P.solver == BSC_SOLVER_FGMRES)
                 ? run_fgmres<CsrOp, double>(c, n, A, w, P.tol, rel_r0, P.maxit, c->fg_m, &iters, &rr)
                 : run_bicgstab<CsrOp, double>(c, n, A, w, P.tol, rel_r0, P.maxit, &iters, &rr);
    if (rc) return rc;
    k_resid<CsrOp, double><<<RED_GRID, RED_BLOCK, 0, c->stream>>>(n, A, x, b, work, c->part);
    BSC_LAUNCH(c);
    double* norms = c->Hd + FgLayout{c->fg_m}.size();
    k_ir_norms<<<1, RED_BLOCK, 0, c->stream>>>(c->part, norms);
    BSC_LAUNCH(c);
    double nrm[2];
    BSC_CUDA(c, cudaMemcpyAsync(nrm, norms, 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    info->iterations = iters;
    info->outer = 1;
    info->b_norm = c->h_sc->bnorm;
    info->r0_norm = c->h_sc->r0norm;
    info->rel_residual = nrm[1] > 0 ? nrm[0] / nrm[1] : nrm[0];
    const double ref = rel_r0 ? info->r0_norm : info->b_norm;
    info->converged = (c->h_sc->done != 0) || nrm[0] <= P.tol * ref;
    info->status = info->converged ? BSC_OK : (c->h_sc->breakdown ? BSC_E_BREAKDOWN : BSC_E_NOT_CONVERGED);
    return info->status;
}

int fg_layout_size(int m) { return FgLayout{m}.size() + 8; }

}  // namespace bsc
