// pairs.cu -- neighbour search and the per-pair SPH operators.
//
// One thread per particle.  Candidates come from the 3x3 block of 2h cells
// around the particle (the reference scans the 2x2 block of 4h cells picked
// by the particle's quadrant, search.f90:328-388; both blocks contain the
// whole 2h disc, so the neighbour sets are the same).  The neighbour test is
// the reference's sqrt((xi-xj)^2+(yi-yj)^2) < 2h (functions.f90:38,
// search.f90:59) evaluated with correctly rounded FP64 operations and no
// contraction, so the sets are bit-identical to the CPU restatement; an FP32
// pre-test with a 1e-5 relative margin rejects the far candidates first.
//
// Every operator is templated on R, the type of the pair arithmetic: double
// for the FP64 drop-in path, float for the mixed path (which keeps the
// particle state, the neighbour predicate and the 2x2 inversion in FP64).
#include <algorithm>
#include <cmath>

#include "bsc_internal.cuh"
#include "dfloat.cuh"
#include "sph_kernel.cuh"

namespace bsc {

// vis(oden) of porous.f90:12-30 / integrator.f90:12-30
__device__ __forceinline__ double vis_of(double oden) {
    double Sp = oden - 1000.0;
    return (1.002 + 0.001652 * Sp + 0.0000083 * (Sp * Sp)) * 0.001;
}

__device__ __forceinline__ double porosity_at(const KParams& K, double x, double y) {
    if (K.pnx <= 0) return K.por;
    double fx = floor((x - K.px0) / K.pdx), fy = floor((y - K.py0) / K.pdy);
    if (!(fx >= 0.0 && fx < (double)K.pnx && fy >= 0.0 && fy < (double)K.pny)) return K.por;
    return K.pgrid[(int64_t)fy * K.pnx + (int64_t)fx];
}

// ---- FP32 pre-test of the pair searches -----------------------------------------------
// Positions are kept as float offsets from the origin of their own cell, so
// a candidate in the neighbouring cell (ax, ay) sits at its offset plus an
// exact shift of 0 or +-cs.  With offsets below PRE_GUARD cells the float
// estimate of r^2 is within ~1e-6 (relative) of the exact one, far inside
// the 1e-5 margin: the pre-test only rejects candidates that the exact FP64
// test would reject too.  Particles farther from their binned cell skip it.
constexpr float PRE_GUARD = 4.0f;
constexpr double PRE_MARGIN = 1e-5;

__device__ __forceinline__ bool pre_ok(float2 p, float csf) {
    return fabsf(p.x) < PRE_GUARD * csf && fabsf(p.y) < PRE_GUARD * csf;
}

// (mixed path: also V as a double-float, {f_vol, f_vol_lo}: its FP32 twin
// for the neighbour search's M sum; and the offsets as double-floats,
// (hi x, lo x, hi y, lo y))
__global__ void k_posf(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                       const int32_t* __restrict__ pcell, KParams K, float2* __restrict__ posf,
                       const double* __restrict__ vol, float* __restrict__ f_vol, float* __restrict__ f_vol_lo,
                       float4* __restrict__ posd) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = pcell[i], cx = c / K.ny, cy = c - cx * K.ny;
    const double ox = x[i] - (K.gx0 + cx * K.cs), oy = y[i] - (K.gy0 + cy * K.cs);
    posf[i] = make_float2((float)ox, (float)oy);
    if (f_vol) {
        const df2 vd = df_of(vol[i]);
        f_vol[i] = vd.hi;
        f_vol_lo[i] = vd.lo;
    }
    if (posd) {
        const df2 dx = df_of(ox), dy = df_of(oy);
        posd[i] = make_float4(dx.hi, dx.lo, dy.hi, dy.lo);
    }
}

// ---- search.f90:13-399 neighbour / nsearch2 ----------------------------------------
// PRE: the candidate phase already ran (k_cand_warpcell): `cand_nc` holds
// each row's number of survivors in its list slots, or -1 for a row that
// takes the one-pass loop.
template <typename R, bool PRE = false>
__global__ void __launch_bounds__(NB_BLOCK) k_neighbour(int64_t n, State S, KParams K,
                                                         const int32_t* __restrict__ cstart,
                                                         const int32_t* __restrict__ ccount,
                                                         const int32_t* __restrict__ sorted,
                                                         const int32_t* __restrict__ pcell,
                                                         const float2* __restrict__ posf,
                                                         const float4* __restrict__ posd,
                                                         int32_t* __restrict__ nbr, double2* __restrict__ gw,
                                                         float2* __restrict__ gwf, float2* __restrict__ gwl,
                                                         const float* __restrict__ f_vol,
                                                         double* __restrict__ ndist, int32_t* __restrict__ cnt,
                                                         int32_t* __restrict__ flag,
                                                         const int32_t* __restrict__ cand_nc = nullptr) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = S.x[i], yi = S.y[i];
    const int c = pcell[i], cx = c / K.ny, cy = c - cx * K.ny;
    const float H2f = (float)(K.H2 * (1.0 + PRE_MARGIN));
    const float csf = (float)K.cs;
    const float2 pi = posf[i];
    const bool pre_i = pre_ok(pi, csf);
    R m0 = 0, m1 = 0, m2 = 0, m3 = 0;
    int count = 0, nc = 0;
    // Mixed path, Wendland kernel: the pair's geometry and grad W in
    // double-float arithmetic (dfloat.cuh) from the double-float offsets to
    // the cells' origins.  r^2 comes out within ~1e-12 of the r^2 of the
    // FP64 positions (the offsets keep 2^-48 of a cell; the FP64 cell
    // origins round by ~4e-16 m), and the FP64 test rounds d^2 by ~4e-16 of
    // itself, so wherever r^2 lies more than 1e-10 of T from the threshold
    // the two agree: only candidates inside that band take the exact FP64
    // test, and the sets stay those of the FP64 predicate.  Per pair the
    // FP64 pipe keeps the widening of the stored grad W (2 operations, ~14
    // before).  Particles far from their binned cell (no pre-test) take the
    // FP64 work below.
    [[maybe_unused]] const bool use_df = sizeof(R) == 4 && posd && K.kernel == BSC_KERNEL_WENDLAND_C2 && pre_i;
    [[maybe_unused]] df2 oxi{0.f, 0.f}, oyi{0.f, 0.f};
    [[maybe_unused]] df2 cs_df{0.f, 0.f}, T_df{0.f, 0.f}, hih{0.f, 0.f}, mwF{0.f, 0.f};
    [[maybe_unused]] float band = 0.f;
    if constexpr (sizeof(R) == 4) {
        if (use_df) {
            const float4 oi = posd[i];
            oxi = {oi.x, oi.y};
            oyi = {oi.z, oi.w};
            cs_df = df_of(K.cs);
            T_df = df_of(K.H2x);
            hih = df_of(K.half_inv_h);
            mwF = df_of(-K.wend_F);
            band = (float)(1e-10 * K.H2);
        }
    }
    // the FP64 work of one candidate: the exact test, grad W, the list entry
    // and the M sum
    auto pair = [&](int j) {
        if constexpr (sizeof(R) == 4) {
            if (use_df) {
                const float4 oj = posd[j];
                if (pre_ok(make_float2(oj.x, oj.z), csf)) {
                    const int cj = pcell[j], cxj = cj / K.ny, cyj = cj - cxj * K.ny;
                    const df2 ddx = df_pair_offset(oxi, make_float2(oj.x, oj.y), cx - cxj, cs_df);
                    const df2 ddy = df_pair_offset(oyi, make_float2(oj.z, oj.w), cy - cyj, cs_df);
                    const df2 r2 = df_add(df_sqr(ddx), df_sqr(ddy));
                    const float side = df_sub(r2, T_df).hi;
                    bool in = side < -band;
                    if (!in && !(side > band)) {  // within the band: the FP64 predicate decides
                        const double dx = xi - S.x[j], dy = yi - S.y[j];
                        in = nonneg_below(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), K.H2x);
                    }
                    if (!in) return;
                    const df2 r = r2.hi > 0.f ? df_sqrt(r2) : df2{0.f, 0.f};
                    const df2 a = df_sub(df2{1.f, 0.f}, df_mul(r, hih));
                    const df2 F = df_mul(df_mul(mwF, a), df_sqr(a));  // -F_W (1 - r/2h)^3
                    const df2 gx = df_mul(F, ddx), gy = df_mul(F, ddy);
                    if (count < K.kmax) {
                        const int64_t e = ell(i, count, K.kmax);
                        nbr[e] = j;
                        // grad W stored as the double-float it is; the FP64
                        // copy only for the FP64 assembly variants
                        if (gw) gw[e] = {df_to_double(gx), df_to_double(gy)};
                        gwf[e] = {gx.hi, gy.hi};
                        if (gwl) gwl[e] = {gx.lo, gy.lo};
                        if (ndist) ndist[e] = df_to_double(r);
                    }
                    ++count;
                    const float vj = f_vol[j];
                    const float rx = -vj * ddx.hi, ry = -vj * ddy.hi;  // m_j (x_j - x_i) / rho_j
                    m0 += gx.hi * rx;
                    m1 += gy.hi * rx;
                    m2 += gx.hi * ry;
                    m3 += gy.hi * ry;
                    return;
                }
            }
        }
        const double dx = xi - S.x[j], dy = yi - S.y[j];
        const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
        // exactly sqrt(d2) < 2h, no FMA contraction; the comparison on the
        // integer pipe (d2 >= 0)
        if (!nonneg_below(d2, K.H2x)) return;
        // the mixed path's root by Newton from an FP32 seed (within 2^-42;
        // the FP64 pipe is this kernel's bound), the FP64 path's correctly
        // rounded
        const double r = sizeof(R) == 4 ? (__double_as_longlong(d2) != 0 ? sqrt_nr(d2) : 0.0) : __dsqrt_rn(d2);
        // grad W per pair in FP64 (stored in FP64, and in FP32 for the FP32
        // pair sums of the mixed path); the M sum runs in R
        const double F = grad_factor<double>(K, r);
        const double gx64 = F * dx, gy64 = F * dy;
        // the FP32 path's values come from the integer-pipe rounding (f32_of)
        // and the FP32 twin of V: no per-pair conversion on the FP64 pipe
        constexpr bool F32 = sizeof(R) == 4;
        const R gx = F32 ? (R)f32_of(gx64) : (R)gx64, gy = F32 ? (R)f32_of(gy64) : (R)gy64;
        if (count < K.kmax) {
            const int64_t e = ell(i, count, K.kmax);
            nbr[e] = j;
            if (gw) gw[e] = {gx64, gy64};
            if (gwl) {  // the mixed path's double-float grad W (hi: the FP32 rounding)
                const df2 ax = df_of(gx64), ay = df_of(gy64);
                gwf[e] = {ax.hi, ay.hi};
                gwl[e] = {ax.lo, ay.lo};
            } else if (gwf) {
                gwf[e] = {(float)gx, (float)gy};
            }
            if (ndist) ndist[e] = r;
        }
        ++count;
        const R vj = F32 ? (R)f_vol[j] : (R)S.vol[j];
        const R fdx = F32 ? (R)f32_of(dx) : (R)dx, fdy = F32 ? (R)f32_of(dy) : (R)dy;
        const R rx = -vj * fdx, ry = -vj * fdy;  // m_j (x_j - x_i) / rho_j
        m0 += gx * rx;
        m1 += gy * rx;
        m2 += gx * ry;
        m3 += gy * ry;
    };
    if constexpr (PRE) {
        nc = cand_nc[i];
        const bool ok = nc >= 0 && nc <= K.kmax;
        if (ok)
            for (int k = 0; k < nc; ++k) pair(nbr[ell(i, k, K.kmax)]);
        else
            nc = K.kmax + 1;  // the one-pass loop below
    } else if (pre_i) {
        // Two phases, so the FP64 work runs on full warps: (1) the FP32
        // pre-test compacts the surviving candidates, in cell-list order,
        // into this row's list slots; (2) the FP64 pair work walks them.  A
        // warp's lanes would otherwise take their FP64 branches at different
        // candidates, and the FP64 pipe (2 lanes a clock per SM here) would
        // run mostly idle lanes.  The pre-test margin lets through only
        // candidates within 1e-5 of the support, so phase 2 rejects almost
        // none.  A row whose survivors exceed the list capacity takes the
        // one-pass loop below, which counts the true neighbours.
        for (int ax = cx - 1; ax <= cx + 1; ++ax) {
            if (ax < 0 || ax >= K.nx) continue;
            const float shx = (float)(ax - cx) * csf;
            for (int ay = cy - 1; ay <= cy + 1; ++ay) {
                if (ay < 0 || ay >= K.ny) continue;
                const float shy = (float)(ay - cy) * csf;
                const int cc = ax * K.ny + ay;
                const int s0 = cstart[cc], s1 = s0 + ccount[cc];
                for (int s = s0; s < s1; ++s) {
                    const int j = sorted[s];
                    if (j == (int)i) continue;  // (tid,matid) self test, search.f90:53-55
                    const float2 pj = posf[j];
                    if (pre_ok(pj, csf)) {
                        const float fdx = pi.x - (pj.x + shx), fdy = pi.y - (pj.y + shy);
                        if (fdx * fdx + fdy * fdy > H2f) continue;
                    }
                    if (nc < K.kmax) nbr[ell(i, nc, K.kmax)] = j;
                    ++nc;
                }
            }
        }
        // slot `count` <= k is written only after slot k is read
        if (nc <= K.kmax)
            for (int k = 0; k < nc; ++k) pair(nbr[ell(i, k, K.kmax)]);
    }
    if ((!PRE && !pre_i) || nc > K.kmax) {
        // far from its binned cell (no pre-test), or too many survivors: one
        // pass over the 3x3 cells
        for (int ax = cx - 1; ax <= cx + 1; ++ax) {
            if (ax < 0 || ax >= K.nx) continue;
            for (int ay = cy - 1; ay <= cy + 1; ++ay) {
                if (ay < 0 || ay >= K.ny) continue;
                const int cc = ax * K.ny + ay;
                const int s0 = cstart[cc], s1 = s0 + ccount[cc];
                for (int s = s0; s < s1; ++s) {
                    const int j = sorted[s];
                    if (j != (int)i) pair(j);
                }
            }
        }
    }
    if (count > K.kmax) {
        atomicOr(flag, 1);
        count = K.kmax;
    }
    cnt[i] = count;
    uint8_t f = S.flags[i] & (uint8_t)~BSC_FLAG_FREE;  // search.f90:41
    double gv = 0.0;
    if (S.tid[i] == BSC_TID_FLUID) {  // search.f90:268-306
        f &= (uint8_t)~BSC_FLAG_VICINITY;
        const double a0 = m0, a1 = m1, a2 = m2, a3 = m3;
        gv = a0 + a3;
        // invertmat2D (functions.f90:62-96), FP64 in both precisions
        const double det = __dsub_rn(__dmul_rn(a0, a3), __dmul_rn(a1, a2));
        double l0 = 1.0, l1 = 0.0, l2 = 0.0, l3 = 1.0;
        if (fabs(det) >= (double)1e-5f && isfinite(det)) {
            l0 = a3 / det;
            l1 = -a1 / det;
            l2 = -a2 / det;
            l3 = a0 / det;
        }
        S.L0[i] = l0; S.L1[i] = l1; S.L2[i] = l2; S.L3[i] = l3;
        if (gv <= K.free_thr && !(f & BSC_FLAG_BUFFER)) f |= BSC_FLAG_FREE;
    }
    S.gradvx[i] = gv;
    S.flags[i] = f;
}

// ---- warp-per-cell candidate phase (BSC_NEIGHBOUR=warpcell) ----------------------
// One warp per cell of the grid.  The warp stages the candidates of the 3x3
// cells around its cell in shared memory (their indices and float offsets
// from the cell's origin), with coalesced loads of the cell lists; then, for
// each particle of the cell in turn, its 32 lanes pre-test 32 staged
// candidates at a time and a ballot compacts the survivors, in the same cell
// order as the thread-per-particle kernel, into the particle's list slots.
// k_neighbour<R, true> then runs the FP64 phase over those slots, so the
// lists and results are the same as the one-kernel search.  A row is handed
// to the one-pass loop (cand_nc = -1) when its cell's candidates exceed the
// staging capacity or the particle sits too far from its binned cell.
constexpr int WC_WARPS = 4, WC_CAP = 192;

__global__ void __launch_bounds__(WC_WARPS * 32) k_cand_warpcell(int ncell, KParams K,
                                                                   const int32_t* __restrict__ cstart,
                                                                   const int32_t* __restrict__ ccount,
                                                                   const int32_t* __restrict__ sorted,
                                                                   const float2* __restrict__ posf,
                                                                   int32_t* __restrict__ nbr,
                                                                   int32_t* __restrict__ cand_nc) {
    __shared__ int32_t sj[WC_WARPS][WC_CAP];
    __shared__ float2 sp[WC_WARPS][WC_CAP];
    const int wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    const float csf = (float)K.cs;
    const float H2f = (float)(K.H2 * (1.0 + PRE_MARGIN));
    const float far = __int_as_float(0x7f800000);  // +inf: a candidate that skips the pre-test
    for (int c = blockIdx.x * WC_WARPS + wib; c < ncell; c += gridDim.x * WC_WARPS) {
        const int mc = ccount[c];
        if (mc == 0) continue;
        const int cx = c / K.ny, cy = c - cx * K.ny;
        int total = 0;
        for (int ax = cx - 1; ax <= cx + 1; ++ax) {
            if (ax < 0 || ax >= K.nx) continue;
            const float shx = (float)(ax - cx) * csf;
            for (int ay = cy - 1; ay <= cy + 1; ++ay) {
                if (ay < 0 || ay >= K.ny) continue;
                const float shy = (float)(ay - cy) * csf;
                const int cc = ax * K.ny + ay;
                const int s0 = cstart[cc], m = ccount[cc];
                for (int q = lane; q < m; q += 32) {
                    const int idx = total + q;
                    if (idx < WC_CAP) {
                        const int j = sorted[s0 + q];
                        const float2 pj = posf[j];
                        sj[wib][idx] = j;
                        sp[wib][idx] = pre_ok(pj, csf) ? make_float2(pj.x + shx, pj.y + shy) : make_float2(far, 0.f);
                    }
                }
                total += m;
            }
        }
        __syncwarp();
        const int s0c = cstart[c];
        for (int q = 0; q < mc; ++q) {
            const int i = sorted[s0c + q];
            const float2 pi = posf[i];
            if (total > WC_CAP || !pre_ok(pi, csf)) {
                if (lane == 0) cand_nc[i] = -1;
                continue;
            }
            int nc = 0;
            for (int base = 0; base < total; base += 32) {
                const int k = base + lane;
                int j = -1;
                bool keep = false;
                if (k < total) {
                    j = sj[wib][k];
                    if (j != i) {
                        const float2 p = sp[wib][k];
                        if (p.x == far) {
                            keep = true;
                        } else {
                            const float fdx = pi.x - p.x, fdy = pi.y - p.y;
                            keep = !(fdx * fdx + fdy * fdy > H2f);
                        }
                    }
                }
                const unsigned bal = __ballot_sync(0xffffffffu, keep);
                if (keep) {
                    const int pos = nc + __popc(bal & below);
                    if (pos < K.kmax) nbr[ell(i, pos, K.kmax)] = j;
                }
                nc += __popc(bal);
            }
            if (lane == 0) cand_nc[i] = nc;
        }
        __syncwarp();
    }
}

int op_neighbour(Ctx* c) {
    k_posf<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S.x, c->S.y, c->pcell, c->K, c->posf, c->S.vol,
                                                         c->mixed ? c->f_vol : nullptr,
                                                         c->mixed ? c->f_vol_lo : nullptr,
                                                         c->mixed ? c->posd : nullptr);
    BSC_LAUNCH(c);
    const unsigned g = blocks_for(c->n, NB_BLOCK);
    // mixed path: grad W as a double-float only, unless an FP64 assembly
    // variant (BSC_ASSEMBLY=rcp, BSC_EXACT_DIV=1) reads the FP64 copy
    double2* gw64 = (c->asm_rcp || c->exact_div) ? c->gw : nullptr;
    StageTimer tk(c, BSC_T_K_NEIGHBOUR);
    if (c->nb_warpcell) {
        const unsigned gc = (unsigned)std::min<int64_t>((c->ncell + WC_WARPS - 1) / WC_WARPS, 152 * 32);
        k_cand_warpcell<<<gc, WC_WARPS * 32, 0, c->stream>>>((int)c->ncell, c->K, c->cell_start, c->cell_count,
                                                              c->sorted, c->posf, c->nbr, c->cand_nc);
        BSC_LAUNCH(c);
        if (c->mixed)
            k_neighbour<float, true><<<g, NB_BLOCK, 0, c->stream>>>(
                c->n, c->S, c->K, c->cell_start, c->cell_count, c->sorted, c->pcell, c->posf, c->posd, c->nbr, gw64,
                c->gwf, c->gwl, c->f_vol, c->ndist, c->cnt, c->d_flag, c->cand_nc);
        else
            k_neighbour<double, true><<<g, NB_BLOCK, 0, c->stream>>>(
                c->n, c->S, c->K, c->cell_start, c->cell_count, c->sorted, c->pcell, c->posf, nullptr, c->nbr, c->gw,
                nullptr, nullptr, nullptr, c->ndist, c->cnt, c->d_flag, c->cand_nc);
    } else if (c->mixed)
        k_neighbour<float><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->cell_start, c->cell_count, c->sorted,
                                                          c->pcell, c->posf, c->posd, c->nbr, gw64, c->gwf, c->gwl,
                                                          c->f_vol, c->ndist, c->cnt, c->d_flag);
    else
        k_neighbour<double><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->cell_start, c->cell_count,
                                                           c->sorted, c->pcell, c->posf, nullptr, c->nbr, c->gw,
                                                           nullptr, nullptr, nullptr, c->ndist, c->cnt, c->d_flag);
    BSC_LAUNCH(c);
    c->have_lists = true;
    return BSC_OK;
}

// ---- isph.f90:49-86 freesurf, gather form --------------------------------------
// vicinity_j |= (exists neighbour i: fluid, not buffer, tr M_i <= threshold).
// The neighbour relation is symmetric, so j's own list enumerates the i that
// would have scattered to it; this removes the reference's racy scatter.
__global__ void k_freesurf(int64_t n, State S, KParams K, const int32_t* __restrict__ nbr,
                           const int32_t* __restrict__ cnt) {
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    const int m = cnt[j];
    bool hit = false;
    for (int k = 0; k < m && !hit; ++k) {
        const int i = nbr[ell(j, k, K.kmax)];
        hit = (S.tid[i] == BSC_TID_FLUID) && !(S.flags[i] & BSC_FLAG_BUFFER) && (S.gradvx[i] <= K.free_thr);
    }
    if (hit) S.flags[j] |= BSC_FLAG_VICINITY;
}

int op_freesurf(Ctx* c) {
    k_freesurf<<<blocks_for(c->n, NB_BLOCK), NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->cnt);
    BSC_LAUNCH(c);
    return BSC_OK;
}

// ---- porous.f90:107-224 effpor ---------------------------------------------------
template <typename R>
__global__ void __launch_bounds__(NB_BLOCK) k_effpor(int64_t n, State S, KParams K, const int32_t* __restrict__ pcell,
                                                      const int32_t* __restrict__ scs, const int32_t* __restrict__ scc,
                                                      const double* __restrict__ sx, const double* __restrict__ sy,
                                                      const float2* __restrict__ sposf,
                                                      const float* __restrict__ swf,
                                                      const double* __restrict__ svol,
                                                      const double* __restrict__ spor,
                                                      float* __restrict__ f_vol = nullptr,
                                                      float* __restrict__ f_vol_lo = nullptr) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    S.resist[i] = 0.0;
    if (S.tid[i] != BSC_TID_FLUID) return;
    const double xi = S.x[i], yi = S.y[i];
    const int c = pcell[i], cx = c / K.ny, cy = c - cx * K.ny;
    const float H2f = (float)(K.H2 * (1.0 + PRE_MARGIN));
    const float csf = (float)K.cs;
    const float2 pi = make_float2((float)(xi - (K.gx0 + cx * K.cs)), (float)(yi - (K.gy0 + cy * K.cs)));
    const bool pre_i = pre_ok(pi, csf);
    R frac = 0;
    // mixed path: the FP32 terms summed as a double-float (TwoSum on the FP32
    // pipe; ~48 bits, more than the FP64 sum of FP32 terms needed, with no
    // FP64 work inside the divergent candidate loop)
    df2 fsum{0.0f, 0.0f};
    // the FP64 work of one solid: the exact test and its weighted W
    auto solid_term = [&](int s) {
        const double dx = xi - sx[s], dy = yi - sy[s];
        const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
        if (!nonneg_below(d2, K.H2x)) return;  // exactly sqrt(d2) < 2h
        // W(r) in R: an FP32 root for the FP32 sum, the exact one for FP64
        const R r = sizeof(R) == 4 ? (R)sqrtf((float)d2) : (R)__dsqrt_rn(d2);
        frac += ((R)1 - (R)spor[s]) * kern_w<R>(K, r) * (R)svol[s];
    };
    // FP64 path, two phases as in the neighbour search: the FP32 pre-test
    // first compacts the surviving solids (in cell order) into this thread's
    // column of shared memory, then the FP64 terms run over them on full
    // warps.  In one pass the FP64 work sat inside the divergent candidate
    // loop, at about half the lanes of each FP64 instruction.  The sum keeps
    // its order, so the result is the same.  A particle with more survivors
    // than the column holds, or far from its binned cell, takes the one pass.
    constexpr int EP_CAP = 32;
    __shared__ int32_t cand[sizeof(R) == 8 ? EP_CAP * NB_BLOCK : 1];
    bool one_pass = true;
    if constexpr (sizeof(R) == 8) {
        if (pre_i) {
            int nc = 0;
            for (int ax = cx - 1; ax <= cx + 1; ++ax) {
                if (ax < 0 || ax >= K.nx) continue;
                const float shx = (float)(ax - cx) * csf;
                for (int ay = cy - 1; ay <= cy + 1; ++ay) {
                    if (ay < 0 || ay >= K.ny) continue;
                    const float shy = (float)(ay - cy) * csf;
                    const int cc = ax * K.ny + ay;
                    const int s0 = scs[cc], s1 = s0 + scc[cc];
                    for (int s = s0; s < s1; ++s) {
                        const float2 ps = sposf[s];
                        if (pre_ok(ps, csf)) {
                            const float fdx = pi.x - (ps.x + shx), fdy = pi.y - (ps.y + shy);
                            if (fdx * fdx + fdy * fdy > H2f) continue;
                        }
                        if (nc < EP_CAP) cand[nc * NB_BLOCK + threadIdx.x] = s;
                        ++nc;
                    }
                }
            }
            if (nc <= EP_CAP) {
                one_pass = false;
                for (int k = 0; k < nc; ++k) solid_term(cand[k * NB_BLOCK + threadIdx.x]);
            }
        }
    }
    if (one_pass) {
        for (int ax = cx - 1; ax <= cx + 1; ++ax) {
            if (ax < 0 || ax >= K.nx) continue;
            const float shx = (float)(ax - cx) * csf;
            for (int ay = cy - 1; ay <= cy + 1; ++ay) {
                if (ay < 0 || ay >= K.ny) continue;
                const float shy = (float)(ay - cy) * csf;
                const int cc = ax * K.ny + ay;
                const int s0 = scs[cc], s1 = s0 + scc[cc];
                for (int s = s0; s < s1; ++s) {
                    const float2 ps = sposf[s];
                    if (pre_i && pre_ok(ps, csf)) {
                        const float fdx = pi.x - (ps.x + shx), fdy = pi.y - (ps.y + shy);
                        const float r2f = fdx * fdx + fdy * fdy;
                        if (r2f > H2f) continue;
                        if constexpr (sizeof(R) == 4) {
                            // Mixed path: each term in FP32 (W is continuous
                            // and vanishes at r = 2h, so the FP32 distance
                            // decides nothing that matters; weight
                            // (1-n_s) V_s), the sum as a double-float. The
                            // FP32 running sum was the main error of the mixed
                            // velocities (1.1e-6 against FP64 after the
                            // benchmark's steps; 6.7e-7 with a wide sum).
                            if (r2f < (float)K.H2)
                                fsum = df_add_f(fsum, swf[s] * kern_w<float>(K, sqrtf(r2f)));
                            continue;
                        }
                    }
                    solid_term(s);
                }
            }
        }
    }
    double sf = (double)frac + df_to_double(fsum);
    const double cap = 1.0 - porosity_at(K, xi, yi);
    if (sf > cap) sf = cap;
    const double nn = 1.0 - sf;
    const double oden = S.oden[i];
    const double rho = nn * oden;
    S.por[i] = nn;
    S.rho[i] = rho;
    S.vol[i] = S.mass[i] / rho;
    if (f_vol) {  // mixed path: V's double-float twin follows V
        const df2 vd = df_of(S.vol[i]);
        f_vol[i] = vd.hi;
        f_vol_lo[i] = vd.lo;
    }
    // Ergun/Darcy-Forchheimer coefficient (porous.f90:192,204-212),
    // Fch*sqrt(lamk) written as beta/sqrt(n^3)
    if constexpr (sizeof(R) == 4) {
        // FP32 on the mixed path (its divisions and roots would dominate this
        // kernel on the FP64 pipe); the coefficient only enters the implicit
        // drag factor 1/(1 - dt R n)
        const float nf = (float)nn, n3 = nf * nf * nf, d = (float)K.d50, od = (float)oden;
        const float vx = (float)S.vx[i], vy = (float)S.vy[i];
        const float vmag = sqrtf(vx * vx + vy * vy), sp = od - 1000.f;
        const float mu = (1.002f + 0.001652f * sp + 0.0000083f * (sp * sp)) * 0.001f;
        const float rn3 = sqrtf(n3);
        S.resist[i] = (double)(-((mu / od) * (float)K.alpha * ((1.f - nf) * (1.f - nf)) / (n3 * (d * d))) -
                               ((float)K.beta / rn3) * vmag * (1.f - nf) / (rn3 * d));
    } else {
        const double n3 = nn * nn * nn, d = K.d50;
        const double vx = S.vx[i], vy = S.vy[i];
        const double vmag = sqrt(vx * vx + vy * vy);
        S.resist[i] = -((vis_of(oden) / oden) * K.alpha * ((1.0 - nn) * (1.0 - nn)) / (n3 * (d * d))) -
                      ((K.beta / sqrt(n3)) * vmag * (1.0 - nn)) / (sqrt(n3) * d);
    }
}

int op_effpor(Ctx* c) {
    const unsigned g = blocks_for(c->n, NB_BLOCK);
    StageTimer tk(c, BSC_T_K_EFFPOR);
    if (c->mixed)
        k_effpor<float><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->pcell, c->scell_start, c->scell_count,
                                                       c->sx, c->sy, c->sposf, c->swf, c->svol, c->spor, c->f_vol,
                                                       c->f_vol_lo);
    else
        k_effpor<double><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->pcell, c->scell_start, c->scell_count,
                                                        c->sx, c->sy, c->sposf, c->swf, c->svol, c->spor);
    BSC_LAUNCH(c);
    return BSC_OK;
}

// per-particle quotients shared by the pair loops: u = v/n (eddyvis, int_vel)
// (mixed path: also the FP32 twin of V and u as double-floats)
__global__ void k_vel_over_por(int64_t n, State S, double* __restrict__ ux, double* __restrict__ uy,
                               float* __restrict__ f_vol, float4* __restrict__ udf) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double nn = S.por[i];
    const double a = S.vx[i] / nn, b = S.vy[i] / nn;
    ux[i] = a;
    uy[i] = b;
    if (f_vol) f_vol[i] = (float)S.vol[i];
    if (udf) {
        const df2 ad = df_of(a), bd = df_of(b);
        udf[i] = make_float4(ad.hi, ad.lo, bd.hi, bd.lo);
    }
}

// u_j - u_i from the double-float twins, rounded to FP32: the FP32 rounding
// of the FP64 difference to ~2^-48 of |u| (the differences cancel, so they
// must not come from FP32 roundings of u), on the FP32 pipe
__device__ __forceinline__ float2 udf_diff(float4 uj, float4 ui) {
    return make_float2(df_sub(df2{uj.x, uj.y}, df2{ui.x, ui.y}).hi, df_sub(df2{uj.z, uj.w}, df2{ui.z, ui.w}).hi);
}

// ---- turbulence.f90:12-110 eddyvis -----------------------------------------------
template <typename R>
__global__ void __launch_bounds__(NB_BLOCK) k_eddyvis(int64_t n, State S, KParams K, const int32_t* __restrict__ nbr,
                                                       const typename Vec2<R>::type* __restrict__ gw,
                                                       const int32_t* __restrict__ cnt, const double* __restrict__ ux,
                                                       const double* __restrict__ uy, const float* __restrict__ f_vol,
                                                       const float4* __restrict__ udf) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || S.tid[i] != BSC_TID_FLUID) return;
    const R L0 = to_r<R>(S.L0[i]), L1 = to_r<R>(S.L1[i]), L2 = to_r<R>(S.L2[i]), L3 = to_r<R>(S.L3[i]);
    const double uxi = ux[i], uyi = uy[i];
    [[maybe_unused]] const float4 udi = sizeof(R) == 4 ? udf[i] : float4{};
    R t1 = 0, t2 = 0, t3 = 0;
    const int m = cnt[i];
    // FP32 sums: four entries' gathers in flight (measured 3-7 % faster)
    #pragma unroll(sizeof(R) == 4 ? 4 : 1)
    for (int k = 0; k < m; ++k) {
        const int64_t e = ell(i, k, K.kmax);
        const int j = nbr[e];
        const auto g = gw[e];
        R vj;
        if constexpr (sizeof(R) == 4)
            vj = f_vol[j];
        else
            vj = S.vol[j];
        // differences in FP64 (they cancel); for R = float in double-float
        // arithmetic, rounded
        R du, dv;
        if constexpr (sizeof(R) == 4) {
            const float2 d = udf_diff(udf[j], udi);
            du = d.x;
            dv = d.y;
        } else {
            du = ux[j] - uxi;
            dv = uy[j] - uyi;
        }
        const R gx = L0 * g.x + L1 * g.y, gy = L2 * g.x + L3 * g.y;
        t1 += vj * du * gx;
        t2 += vj * dv * gy;
        t3 += (R)0.5 * vj * (du * gy + dv * gx);
    }
    const double T1 = t1, T2 = t2, T3 = t3;
    const double t4 = sqrt(2 * (T1 * T1 + T2 * T2) + (2 * T3) * (2 * T3));
    const double csdl = K.eddy_cs * K.dl, dlt = K.dl * t4;
    S.nut[i] = (csdl * csdl) * t4;
    S.tke[i] = (K.eddy_cv / K.eddy_ce) * (dlt * dlt);
}

int op_eddyvis(Ctx* c) {
    if (!c->have_lists) return set_err(c, BSC_E_INVALID, "eddyvis before neighbour");
    double *ux = c->r, *uy = c->rh;  // Krylov work vectors double as scratch outside the solve
    k_vel_over_por<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, ux, uy, c->mixed ? c->f_vol : nullptr,
                                                                 c->mixed ? c->udf : nullptr);
    BSC_LAUNCH(c);
    const unsigned g = blocks_for(c->n, NB_BLOCK);
    if (c->mixed)
        k_eddyvis<float><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gwf, c->cnt, ux, uy, c->f_vol,
                                                        c->udf);
    else
        k_eddyvis<double><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gw, c->cnt, ux, uy, nullptr,
                                                         nullptr);
    BSC_LAUNCH(c);
    return BSC_OK;
}

// ---- integrator.f90:458-713 int_vel ------------------------------------------------
// pass 1: free-surface artificial viscosity (:467-506)
template <typename R>
__global__ void __launch_bounds__(NB_BLOCK) k_varts(int64_t n, State S, KParams K, const int32_t* __restrict__ nbr,
                                                     const typename Vec2<R>::type* __restrict__ gw,
                                                     const int32_t* __restrict__ cnt, const double* __restrict__ ux,
                                                     const double* __restrict__ uy, const double* __restrict__ umax,
                                                     const float* __restrict__ f_vol, float* __restrict__ f_varts,
                                                     const float4* __restrict__ udf) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || !(S.flags[i] & BSC_FLAG_FREE)) return;
    const R L0 = to_r<R>(S.L0[i]), L1 = to_r<R>(S.L1[i]), L2 = to_r<R>(S.L2[i]), L3 = to_r<R>(S.L3[i]);
    const double uxi = ux[i], uyi = uy[i];
    [[maybe_unused]] const float4 udi = sizeof(R) == 4 ? udf[i] : float4{};
    R t1 = 0, t2 = 0;
    const int m = cnt[i];
    for (int k = 0; k < m; ++k) {
        const int64_t e = ell(i, k, K.kmax);
        const int j = nbr[e];
        const auto g = gw[e];
        R vj;
        if constexpr (sizeof(R) == 4)
            vj = f_vol[j];
        else
            vj = S.vol[j];
        R du, dv;
        if constexpr (sizeof(R) == 4) {
            const float2 d = udf_diff(udf[j], udi);
            du = d.x;
            dv = d.y;
        } else {
            du = ux[j] - uxi;
            dv = uy[j] - uyi;
        }
        t1 += du * (L0 * g.x + L1 * g.y) * vj;
        t2 += dv * (L2 * g.x + L3 * g.y) * vj;
    }
    const double T1 = t1, T2 = t2, vx = S.vx[i], vy = S.vy[i];
    const double va = K.varts_ps * (K.dl * K.dl) * sqrt(T1 * T1 + T2 * T2) * sqrt(vx * vx + vy * vy) /
                      ((*umax + (double)1e-6f) * S.por[i]);
    S.varts[i] = va;
    if (f_varts) f_varts[i] = (float)va;
}

// pass 2: viscous (Morris, harmonic mu/oden), eddy viscosity, SPS k gradient,
// implicit porous drag and gravity (:509-711)
template <typename R>
__global__ void __launch_bounds__(NB_BLOCK) k_int_vel(int64_t n, State S, KParams K, const int32_t* __restrict__ nbr,
                                                       const typename Vec2<R>::type* __restrict__ gw,
                                                       const int32_t* __restrict__ cnt,
                                                       const double* __restrict__ nu, double dt, const float* __restrict__ f_vol,
                                                       const float* __restrict__ f_nu, const float* __restrict__ f_nut,
                                                       const float* __restrict__ f_tke, const float* __restrict__ f_varts,
                                                       const float2* __restrict__ posf, const int32_t* __restrict__ pcell) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    constexpr bool F32 = sizeof(R) == 4;  // FP32 sums: the per-particle fields come from their FP32 twins
    const uint8_t fi = S.flags[i];
    if (S.tid[i] == BSC_TID_FLUID && !(fi & (BSC_FLAG_BUFFER | BSC_FLAG_DEAD))) {
        const R L0 = to_r<R>(S.L0[i]), L1 = to_r<R>(S.L1[i]), L2 = to_r<R>(S.L2[i]), L3 = to_r<R>(S.L3[i]);
        const double xi = S.x[i], yi = S.y[i], vxi = S.vx[i], vyi = S.vy[i];
        // FP32 path: the pair offsets from the particles' FP32 offsets to
        // their cells' origins (as the neighbour search wrote them) and the
        // cells' column and row differences,
        // the velocity differences from FP32 roundings of the velocities
        // (their error, ~1e-7 of |v| per difference, reaches v* through
        // dt nu / h^2 ~ 1e-3): no FP64 operation per pair
        [[maybe_unused]] float2 pfi{};
        [[maybe_unused]] int cxi = 0, cyi = 0;
        [[maybe_unused]] float vxif = 0.f, vyif = 0.f;
        [[maybe_unused]] const float csf = (float)K.cs;
        if constexpr (F32) {
            pfi = posf[i];
            const int ci = pcell[i];
            cxi = ci / K.ny;
            cyi = ci - cxi * K.ny;
            vxif = f32_of(vxi);
            vyif = f32_of(vyi);
        }
        const R nui = to_r<R>(nu[i]), nuti = to_r<R>(S.nut[i]), tkei = to_r<R>(S.tke[i]), ni = to_r<R>(S.por[i]);
        const bool free_i = fi & BSC_FLAG_FREE;
        const R varts_i = to_r<R>(S.varts[i]);
        const R inv_w0 = (R)K.inv_w0;
        const R eps6 = (R)(double)1e-6f;
        R ax = 0, ay = 0, kx = 0, ky = 0;  // kx, ky: the SPS sum, scaled by (2/3) n_i once
        const int m = cnt[i];
        // FP32 sums: four entries' gathers in flight (measured 3-7 % faster)
        #pragma unroll(sizeof(R) == 4 ? 4 : 1)
        for (int k = 0; k < m; ++k) {
            const int64_t e = ell(i, k, K.kmax);
            const int j = nbr[e];
            const auto g = gw[e];
            const bool fluid_j = S.tid[j] == BSC_TID_FLUID;
            R cmu;
            if (fluid_j) {
                const R nuj = F32 ? (R)f_nu[j] : (R)nu[j];
                cmu = (R)2 * nui * nuj / (nui + nuj);
            } else {
                cmu = nui;
            }
            R fx, fy, r2;
            [[maybe_unused]] double dx = 0.0, dy = 0.0;
            if constexpr (F32) {
                const float2 pfj = posf[j];
                const int cj = pcell[j], cxj = cj / K.ny, cyj = cj - cxj * K.ny;
                fx = (pfi.x - pfj.x) + (float)(cxi - cxj) * csf;
                fy = (pfi.y - pfj.y) + (float)(cyi - cyj) * csf;
                r2 = fx * fx + fy * fy;
            } else {
                dx = xi - S.x[j];
                dy = yi - S.y[j];
                fx = dx;
                fy = dy;
                r2 = dx * dx + dy * dy;
            }
            R vart = 0;
            if (free_i) {
                vart = varts_i;
            } else if ((S.flags[j] & BSC_FLAG_FREE) && !(fi & BSC_FLAG_BUFFER)) {
                R r;
                if constexpr (F32)
                    r = sqrtf(r2);
                else
                    r = sqrt(dx * dx + dy * dy);
                vart = kern_w<R>(K, r) * (F32 ? (R)f_varts[j] : (R)S.varts[j]) * inv_w0;
            }
            const R pvol = F32 ? (R)f_vol[j] : (R)S.vol[j];
            const R p_dist = (R)1 / (r2 + (R)K.lam);
            const R gx = L0 * g.x + L1 * g.y, gy = L2 * g.x + L3 * g.y;
            const R geo = (R)2 * pvol * (fx * gx + fy * gy) * p_dist;
            R dvx, dvy;
            if constexpr (F32) {
                dvx = vxif - f32_of(S.vx[j]);
                dvy = vyif - f32_of(S.vy[j]);
            } else {
                dvx = vxi - S.vx[j];
                dvy = vyi - S.vy[j];
            }
            R visc = cmu + vart;
            if (fluid_j) {
                const R nutj = F32 ? (R)f_nut[j] : (R)S.nut[j];
                if (nuti < eps6 && nutj < eps6) visc += (nuti + nutj) * (R)0.5;
                else visc += ((R)2 * nuti * nutj) / (nuti + nutj);
            }
            ax += geo * dvx * visc;
            ay += geo * dvy * visc;
            // SPS turbulence (:645-666): -(2/3) n_i sum_j V_j (k_j - k_i) L grad W
            const R dk = pvol * ((F32 ? (R)f_tke[j] : (R)S.tke[j]) - tkei);
            kx += dk * gx;
            ky += dk * gy;
        }
        const R sps = ni * (R)2 / (R)3;
        ax -= kx * sps;
        ay -= ky * sps;
        const double nn = S.por[i], R_ = S.resist[i];
        double vxs, vys;
        if constexpr (F32) {
            const double inv = 1.0 / (1.0 - dt * R_ * nn);  // one FP64 division for both components
            vxs = (vxi + dt * (double)ax) * inv;
            vys = (vyi + dt * (double)ay) * inv;
        } else {
            vxs = (vxi + dt * (double)ax) / (1.0 - dt * R_ * nn);
            vys = (vyi + dt * (double)ay) / (1.0 - dt * R_ * nn);
        }
        vys = vys + K.g * nn * dt;
        S.vxs[i] = vxs;
        S.vys[i] = vys;
    }
    if (fi & BSC_FLAG_BUFFER) {  // :691-698
        S.vxs[i] = S.vx[i];
        S.vys[i] = K.g * S.por[i] * dt;
    }
}

// nu = mu(oden)/oden; on the mixed path also the FP32 twins the pair sum reads
__global__ void k_kin_visc(int64_t n, State S, double* __restrict__ nu, float* __restrict__ f_nu,
                           float* __restrict__ f_nut, float* __restrict__ f_tke) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double o = S.oden[i];
    const double v = vis_of(o) / o;
    nu[i] = v;
    if (f_nu) {
        f_nu[i] = (float)v;
        f_nut[i] = (float)S.nut[i];
        f_tke[i] = (float)S.tke[i];
    }
}

int op_int_vel(Ctx* c, const double* d_umax) {
    if (!c->have_lists) return set_err(c, BSC_E_INVALID, "int_vel before neighbour");
    double *ux = c->r, *uy = c->rh, *nu = c->pd;
    const unsigned g = blocks_for(c->n, NB_BLOCK);
    const bool mx = c->mixed;
    k_vel_over_por<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, ux, uy, mx ? c->f_vol : nullptr,
                                                                 mx ? c->udf : nullptr);
    BSC_LAUNCH(c);
    if (mx)
        k_varts<float><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gwf, c->cnt, ux, uy, d_umax,
                                                      c->f_vol, c->f_varts, c->udf);
    else
        k_varts<double><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gw, c->cnt, ux, uy, d_umax,
                                                       nullptr, nullptr, nullptr);
    BSC_LAUNCH(c);
    k_kin_visc<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, nu, mx ? c->f_nu : nullptr,
                                                             mx ? c->f_nut : nullptr, mx ? c->f_tke : nullptr);
    BSC_LAUNCH(c);
    StageTimer tk(c, BSC_T_K_INT_VEL);
    if (mx)
        k_int_vel<float><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gwf, c->cnt, nu, c->dt,
                                                        c->f_vol, c->f_nu, c->f_nut, c->f_tke, c->f_varts, c->posf,
                                                        c->pcell);
    else
        k_int_vel<double><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gw, c->cnt, nu, c->dt,
                                                         nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                                         nullptr);
    BSC_LAUNCH(c);
    return BSC_OK;
}

// ---- integrator.f90:715-865 comp_vel (comp_pos is separate, cells.cu) ---------------
// (mixed path: also the FP32 twins of q and V)
__global__ void k_rho_over_por(int64_t n, State S, double* __restrict__ q, float* __restrict__ f_q,
                               float* __restrict__ f_vol, float* __restrict__ f_vol_lo) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = S.rho[i] / S.por[i];
    q[i] = v;
    if (f_q) {
        f_q[i] = (float)v;
        const df2 vd = df_of(S.vol[i]);
        f_vol[i] = vd.hi;
        f_vol_lo[i] = vd.lo;
    }
}

template <typename R>
__global__ void __launch_bounds__(NB_BLOCK) k_comp_vel(int64_t n, State S, KParams K, const int32_t* __restrict__ nbr,
                                                        const typename Vec2<R>::type* __restrict__ gw,
                                                        const int32_t* __restrict__ cnt,
                                                        const double* __restrict__ q, double dt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint8_t fi = S.flags[i];
    if (S.tid[i] == BSC_TID_FLUID && !(fi & (BSC_FLAG_BUFFER | BSC_FLAG_DEAD))) {
        const R L0 = to_r<R>(S.L0[i]), L1 = to_r<R>(S.L1[i]), L2 = to_r<R>(S.L2[i]), L3 = to_r<R>(S.L3[i]);
        const R ni = (R)S.por[i], rhoi = (R)S.rho[i], pi = (R)S.p[i], qi = (R)q[i];
        const R c0 = ni * ni / rhoi;
        R wgx = 0, wgy = 0;  // sums of w grad W; the row's L is applied after them
        const int m = cnt[i];
        for (int k = 0; k < m; ++k) {
            const int64_t e = ell(i, k, K.kmax);
            const int j = nbr[e];
            const auto g = gw[e];
            const R vj = (R)S.vol[j], pj = (R)S.p[j];
            R w;
            if (S.tid[j] == BSC_TID_FLUID) {
                const R qj = (R)q[j];
                w = (R)2 * vj * c0 * (pj * qi + pi * qj) / (qi + qj);
            } else {
                w = vj * c0 * (pj + pi);
            }
            wgx += w * g.x;
            wgy += w * g.y;
        }
        const R ax = L0 * wgx + L1 * wgy, ay = L2 * wgx + L3 * wgy;
        const double vx = S.vxs[i] - dt * (double)ax;
        const double vy = S.vys[i] - dt * (double)ay;
        S.vx[i] = vx;
        S.vy[i] = vy;
        S.vel[i] = sqrt(vx * vx + vy * vy) / S.por[i];
    }
    if (fi & BSC_FLAG_BUFFER) {
        S.vx[i] = S.vxs[i];
        S.vy[i] = 0.0;
    }
    if ((fi & BSC_FLAG_DEAD) && !(fi & BSC_FLAG_BUFFER)) {
        S.vx[i] = 0.0; S.vy[i] = 0.0; S.vxs[i] = 0.0; S.vys[i] = 0.0;
    }
}

// Mixed path.  The pressure force is a sum of terms ~p/h that cancel down to
// ~rho g (a factor ~200 in a hydrostatic column), so FP32 there costs ~5e-5
// in the velocity.  The term is split exactly:
//   fluid j: (p_j q_i + p_i q_j)/(q_i+q_j) = p_i + q_i (p_j - p_i)/(q_i+q_j)
//   wall j:  p_j + p_i = 2 p_i + (p_j - p_i)
// so a_i = c0 [ 2 p_i sum_j V_j g_j  +  sum_j w_j (p_j - p_i) g_j ]; the first
// (cancelling) sum runs in double-float arithmetic from the double-float V
// and grad W (~48 bits, on the FP32 pipe), the second (difference) sum in FP32.
__global__ void __launch_bounds__(NB_BLOCK) k_comp_vel_mixed(int64_t n, State S, KParams K,
                                                              const int32_t* __restrict__ nbr,
                                                              const float2* __restrict__ gwf,
                                                              const float2* __restrict__ gwl,
                                                              const int32_t* __restrict__ cnt,
                                                              const float* __restrict__ f_q,
                                                              const float* __restrict__ f_vol,
                                                              const float* __restrict__ f_vol_lo, double dt) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint8_t fi = S.flags[i];
    if (S.tid[i] == BSC_TID_FLUID && !(fi & (BSC_FLAG_BUFFER | BSC_FLAG_DEAD))) {
        const double L0 = S.L0[i], L1 = S.L1[i], L2 = S.L2[i], L3 = S.L3[i];
        const float L0f = f32_of(L0), L1f = f32_of(L1), L2f = f32_of(L2), L3f = f32_of(L3);
        const double pi = S.p[i];
        const float qi = f_q[i];
        df2 sxd{0.f, 0.f}, syd{0.f, 0.f};
        float ax = 0.f, ay = 0.f;
        const int m = cnt[i];
        for (int k = 0; k < m; ++k) {
            const int64_t e = ell(i, k, K.kmax);
            const int j = nbr[e];
            const float2 gf = gwf[e], gl = gwl[e];
            const float vjf = f_vol[j];
            const df2 vj{vjf, f_vol_lo[j]};
            sxd = df_add(sxd, df_mul(vj, df2{gf.x, gl.x}));  // sum V grad W; L applied after the loop
            syd = df_add(syd, df_mul(vj, df2{gf.y, gl.y}));
            const float w = (S.tid[j] == BSC_TID_FLUID) ? 2.f * vjf * qi / (qi + f_q[j]) : vjf;
            const float dp = f32_of(S.p[j] - pi);  // FP64 difference (pressures cancel), rounded on the integer pipe
            ax += w * dp * (L0f * gf.x + L1f * gf.y);
            ay += w * dp * (L2f * gf.x + L3f * gf.y);
        }
        const double sx = df_to_double(sxd), sy = df_to_double(syd);
        const double hx = L0 * sx + L1 * sy, hy = L2 * sx + L3 * sy;
        const double ni = S.por[i], c0 = ni * ni / S.rho[i];
        const double vx = S.vxs[i] - dt * c0 * (2.0 * pi * hx + (double)ax);
        const double vy = S.vys[i] - dt * c0 * (2.0 * pi * hy + (double)ay);
        S.vx[i] = vx;
        S.vy[i] = vy;
        S.vel[i] = sqrt(vx * vx + vy * vy) / ni;
    }
    if (fi & BSC_FLAG_BUFFER) {
        S.vx[i] = S.vxs[i];
        S.vy[i] = 0.0;
    }
    if ((fi & BSC_FLAG_DEAD) && !(fi & BSC_FLAG_BUFFER)) {
        S.vx[i] = 0.0; S.vy[i] = 0.0; S.vxs[i] = 0.0; S.vys[i] = 0.0;
    }
}

int op_comp_vel(Ctx* c) {
    if (!c->have_lists) return set_err(c, BSC_E_INVALID, "comp_vel before neighbour");
    double* q = c->r;
    k_rho_over_por<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, q, c->mixed ? c->f_q : nullptr,
                                                                 c->mixed ? c->f_vol : nullptr,
                                                                 c->mixed ? c->f_vol_lo : nullptr);
    BSC_LAUNCH(c);
    const unsigned g = blocks_for(c->n, NB_BLOCK);
    if (c->mixed)
        k_comp_vel_mixed<<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gwf, c->gwl, c->cnt, c->f_q,
                                                        c->f_vol, c->f_vol_lo, c->dt);
    else
        k_comp_vel<double><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gw, c->cnt, q, c->dt);
    BSC_LAUNCH(c);
    return BSC_OK;
}

// ---- part_shift.f90:12-192 opt2_shift ------------------------------------------------
// The surface normal and pint are forced to zero in the reference
// (part_shift.f90:68-70), so the shift is -csh h^2 frac sum V_j grad W
// (uncorrected), clamped per component to maxshift*dl; the velocity is
// corrected with the unclamped shift and the corrected gradient.
// R: type of the velocity-gradient sums of the Taylor correction.  The
// position shift sum_j V_j grad W cancels to ~1e-3 of its terms inside the
// fluid: FP64 on the FP64 path, double-float (~48 bits, from the
// double-float V and grad W) on the mixed path.  The gradient sums only
// scale the correction grad(v).delta, a fraction ~|delta|/L of v (1e-3 and
// below here): on the mixed path they run in FP32 from the FP32 roundings
// of the velocities (taken on the integer pipe) and the FP32 grad W (an
// error of ~1e-8 of v in the correction), so the kernel issues no FP64
// operation per pair (ten on the FP64 path).
template <typename R>
__global__ void __launch_bounds__(NB_BLOCK) k_shift(int64_t n, State S, KParams K, const int32_t* __restrict__ nbr,
                                                     const double2* __restrict__ gw, const float2* __restrict__ gwf,
                                                     const float2* __restrict__ gwl, const float* __restrict__ f_vol,
                                                     const float* __restrict__ f_vol_lo,
                                                     const int32_t* __restrict__ cnt, int8_t* __restrict__ mark) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    mark[i] = 0;
    const uint8_t fi = S.flags[i];
    if (!(S.tid[i] == BSC_TID_FLUID && !(fi & (BSC_FLAG_BUFFER | BSC_FLAG_DEAD)))) return;
    const int m = cnt[i];
    if (m == 0) return;
    constexpr bool F32 = sizeof(R) == 4;
    const R L0 = to_r<R>(S.L0[i]), L1 = to_r<R>(S.L1[i]), L2 = to_r<R>(S.L2[i]), L3 = to_r<R>(S.L3[i]);
    const double vxi = S.vx[i], vyi = S.vy[i];
    // the corrected gradient L grad W enters linearly and L is the row's own,
    // so L is applied once to the four sums of grad W (dv V) rather than per
    // pair
    double sx = 0, sy = 0;
    [[maybe_unused]] df2 sxd{0.f, 0.f}, syd{0.f, 0.f};
    [[maybe_unused]] const float vxif = f32_of(vxi), vyif = f32_of(vyi);
    R ax = 0, bx = 0, ay = 0, by = 0;
    // FP32 sums: four entries' gathers in flight (measured 3-7 % faster)
    #pragma unroll(sizeof(R) == 4 ? 4 : 1)
    for (int k = 0; k < m; ++k) {
        const int64_t e = ell(i, k, K.kmax);
        const int j = nbr[e];
        R gx, gy, dvx, dvy;
        if constexpr (F32) {
            const float2 gf = gwf[e], gl = gwl[e];
            const float vf = f_vol[j];
            const df2 vjd{vf, f_vol_lo[j]};
            sxd = df_add(sxd, df_mul(df2{gf.x, gl.x}, vjd));
            syd = df_add(syd, df_mul(df2{gf.y, gl.y}, vjd));
            gx = gf.x;
            gy = gf.y;
            dvx = (f32_of(S.vx[j]) - vxif) * vf;
            dvy = (f32_of(S.vy[j]) - vyif) * vf;
        } else {
            const double2 g = gw[e];
            const double vj = S.vol[j];
            sx += g.x * vj;
            sy += g.y * vj;
            gx = g.x;
            gy = g.y;
            dvx = (S.vx[j] - vxi) * vj;
            dvy = (S.vy[j] - vyi) * vj;
        }
        ax += gx * dvx;
        bx += gy * dvx;
        ay += gx * dvy;
        by += gy * dvy;
    }
    if constexpr (F32) {
        sx = df_to_double(sxd);
        sy = df_to_double(syd);
    }
    const R tx1 = L0 * ax + L1 * bx, tx2 = L2 * ax + L3 * bx;
    const R ty1 = L0 * ay + L1 * by, ty2 = L2 * ay + L3 * by;
    const double frac = (fi & BSC_FLAG_FREE) ? 0.01 : 1.0;
    const double coef = -K.csh * (K.h * K.h) * frac;
    const double xs = coef * sx, ys = coef * sy;
    const double lim = K.maxshift * K.dl;
    const double cx = (xs == 0.0) ? 0.0 : fmin(fabs(xs), lim) * xs / fabs(xs);
    const double cy = (ys == 0.0) ? 0.0 : fmin(fabs(ys), lim) * ys / fabs(ys);
    S.xs[i] = cx;
    S.ys[i] = cy;
    S.vxs[i] = (double)tx1 * xs + (double)tx2 * ys;
    S.vys[i] = (double)ty1 * xs + (double)ty2 * ys;
    mark[i] = 1;
}

__global__ void k_shift_apply(int64_t n, State S, const int8_t* __restrict__ mark) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || !mark[i]) return;
    S.x[i] += S.xs[i];
    S.y[i] += S.ys[i];
    S.vx[i] += S.vxs[i];
    S.vy[i] += S.vys[i];
}

int op_opt2_shift(Ctx* c) {
    if (!c->have_lists) return set_err(c, BSC_E_INVALID, "opt2_shift before neighbour");
    int8_t* mark = (int8_t*)c->pslot;  // scratch: pslot is free between cell builds
    const unsigned g = blocks_for(c->n, NB_BLOCK);
    // The position shift's sum is FP64 on the FP64 path and double-float on
    // the mixed one (with it in FP32 the mixed path's velocities moved by
    // ~7e-6 from the FP64 path's after 8 c3 steps, against ~1e-6 with a wide
    // sum); on the mixed path the velocity gradient of the Taylor correction
    // runs in FP32 (see k_shift).  V is the one effpor just wrote (with its
    // double-float twin).
    {
        StageTimer tk(c, BSC_T_K_SHIFT);
        if (c->mixed)
            k_shift<float><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, nullptr, c->gwf, c->gwl,
                                                          c->f_vol, c->f_vol_lo, c->cnt, mark);
        else
            k_shift<double><<<g, NB_BLOCK, 0, c->stream>>>(c->n, c->S, c->K, c->nbr, c->gw, nullptr, nullptr,
                                                           nullptr, nullptr, c->cnt, mark);
        BSC_LAUNCH(c);
    }
    k_shift_apply<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, mark);
    BSC_LAUNCH(c);
    return BSC_OK;
}

// ---- integrator.f90:908-976 timestep: max |vel|, max |nut| (comp_vel :853-861) --------
__global__ void k_maxred(int64_t n, const double* __restrict__ a, const double* __restrict__ b,
                         double* __restrict__ part) {
    __shared__ double sa[RED_BLOCK], sb[RED_BLOCK];
    double ma = 0.0, mb = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        ma = fmax(ma, fabs(a[i]));
        mb = fmax(mb, fabs(b[i]));
    }
    sa[threadIdx.x] = ma;
    sb[threadIdx.x] = mb;
    __syncthreads();
    for (int s = RED_BLOCK / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sa[threadIdx.x] = fmax(sa[threadIdx.x], sa[threadIdx.x + s]);
            sb[threadIdx.x] = fmax(sb[threadIdx.x], sb[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = sa[0];
        part[2 * blockIdx.x + 1] = sb[0];
    }
}

// one block: strided maxima of the block partials, then a tree (a single
// thread walking them serially waited on each load)
__global__ void __launch_bounds__(RED_BLOCK) k_maxfin(int nb, const double* __restrict__ part,
                                                      double* __restrict__ out) {
    __shared__ double sa[RED_BLOCK], sb[RED_BLOCK];
    double ma = 0.0, mb = 0.0;
    for (int k = threadIdx.x; k < nb; k += blockDim.x) {
        ma = fmax(ma, part[2 * k]);
        mb = fmax(mb, part[2 * k + 1]);
    }
    sa[threadIdx.x] = ma;
    sb[threadIdx.x] = mb;
    __syncthreads();
    for (int s = RED_BLOCK / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            sa[threadIdx.x] = fmax(sa[threadIdx.x], sa[threadIdx.x + s]);
            sb[threadIdx.x] = fmax(sb[threadIdx.x], sb[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = sa[0];
        out[1] = sb[0];
    }
}

// ---- free-surface elevation probes (greenfield) ------------------------------------
__global__ void k_probe(int64_t n, State S, double R, int np, const double* __restrict__ xp,
                        double* __restrict__ part) {
    extern __shared__ double sh[];
    double acc[16];
    for (int k = 0; k < np; ++k) acc[k] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (S.tid[i] != BSC_TID_FLUID) continue;
        const double xi = S.x[i], vi = S.vol[i];
        for (int k = 0; k < np; ++k) {
            const double q = fabs(xi - xp[k]) / R;
            if (q < 1.0) {
                const double a = 1.0 - q;
                acc[k] += vi * (1.25 / R) * (a * a * a) * (1.0 + 3.0 * q);
            }
        }
    }
    for (int k = 0; k < np; ++k) {
        sh[threadIdx.x] = acc[k];
        __syncthreads();
        for (int s = RED_BLOCK / 2; s > 0; s >>= 1) {
            if (threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[blockIdx.x * np + k] = sh[0];
        __syncthreads();
    }
}

int op_probe_eta(Ctx* c, int np, const double* xp, double depth, double* eta) {
    if (np <= 0 || np > 16) return set_err(c, BSC_E_INVALID, "probe_eta: 1..16 probes");
    double* dxp = c->tv;
    BSC_CUDA(c, cudaMemcpyAsync(dxp, xp, sizeof(double) * np, cudaMemcpyHostToDevice, c->stream));
    k_probe<<<RED_GRID, RED_BLOCK, RED_BLOCK * sizeof(double), c->stream>>>(c->n, c->S, 2 * c->K.h, np, dxp, c->part);
    BSC_LAUNCH(c);
    std::vector<double> h((size_t)RED_GRID * np);
    BSC_CUDA(c, cudaMemcpyAsync(h.data(), c->part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    for (int k = 0; k < np; ++k) {
        double s = 0.0;
        for (int b = 0; b < RED_GRID; ++b) s += h[(size_t)b * np + k];
        eta[k] = s - depth;
    }
    return BSC_OK;
}

}  // namespace bsc

namespace bsc {
// max |vel| and max |nut| over all particles -> stepsc[0..1] (device)
int op_timestep_reduce(Ctx* c) {
    k_maxred<<<RED_GRID, RED_BLOCK, 0, c->stream>>>(c->n, c->S.vel, c->S.nut, c->part);
    BSC_LAUNCH(c);
    k_maxfin<<<1, RED_BLOCK, 0, c->stream>>>(RED_GRID, c->part, c->stepsc);
    BSC_LAUNCH(c);
    return BSC_OK;
}
}  // namespace bsc
