// mg.cu -- cell-aggregation multigrid preconditioner for the PPE.
//
// The reference solves the PPE with unpreconditioned Krylov methods (MKL
// dfgmres, solver.f90:306-347; BiCGSTAB, solver.f90:129-254), whose iteration
// count grows with the resolution (about 1400 BiCGSTAB iterations at 0.85 M
// particles).  This preconditioner keeps the same matrix and the same
// stopping test and only changes how fast the Krylov method gets there.
//
// Hierarchy (rebuilt for every assembled matrix):
//  - level 0: the Jacobi-scaled PPE I + N in the neighbour-list layout;
//  - level 1: one unknown per neighbour-search cell (side >= 2h), the sum of
//    its particles' unknowns (piecewise-constant aggregation).  Every
//    neighbour of a particle lies in the 3x3 cells around it, so the Galerkin
//    operator P^T A P is a 9-point stencil on the cell grid;
//  - level l+1: 2x2 blocks of level-l cells, again a 9-point stencil;
//  - the coarsest level (<= mg_coarse_max cells) is inverted densely.
// Every coarse operator is summed by one thread per coarse cell in a fixed
// order, so the hierarchy is deterministic.
//
// V-cycle: mg_sweeps damped-Jacobi sweeps before and after the coarse
// correction on every level (weight mg_omega), the correction prolonged by
// injection and scaled by mg_scale (plain aggregation under-corrects smooth
// error; a factor of about 1.5 restores it).  The first pre-sweep from a
// zero guess and the prolongation are folded into the neighbouring sweep.
#include <algorithm>
#include <cmath>

#include "bsc_internal.cuh"
#include "ellop.cuh"

namespace bsc {

namespace {

constexpr int MG_BLOCK = 256;

__device__ __forceinline__ int stencil_slot(int dx, int dy) { return (dx + 1) * 3 + (dy + 1); }

// ---- hierarchy ----------------------------------------------------------------
// level 1 from the fine matrix, in two coalesced passes: (1) thread per row,
// the row's entries summed into the 9 neighbour-cell slots of its own cell
// (every neighbour lies in the 3x3 cells around it); (2) thread per cell, its
// rows' slot sums added in the cell list's (id-sorted) order
__global__ void k_mg_rowslots(int64_t n, int ny, const int32_t* __restrict__ pcell, EllOp<double> A,
                              double* __restrict__ rs, float* __restrict__ rsf) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int ci = pcell[i], cx = ci / ny, cy = ci % ny;
    double acc[9] = {0, 0, 0, 0, 1.0, 0, 0, 0, 0};  // the unit diagonal
    const int m = A.cnt[i];
    const int64_t e0 = ell(i, 0, A.kmax);
    for (int k = 0; k < m; ++k) {
        const int64_t e = e0 + (int64_t)k * 32;
        const int cj = pcell[A.nbr[e]];
        const int dx = cj / ny - cx, dy = cj % ny - cy;
        if (dx < -1 || dx > 1 || dy < -1 || dy > 1) continue;  // cannot happen: lists come from the 3x3 cells
        acc[stencil_slot(dx, dy)] += A.aval[e];
    }
#pragma unroll
    for (int s = 0; s < 9; ++s) rs[s * n + i] = acc[s];
    if (rsf)
#pragma unroll
        for (int s = 0; s < 9; ++s) rsf[s * n + i] = (float)acc[s];
}

__global__ void k_mg_galerkin0(int nx, int ny, int64_t n, const int32_t* __restrict__ cell_start,
                               const int32_t* __restrict__ cell_count, const int32_t* __restrict__ sorted,
                               const double* __restrict__ rs, double* __restrict__ Ac, double* __restrict__ dinv,
                               float* __restrict__ Acf, float* __restrict__ dinvf) {
    const int64_t nc = (int64_t)nx * ny;
    const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (c >= nc) return;
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int q0 = cell_start[c], qn = cell_count[c];
    for (int q = q0; q < q0 + qn; ++q) {
        const int i = sorted[q];
#pragma unroll
        for (int s = 0; s < 9; ++s) acc[s] += rs[s * n + i];
    }
#pragma unroll
    for (int s = 0; s < 9; ++s) Ac[s * nc + c] = acc[s];
    dinv[c] = acc[4] != 0.0 ? 1.0 / acc[4] : 0.0;
    if (Acf) {  // the mixed path's FP32 copies
#pragma unroll
        for (int s = 0; s < 9; ++s) Acf[s * nc + c] = (float)acc[s];
        dinvf[c] = (float)dinv[c];
    }
}

// level l -> l+1 over 2x2 blocks
__global__ void k_mg_galerkin(int nxf, int nyf, const double* __restrict__ Af, int nxc, int nyc,
                              double* __restrict__ Ac, double* __restrict__ dinv, float* __restrict__ Acf,
                              float* __restrict__ dinvf) {
    const int64_t ncc = (int64_t)nxc * nyc, ncf = (int64_t)nxf * nyf;
    const int64_t C = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (C >= ncc) return;
    const int CX = (int)(C / nyc), CY = (int)(C % nyc);
    double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = 0; a < 2; ++a) {
        const int fx = 2 * CX + a;
        if (fx >= nxf) continue;
        for (int b = 0; b < 2; ++b) {
            const int fy = 2 * CY + b;
            if (fy >= nyf) continue;
            const int64_t f = (int64_t)fx * nyf + fy;
            for (int s = 0; s < 9; ++s) {
                const double v = Af[s * ncf + f];
                if (v == 0.0) continue;
                const int gx = fx + s / 3 - 1, gy = fy + s % 3 - 1;
                if (gx < 0 || gx >= nxf || gy < 0 || gy >= nyf) continue;
                acc[stencil_slot((gx >> 1) - CX, (gy >> 1) - CY)] += v;
            }
        }
    }
#pragma unroll
    for (int s = 0; s < 9; ++s) Ac[s * ncc + C] = acc[s];
    dinv[C] = acc[4] != 0.0 ? 1.0 / acc[4] : 0.0;
    if (Acf) {
#pragma unroll
        for (int s = 0; s < 9; ++s) Acf[s * ncc + C] = (float)acc[s];
        dinvf[C] = (float)dinv[C];
    }
}

// Dense inverse of the coarsest level by Gauss-Jordan elimination with
// partial (row) pivoting, in place in shared memory, one CTA.  Empty cells
// (all-zero rows) become identity rows.  A zero pivot is replaced by a tiny
// one: the preconditioner then loses that direction but stays finite.
// Computed in FP32 (R below) on both paths and written as O: one SM runs
// it, where FP64 is ~60x slower, and the coarsest solve is part of a
// preconditioner, whose rounding costs iterations, never accuracy.
template <typename O>
__global__ void __launch_bounds__(1024) k_mg_dense_inverse(int nx, int ny, const double* __restrict__ A,
                                                            O* __restrict__ cinv) {
    using R = float;
    extern __shared__ __align__(16) unsigned char dense_sm[];
    R* M = reinterpret_cast<R*>(dense_sm);  // n x n, row-major
    __shared__ int perm[MG_COARSE_MAX];
    __shared__ R fcol[MG_COARSE_MAX];
    __shared__ int piv_row;
    __shared__ R piv_inv;
    const int n = nx * ny;
    const int t = threadIdx.x, T = blockDim.x;
    const int lane = t & 31, warp = t >> 5, nwarps = T >> 5;
    for (int q = t; q < n * n; q += T) M[q] = (R)0;
    __syncthreads();
    for (int c = t; c < n; c += T) {
        const int cx = c / ny, cy = c % ny;
        bool any = false;
        for (int s = 0; s < 9; ++s) {
            const double v = A[(int64_t)s * n + c];
            const int gx = cx + s / 3 - 1, gy = cy + s % 3 - 1;
            if (v == 0.0 || gx < 0 || gx >= nx || gy < 0 || gy >= ny) continue;
            M[c * n + gx * ny + gy] += (R)v;
            any = true;
        }
        if (!any) M[c * n + c] = (R)1;
    }
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        // pivot: the largest |M[i][k]| over i >= k (warp 0)
        if (t < 32) {
            R best = (R)-1;
            int bi = k;
            for (int i = k + t; i < n; i += 32) {
                const R a = fabs(M[i * n + k]);
                if (a > best) { best = a; bi = i; }
            }
            for (int o = 16; o > 0; o >>= 1) {
                const R ob = __shfl_down_sync(0xffffffffu, best, o);
                const int oi = __shfl_down_sync(0xffffffffu, bi, o);
                if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
            }
            if (t == 0) { piv_row = bi; perm[k] = bi; }
        }
        __syncthreads();
        const int p = piv_row;
        if (p != k)
            for (int j = t; j < n; j += T) {
                const R a = M[k * n + j];
                M[k * n + j] = M[p * n + j];
                M[p * n + j] = a;
            }
        __syncthreads();
        if (t == 0) {
            R pv = M[k * n + k];
            if (pv == (R)0) pv = (R)1e-30f;
            piv_inv = (R)1 / pv;
            M[k * n + k] = (R)1;
        }
        __syncthreads();
        for (int j = t; j < n; j += T) M[k * n + j] *= piv_inv;
        for (int i = t; i < n; i += T) fcol[i] = (i == k) ? (R)0 : M[i * n + k];
        __syncthreads();
        for (int i = t; i < n; i += T)
            if (i != k) M[i * n + k] = (R)0;
        __syncthreads();
        // eliminate column k from every other row: a warp per row, lanes
        // along it
        for (int i = warp; i < n; i += nwarps) {
            if (i == k) continue;
            const R f = fcol[i];
            for (int j = lane; j < n; j += 32) M[i * n + j] -= f * M[k * n + j];
        }
        __syncthreads();
    }
    // undo the row interchanges as column interchanges, last first
    for (int k = n - 1; k >= 0; --k) {
        const int p = perm[k];
        if (p != k)
            for (int i = t; i < n; i += T) {
                const R a = M[i * n + k];
                M[i * n + k] = M[i * n + p];
                M[i * n + p] = a;
            }
        __syncthreads();
    }
    for (int q = t; q < n * n; q += T) cinv[q] = (O)M[q];
}

// ---- V-cycle, structured levels (l >= 1) -------------------------------------------
// The per-cell helpers take plain (not __restrict__) pointers: the tail
// kernel reads, in later phases, vectors it wrote in earlier ones, so those
// loads must stay on the coherent path (within one CTA, a block barrier makes
// the writes visible).

// One damped-Jacobi update of cell c: x + w D^-1 (b - A x), where the input x is
//   MODE 0: xin;
//   MODE 1: w D^-1 b (the first sweep from a zero guess, folded in);
//   MODE 2: xin + scale * xc[parent] (the prolonged coarse correction, folded in).
// Cell indices fit 32 bits (grids are capped at 16M cells, stencils at 9 x
// that); 32-bit index arithmetic keeps these latency-bound chains short.
template <typename T, int MODE>
__device__ __forceinline__ T smooth_at(int nx, int ny, int c, const T* A, const T* dinv, const T* b,
                                       const T* xin, const T* xc, int nyc, T scale, T w, T w0 = 0) {
    const int nc = nx * ny;
    const int cx = c / ny, cy = c - cx * ny;
    auto xv = [&](int gx, int gy) -> T {
        const int g = gx * ny + gy;
        if (MODE == 1) return w0 * dinv[g] * b[g];
        if (MODE == 2) return xin[g] + scale * xc[(gx >> 1) * nyc + (gy >> 1)];
        return xin[g];
    };
    T ax = 0;
#pragma unroll
    for (int s = 0; s < 9; ++s) {
        const int gx = cx + s / 3 - 1, gy = cy + s % 3 - 1;
        if (gx < 0 || gx >= nx || gy < 0 || gy >= ny) continue;
        ax += A[s * nc + c] * xv(gx, gy);  // no test on the loaded value: loads stay independent
    }
    return xv(cx, cy) + w * dinv[c] * (b[c] - ax);
}

// the residual b - A x summed over the 2x2 children of coarse cell C
template <typename T>
__device__ __forceinline__ T restrict_at(int nx, int ny, const T* A, const T* b, const T* x, int C, int nyc) {
    const int nc = nx * ny;
    const int CX = C / nyc, CY = C - CX * nyc;
    T sum = 0;
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        const int fx = 2 * CX + a;
        if (fx >= nx) continue;
#pragma unroll
        for (int bb = 0; bb < 2; ++bb) {
            const int fy = 2 * CY + bb;
            if (fy >= ny) continue;
            const int f = fx * ny + fy;
            T ax = 0;
#pragma unroll
            for (int s = 0; s < 9; ++s) {
                const int gx = fx + s / 3 - 1, gy = fy + s % 3 - 1;
                if (gx < 0 || gx >= nx || gy < 0 || gy >= ny) continue;
                ax += A[s * nc + f] * x[gx * ny + gy];
            }
            sum += b[f] - ax;
        }
    }
    return sum;
}

template <typename T, int MODE>
__global__ void __launch_bounds__(MG_BLOCK) k_mg_smooth(int nx, int ny, const T* __restrict__ A,
                                                         const T* __restrict__ dinv, const T* __restrict__ b,
                                                         const T* __restrict__ xin, const T* __restrict__ xc, int nyc,
                                                         T scale, T w, T w0, T* __restrict__ xout,
                                                         const Scalars* __restrict__ sk) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= nx * ny) return;
    // the loads are in bounds whatever the solver state: they go out before
    // the skip test's own load returns
    const T v = smooth_at<T, MODE>(nx, ny, c, A, dinv, b, xin, xc, nyc, scale, w, w0);
    if (!mg_skip(sk)) xout[c] = v;
}

// Both post-sweeps of a cell level in one launch: a block owns a tile of
// PT_X x PT_Y cells (PT_Y along the grid's contiguous y index) and computes
// the first sweep (prolonged correction folded in, weight w) on the tile and
// its one-cell ring into shared memory, then the second sweep (weight w1) on
// the tile from there.  The ring's first sweep is recomputed by the
// neighbouring blocks (a third more first-sweep work) and one launch of the
// latency-bound chain is saved per level.
constexpr int PT_X = 8, PT_Y = 32;
constexpr int PT_HX = PT_X + 2, PT_HY = PT_Y + 2;
template <typename T>
__global__ void __launch_bounds__(PT_X * PT_Y) k_mg_post2(int nx, int ny, const T* __restrict__ A,
                                                           const T* __restrict__ dinv, const T* __restrict__ b,
                                                           const T* __restrict__ xin, const T* __restrict__ xc,
                                                           int nyc, T scale, T w, T w1, T* __restrict__ xout,
                                                           const Scalars* __restrict__ sk) {
    __shared__ T y1[PT_HX * PT_HY];
    const int nc = nx * ny;
    const int x0 = blockIdx.x * PT_X - 1, y0 = blockIdx.y * PT_Y - 1;  // ring origin
    for (int h = threadIdx.x; h < PT_HX * PT_HY; h += blockDim.x) {
        const int gx = x0 + h / PT_HY, gy = y0 + h % PT_HY;
        T v = 0;
        if (gx >= 0 && gx < nx && gy >= 0 && gy < ny)
            v = smooth_at<T, 2>(nx, ny, gx * ny + gy, A, dinv, b, xin, xc, nyc, scale, w);
        y1[h] = v;
    }
    __syncthreads();
    const int tx = threadIdx.x / PT_Y, ty = threadIdx.x % PT_Y;
    const int cx = x0 + 1 + tx, cy = y0 + 1 + ty;
    if (cx >= nx || cy >= ny) return;
    const int c = cx * ny + cy;
    T ax = 0;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const int gx = cx + q / 3 - 1, gy = cy + q % 3 - 1;
        if (gx < 0 || gx >= nx || gy < 0 || gy >= ny) continue;
        ax += A[q * nc + c] * y1[(tx + q / 3) * PT_HY + (ty + q % 3)];
    }
    const T v = y1[(tx + 1) * PT_HY + (ty + 1)] + w1 * dinv[c] * (b[c] - ax);
    if (!mg_skip(sk)) xout[c] = v;
}

// Four sweeps per cell level (BSC_MG_CELL_SWEEPS=4), each direction in one
// launch on the same PT_X x PT_Y tiles: a stage on ring r (the tile and r
// cells around it) is one damped-Jacobi sweep whose neighbours' values come
// from the previous stage on ring r + 1, in shared memory.  The weights
// alternate w, w1, w, w1 as the two-sweep pair does.
// out on ring r from prev on ring r + 1 (both tile-relative arrays)
template <typename T>
__device__ __forceinline__ void pt_sweep(int nx, int ny, const T* __restrict__ A, const T* __restrict__ dinv,
                                         const T* __restrict__ b, int x0, int y0, int r, const T* prev, T* out,
                                         T wgt) {
    const int nc = nx * ny;
    const int HY = PT_Y + 2 * r, HN = (PT_X + 2 * r) * HY, PY = PT_Y + 2 * (r + 1);
    for (int h = threadIdx.x; h < HN; h += blockDim.x) {
        const int gx = x0 - r + h / HY, gy = y0 - r + h % HY;
        T v = 0;
        if (gx >= 0 && gx < nx && gy >= 0 && gy < ny) {
            const int c = gx * ny + gy;
            const int px = h / HY + 1, py = h % HY + 1;  // (gx, gy) in prev's ring r + 1
            T ax = 0;
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                const int hx = gx + q / 3 - 1, hy = gy + q % 3 - 1;
                if (hx < 0 || hx >= nx || hy < 0 || hy >= ny) continue;
                ax += A[q * nc + c] * prev[(px + q / 3 - 1) * PY + (py + q % 3 - 1)];
            }
            v = prev[px * PY + py] + wgt * dinv[c] * (b[c] - ax);
        }
        out[h] = v;
    }
}

constexpr int PT_R3 = (PT_X + 6) * (PT_Y + 6), PT_R2 = (PT_X + 4) * (PT_Y + 4), PT_R1 = (PT_X + 2) * (PT_Y + 2),
              PT_R0 = PT_X * PT_Y;

// pre-smoothing from zero (x1 = w D^-1 b folded into x2 on ring 3, then x3
// on ring 2, x4 on ring 1), x4 on the tile into xout, the residual
// b - A x4 on the tile, and its sums over each coarse cell's 2x2 children
// (the tile holds whole coarse cells: its origin is even) into bc
template <typename T>
__global__ void __launch_bounds__(PT_X * PT_Y) k_mg_pre4_restrict(int nx, int ny, const T* __restrict__ A,
                                                                   const T* __restrict__ dinv,
                                                                   const T* __restrict__ b, T w, T w1,
                                                                   T* __restrict__ xout, int nxc, int nyc,
                                                                   T* __restrict__ bc,
                                                                   const Scalars* __restrict__ sk) {
    __shared__ T s3[PT_R3], s2[PT_R2], s1[PT_R1], s0[PT_R0];
    const int x0 = blockIdx.x * PT_X, y0 = blockIdx.y * PT_Y;
    {   // x2 on ring 3, from b alone (the first sweep from zero is pointwise)
        const int HY = PT_Y + 6;
        for (int h = threadIdx.x; h < PT_R3; h += blockDim.x) {
            const int gx = x0 - 3 + h / HY, gy = y0 - 3 + h % HY;
            T v = 0;
            if (gx >= 0 && gx < nx && gy >= 0 && gy < ny)
                v = smooth_at<T, 1>(nx, ny, gx * ny + gy, A, dinv, b, nullptr, nullptr, 0, (T)0, w1, w);
            s3[h] = v;
        }
    }
    __syncthreads();
    pt_sweep<T>(nx, ny, A, dinv, b, x0, y0, 2, s3, s2, w);
    __syncthreads();
    pt_sweep<T>(nx, ny, A, dinv, b, x0, y0, 1, s2, s1, w1);
    __syncthreads();
    // the tile: x4 out, and the residual b - A x4 into s0
    const int nc = nx * ny;
    {
        const int tx = threadIdx.x / PT_Y, ty = threadIdx.x % PT_Y;
        const int cx = x0 + tx, cy = y0 + ty;
        T rv = 0;
        if (cx < nx && cy < ny) {
            const int c = cx * ny + cy;
            T ax = 0;
#pragma unroll
            for (int q = 0; q < 9; ++q) {
                const int hx = cx + q / 3 - 1, hy = cy + q % 3 - 1;
                if (hx < 0 || hx >= nx || hy < 0 || hy >= ny) continue;
                ax += A[q * nc + c] * s1[(tx + q / 3) * (PT_Y + 2) + (ty + q % 3)];
            }
            rv = b[c] - ax;
            if (!mg_skip(sk)) xout[c] = s1[(tx + 1) * (PT_Y + 2) + (ty + 1)];
        }
        s0[threadIdx.x] = rv;
    }
    __syncthreads();
    // the tile's PT_X/2 x PT_Y/2 coarse cells
    if (threadIdx.x < (PT_X / 2) * (PT_Y / 2)) {
        const int a = threadIdx.x / (PT_Y / 2), q = threadIdx.x % (PT_Y / 2);
        const int X = x0 / 2 + a, Y = y0 / 2 + q;
        if (X < nxc && Y < nyc) {
            T sum = 0;
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j)
                    if (2 * X + i < nx && 2 * Y + j < ny) sum += s0[(2 * a + i) * PT_Y + (2 * q + j)];
            if (!mg_skip(sk)) bc[X * nyc + Y] = sum;
        }
    }
}

// post-smoothing: y1 on ring 3 (the prolonged correction folded in, as
// k_mg_post2's first sweep), y2 on ring 2, y3 on ring 1, y4 on the tile
template <typename T>
__global__ void __launch_bounds__(PT_X * PT_Y) k_mg_post4(int nx, int ny, const T* __restrict__ A,
                                                           const T* __restrict__ dinv, const T* __restrict__ b,
                                                           const T* __restrict__ xin, const T* __restrict__ xc,
                                                           int nyc, T scale, T w, T w1, T* __restrict__ xout,
                                                           const Scalars* __restrict__ sk) {
    __shared__ T s3[PT_R3], s2[PT_R2], s1[PT_R1], s0[PT_R0];
    const int x0 = blockIdx.x * PT_X, y0 = blockIdx.y * PT_Y;
    {
        const int HY = PT_Y + 6;
        for (int h = threadIdx.x; h < PT_R3; h += blockDim.x) {
            const int gx = x0 - 3 + h / HY, gy = y0 - 3 + h % HY;
            T v = 0;
            if (gx >= 0 && gx < nx && gy >= 0 && gy < ny)
                v = smooth_at<T, 2>(nx, ny, gx * ny + gy, A, dinv, b, xin, xc, nyc, scale, w);
            s3[h] = v;
        }
    }
    __syncthreads();
    pt_sweep<T>(nx, ny, A, dinv, b, x0, y0, 2, s3, s2, w1);
    __syncthreads();
    pt_sweep<T>(nx, ny, A, dinv, b, x0, y0, 1, s2, s1, w);
    __syncthreads();
    pt_sweep<T>(nx, ny, A, dinv, b, x0, y0, 0, s1, s0, w1);
    const int tx = threadIdx.x / PT_Y, ty = threadIdx.x % PT_Y;
    const int cx = x0 + tx, cy = y0 + ty;
    if (cx < nx && cy < ny && !mg_skip(sk)) xout[cx * ny + cy] = s0[threadIdx.x];
}

// one sweep from a zero guess: x = w D^-1 b
template <typename T>
__global__ void k_mg_jacobi0(int64_t nc, const T* __restrict__ dinv, const T* __restrict__ b, T w, T* __restrict__ x,
                             const Scalars* __restrict__ sk) {
    if (mg_skip(sk)) return;
    GRID_LOOP(c, nc) x[c] = w * dinv[c] * b[c];
}

template <typename T>
__global__ void __launch_bounds__(MG_BLOCK) k_mg_restrict(int nx, int ny, const T* __restrict__ A,
                                                           const T* __restrict__ b, const T* __restrict__ x, int nxc,
                                                           int nyc, T* __restrict__ bc, const Scalars* __restrict__ sk) {
    const int C = blockIdx.x * blockDim.x + threadIdx.x;
    if (C >= nxc * nyc) return;
    const T v = restrict_at<T>(nx, ny, A, b, x, C, nyc);
    if (!mg_skip(sk)) bc[C] = v;
}

// ---- restriction of the pre-smoothed residual as an operator -------------------------
// With two pre-sweeps from zero (weights w0, then w1) the residual is
//   r = (I - w1 B)(I - w0 B) b,  B = A D^-1,
// so the coarse right-hand side P^T r is a fixed 36-point stencil on b (the
// 6x6 patch of fine cells within two of the coarse cell's 2x2 children).
// Built once per hierarchy; the V-cycle then computes it from b alone, in the
// same launch as the pre-smoothing (the two only read b).
constexpr int MG_RPATCH = 6;
constexpr int MG_RW = MG_RPATCH * MG_RPATCH;

template <typename T>
__global__ void k_mg_build_R(int nx, int ny, const T* __restrict__ A, const T* __restrict__ dinv, int nxc, int nyc,
                             T w0, T w1, T* __restrict__ R) {
    const int C = blockIdx.x * blockDim.x + threadIdx.x;
    if (C >= nxc * nyc) return;
    const int CX = C / nyc, CY = C - CX * nyc, nc = nx * ny, ncc = nxc * nyc;
    const int x0 = 2 * CX - 2, y0 = 2 * CY - 2;  // patch origin
    T acc[MG_RW];
#pragma unroll
    for (int k = 0; k < MG_RW; ++k) acc[k] = 0;
    const T wsum = w0 + w1, wprod = w0 * w1;
    // fully unrolled: every accumulator index is a compile-time constant, so
    // acc stays in registers
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int fx = 2 * CX + a, fy = 2 * CY + q;
            if (fx >= nx || fy >= ny) continue;
            const int f = fx * ny + fy;
            acc[(a + 2) * MG_RPATCH + (q + 2)] += (T)1;
#pragma unroll
            for (int s = 0; s < 9; ++s) {
                const int hx = fx + s / 3 - 1, hy = fy + s % 3 - 1;
                if (hx < 0 || hx >= nx || hy < 0 || hy >= ny) continue;
                const int h = hx * ny + hy;
                const T bfh = A[s * nc + f] * dinv[h];
                acc[(a + 1 + s / 3) * MG_RPATCH + (q + 1 + s % 3)] -= wsum * bfh;
#pragma unroll
                for (int s2 = 0; s2 < 9; ++s2) {
                    const int gx = hx + s2 / 3 - 1, gy = hy + s2 % 3 - 1;
                    if (gx < 0 || gx >= nx || gy < 0 || gy >= ny) continue;
                    acc[(a + s / 3 + s2 / 3) * MG_RPATCH + (q + s % 3 + s2 % 3)] +=
                        wprod * bfh * A[s2 * nc + h] * dinv[gx * ny + gy];
                }
            }
        }
#pragma unroll
    for (int k = 0; k < MG_RW; ++k) R[k * ncc + C] = acc[k];
}

// pre-smoothing of level l (blocks [0, nbs): two sweeps from zero, as
// k_mg_smooth<1>) and the restriction to level l+1 through R (the other
// blocks), in one launch
template <typename T>
__global__ void __launch_bounds__(MG_BLOCK) k_mg_pre_restrict(int nx, int ny, const T* __restrict__ A,
                                                               const T* __restrict__ dinv, const T* __restrict__ b,
                                                               T scale, T w, T w0, T* __restrict__ xout, int nbs,
                                                               int nxc, int nyc, const T* __restrict__ R,
                                                               T* __restrict__ bc, const Scalars* __restrict__ sk) {
    if ((int)blockIdx.x < nbs) {
        const int c = blockIdx.x * blockDim.x + threadIdx.x;
        if (c >= nx * ny) return;
        const T v = smooth_at<T, 1>(nx, ny, c, A, dinv, b, nullptr, nullptr, 0, scale, w, w0);
        if (!mg_skip(sk)) xout[c] = v;
        return;
    }
    const int C = (blockIdx.x - nbs) * blockDim.x + threadIdx.x, ncc = nxc * nyc;
    if (C >= ncc) return;
    const int CX = C / nyc, CY = C - CX * nyc, x0 = 2 * CX - 2, y0 = 2 * CY - 2;
    // the weights of patch cells outside the grid are exactly zero: clamped,
    // unconditional loads keep all 72 in flight
    T sum = 0;
#pragma unroll
    for (int k = 0; k < MG_RW; ++k) {
        const int gx = min(max(x0 + k / MG_RPATCH, 0), nx - 1), gy = min(max(y0 + k % MG_RPATCH, 0), ny - 1);
        sum += R[k * ncc + C] * b[gx * ny + gy];
    }
    if (!mg_skip(sk)) bc[C] = sum;
}

// The small levels l0..nlev in one CTA: the same sweeps, restrictions, dense
// solve and prolongations as the per-level kernels, phase by phase with a
// block barrier between phases (each phase reads what the previous one
// wrote).  Saves two to four launches per level where a level is too small
// to fill the GPU; the thresholds are measured (a single SM is latency-bound
// above about a thousand FP32 cells, and FP64 runs at a small fraction of
// the FP32 rate on this GPU).
// With `smem` set, the kernel first copies every tail level's stencil and
// diagonal and the coarsest level's inverse into shared memory and keeps the
// tail's vectors there: the phases then wait on shared-memory latency, not
// on L2's.  Only the first level's right-hand side comes in from global
// memory and only its solution goes out (the level above prolongs it).
constexpr int MG_TAIL_CELLS = 1100;
constexpr int MG_TAIL_CELLS_F64 = 300;
constexpr int MG_TAIL_THREADS = 1024;
template <typename T>
struct TailLevel {
    int nx, ny;
    const T* A;
    const T* dinv;
    T *b, *x, *y, *t;
};
template <typename T>
struct TailArgs {
    int l0, nlev, nu, nu_post, smem;
    T w, w1, scale;  // weights of the first and of the later sweeps
    T wpost;         // weight of the first post-sweep
    const T* cinv;
    const Scalars* sk;
    TailLevel<T> L[MG_MAX_LEVELS + 1];
    int64_t off[MG_MAX_LEVELS + 2];  // shared-memory words: level q's block; off[nlev+1] the inverse
};

// shared-memory words (of T) the tail stages for levels l0..nlev: per level
// the 9-point stencil, the diagonal and four vectors, each segment rounded
// to 16 bytes; then the coarsest inverse
template <typename T>
__host__ __device__ inline int64_t tail_seg(int64_t count) {
    const int64_t per16 = 16 / sizeof(T);
    return (count + per16 - 1) / per16 * per16;
}
template <typename T>
inline int64_t tail_words(const int64_t* nc, int l0, int nlev, int64_t* off) {
    int64_t w = 0;
    for (int q = l0; q <= nlev; ++q) {
        if (off) off[q] = w;
        w += tail_seg<T>(9 * nc[q]) + 5 * tail_seg<T>(nc[q]);
    }
    if (off) off[nlev + 1] = w;
    return w + tail_seg<T>(nc[nlev] * nc[nlev]);
}

// bytes from global to shared memory (both 16-byte aligned), all threads
__device__ __forceinline__ void tail_copy(void* dst, const void* src, int64_t bytes) {
    const int64_t n16 = bytes / 16;
    for (int64_t k = threadIdx.x; k < n16; k += blockDim.x) ((uint4*)dst)[k] = ((const uint4*)src)[k];
    for (int64_t k = n16 * 16 + threadIdx.x; k < bytes; k += blockDim.x)
        ((unsigned char*)dst)[k] = ((const unsigned char*)src)[k];
}

template <typename T>
__device__ __forceinline__ void tail_body(const TailArgs<T>& P, unsigned char* tail_sm, const Scalars* sk) {
    const int t = threadIdx.x, NT = blockDim.x;
    const T w = P.w, w1 = P.w1, sc = P.scale;
    const int nu = P.nu, nup = P.nu_post;
    const T wp = P.wpost;
    // level q as the phases see it: in global memory, or staged
    auto lv = [&](int q) -> TailLevel<T> {
        TailLevel<T> L = P.L[q];
        if (P.smem) {
            const int64_t nc = (int64_t)L.nx * L.ny, sn = tail_seg<T>(nc);
            T* s = (T*)tail_sm + P.off[q];
            L.A = s;
            L.dinv = s + tail_seg<T>(9 * nc);
            T* v = s + tail_seg<T>(9 * nc) + sn;
            L.b = v;
            L.x = v + sn;
            L.y = v + 2 * sn;
            L.t = v + 3 * sn;
        }
        return L;
    };
    const T* cinv = P.smem ? (const T*)((T*)tail_sm + P.off[P.nlev + 1]) : P.cinv;
    if (P.smem) {
        for (int l = P.l0; l <= P.nlev; ++l) {
            const TailLevel<T> L = lv(l);
            const int64_t nc = (int64_t)L.nx * L.ny;
            tail_copy((void*)L.A, P.L[l].A, 9 * nc * sizeof(T));
            tail_copy((void*)L.dinv, P.L[l].dinv, nc * sizeof(T));
            if (l == P.l0) tail_copy(L.b, P.L[l].b, nc * sizeof(T));
        }
        const int64_t nco = (int64_t)P.L[P.nlev].nx * P.L[P.nlev].ny;
        tail_copy((void*)cinv, P.cinv, nco * nco * sizeof(T));
        __syncthreads();
    }
    if (mg_skip(sk)) return;  // after the staging loads went out; the same for every thread
    T* cur[MG_MAX_LEVELS + 1];
    for (int l = P.l0; l < P.nlev; ++l) {
        const TailLevel<T> L = lv(l);
        const int64_t nc = (int64_t)L.nx * L.ny;
        T* c0 = L.y;
        for (int c = t; c < nc; c += NT)
            c0[c] = nu == 1 ? w * L.dinv[c] * L.b[c]
                            : smooth_at<T, 1>(L.nx, L.ny, c, L.A, L.dinv, L.b, nullptr, nullptr, 0, sc, w1, w);
        __syncthreads();
        for (int k = 2; k < nu; ++k) {
            T* out = c0 == L.y ? L.t : L.y;
            for (int c = t; c < nc; c += NT)
                out[c] = smooth_at<T, 0>(L.nx, L.ny, c, L.A, L.dinv, L.b, c0, nullptr, 0, sc, w1);
            __syncthreads();
            c0 = out;
        }
        cur[l] = c0;
        const TailLevel<T> C = lv(l + 1);
        const int64_t ncc = (int64_t)C.nx * C.ny;
        for (int q = t; q < ncc; q += NT) C.b[q] = restrict_at<T>(L.nx, L.ny, L.A, L.b, c0, q, C.ny);
        __syncthreads();
    }
    {   // coarsest level: x = C^-1 b, a warp per row, lanes along the row
        const TailLevel<T> L = lv(P.nlev);
        const int n = L.nx * L.ny;
        const int lane = t & 31;
        for (int r = t >> 5; r < n; r += NT >> 5) {
            T s = 0;
            for (int q = lane; q < n; q += 32) s += cinv[r * n + q] * L.b[q];
            for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
            if (lane == 0) L.x[r] = s;
        }
        __syncthreads();
    }
    for (int l = P.nlev - 1; l >= P.l0; --l) {
        const TailLevel<T> L = lv(l);
        const TailLevel<T> C = lv(l + 1);
        const int64_t nc = (int64_t)L.nx * L.ny;
        T* c0 = cur[l];
        for (int k = 0; k < nup; ++k) {
            T* out = (k == nup - 1) ? L.x : (c0 == L.y ? L.t : L.y);
            for (int c = t; c < nc; c += NT)
                out[c] = k == 0 ? smooth_at<T, 2>(L.nx, L.ny, c, L.A, L.dinv, L.b, c0, C.x, C.ny, sc, wp)
                                : smooth_at<T, 0>(L.nx, L.ny, c, L.A, L.dinv, L.b, c0, nullptr, 0, sc, w1);
            __syncthreads();
            c0 = out;
        }
    }
    if (P.smem) {  // the first level's solution, for the level above
        const TailLevel<T> L = lv(P.l0);
        const int64_t nc = (int64_t)L.nx * L.ny;
        for (int64_t c = t; c < nc; c += NT) P.L[P.l0].x[c] = L.x[c];
    }
}

template <typename T>
__global__ void __launch_bounds__(MG_TAIL_THREADS) k_mg_tail(TailArgs<T> P) {
    extern __shared__ __align__(16) unsigned char tail_sm[];
    tail_body<T>(P, tail_sm, P.sk);
}

// ---- V-cycle, level 0 (the PPE, unit diagonal) ---------------------------------------
// VI: type of the right-hand side v; O: type of the result z (the last sweep)
// two sweeps from a zero guess: x1 = w v; x2 = x1 + w (v - A x1)
template <typename T, typename VI, typename Op>
__global__ void __launch_bounds__(MG_BLOCK) k_mg0_pre2(int64_t n, Op A, const VI* __restrict__ v, T w,
                                                        T w1, T* __restrict__ x, const Scalars* __restrict__ sk) {
    if (mg_skip(sk)) return;
    GRID_LOOP(i, n) {
        const T Av = A.template row<VI, T>(i, v);
        const T vi = (T)v[i];
        x[i] = w * vi + w1 * (vi - w * Av);  // x1 = w v; x2 = x1 + w1 (v - A x1)
    }
}

template <typename T, typename VI>
__global__ void k_mg0_scale(int64_t n, const VI* __restrict__ v, T w, T* __restrict__ x,
                            const Scalars* __restrict__ sk) {
    if (mg_skip(sk)) return;
    GRID_LOOP(i, n) x[i] = w * (T)v[i];
}

// x_out = x + w (v - A x)
template <typename T, typename VI, typename O, typename Op>
__global__ void __launch_bounds__(MG_BLOCK) k_mg0_sweep(int64_t n, Op A, const VI* __restrict__ v,
                                                         const T* __restrict__ x, T w, O* __restrict__ xout,
                                                         const Scalars* __restrict__ sk) {
    if (mg_skip(sk)) return;
    GRID_LOOP(i, n) xout[i] = (O)(x[i] + w * ((T)v[i] - A.template row<T, T>(i, x)));
}

// r = v - A x
template <typename T, typename VI, typename Op>
__global__ void __launch_bounds__(MG_BLOCK) k_mg0_resid(int64_t n, Op A, const VI* __restrict__ v,
                                                         const T* __restrict__ x, T* __restrict__ r,
                                                         const Scalars* __restrict__ sk) {
    if (mg_skip(sk)) return;
    GRID_LOOP(i, n) r[i] = (T)v[i] - A.template row<T, T>(i, x);
}

// level-1 right-hand side: the residual summed over each cell's particles
template <typename T>
__global__ void k_mg0_restrict(int64_t nc, const int32_t* __restrict__ cell_start, const int32_t* __restrict__ cell_count,
                               const int32_t* __restrict__ sorted, const T* __restrict__ r, T* __restrict__ b1,
                               const Scalars* __restrict__ sk) {
    if (mg_skip(sk)) return;
    GRID_LOOP(c, nc) {
        const int q0 = cell_start[c], qn = cell_count[c];
        T s = 0;
        for (int q = q0; q < q0 + qn; ++q) s += r[sorted[q]];
        b1[c] = s;
    }
}

// First post-sweep, with the prolonged level-1 correction folded in and no
// pass over the matrix.  With y = x + s P x1 and r = v - A x (the residual
// restricted on the way down, still in place):
//   v - A y = r - s (A P x1),   (A P x1)_i = sum_k rs_k(i) x1[cell k of i's 3x3],
// rs_k(i) being row i's sums over its 3x3 neighbour cells (with the unit
// diagonal), the same sums the level-1 Galerkin product is built from.
// Reads 9 sums and 9 cell values per row instead of the row's entries.
template <typename T, typename O>
__global__ void __launch_bounds__(MG_BLOCK) k_mg0_post(int64_t n, int nx, int ny, const T* __restrict__ x,
                                                        const T* __restrict__ r, const T* __restrict__ x1,
                                                        const int32_t* __restrict__ pcell, const T* __restrict__ rs,
                                                        T scale, T w, O* __restrict__ xout,
                                                        const Scalars* __restrict__ sk) {
    if (mg_skip(sk)) return;
    GRID_LOOP(i, n) {
        const int c = pcell[i], cx = c / ny, cy = c - cx * ny;
        T apx = 0;
#pragma unroll
        for (int s = 0; s < 9; ++s) {
            const int gx = cx + s / 3 - 1, gy = cy + s % 3 - 1;
            if (gx < 0 || gx >= nx || gy < 0 || gy >= ny) continue;
            apx += rs[s * n + i] * x1[(int64_t)gx * ny + gy];
        }
        const T yi = x[i] + scale * x1[c];
        xout[i] = (O)(yi + w * (r[i] - scale * apx));
    }
}

template <typename T>
struct Lv {
    const T* A;
    const T* dinv;
    T *b, *x, *y, *t;
};

template <typename T>
Lv<T> level_view(const MgLevel& L) {
    if constexpr (sizeof(T) == 4)
        return {L.Af, L.dinvf, (T*)L.b, (T*)L.x, (T*)L.y, (T*)L.t};
    else
        return {L.A, L.dinv, (T*)L.b, (T*)L.x, (T*)L.y, (T*)L.t};
}

// the fine-level operator of the V-cycle: the FP64 matrix on the FP64 path;
// on the mixed path an FP16 copy of the Jacobi-scaled off-diagonals (all of
// magnitude below about one).  The V-cycle is only a preconditioner of a
// flexible Krylov method whose residuals use the FP32 and FP64 operators, so
// the FP16 rounding (2^-11 relative) can cost iterations, never accuracy;
// it cuts the bytes of the three matrix passes per V-cycle by a quarter.
// (The packed FP32 entries of the FP32 SpMV, one 8-byte load per entry, made
// these passes slower: 10.29 against 10.17 ms per c3 step.)
template <typename T>
struct FineOp;
template <>
struct FineOp<double> { using type = EllOp<double>; };
template <>
struct FineOp<float> { using type = EllPack16; };

template <typename T>
typename FineOp<T>::type fine_op(Ctx* c);
template <>
EllOp<double> fine_op<double>(Ctx* c) {
    return EllOp<double>{c->aval, c->nbr, c->cnt, c->K.kmax, c->spmv_unroll};
}
template <>
EllPack16 fine_op<float>(Ctx* c) {
    return EllPack16{c->ellh, c->ellh_ok, c->nbr, c->avalh, c->cnt, c->K.kmax};
}

// approximate solve of level l >= 1 (b_l -> x_l)
template <typename T>
int cycle_level(Ctx* c, int l) {
    Mg& mg = c->mg;
    const MgLevel& L = mg.L[l];
    Lv<T> v = level_view<T>(L);
    const unsigned g = blocks_for(L.nc, MG_BLOCK);
    const T w = (T)c->mg_w[0], w1 = (T)c->mg_w[1], sc = (T)c->P.mg_scale;
    const T wp = c->mg_wpost > 0 ? (T)c->mg_wpost : w;
    const int nu = c->P.mg_sweeps, nup = c->mg_post[0] > 0 ? c->mg_post[0] : nu;
    if (l >= mg.tail_l0) {  // this level and all coarser ones in one CTA
        TailArgs<T> P{};
        P.l0 = l;
        P.nlev = mg.nlev;
        P.nu = nu;
        P.nu_post = nup;
        P.wpost = wp;
        P.w = w;
        P.w1 = w1;
        P.scale = sc;
        if constexpr (sizeof(T) == 4)
            P.cinv = mg.cinvf;
        else
            P.cinv = mg.cinv;
        P.sk = mg.skip;
        P.smem = mg.tail_smem > 0;
        {
            int64_t nc[MG_MAX_LEVELS + 1] = {};
            for (int q = l; q <= mg.nlev; ++q) nc[q] = mg.L[q].nc;
            tail_words<T>(nc, l, mg.nlev, P.off);
        }
        for (int q = l; q <= mg.nlev; ++q) {
            Lv<T> u = level_view<T>(mg.L[q]);
            P.L[q] = TailLevel<T>{mg.L[q].nx, mg.L[q].ny, u.A, u.dinv, u.b, u.x, u.y, u.t};
        }
        k_mg_tail<T><<<1, MG_TAIL_THREADS, mg.tail_smem, c->stream>>>(P);
        BSC_LAUNCH(c);
        return BSC_OK;
    }
    // pre-smoothing from a zero guess: one sweep is x = w D^-1 b; with two or
    // more, the first is folded into the second
    T* cur = v.y;
    const MgLevel& Lc = mg.L[l + 1];
    Lv<T> vc = level_view<T>(Lc);
    if (c->mg_cell4 && nu == 2) {  // four sweeps each way, one launch each
        const dim3 gt((unsigned)((L.nx + PT_X - 1) / PT_X), (unsigned)((L.ny + PT_Y - 1) / PT_Y));
        k_mg_pre4_restrict<T><<<gt, PT_X * PT_Y, 0, c->stream>>>(L.nx, L.ny, v.A, v.dinv, v.b, w, w1, cur, Lc.nx,
                                                                  Lc.ny, vc.b, c->mg.skip);
        BSC_LAUNCH(c);
        if (int rc = cycle_level<T>(c, l + 1)) return rc;
        k_mg_post4<T><<<gt, PT_X * PT_Y, 0, c->stream>>>(L.nx, L.ny, v.A, v.dinv, v.b, cur, vc.x, Lc.ny, sc, w, w1,
                                                          v.x, c->mg.skip);
        BSC_LAUNCH(c);
        return BSC_OK;
    }
    if (nu == 2 && L.R) {
        // both sweeps and the restriction in one launch
        k_mg_pre_restrict<T><<<g + blocks_for(Lc.nc, MG_BLOCK), MG_BLOCK, 0, c->stream>>>(
            L.nx, L.ny, v.A, v.dinv, v.b, sc, w1, w, cur, (int)g, Lc.nx, Lc.ny, (const T*)L.R, vc.b, c->mg.skip);
        BSC_LAUNCH(c);
    } else {
    if (nu == 1)
        k_mg_jacobi0<T><<<g, MG_BLOCK, 0, c->stream>>>(L.nc, v.dinv, v.b, w, cur, c->mg.skip);
    else
        k_mg_smooth<T, 1><<<g, MG_BLOCK, 0, c->stream>>>(L.nx, L.ny, v.A, v.dinv, v.b, nullptr, nullptr, 0, sc, w1, w,
                                                          cur, c->mg.skip);
    BSC_LAUNCH(c);
    for (int k = 2; k < nu; ++k) {
        T* out = cur == v.y ? v.t : v.y;
        k_mg_smooth<T, 0><<<g, MG_BLOCK, 0, c->stream>>>(L.nx, L.ny, v.A, v.dinv, v.b, cur, nullptr, 0, sc, w1, w1,
                                                          out, c->mg.skip);
        BSC_LAUNCH(c);
        cur = out;
    }
    k_mg_restrict<T><<<blocks_for(Lc.nc, MG_BLOCK), MG_BLOCK, 0, c->stream>>>(L.nx, L.ny, v.A, v.b, cur, Lc.nx, Lc.ny, vc.b, c->mg.skip);
    BSC_LAUNCH(c);
    }
    if (int rc = cycle_level<T>(c, l + 1)) return rc;
    // post-smoothing: the prolongation folded into the first sweep; the last
    // sweep writes x_l
    if (nup == 2 && c->mg_post_fused) {  // both sweeps in one launch
        const dim3 gt((unsigned)((L.nx + PT_X - 1) / PT_X), (unsigned)((L.ny + PT_Y - 1) / PT_Y));
        k_mg_post2<T><<<gt, PT_X * PT_Y, 0, c->stream>>>(L.nx, L.ny, v.A, v.dinv, v.b, cur, vc.x, Lc.ny, sc, wp, w1,
                                                          v.x, c->mg.skip);
        BSC_LAUNCH(c);
        return BSC_OK;
    }
    for (int k = 0; k < nup; ++k) {
        T* out = (k == nup - 1) ? v.x : (cur == v.y ? v.t : v.y);
        if (k == 0)
            k_mg_smooth<T, 2><<<g, MG_BLOCK, 0, c->stream>>>(L.nx, L.ny, v.A, v.dinv, v.b, cur, vc.x, Lc.ny, sc, wp, wp,
                                                              out, c->mg.skip);
        else
            k_mg_smooth<T, 0><<<g, MG_BLOCK, 0, c->stream>>>(L.nx, L.ny, v.A, v.dinv, v.b, cur, nullptr, 0, sc, w1, w1,
                                                              out, c->mg.skip);
        BSC_LAUNCH(c);
        cur = out;
    }
    return BSC_OK;
}

// z = M v: V-cycle arithmetic in T, right-hand side in VI, result in O
template <typename T, typename VI, typename O>
int vcycle(Ctx* c, const VI* vin, O* z) {
    Mg& mg = c->mg;
    const int64_t n = c->n;
    using AV = typename FineOp<T>::type;  // the fine operator's type
    const AV A = fine_op<T>(c);
    const T w = (T)c->mg_w[0], w1 = (T)c->mg_w[1], sc = (T)c->P.mg_scale;
    const T wp = c->mg_wpost > 0 ? (T)c->mg_wpost : w;
    const int nu = c->P.mg_sweeps, nup = c->mg_post[1] > 0 ? c->mg_post[1] : nu;
    T *P0 = (T*)mg.y0, *Q0 = (T*)mg.t0, *R0 = (T*)mg.r0;
    // one row per thread: the fine-level passes have no reduction, and a full
    // grid keeps more rows' loads in flight than a grid-stride loop over a
    // fixed grid (measured: 10% faster fine passes at 846k rows)
    const int G = (int)blocks_for(n, MG_BLOCK);
    if (c->prof_iter) record_event(c, c->ev_it[0]);
    T* cur = P0;
    const int nupre = c->mg_pre_fine > 0 ? c->mg_pre_fine : nu;
    if (nupre == 1)
        k_mg0_scale<T, VI><<<G, MG_BLOCK, 0, c->stream>>>(n, vin, w, cur, c->mg.skip);
    else
        k_mg0_pre2<T, VI, AV><<<G, MG_BLOCK, 0, c->stream>>>(n, A, vin, w, w1, cur, c->mg.skip);
    BSC_LAUNCH(c);
    for (int k = 2; k < nupre; ++k) {
        T* out = cur == P0 ? Q0 : P0;
        k_mg0_sweep<T, VI, T, AV><<<G, MG_BLOCK, 0, c->stream>>>(n, A, vin, cur, w1, out, c->mg.skip);
        BSC_LAUNCH(c);
        cur = out;
    }
    k_mg0_resid<T, VI, AV><<<G, MG_BLOCK, 0, c->stream>>>(n, A, vin, cur, R0, c->mg.skip);
    BSC_LAUNCH(c);
    const MgLevel& L1 = mg.L[1];
    Lv<T> v1 = level_view<T>(L1);
    k_mg0_restrict<T><<<blocks_for(L1.nc, MG_BLOCK), MG_BLOCK, 0, c->stream>>>(L1.nc, c->cell_start, c->cell_count, c->sorted, R0, v1.b, c->mg.skip);
    BSC_LAUNCH(c);
    if (c->prof_iter) record_event(c, c->ev_it[1]);
    if (int rc = cycle_level<T>(c, 1)) return rc;
    if (c->prof_iter) record_event(c, c->ev_it[2]);
    // post-smoothing; the last sweep writes z
    const T* rs;
    if constexpr (sizeof(T) == 4)
        rs = mg.rowslotsf;
    else
        rs = mg.rowslots;
    for (int k = 0; k < nup; ++k) {
        const bool last = k == nup - 1;
        T* out = cur == P0 ? Q0 : P0;
        if (k == 0 && last)
            k_mg0_post<T, O><<<G, MG_BLOCK, 0, c->stream>>>(n, L1.nx, L1.ny, cur, R0, v1.x, c->pcell, rs, sc, wp, z,
                                                            c->mg.skip);
        else if (k == 0)
            k_mg0_post<T, T><<<G, MG_BLOCK, 0, c->stream>>>(n, L1.nx, L1.ny, cur, R0, v1.x, c->pcell, rs, sc, wp,
                                                            out, c->mg.skip);
        else if (last)
            k_mg0_sweep<T, VI, O, AV><<<G, MG_BLOCK, 0, c->stream>>>(n, A, vin, cur, w1, z, c->mg.skip);
        else
            k_mg0_sweep<T, VI, T, AV><<<G, MG_BLOCK, 0, c->stream>>>(n, A, vin, cur, w1, out, c->mg.skip);
        BSC_LAUNCH(c);
        cur = out;
    }
    if (c->prof_iter) record_event(c, c->ev_it[3]);
    return BSC_OK;
}

template <typename T>
int mg_dalloc(Ctx* c, T** p, int64_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, (size_t)std::max<int64_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return cuda_err(c, e, "cudaMalloc (multigrid)");
    c->mg.allocs.push_back(q);
    *p = (T*)q;
    return BSC_OK;
}

// buffers for the grid, the row count, the restart length and the precision
int mg_alloc(Ctx* c) {
    Mg& mg = c->mg;
    const int64_t n = c->n;
    const int m = std::max(1, std::min(c->P.restart, 64));
    const bool f32 = c->mixed;
    if (mg.n == n && mg.gx == c->K.nx && mg.gy == c->K.ny && mg.m == m && mg.f32 == f32 && !mg.allocs.empty())
        return BSC_OK;
    drop_graphs(c);  // captured iterations point into the buffers replaced here
    mg_free(c);
    // the level dimensions
    int nlev = 1;
    mg.L[1].nx = c->K.nx;
    mg.L[1].ny = c->K.ny;
    const int64_t cmax = std::max(4, std::min(c->P.mg_coarse_max, MG_COARSE_MAX));
    while ((int64_t)mg.L[nlev].nx * mg.L[nlev].ny > cmax) {
        if (nlev == MG_MAX_LEVELS) return set_err(c, BSC_E_CAPACITY, "multigrid: too many levels");
        mg.L[nlev + 1].nx = (mg.L[nlev].nx + 1) / 2;
        mg.L[nlev + 1].ny = (mg.L[nlev].ny + 1) / 2;
        ++nlev;
    }
    mg.nlev = nlev;
    // one SM runs the tail: FP32 levels up to MG_TAIL_CELLS cells, FP64 ones
    // up to MG_TAIL_CELLS_F64
    int64_t tail_cells = f32 ? MG_TAIL_CELLS : MG_TAIL_CELLS_F64;
    if (c->mg_tail_cells >= 0) tail_cells = c->mg_tail_cells;
    mg.tail_l0 = nlev;
    while (mg.tail_l0 > 1 && (int64_t)mg.L[mg.tail_l0 - 1].nx * mg.L[mg.tail_l0 - 1].ny <= tail_cells)
        --mg.tail_l0;
    const size_t vs = f32 ? sizeof(float) : sizeof(double);
    int rc;
    for (int l = 1; l <= nlev; ++l) {
        MgLevel& L = mg.L[l];
        L.nc = (int64_t)L.nx * L.ny;
        if ((rc = mg_dalloc(c, &L.A, 9 * L.nc)) || (rc = mg_dalloc(c, &L.dinv, L.nc))) return rc;
        if (f32 && ((rc = mg_dalloc(c, &L.Af, 9 * L.nc)) || (rc = mg_dalloc(c, &L.dinvf, L.nc)))) return rc;
        // four vectors, each on a 256-byte boundary (no cache line shared)
        const int64_t stride = ((L.nc * (int64_t)vs + 255) / 256) * 256;
        unsigned char* vec = nullptr;
        if ((rc = mg_dalloc(c, &vec, 4 * stride))) return rc;
        L.b = vec;
        L.x = vec + stride;
        L.y = vec + 2 * stride;
        L.t = vec + 3 * stride;
    }
    for (int l = 1; l < mg.tail_l0; ++l)  // the restriction operators of the per-level kernels
        if ((rc = mg_dalloc(c, (unsigned char**)&mg.L[l].R, (int64_t)MG_RW * mg.L[l + 1].nc * (int64_t)vs))) return rc;
    if ((rc = mg_dalloc(c, &mg.rowslots, 9 * n))) return rc;  // the level-1 Galerkin pass
    if (f32 && (rc = mg_dalloc(c, &mg.rowslotsf, 9 * n))) return rc;
    const int64_t nco = mg.L[nlev].nc;
    if ((rc = mg_dalloc(c, &mg.cinv, nco * nco))) return rc;
    if (f32 && (rc = mg_dalloc(c, &mg.cinvf, nco * nco))) return rc;
    // stage the tail in shared memory when it fits
    {
        int64_t nc[MG_MAX_LEVELS + 1] = {};
        for (int l = 1; l <= nlev; ++l) nc[l] = mg.L[l].nc;
        const int64_t bytes = f32 ? tail_words<float>(nc, mg.tail_l0, nlev, nullptr) * (int64_t)sizeof(float)
                                  : tail_words<double>(nc, mg.tail_l0, nlev, nullptr) * (int64_t)sizeof(double);
        int optin = 0;
        BSC_CUDA(c, cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
        mg.tail_smem = bytes <= optin ? (int)bytes : 0;
        // the attribute is per function, process-wide: allow the device's
        // maximum, whatever this context needs
        if (mg.tail_smem > 0) {
            if (f32)
                BSC_CUDA(c, cudaFuncSetAttribute(k_mg_tail<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
            else
                BSC_CUDA(c, cudaFuncSetAttribute(k_mg_tail<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
        }
    }
    unsigned char* fine = nullptr;
    if ((rc = mg_dalloc(c, &fine, 3 * n * (int64_t)vs))) return rc;
    mg.r0 = fine;
    mg.y0 = fine + n * vs;
    mg.t0 = fine + 2 * n * vs;
    if (f32) {
        // FP32 inner FGMRES of the iterative refinement: basis, preconditioned
        // vectors, and the work vectors w, r
        if ((rc = mg_dalloc(c, &mg.Vf, (int64_t)(m + 1) * n)) || (rc = mg_dalloc(c, &mg.Zf, (int64_t)m * n)) ||
            (rc = mg_dalloc(c, &mg.wf, 2 * n)))
            return rc;
        mg.rf = mg.wf + n;
    } else {
        if ((rc = mg_dalloc(c, &mg.V, (int64_t)(m + 1) * n)) || (rc = mg_dalloc(c, &mg.Z, (int64_t)m * n))) return rc;
    }
    mg.n = n;
    mg.gx = c->K.nx;
    mg.gy = c->K.ny;
    mg.m = m;
    mg.f32 = f32;
    return BSC_OK;
}

}  // namespace

void mg_free(Ctx* c) {
    Mg& mg = c->mg;
    if (!mg.allocs.empty() && c->stream) cudaStreamSynchronize(c->stream);
    for (void* p : mg.allocs) cudaFree(p);
    mg.allocs.clear();
    mg = Mg{};
}

int mg_setup(Ctx* c) {
    if (!c->have_csr) return set_err(c, BSC_E_INVALID, "multigrid setup before assembly");
    if (int rc = mg_alloc(c)) return rc;
    Mg& mg = c->mg;
    const EllOp<double> A{c->aval, c->nbr, c->cnt, c->K.kmax, 0};
    MgLevel& L1 = mg.L[1];
    k_mg_rowslots<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, L1.ny, c->pcell, A, mg.rowslots,
                                                                mg.f32 ? mg.rowslotsf : nullptr);
    BSC_LAUNCH(c);
    const bool f32 = mg.f32;
    k_mg_galerkin0<<<blocks_for(L1.nc, 128), 128, 0, c->stream>>>(L1.nx, L1.ny, c->n, c->cell_start,
                                                                   c->cell_count, c->sorted, mg.rowslots, L1.A,
                                                                   L1.dinv, f32 ? L1.Af : nullptr,
                                                                   f32 ? L1.dinvf : nullptr);
    BSC_LAUNCH(c);
    for (int l = 1; l < mg.nlev; ++l) {
        const MgLevel &F = mg.L[l], &C = mg.L[l + 1];
        k_mg_galerkin<<<blocks_for(C.nc, 128), 128, 0, c->stream>>>(F.nx, F.ny, F.A, C.nx, C.ny, C.A, C.dinv,
                                                                     f32 ? C.Af : nullptr, f32 ? C.dinvf : nullptr);
        BSC_LAUNCH(c);
    }
    // the coarsest inverse (FP32 Gauss-Jordan), in the V-cycle's precision
    const MgLevel& Lc = mg.L[mg.nlev];
    const int smem = (int)(Lc.nc * Lc.nc * sizeof(float));
    const int smem_max = MG_COARSE_MAX * MG_COARSE_MAX * (int)sizeof(float);
    BSC_CUDA(c, cudaFuncSetAttribute(k_mg_dense_inverse<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
    BSC_CUDA(c, cudaFuncSetAttribute(k_mg_dense_inverse<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_max));
    if (f32)
        k_mg_dense_inverse<float><<<1, 1024, smem, c->stream>>>(Lc.nx, Lc.ny, Lc.A, mg.cinvf);
    else
        k_mg_dense_inverse<double><<<1, 1024, smem, c->stream>>>(Lc.nx, Lc.ny, Lc.A, mg.cinv);
    BSC_LAUNCH(c);
    // the restriction operators of the levels swept by per-level kernels
    if (c->P.mg_sweeps == 2 && !c->mg_cell4)
        for (int l = 1; l < mg.tail_l0; ++l) {
            const MgLevel &F = mg.L[l], &C = mg.L[l + 1];
            const unsigned gb = blocks_for(C.nc, 128);
            if (f32)
                k_mg_build_R<float><<<gb, 128, 0, c->stream>>>(F.nx, F.ny, F.Af, F.dinvf, C.nx, C.ny,
                                                               (float)c->mg_w[0], (float)c->mg_w[1], (float*)F.R);
            else
                k_mg_build_R<double><<<gb, 128, 0, c->stream>>>(F.nx, F.ny, F.A, F.dinv, C.nx, C.ny, c->mg_w[0],
                                                                c->mg_w[1], (double*)F.R);
            BSC_LAUNCH(c);
        }
    return BSC_OK;
}

int mg_vcycle_f64(Ctx* c, const double* v, double* z) { return vcycle<double, double, double>(c, v, z); }
int mg_vcycle_f32(Ctx* c, const float* v, float* z) { return vcycle<float, float, float>(c, v, z); }

}  // namespace bsc
