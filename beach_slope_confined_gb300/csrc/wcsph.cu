// wcsph.cu -- the differentiable weakly compressible SPH step and its
// hand-written adjoint (the calibration workload: gradients of a wave-probe
// misfit with respect to the porous-drag coefficients and a porosity grid).
//
// Forward step (FP64, one thread per particle, gathers over the frozen
// neighbour lists of the step):
//   rt = max(rho, rho0) (fluid; the reference's dentopress reset of negative
//        pressure, wcsph.f90:36-62), p = B((rt/rho0)^gamma - 1), B = rho0 c0^2/gamma
//   n_i  = 1 - sum_s (1 - phi_s) V_s W(r_is)           porosity from the solids
//   Drho = sum_j m_j (rt_i/rt_j) (v_i - v_j).gW
//        + c2 sum_j (rt_j - rt_i - rhoH_j + rhoH_i) (x_j - x_i).gW V_j/(r^2+lam)
//                                    (wcsph.f90:66-133, c2 = delta 2h c0; the
//                                     diffusion written with x_j - x_i)
//   a    = -n_i sum_j m_j (p_i/rt_i^2 + p_j/rt_j^2) gW
//        + sum_j 2 nu V_j (x_ij.gW)/(r^2+lam) (v_i - v_j) + n_i g
//   R    = -nu alpha (1-n)^2/(n^3 d^2) - beta |v| (1-n)/(n^3 d)   (Ergun, porous.f90:192-212)
//   v'   = (v + dt a)/(1 - dt R n),  x' = x + dt v'/n,  rho' = rt + dt Drho
// with gW = F(r) (x_i - x_j) the Wendland C2 gradient and rhoH(y) the
// hydrostatic density below the still-water level.  Walls are prescribed
// (fixed hydrostatic density; the piston moves its wall particles).  The
// model carries its own particle masses m = rho_init dl^2, so that every
// volume m/rho starts at the lattice volume dl^2, inside the porous layer too
// (the ISPH masses rho0 n dl^2 would leave the kernel sums there short by n
// and the layer out of hydrostatic balance); v is the superficial velocity,
// the particles move at the pore velocity v/n.
//
// Adjoint: the exact reverse of that map for the fluid state (x, y, vx, vy,
// rho), geometry included (the derivative of gW through F'(r)); lists are
// symmetric, so each particle gathers the terms of its own sums and of its
// neighbours' sums without atomics.  Reverse sweep by segments: each segment
// of `ckpt_every` steps is recomputed from its checkpoint, keeping the
// per-step states, lists, porosities and pressure sums the adjoint reads.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "bsc_internal.cuh"

struct bsc_ctx : bsc::Ctx {};  // the same definition as in api.cu

namespace bsc {

struct WcK {
    double rho0, B, gam, inv_gam, grav_c, ys;  // EOS; rhoH(y) = rho0 (1 + grav_c (ys - y))^(1/gamma)
    double c2;                                 // delta 2h c0
    double nu, lam, g, dt, d50, H2;
    double alpha, beta;
    double inv_h, wend_F, wend_W;
    double gx0, gy0, gdx, gdy, por_default;
    int gnx, gny, kmax, np, gc;  // gc: grid cells one support can overlap
    double R1, depth;                          // probe kernel radius, probe depth
};

struct WcState {
    WcK K{};
    int64_t n = 0, ns = 0;
    int G = 0;                                 // grid cells
    double t0 = 0.0;
    double* init = nullptr;                    // initial state: x y vx vy rho (5n)
    double* mass = nullptr;                    // particle masses rho_init dl^2
    double *theta = nullptr, *sw = nullptr;    // grid porosities; (1 - phi_s) V_s
    int32_t* sg = nullptr;                     // solid -> grid cell or -1
    double *rt = nullptr, *pp = nullptr, *rh = nullptr, *drh = nullptr;  // per step
    double *vol = nullptr, *pr = nullptr;      // m/rt, p/rt^2 (per step)
    double* dpdr = nullptr;                    // dp/drt (per step)
    double* nxt = nullptr;                     // next state (5n)
    double *xp = nullptr, *eta = nullptr, *part = nullptr;  // probes, eta history, partials
    // forward record
    int nsteps = 0, every = 0;
    bool last_kept = false;                    // the forward run kept its last segment
    std::vector<double> tck;
    double* ck = nullptr;                      // checkpoints (5n each)
    int ck_cap = 0, seg_cap = 0, eta_cap = 0;
    double *seg = nullptr, *segn = nullptr, *segP = nullptr;  // (K+1) states; n; P (2n)
    int32_t *segnbr = nullptr, *segcnt = nullptr, *segpc = nullptr;  // lists, counts, cells
    // what the reverse sweep reads from the recomputation, per step: the
    // per-particle quotients, per-pair kernel values (F, F'/r, G, G'/r), the
    // porosity gradient and the per-grid-cell kernel sums of the porosity
    double *segpre = nullptr, *seggeo = nullptr, *segdn = nullptr, *segpgv = nullptr;
    int32_t* segpgi = nullptr;
    // adjoint
    double *lam = nullptr, *lamn = nullptr;    // 5n each
    double *la = nullptr, *lD = nullptr, *ln = nullptr, *lvl = nullptr, *lrl = nullptr;
    double *dJ = nullptr, *grad = nullptr;
    std::vector<void*> allocs;
};

namespace {

constexpr int WB = 128;
constexpr int GCMAX = 9;  // grid cells one particle's kernel support can overlap (checked at setup)

template <typename T>
int wc_alloc(Ctx* c, WcState* w, T** p, int64_t count) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, (size_t)std::max<int64_t>(count, 1) * sizeof(T));
    if (e != cudaSuccess) return cuda_err(c, e, "cudaMalloc (wcsph)");
    w->allocs.push_back(q);
    *p = (T*)q;
    return BSC_OK;
}

// Wendland C2: grad W = F(r) d, F' = dF/dr
__device__ __forceinline__ double wF(const WcK& K, double r) {
    const double a = 1.0 - 0.5 * r * K.inv_h;
    return -K.wend_F * a * a * a;
}
__device__ __forceinline__ double wdF(const WcK& K, double r) {
    const double a = 1.0 - 0.5 * r * K.inv_h;
    return 1.5 * K.wend_F * a * a * K.inv_h;
}
__device__ __forceinline__ double wW(const WcK& K, double r) {
    const double q = r * K.inv_h, a = 1.0 - 0.5 * q, a2 = a * a;
    return K.wend_W * (1.0 + 2.0 * q) * a2 * a2;
}
// the 1-D Wendland C2 kernel of the probes (radius R1, unit integral)
__device__ __forceinline__ double w1(double q, double R1) {
    const double a = 1.0 - q;
    return (1.25 / R1) * (a * a * a) * (1.0 + 3.0 * q);
}
__device__ __forceinline__ double w1q(double q, double R1) {  // d w1 / dq
    const double a = 1.0 - q;
    return -(15.0 / R1) * q * a * a;
}

__device__ __forceinline__ bool is_fluid(const State& S, int64_t i) { return S.tid[i] == BSC_TID_FLUID; }

// fields of a 5n state block
struct St {
    double *x, *y, *vx, *vy, *rho;
};
__host__ __device__ inline St st_of(double* b, int64_t n) { return {b, b + n, b + 2 * n, b + 3 * n, b + 4 * n}; }

__global__ void k_wc_init(int64_t n, State S, WcK K, double vol0, double* __restrict__ mass) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s = 1.0 + K.grav_c * (K.ys - S.y[i]);
    // hydrostatic density below the level, rho0 above it
    const double r = S.y[i] < K.ys ? K.rho0 * pow(s, K.inv_gam) : K.rho0;
    S.rho[i] = r;
    mass[i] = r * vol0;
}

__global__ void k_wc_solids(int64_t ns, const double* __restrict__ sx, const double* __restrict__ sy,
                            const double* __restrict__ svol, const double* __restrict__ theta, WcK K,
                            double* __restrict__ sw, int32_t* __restrict__ sg) {
    const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (s >= ns) return;
    const double fx = floor((sx[s] - K.gx0) / K.gdx), fy = floor((sy[s] - K.gy0) / K.gdy);
    int g = -1;
    if (fx >= 0.0 && fx < (double)K.gnx && fy >= 0.0 && fy < (double)K.gny) g = (int)fy * K.gnx + (int)fx;
    const double phi = g >= 0 ? theta[g] : K.por_default;
    sw[s] = (1.0 - phi) * svol[s];
    sg[s] = g;
}

// clamped density, pressure, hydrostatic density and its slope, and the
// per-particle quotients the pair loops read (volume m/rt, p/rt^2)
struct Pre {
    double *rt, *pp, *rh, *drh, *vol, *pr, *dpdr;  // dpdr: dp/drt of the EOS
};

__global__ void k_wc_pre(int64_t n, const int8_t* __restrict__ tid, const double* __restrict__ mass,
                         const double* __restrict__ y, const double* __restrict__ rho, WcK K, Pre o) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double r = tid[i] == BSC_TID_FLUID ? fmax(rho[i], K.rho0) : rho[i];
    const double qg = pow(r / K.rho0, K.gam);
    double p = K.B * (qg - 1.0);
    if (p < 0.0) p = 0.0;
    const double ir = 1.0 / r;
    o.dpdr[i] = K.B * K.gam * qg * ir;  // B gamma (rt/rho0)^(gamma-1) / rho0
    o.rt[i] = r;
    o.pp[i] = p;
    o.vol[i] = mass[i] * ir;
    o.pr[i] = p * ir * ir;
    double* rh = o.rh;
    double* drh = o.drh;
    const double s = 1.0 + K.grav_c * (K.ys - y[i]);
    const double q = pow(s, K.inv_gam);
    rh[i] = K.rho0 * q;
    drh[i] = -K.rho0 * K.grav_c * K.inv_gam * q / s;
}

// the five state fields, one launch
__global__ void k_wc_copy(int64_t n, St src, St dst) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst.x[i] = src.x[i];
    dst.y[i] = src.y[i];
    dst.vx[i] = src.vx[i];
    dst.vy[i] = src.vy[i];
    dst.rho[i] = src.rho[i];
}

// what the porosity pass keeps for the adjoint (null when not kept)
struct PorKeep {
    double* dn;    // grad n_i (2n)
    int32_t* pgi;  // grid cell u of particle i at [u * n + i], -1 past the last
    double* pgv;   // sum over that cell's solids of V_s W(r_is)
};

// porosity n_i from the solids in the 3x3 cells (fluid; 1 elsewhere)
__global__ void __launch_bounds__(WB) k_wc_por(int64_t n, State S, KParams KP, WcK K, const int32_t* __restrict__ pcell,
                                               const int32_t* __restrict__ scs, const int32_t* __restrict__ scc,
                                               const double* __restrict__ sx, const double* __restrict__ sy,
                                               const double* __restrict__ sw, const double* __restrict__ svol,
                                               const int32_t* __restrict__ sg, double* __restrict__ nout, PorKeep kp) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    int cg[GCMAX];
    double cv[GCMAX];
#pragma unroll
    for (int u = 0; u < GCMAX; ++u) {
        cg[u] = -1;
        cv[u] = 0.0;
    }
    double frac = 0.0, gx = 0.0, gy = 0.0;
    if (is_fluid(S, i)) {
        const double xi = S.x[i], yi = S.y[i];
        const int c = pcell[i], cx = c / KP.ny, cy = c - cx * KP.ny;
        for (int ax = cx - 1; ax <= cx + 1; ++ax) {
            if (ax < 0 || ax >= KP.nx) continue;
            for (int ay = cy - 1; ay <= cy + 1; ++ay) {
                if (ay < 0 || ay >= KP.ny) continue;
                const int cc = ax * KP.ny + ay;
                for (int s = scs[cc], e = scs[cc] + scc[cc]; s < e; ++s) {
                    const double dx = xi - sx[s], dy = yi - sy[s], d2 = dx * dx + dy * dy;
                    if (!(d2 < K.H2)) continue;
                    const double r = sqrt(d2), W = wW(K, r);
                    frac += sw[s] * W;
                    if (kp.dn) {
                        const double F = wF(K, r);
                        gx -= sw[s] * F * dx;  // grad n = -sum sw grad W
                        gy -= sw[s] * F * dy;
                        const int g = sg[s];
                        if (g < 0) continue;
                        const double v = svol[s] * W;
                        bool kept = false;
#pragma unroll
                        for (int u = 0; u < GCMAX; ++u) {
                            if (!kept && u < K.gc && (cg[u] == g || cg[u] < 0)) {
                                cg[u] = g;
                                cv[u] += v;
                                kept = true;
                            }
                        }
                    }
                }
            }
        }
    }
    nout[i] = is_fluid(S, i) ? 1.0 - frac : 1.0;
    if (kp.dn) {
        kp.dn[i] = gx;
        kp.dn[n + i] = gy;
#pragma unroll
        for (int u = 0; u < GCMAX; ++u) {
            if (u < K.gc) {
                kp.pgi[u * n + i] = cg[u];
                kp.pgv[u * n + i] = cv[u];
            }
        }
    }
}

// one step: next state; the porosity (in nbuf) and the pressure sum P
// (2 per particle, for the adjoint) are kept
__global__ void __launch_bounds__(WB) k_wc_step(int64_t n, State S, WcK K, const int32_t* __restrict__ nbr,
                                                const int32_t* __restrict__ cnt, Pre pq,
                                                const double* __restrict__ nbuf, St out, double* __restrict__ Pbuf,
                                                double* __restrict__ geo, int64_t slots) {
    const double* __restrict__ rt = pq.rt;
    const double* __restrict__ rh = pq.rh;
    const double* __restrict__ vol = pq.vol;
    const double* __restrict__ pr = pq.pr;
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = S.x[i], yi = S.y[i], vxi = S.vx[i], vyi = S.vy[i];
    if (!is_fluid(S, i)) {
        out.x[i] = xi;
        out.y[i] = yi;
        out.vx[i] = vxi;
        out.vy[i] = vyi;
        out.rho[i] = S.rho[i];
        Pbuf[i] = Pbuf[n + i] = 0.0;
        return;
    }
    const double rti = rt[i], rhi = rh[i], ni = nbuf[i];
    const double pri = pr[i];
    double Dr = 0.0, Px = 0.0, Py = 0.0, vx = 0.0, vy = 0.0;
    const int m = cnt[i];
    for (int k = 0; k < m; ++k) {
        const int j = nbr[ell(i, k, K.kmax)];
        const double dx = xi - S.x[j], dy = yi - S.y[j];
        const double r2 = dx * dx + dy * dy, r = sqrt(r2);
        const double iden = rcp_nr(r2 + K.lam);
        const double F = wF(K, r), G = F * r2 * iden;
        if (geo) {  // F, F'/r, G, G'/r for the reverse sweep
            const int64_t e = ell(i, k, K.kmax);
            const double ir = rcp_nr(r), dF = wdF(K, r);
            geo[e] = F;
            geo[slots + e] = dF * ir;
            geo[2 * slots + e] = G;
            geo[3 * slots + e] = (dF * r2 + F * 2.0 * r * K.lam * iden) * iden * ir;
        }
        const double rtj = rt[j], mj = S.mass[j], Vj = vol[j];
        const double dvx = vxi - S.vx[j], dvy = vyi - S.vy[j];
        Dr += rti * Vj * F * (dvx * dx + dvy * dy);  // m_j (rt_i / rt_j) F (v_ij . x_ij)
        Dr += K.c2 * (rtj - rti - rh[j] + rhi) * (-G) * Vj;
        const double pc = mj * (pri + pr[j]) * F;
        Px += pc * dx;
        Py += pc * dy;
        const double vc = 2.0 * K.nu * Vj * G;
        vx += vc * dvx;
        vy += vc * dvy;
    }
    const double ax = -ni * Px + vx, ay = -ni * Py + vy + ni * K.g;
    const double vm = sqrt(vxi * vxi + vyi * vyi), on = 1.0 - ni, n3 = ni * ni * ni;
    const double R = -K.nu * K.alpha * on * on / (n3 * K.d50 * K.d50) - K.beta * vm * on / (n3 * K.d50);
    const double D = 1.0 - K.dt * R * ni;
    const double vxn = (vxi + K.dt * ax) / D, vyn = (vyi + K.dt * ay) / D;
    out.vx[i] = vxn;
    out.vy[i] = vyn;
    out.x[i] = xi + K.dt * vxn / ni;
    out.y[i] = yi + K.dt * vyn / ni;
    out.rho[i] = rti + K.dt * Dr;
    Pbuf[i] = Px;
    Pbuf[n + i] = Py;
}

// probe elevations of a state: per-block partials of sum_i V_i w1(x_i - x_p)
__global__ void __launch_bounds__(WB) k_wc_eta(int64_t n, const int8_t* __restrict__ tid, const double* __restrict__ mass,
                                               St s, WcK K, const double* __restrict__ xp, double* __restrict__ part) {
    __shared__ double sh[WB];
    double acc[BSC_WCSPH_MAX_PROBES];
    for (int p = 0; p < K.np; ++p) acc[p] = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (tid[i] != BSC_TID_FLUID) continue;
        const double V = mass[i] / s.rho[i];
        for (int p = 0; p < K.np; ++p) {
            const double q = fabs(s.x[i] - xp[p]) / K.R1;
            if (q < 1.0) acc[p] += V * w1(q, K.R1);
        }
    }
    for (int p = 0; p < K.np; ++p) {
        sh[threadIdx.x] = acc[p];
        __syncthreads();
        for (int o = WB / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) part[blockIdx.x * K.np + p] = sh[0];
        __syncthreads();
    }
}

// one block per probe, fixed summation order
__global__ void k_wc_eta_fin(int nb, WcK K, const double* __restrict__ part, double* __restrict__ eta) {
    __shared__ double sh[WB];
    const int p = blockIdx.x;
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += WB) s += part[b * K.np + p];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = WB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) eta[p] = sh[0] - K.depth;
}

// ---- adjoint ---------------------------------------------------------------------
// the loss's direct dependence on a state: lam += dJ/deta . d eta/d(x, rho)
__global__ void k_wc_adj_probe(int64_t n, const int8_t* __restrict__ tid, const double* __restrict__ mass, St s,
                               WcK K, const double* __restrict__ xp, const double* __restrict__ dJ, St lam) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || tid[i] != BSC_TID_FLUID) return;
    const double V = mass[i] / s.rho[i];
    double gx = 0.0, gr = 0.0;
    for (int p = 0; p < K.np; ++p) {
        const double d = s.x[i] - xp[p], q = fabs(d) / K.R1;
        if (q >= 1.0) continue;
        gx += dJ[p] * V * w1q(q, K.R1) * (d >= 0.0 ? 1.0 : -1.0) / K.R1;
        gr += dJ[p] * (-V / s.rho[i]) * w1(q, K.R1);
    }
    lam.x[i] += gx;
    lam.rho[i] += gr;
}

// block sum of two values into part[block][0..1]
__device__ __forceinline__ void block_sum2(double a, double b, double* __restrict__ part) {
    __shared__ double sa[WB], sb[WB];
    sa[threadIdx.x] = a;
    sb[threadIdx.x] = b;
    __syncthreads();
    for (int o = WB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            sa[threadIdx.x] += sa[threadIdx.x + o];
            sb[threadIdx.x] += sb[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[0] = sa[0];
        part[1] = sb[0];
    }
}

// the per-particle part of the reverse step: position update, drag, the
// porosity's direct roles; writes lam_a, lam_Drho, lam_n, and the particle's
// own contributions to lam_v and lam_rt; drag-coefficient partials per block
__global__ void __launch_bounds__(WB) k_wc_adj_local(int64_t n, const int8_t* __restrict__ tid, WcK K, St s0, St s1,
                                                     const double* __restrict__ nbuf, const double* __restrict__ Pbuf,
                                                     St lam, double* __restrict__ la, double* __restrict__ lD,
                                                     double* __restrict__ ln, double* __restrict__ lvl,
                                                     double* __restrict__ lrl, double* __restrict__ part, int pstride) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    double ga = 0.0, gb = 0.0;
    if (i < n && tid[i] == BSC_TID_FLUID) {
        // the quotients by n, n^3, d and D as products with reciprocals taken once
        const double ni = nbuf[i], vx = s0.vx[i], vy = s0.vy[i], vxn = s1.vx[i], vyn = s1.vy[i];
        const double in = 1.0 / ni, in3 = in * in * in, in4 = in3 * in, id = 1.0 / K.d50;
        const double vm = sqrt(vx * vx + vy * vy), on = 1.0 - ni;
        const double cA = K.nu * on * on * in3 * id * id, cB = vm * on * in3 * id;  // dR/dalpha, dR/dbeta (negated)
        const double R = -K.alpha * cA - K.beta * cB;
        const double iD = 1.0 / (1.0 - K.dt * R * ni);
        const double lx = lam.x[i], ly = lam.y[i];
        const double lpx = lam.vx[i] + K.dt * lx * in, lpy = lam.vy[i] + K.dt * ly * in;
        double lni = -K.dt * (lx * vxn + ly * vyn) * in * in;
        const double lax = K.dt * lpx * iD, lay = K.dt * lpy * iD;
        const double lDD = -(lpx * vxn + lpy * vyn) * iD;
        const double lR = -K.dt * ni * lDD;
        lni += -K.dt * R * lDD;
        const double dRdn = -K.nu * K.alpha * id * id * (-2.0 * on * in3 - 3.0 * on * on * in4) -
                            K.beta * vm * id * (-in3 - 3.0 * on * in4);
        lni += lR * dRdn;
        double lvx = lpx * iD, lvy = lpy * iD;
        if (vm > 0.0) {
            const double cv = lR * (-K.beta * on * in3 * id) / vm;
            lvx += cv * vx;
            lvy += cv * vy;
        }
        ga = lR * (-cA);
        gb = lR * (-cB);
        // a = -n P + visc + n g: d a / d n = -P + g
        lni += lax * (-Pbuf[i]) + lay * (-Pbuf[n + i] + K.g);
        la[i] = lax;
        la[n + i] = lay;
        lD[i] = K.dt * lam.rho[i];
        ln[i] = lni;
        lvl[i] = lvx;
        lvl[n + i] = lvy;
        lrl[i] = lam.rho[i];
    } else if (i < n) {
        la[i] = la[n + i] = 0.0;
        lD[i] = ln[i] = 0.0;
    }
    block_sum2(ga, gb, part + (int64_t)blockIdx.x * pstride);
}

// the pair part: for fluid particle k, the terms of its own sums (k as i) and
// of its neighbours' sums (k as j), with the per-pair kernel values and the
// porosity's gradient and per-grid-cell sums that the recomputation kept;
// writes the state adjoint lam_out for the state before the step and the
// block's porosity-grid partials
__global__ void __launch_bounds__(WB) k_wc_adj_pair(
    int64_t n, State S, WcK K, St s0, const int32_t* __restrict__ nbr, const int32_t* __restrict__ cnt, Pre pq,
    const double* __restrict__ geo, int64_t slots, const double* __restrict__ nbuf, const double* __restrict__ la,
    const double* __restrict__ lD, const double* __restrict__ ln, const double* __restrict__ lvl,
    const double* __restrict__ lrl, St lam_in, St lam_out, const double* __restrict__ dn,
    const int32_t* __restrict__ pgi, const double* __restrict__ pgv, double* __restrict__ part, int pstride) {
    // grid-porosity partials per warp, then summed over the warps in order
    __shared__ double wb[WB / 32][BSC_WCSPH_MAX_GRID];
    const int G = K.gnx * K.gny;
    for (int e = threadIdx.x; e < (WB / 32) * BSC_WCSPH_MAX_GRID; e += WB) (&wb[0][0])[e] = 0.0;
    __syncthreads();
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool act = k < n && S.tid[k] == BSC_TID_FLUID;
    double lnk = 0.0;
    if (act) {
        const double* __restrict__ rt = pq.rt;
        const double* __restrict__ rh = pq.rh;
        const double xk = s0.x[k], yk = s0.y[k], vxk = s0.vx[k], vyk = s0.vy[k];
        const double rtk = rt[k], pk = pq.pp[k], rhk = rh[k], drk = pq.drh[k], nk = nbuf[k], mk = S.mass[k];
        const double Vk = pq.vol[k], prk = pq.pr[k], irk = 1.0 / rtk;
        const double mk_rt2 = mk * irk * irk, pk_rt3 = 2.0 * prk * irk;  // m_k / rt_k^2, 2 p_k / rt_k^3
        const double lDk = lD[k], lax = la[k], lay = la[n + k];
        double lrt = lrl[k], lp = 0.0;
        double lvx = lvl[k], lvy = lvl[n + k];
        double lxx = lam_in.x[k], lyy = lam_in.y[k];
        const int m = cnt[k];
        for (int q = 0; q < m; ++q) {
            const int64_t e = ell(k, q, K.kmax);
            const int j = nbr[e];
            const double dx = xk - s0.x[j], dy = yk - s0.y[j];
            const double F = geo[e], Fr = geo[slots + e], G_ = geo[2 * slots + e], Gr = geo[3 * slots + e];
            const double rtj = rt[j], prj = pq.pr[j], mj = S.mass[j], Vj = pq.vol[j];
            const double dvx = vxk - s0.vx[j], dvy = vyk - s0.vy[j], dvd = dvx * dx + dvy * dy;
            double gx = 0.0, gy = 0.0;  // adjoint of d = x_k - x_j
            // -- k's own continuity sum
            {
                const double c1 = rtk * Vj;  // m_j rt_k / rt_j
                lrt += lDk * Vj * F * dvd;
                lvx += lDk * c1 * F * dx;
                lvy += lDk * c1 * F * dy;
                const double t = lDk * c1 * Fr * dvd;
                gx += lDk * c1 * F * dvx + t * dx;
                gy += lDk * c1 * F * dvy + t * dy;
                const double del = rtj - rtk - rh[j] + rhk;
                lrt += lDk * K.c2 * G_ * Vj;
                lyy += lDk * K.c2 * drk * (-G_) * Vj;
                const double u = -lDk * K.c2 * del * Gr * Vj;
                gx += u * dx;
                gy += u * dy;
            }
            // -- k's own momentum sum
            {
                const double lad = lax * dx + lay * dy;
                const double pc = mj * (prk + prj);
                gx += -nk * pc * (F * lax + Fr * lad * dx);
                gy += -nk * pc * (F * lay + Fr * lad * dy);
                lp += -nk * mj * irk * irk * F * lad;
                lrt += nk * mj * pk_rt3 * F * lad;
                const double vc = 2.0 * K.nu * Vj;
                lvx += vc * G_ * lax;
                lvy += vc * G_ * lay;
                const double w = vc * (lax * dvx + lay * dvy) * Gr;
                gx += w * dx;
                gy += w * dy;
            }
            // -- k in the sums of its fluid neighbour j, where the offset is
            // e = x_j - x_k = -d: the adjoint of e (hx, hy) enters lam_x_k with
            // the opposite sign
            if (S.tid[j] == BSC_TID_FLUID) {
                const double lDj = lD[j], lajx = la[j], lajy = la[n + j], nj = nbuf[j];
                const double ex = -dx, ey = -dy;      // x_j - x_k; (v_j - v_k).(x_j - x_k) = dvd
                const double dwx = -dvx, dwy = -dvy;  // v_j - v_k
                double hx = 0.0, hy = 0.0;
                // continuity of j
                const double c1 = rtj * Vk;  // m_k rt_j / rt_k
                lrt += lDj * (-c1 * irk) * F * dvd;
                lvx += lDj * (-c1 * F * ex);
                lvy += lDj * (-c1 * F * ey);
                {
                    const double t = lDj * c1 * Fr * dvd;
                    hx += lDj * c1 * F * dwx + t * ex;
                    hy += lDj * c1 * F * dwy + t * ey;
                }
                const double del = rtk - rtj - rhk + rh[j];
                lrt += lDj * K.c2 * (-G_) * Vk * (1.0 - del * irk);
                lyy += lDj * K.c2 * drk * G_ * Vk;
                {
                    const double u = -lDj * K.c2 * del * Gr * Vk;
                    hx += u * ex;
                    hy += u * ey;
                }
                // momentum of j
                const double lad = lajx * ex + lajy * ey;
                const double pc = mk * (prj + prk);
                hx += -nj * pc * (F * lajx + Fr * lad * ex);
                hy += -nj * pc * (F * lajy + Fr * lad * ey);
                lp += -nj * mk_rt2 * F * lad;
                lrt += nj * mk * pk_rt3 * F * lad;
                const double vc = 2.0 * K.nu * Vk;
                lvx += -vc * G_ * lajx;
                lvy += -vc * G_ * lajy;
                const double ldv = lajx * dwx + lajy * dwy;
                lrt += -2.0 * K.nu * mk_rt2 * G_ * ldv;
                const double w = vc * ldv * Gr;
                hx += w * ex;
                hy += w * ey;
                gx -= hx;
                gy -= hy;
            }
            lxx += gx;
            lyy += gy;
        }
        // porosity n_k = 1 - sum_s (1 - phi_s) V_s W(r_ks)
        lnk = ln[k];
        lxx += lnk * dn[k];
        lyy += lnk * dn[n + k];
        // pressure and the clamp
        lrt += lp * pq.dpdr[k];
        lam_out.x[k] = lxx;
        lam_out.y[k] = lyy;
        lam_out.vx[k] = lvx;
        lam_out.vy[k] = lvy;
        lam_out.rho[k] = s0.rho[k] >= K.rho0 ? lrt : 0.0;
    } else if (k < n) {
        lam_out.x[k] = lam_out.y[k] = lam_out.vx[k] = lam_out.vy[k] = lam_out.rho[k] = 0.0;
    }
    // d n_k / d phi_g = sum over cell g's solids of V_s W(r_ks): lanes with the
    // same cell are summed in lane order by the lowest of them
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int u = 0; u < K.gc; ++u) {
        int g = -1;
        double v = 0.0;
        if (act) {
            g = pgi[u * n + k];
            v = lnk * pgv[u * n + k];
        }
        const unsigned grp = __match_any_sync(0xffffffffu, g);
        double acc = 0.0;
        for (int src = 0; src < 32; ++src) {
            const double t = __shfl_sync(0xffffffffu, v, src);
            if ((grp >> src) & 1u) acc += t;
        }
        if (g >= 0 && lane == __ffs(grp) - 1) wb[warp][g] += acc;
        __syncwarp();
    }
    __syncthreads();
    for (int g = threadIdx.x; g < G; g += WB) {
        double acc = 0.0;
        for (int q = 0; q < WB / 32; ++q) acc += wb[q][g];
        part[(int64_t)blockIdx.x * pstride + 2 + g] = acc;
    }
}

// grad[q] += sum over blocks of part[block][q]: one block per q, fixed order
__global__ void k_wc_grad(int nb, int pstride, const double* __restrict__ part, double* __restrict__ grad) {
    __shared__ double sh[WB];
    const int q = blockIdx.x;
    double s = 0.0;
    for (int b = threadIdx.x; b < nb; b += WB) s += part[(int64_t)b * pstride + q];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = WB / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) grad[q] += sh[0];
}

}  // namespace

void wc_free(Ctx* c) {
    WcState* w = c->wc;
    if (!w) return;
    if (c->stream) cudaStreamSynchronize(c->stream);
    for (void* p : w->allocs) cudaFree(p);
    delete w;
    c->wc = nullptr;
}

namespace {

int wc_params(Ctx* c, WcState* w, double alpha, double beta, const double* grid) {
    w->K.alpha = alpha;
    w->K.beta = beta;
    if (grid) BSC_CUDA(c, cudaMemcpyAsync(w->theta, grid, sizeof(double) * w->G, cudaMemcpyHostToDevice, c->stream));
    if (w->ns > 0) {
        k_wc_solids<<<blocks_for(w->ns, 256), 256, 0, c->stream>>>(w->ns, c->sx, c->sy, c->svol, w->theta, w->K, w->sw,
                                                                 w->sg);
        BSC_LAUNCH(c);
    }
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    return BSC_OK;
}

// one forward step on c->S; keeps n and P in nbuf, Pbuf
Pre wc_pre(WcState* w) { return {w->rt, w->pp, w->rh, w->drh, w->vol, w->pr, w->dpdr}; }

// the context's state with the model's masses
State wc_view(Ctx* c, WcState* w) {
    State S = c->S;
    S.mass = w->mass;
    return S;
}

int launch_check(Ctx* c) {
    c->launches++;
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? BSC_OK : cuda_err(c, e, "wcsph step");
}

St st_ctx(Ctx* c) { return {c->S.x, c->S.y, c->S.vx, c->S.vy, c->S.rho}; }

int wc_copy(Ctx* c, St src, St dst) {
    k_wc_copy<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, src, dst);
    BSC_LAUNCH(c);
    return BSC_OK;
}
int wc_save(Ctx* c, double* dst) { return wc_copy(c, st_ctx(c), st_of(dst, c->n)); }
int wc_load(Ctx* c, const double* src) { return wc_copy(c, st_of(const_cast<double*>(src), c->n), st_ctx(c)); }

// what the recomputation of a segment keeps of one step for the reverse sweep
struct Keep {
    int32_t *nbr, *cnt, *cell;  // neighbour lists, counts, particle cells
    Pre pre;                    // per-particle quotients
    double* geo;                // per-pair kernel values (4 x slots)
    PorKeep por;                // porosity gradient and per-grid-cell sums
};

int64_t list_slots(const Ctx* c) { return ((c->n + 31) / 32) * 32 * (int64_t)c->K.kmax; }

Keep seg_keep(WcState* w, int q, int64_t n, int64_t slots) {
    double* pre = w->segpre + (int64_t)q * 7 * n;
    const int gc = w->K.gc;
    return {w->segnbr + (int64_t)q * slots,
            w->segcnt + (int64_t)q * n,
            w->segpc + (int64_t)q * n,
            {pre, pre + n, pre + 2 * n, pre + 3 * n, pre + 4 * n, pre + 5 * n, pre + 6 * n},
            w->seggeo + (int64_t)q * 4 * slots,
            {w->segdn + (int64_t)q * 2 * n, w->segpgi + (int64_t)q * gc * n, w->segpgv + (int64_t)q * gc * n}};
}

// One step on c->S; keeps the porosity and the pressure sum in nbuf and Pbuf.
// With `keep`, the step's lists, counts and cells are built straight into the
// kept buffers (the context's own are pointed there for the step), and the
// per-particle quotients, per-pair kernel values and porosity derivatives
// are kept too.
int wc_step(Ctx* c, WcState* w, double* nbuf, double* Pbuf, const Keep* keep = nullptr) {
    const int64_t n = c->n;
    c->t += w->K.dt;
    int32_t *own_nbr = c->nbr, *own_cnt = c->cnt, *own_cell = c->pcell;
    if (keep) {
        c->nbr = keep->nbr;
        c->cnt = keep->cnt;
        c->pcell = keep->cell;
    }
    const Pre pre = keep ? keep->pre : wc_pre(w);
    int rc = op_piston(c);
    if (!rc) rc = cells_build(c, false);
    if (!rc) rc = op_neighbour(c);
    if (!rc) {
        const unsigned g = blocks_for(n, WB);
        const State S = wc_view(c, w);
        k_wc_pre<<<g, WB, 0, c->stream>>>(n, S.tid, S.mass, S.y, S.rho, w->K, pre);
        rc = launch_check(c);
        if (!rc) {
            k_wc_por<<<g, WB, 0, c->stream>>>(n, S, c->K, w->K, c->pcell, c->scell_start, c->scell_count, c->sx,
                                              c->sy, w->sw, c->svol, w->sg, nbuf,
                                              keep ? keep->por : PorKeep{nullptr, nullptr, nullptr});
            rc = launch_check(c);
        }
        if (!rc) {
            k_wc_step<<<g, WB, 0, c->stream>>>(n, S, w->K, c->nbr, c->cnt, pre, nbuf, st_of(w->nxt, n), Pbuf,
                                               keep ? keep->geo : nullptr, list_slots(c));
            rc = launch_check(c);
        }
    }
    c->nbr = own_nbr;
    c->cnt = own_cnt;
    c->pcell = own_cell;
    if (rc) return rc;
    // the next state becomes the state
    return wc_copy(c, st_of(w->nxt, n), st_ctx(c));
}

}  // namespace
}  // namespace bsc

using namespace bsc;

extern "C" {

int bsc_wcsph_setup(bsc_ctx* c, const bsc_wcsph_params* p) {
    if (!c || !p) return BSC_E_INVALID;
    if (!c->have_state) return set_err(c, BSC_E_INVALID, "wcsph_setup before upload_state");
    if (c->mixed || c->K.kernel != BSC_KERNEL_WENDLAND_C2)
        return set_err(c, BSC_E_INVALID, "wcsph: an FP64 context with the Wendland C2 kernel");
    const int G = p->grid_nx * p->grid_ny;
    if (p->grid_nx < 1 || p->grid_ny < 1 || G > BSC_WCSPH_MAX_GRID || !p->grid_por || !(p->grid_dx > 0) ||
        !(p->grid_dy > 0) || p->nprobe < 1 || p->nprobe > BSC_WCSPH_MAX_PROBES || !(p->c0 > 0) || !(p->gamma > 0))
        return set_err(c, BSC_E_INVALID, "wcsph_setup: bad parameters");
    wc_free(c);
    WcState* w = new (std::nothrow) WcState();
    if (!w) return BSC_E_NOMEM;
    c->wc = w;
    const int64_t n = c->n;
    w->n = n;
    w->ns = c->ns;
    w->G = G;
    WcK& K = w->K;
    const KParams& KP = c->K;
    K.rho0 = KP.rho0;
    K.gam = p->gamma;
    K.inv_gam = 1.0 / p->gamma;
    K.B = KP.rho0 * p->c0 * p->c0 / p->gamma;
    K.grav_c = std::fabs(KP.g) * p->gamma / (p->c0 * p->c0);
    K.ys = p->surface_y;
    K.c2 = p->delta * 2.0 * KP.h * p->c0;
    K.nu = p->nu;
    K.lam = KP.lam;
    K.g = KP.g;
    K.dt = c->dt;
    K.d50 = KP.d50;
    K.H2 = KP.H2;
    K.inv_h = KP.inv_h;
    K.wend_F = KP.wend_F;
    K.wend_W = KP.wend_W;
    K.gx0 = p->grid_x0;
    K.gy0 = p->grid_y0;
    K.gdx = p->grid_dx;
    K.gdy = p->grid_dy;
    K.gnx = p->grid_nx;
    K.gny = p->grid_ny;
    K.por_default = KP.por;
    K.kmax = KP.kmax;
    K.np = p->nprobe;
    K.R1 = 2.0 * KP.h;
    K.depth = p->probe_depth;
    // grid cells a kernel support (diameter 4h) can overlap
    const int ncx = std::min(p->grid_nx, (int)std::floor(4.0 * KP.h / p->grid_dx) + 2);
    const int ncy = std::min(p->grid_ny, (int)std::floor(4.0 * KP.h / p->grid_dy) + 2);
    K.gc = ncx * ncy;
    if (K.gc > GCMAX) return set_err(c, BSC_E_INVALID, "wcsph_setup: porosity grid cells smaller than 2h");
    int rc;
    if ((rc = wc_alloc(c, w, &w->init, 5 * n)) || (rc = wc_alloc(c, w, &w->mass, n)) ||
        (rc = wc_alloc(c, w, &w->theta, G)) ||
        (rc = wc_alloc(c, w, &w->sw, w->ns)) || (rc = wc_alloc(c, w, &w->sg, w->ns)) ||
        (rc = wc_alloc(c, w, &w->rt, n)) || (rc = wc_alloc(c, w, &w->pp, n)) || (rc = wc_alloc(c, w, &w->rh, n)) ||
        (rc = wc_alloc(c, w, &w->drh, n)) || (rc = wc_alloc(c, w, &w->vol, n)) || (rc = wc_alloc(c, w, &w->pr, n)) ||
        (rc = wc_alloc(c, w, &w->dpdr, n)) ||
        (rc = wc_alloc(c, w, &w->nxt, 5 * n)) ||
        (rc = wc_alloc(c, w, &w->xp, BSC_WCSPH_MAX_PROBES)) ||
        (rc = wc_alloc(c, w, &w->part, (int64_t)blocks_for(n, WB) * (2 + BSC_WCSPH_MAX_GRID))) ||
        (rc = wc_alloc(c, w, &w->lam, 5 * n)) || (rc = wc_alloc(c, w, &w->lamn, 5 * n)) ||
        (rc = wc_alloc(c, w, &w->la, 2 * n)) || (rc = wc_alloc(c, w, &w->lD, n)) || (rc = wc_alloc(c, w, &w->ln, n)) ||
        (rc = wc_alloc(c, w, &w->lvl, 2 * n)) || (rc = wc_alloc(c, w, &w->lrl, n)) ||
        (rc = wc_alloc(c, w, &w->grad, 2 + BSC_WCSPH_MAX_GRID)))
        return rc;
    BSC_CUDA(c, cudaMemcpyAsync(w->xp, p->probe_x, sizeof(double) * p->nprobe, cudaMemcpyHostToDevice, c->stream));
    // hydrostatic densities, then the initial state
    k_wc_init<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, c->S, K, KP.dl * KP.dl, w->mass);
    BSC_LAUNCH(c);
    if ((rc = wc_save(c, w->init))) return rc;
    w->t0 = c->t;
    return wc_params(c, w, p->alpha, p->beta, p->grid_por);
}

int bsc_wcsph_set_params(bsc_ctx* c, double alpha, double beta, const double* grid_por) {
    if (!c || !c->wc) return c ? set_err(c, BSC_E_INVALID, "wcsph_set_params before wcsph_setup") : BSC_E_INVALID;
    return wc_params(c, c->wc, alpha, beta, grid_por);
}

int bsc_wcsph_forward(bsc_ctx* c, int32_t nsteps, int32_t every, double* eta) {
    if (!c || !c->wc) return c ? set_err(c, BSC_E_INVALID, "wcsph_forward before wcsph_setup") : BSC_E_INVALID;
    if (nsteps < 1 || every < 1 || !eta) return set_err(c, BSC_E_INVALID, "wcsph_forward: bad arguments");
    WcState* w = c->wc;
    const int64_t n = c->n;
    int rc;
    const int nck = (nsteps + every - 1) / every;
    if (nck > w->ck_cap) {
        if ((rc = wc_alloc(c, w, &w->ck, (int64_t)nck * 5 * n))) return rc;
        w->ck_cap = nck;
    }
    if (nsteps > w->eta_cap) {
        if ((rc = wc_alloc(c, w, &w->eta, (int64_t)nsteps * w->K.np)) ||
            (rc = wc_alloc(c, w, &w->dJ, (int64_t)nsteps * w->K.np)))
            return rc;
        w->eta_cap = nsteps;
    }
    if (every > w->seg_cap) {
        const int64_t slots = list_slots(c), gc = w->K.gc;
        if ((rc = wc_alloc(c, w, &w->seg, (int64_t)(every + 1) * 5 * n)) ||
            (rc = wc_alloc(c, w, &w->segn, (int64_t)every * n)) || (rc = wc_alloc(c, w, &w->segP, (int64_t)every * 2 * n)) ||
            (rc = wc_alloc(c, w, &w->segnbr, (int64_t)every * slots)) ||
            (rc = wc_alloc(c, w, &w->segcnt, (int64_t)every * n)) ||
            (rc = wc_alloc(c, w, &w->segpc, (int64_t)every * n)) ||
            (rc = wc_alloc(c, w, &w->segpre, (int64_t)every * 7 * n)) ||
            (rc = wc_alloc(c, w, &w->seggeo, (int64_t)every * 4 * slots)) ||
            (rc = wc_alloc(c, w, &w->segdn, (int64_t)every * 2 * n)) ||
            (rc = wc_alloc(c, w, &w->segpgi, (int64_t)every * gc * n)) ||
            (rc = wc_alloc(c, w, &w->segpgv, (int64_t)every * gc * n)))
            return rc;
        w->seg_cap = every;
    }
    w->nsteps = nsteps;
    w->every = every;
    w->tck.assign(nck, 0.0);
    // the last segment keeps what the reverse sweep reads as it runs, so the
    // adjoint recomputes one segment fewer
    const int last0 = (nck - 1) * every;
    const int64_t slots = list_slots(c);
    w->last_kept = false;
    if ((rc = wc_load(c, w->init))) return rc;
    c->t = w->t0;
    const unsigned nb = blocks_for(n, WB);
    for (int s = 0; s < nsteps; ++s) {
        if (s % every == 0) {
            if ((rc = wc_save(c, w->ck + (int64_t)(s / every) * 5 * n))) return rc;
            w->tck[s / every] = c->t;
        }
        if (s >= last0) {
            const int q = s - last0;
            const Keep kq = seg_keep(w, q, n, slots);
            if ((rc = wc_save(c, w->seg + (int64_t)q * 5 * n)) ||
                (rc = wc_step(c, w, w->segn + (int64_t)q * n, w->segP + (int64_t)q * 2 * n, &kq)))
                return rc;
            if (s == nsteps - 1 && (rc = wc_save(c, w->seg + (int64_t)(q + 1) * 5 * n))) return rc;
        } else if ((rc = wc_step(c, w, w->segn, w->segP))) {
            return rc;
        }
        k_wc_eta<<<nb, WB, 0, c->stream>>>(n, c->S.tid, w->mass, st_of(w->nxt, n), w->K, w->xp, w->part);
        BSC_LAUNCH(c);
        k_wc_eta_fin<<<w->K.np, WB, 0, c->stream>>>(nb, w->K, w->part, w->eta + (int64_t)s * w->K.np);
        BSC_LAUNCH(c);
    }
    BSC_CUDA(c, cudaMemcpyAsync(eta, w->eta, sizeof(double) * nsteps * w->K.np, cudaMemcpyDeviceToHost, c->stream));
    int32_t flag = 0;
    BSC_CUDA(c, cudaMemcpyAsync(&flag, c->d_flag, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    if (flag) {
        BSC_CUDA(c, cudaMemsetAsync(c->d_flag, 0, 4 * sizeof(int32_t), c->stream));
        return set_err(c, BSC_E_CAPACITY, "wcsph_forward: neighbour-list capacity or cell grid exceeded");
    }
    w->last_kept = true;
    return BSC_OK;
}

int bsc_wcsph_adjoint(bsc_ctx* c, const double* dJ_deta, double* grad) {
    if (!c || !c->wc) return c ? set_err(c, BSC_E_INVALID, "wcsph_adjoint before wcsph_setup") : BSC_E_INVALID;
    WcState* w = c->wc;
    if (w->nsteps < 1 || !dJ_deta || !grad) return set_err(c, BSC_E_INVALID, "wcsph_adjoint: run wcsph_forward first");
    const int64_t n = c->n;
    const int nsteps = w->nsteps, every = w->every, np = w->K.np, G = w->G;
    const unsigned nb = blocks_for(n, WB);
    const int pstride = 2 + BSC_WCSPH_MAX_GRID;
    const int64_t slots = list_slots(c);
    int rc;
    BSC_CUDA(c, cudaMemcpyAsync(w->dJ, dJ_deta, sizeof(double) * nsteps * np, cudaMemcpyHostToDevice, c->stream));
    BSC_CUDA(c, cudaMemsetAsync(w->lam, 0, sizeof(double) * 5 * n, c->stream));
    BSC_CUDA(c, cudaMemsetAsync(w->grad, 0, sizeof(double) * (2 + BSC_WCSPH_MAX_GRID), c->stream));
    const int nseg = (nsteps + every - 1) / every;
    for (int sgi = nseg - 1; sgi >= 0; --sgi) {
        const int s0 = sgi * every, s1 = std::min(nsteps, s0 + every);
        // recompute the segment, keeping states, lists, porosities, pressure
        // sums (the last one the forward run kept)
        const bool kept = sgi == nseg - 1 && w->last_kept;
        if (!kept && (rc = wc_load(c, w->ck + (int64_t)sgi * 5 * n))) return rc;
        c->t = w->tck[sgi];
        for (int s = s0; s < s1 && !kept; ++s) {
            const int q = s - s0;
            if ((rc = wc_save(c, w->seg + (int64_t)q * 5 * n))) return rc;
            const Keep kq = seg_keep(w, q, n, slots);
            if ((rc = wc_step(c, w, w->segn + (int64_t)q * n, w->segP + (int64_t)q * 2 * n, &kq))) return rc;
        }
        if (!kept && (rc = wc_save(c, w->seg + (int64_t)(s1 - s0) * 5 * n))) return rc;
        // reverse through the segment
        for (int s = s1 - 1; s >= s0; --s) {
            const int q = s - s0;
            const St st0 = st_of(w->seg + (int64_t)q * 5 * n, n), st1 = st_of(w->seg + (int64_t)(q + 1) * 5 * n, n);
            St lam = st_of(w->lam, n), lamn = st_of(w->lamn, n);
            // the loss at the state after step s
            k_wc_adj_probe<<<nb, WB, 0, c->stream>>>(n, c->S.tid, w->mass, st1, w->K, w->xp,
                                                     w->dJ + (int64_t)s * np, lam);
            BSC_LAUNCH(c);
            const State S = wc_view(c, w);
            const Keep kq = seg_keep(w, q, n, slots);
            const double* nq = w->segn + (int64_t)q * n;
            k_wc_adj_local<<<nb, WB, 0, c->stream>>>(n, c->S.tid, w->K, st0, st1, nq, w->segP + (int64_t)q * 2 * n, lam,
                                                     w->la, w->lD, w->ln, w->lvl, w->lrl, w->part, pstride);
            BSC_LAUNCH(c);
            k_wc_adj_pair<<<nb, WB, 0, c->stream>>>(n, S, w->K, st0, kq.nbr, kq.cnt, kq.pre, kq.geo, slots, nq,
                                                    w->la, w->lD, w->ln, w->lvl, w->lrl, lam, lamn, kq.por.dn,
                                                    kq.por.pgi, kq.por.pgv, w->part, pstride);
            BSC_LAUNCH(c);
            k_wc_grad<<<2 + G, WB, 0, c->stream>>>(nb, pstride, w->part, w->grad);
            BSC_LAUNCH(c);
            std::swap(w->lam, w->lamn);
        }
    }
    // the segment buffers now hold the first segment
    if (nseg > 1) w->last_kept = false;
    BSC_CUDA(c, cudaMemcpyAsync(grad, w->grad, sizeof(double) * (2 + G), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    return BSC_OK;
}

}  // extern "C"
