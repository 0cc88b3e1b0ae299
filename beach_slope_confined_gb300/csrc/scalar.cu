// scalar.cu -- salinity transport (scalar.f90): the dispersion flux of
// scalart, the sub-step update of scalarupdate and the density of
// densityupdate.  FP64 in both precisions.
//
// scalart follows scalar.f90:114-240 term by term:
//   D_x = Dm + (al vx^2 + at vy^2 + (al - at) vx vy) / (|v| n), then D_x = Dm
//   unless D_x > 0 (a NaN from |v| = 0 included) and D_x <= 0.12 dl^2/dt;
//   D_y likewise with al and at exchanged;
//   for fluid neighbours j: the harmonic mean of D_i and D_j per axis, or,
//   where either porosity is >= 0.8, the Schmidt-scaled eddy diffusivity
//   (arithmetic mean when both nu_t < 1e-6, harmonic otherwise);
//   cdiff_i = sum_j ovol_i (n_i + n_j) / (n_i n_j) (c_i - c_j)
//             [t1x (x_i - x_j) dW/dx + t1y (y_i - y_j) dW/dy] / (r^2 + lam)
// with the kernel gradient evaluated, as hWabx/hWaby do, at the distance
// stored by the neighbour search and the current positions (the particles
// have moved by opt2_shift since the search).  The neighbour search keeps
// the distance per list slot when params.salinity is set.
#include <cmath>

#include "bsc_internal.cuh"
#include "sph_kernel.cuh"

struct bsc_ctx : bsc::Ctx {};  // the same definition as in api.cu

namespace bsc {
namespace {

// the reference's single-precision literals, promoted to FP64
constexpr double SC_NUT_MIN = (double)1e-6f;  // scalar.f90 `nut < 1e-6`
constexpr double SC_TOR = 1.0;                // scalar.f90 `tor`

struct ScalarK {
    double Dm, al, at, tsc, cap;  // molecular diffusivity, dispersivities, Schmidt number, D cap
};

// directional dispersion coefficient of one particle (scalar.f90:135-154)
__device__ __forceinline__ double disp(double Dm, double a1, double a2, double amx, double vx, double vy, double v,
                                       double n, double cap) {
    double D = Dm + ((a1 * (vx * vx)) + (a2 * (vy * vy)) + (amx * vx * vy)) / (v * n);
    if (!(D > 0.0)) D = Dm;
    if (!(D <= cap)) D = cap;
    return D;
}

// per particle: D_x, D_y and the eddy term Dm + nu_t / Sc, the same values
// scalart forms for a particle as i and as j (one division and root each,
// instead of per pair)
__global__ void k_scalar_pre(int64_t n, State S, ScalarK C, double* __restrict__ Dx, double* __restrict__ Dy,
                             double* __restrict__ E, double* __restrict__ inv_n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double vx = S.vx[i], vy = S.vy[i], v = sqrt(vx * vx + vy * vy), ni = S.por[i];
    const double amx = C.al - C.at;
    Dx[i] = disp(C.Dm, C.al, C.at, amx, vx, vy, v, ni, C.cap);
    Dy[i] = disp(C.Dm, C.at, C.al, amx, vx, vy, v, ni, C.cap);
    E[i] = C.Dm + S.nut[i] / C.tsc;
    inv_n[i] = 1.0 / ni;
}

__global__ void k_scalart(int64_t n, State S, KParams K, ScalarK C, const int32_t* __restrict__ nbr,
                          const double* __restrict__ ndist, const int32_t* __restrict__ cnt,
                          const double* __restrict__ Dx, const double* __restrict__ Dy,
                          const double* __restrict__ E, const double* __restrict__ inv_n) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (S.tid[i] != BSC_TID_FLUID || (S.flags[i] & BSC_FLAG_DEAD)) return;
    const double con1 = S.con[i], ni = S.por[i], nuti = S.nut[i], oi = S.ovol[i];
    const double Dxi = Dx[i], Dyi = Dy[i], Ei = E[i], ini = inv_n[i];
    const double xi = S.x[i], yi = S.y[i];
    double cd = 0.0;
    const int m = cnt[i];
    for (int k = 0; k < m; ++k) {
        const int64_t e = ell(i, k, K.kmax);
        const int j = nbr[e];
        if (S.tid[j] != BSC_TID_FLUID || (S.flags[j] & BSC_FLAG_DEAD)) continue;
        const double con2 = S.con[j], nj = S.por[j];
        double t1x, t1y;
        if (ni >= 0.8 || nj >= 0.8) {
            const double nutj = S.nut[j];
            if (nuti < SC_NUT_MIN && nutj < SC_NUT_MIN) {
                t1x = C.Dm + (nuti + nutj) * 0.50 / C.tsc;
            } else {
                const double Ej = E[j];
                t1x = 2 * ((Ei * Ej) / (Ei + Ej));
            }
            t1y = t1x;
        } else {
            const double Dxj = Dx[j], Dyj = Dy[j];
            t1x = 2.0 * SC_TOR * Dxi * Dxj / (Dxi + Dxj);
            t1y = 2.0 * SC_TOR * Dyi * Dyj / (Dyi + Dyj);
        }
        // t3 = ovol_i (n_i + n_j) / (n_i n_j), written with the reciprocals
        const double t3 = oi * (ini + inv_n[j]);
        const double r = ndist[e];
        const double dx = xi - S.x[j], dy = yi - S.y[j];
        const double F = grad_factor<double>(K, r);  // dW/dx = F (x_i - x_j) at the stored distance
        const double q = t3 * (con1 - con2) * F / (r * r + K.lam);
        cd += q * (t1x * (dx * dx) + t1y * (dy * dy));
    }
    S.cdiff[i] = cd;
}

// scalar.f90:242-275
__global__ void k_scalarupdate(int64_t n, State S, double stime, double bcon, double bxmax) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (S.tid[i] != BSC_TID_FLUID || (S.flags[i] & BSC_FLAG_DEAD)) return;
    S.con[i] = S.con[i] + S.cdiff[i] * stime;
    if ((S.flags[i] & BSC_FLAG_BUFFER) && S.x[i] < bxmax) S.con[i] = bcon;
}

// scalar.f90:277-305: density of the mixture, mass from the original volume
__global__ void k_densityupdate(int64_t n, State S, double rhomin, double rhomax) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (S.tid[i] != BSC_TID_FLUID || (S.flags[i] & BSC_FLAG_DEAD)) return;
    const double od = 0.5 * (rhomax + rhomin) + S.con[i] * (rhomax - rhomin);
    S.oden[i] = od;
    S.mass[i] = od * S.ovol[i];
    S.rho[i] = od * S.por[i];
    S.vol[i] = S.mass[i] / S.rho[i];
}

}  // namespace

int op_scalart(Ctx* c) {
    if (!c->ndist) return set_err(c, BSC_E_INVALID, "scalart needs params.salinity = 1");
    if (!c->have_lists) return set_err(c, BSC_E_INVALID, "scalart before neighbour");
    const bsc_params& P = c->P;
    const ScalarK C{P.diffusivity, P.disp_long, P.disp_trans, P.tschmidt, 0.12 * (P.dl * P.dl) / c->dt};
    double *Dx = c->sdisp, *Dy = c->sdisp + c->n, *E = c->sdisp + 2 * c->n, *inv_n = c->sdisp + 3 * c->n;
    k_scalar_pre<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, C, Dx, Dy, E, inv_n);
    BSC_LAUNCH(c);
    k_scalart<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, c->K, C, c->nbr, c->ndist, c->cnt, Dx, Dy,
                                                             E, inv_n);
    BSC_LAUNCH(c);
    return BSC_OK;
}

int op_scalarupdate(Ctx* c, double stime) {
    k_scalarupdate<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, stime, c->P.buffer_con,
                                                                  c->P.buffer_con_xmax);
    BSC_LAUNCH(c);
    return BSC_OK;
}

// rhomin = rho0 (initialize.f90:22), rhomax = rho0 rel_den (setup.f90:19)
int op_densityupdate(Ctx* c) {
    k_densityupdate<<<blocks_for(c->n, 256), 256, 0, c->stream>>>(c->n, c->S, c->P.rho0, c->P.rho0 * c->P.rel_den);
    BSC_LAUNCH(c);
    return BSC_OK;
}

}  // namespace bsc

using namespace bsc;

extern "C" {

int bsc_scalart(bsc_ctx* c) {
    if (!c) return BSC_E_INVALID;
    if (!c->have_state) return set_err(c, BSC_E_INVALID, "scalart before upload_state");
    return op_scalart(c);
}

int bsc_scalarupdate(bsc_ctx* c, double stime) {
    if (!c) return BSC_E_INVALID;
    if (!c->have_state) return set_err(c, BSC_E_INVALID, "scalarupdate before upload_state");
    return op_scalarupdate(c, stime);
}

int bsc_densityupdate(bsc_ctx* c) {
    if (!c) return BSC_E_INVALID;
    if (!c->have_state) return set_err(c, BSC_E_INVALID, "densityupdate before upload_state");
    return op_densityupdate(c);
}

}  // extern "C"
