// oracle.cpp -- CPU restatement of the reference ISPH step (TEST INFRASTRUCTURE).
//
// This file is the checker, never the product: only the tests, the smoke
// check and the CPU-baseline leg of the benchmark load it.  It restates, in
// FP64 C++ with no floating-point contraction (-ffp-contract=off), the hot
// path of Sinchanrc/Beach_Slope_Confined: the routines called by main.f90:44-65.
// Each routine cites the reference file:line it follows, and keeps the
// reference's loop structure and the order of its floating-point operations:
//   * the 4*h1 cell grid of setup.f90:51-52,120-123 with the 2x2 quadrant
//     block of search.f90:328-388 (and porous.f90:133-178);
//   * resetid numbering (isph.f90:88-113) and the column-sorted PPE rows with
//     the diagonal slotted in by matid (isph.f90:147-176,425-442);
//   * every pair sum in the reference's visiting order.
//
// Parity status.  The reference cannot be compiled here (Fortran, closed MKL),
// and it ships no golden vectors for these routines.  The linear solvers are
// pinned by the reference's only known-answer test (solvertest.f90:10-19, exact
// solution 1..5); the SPH operators are pinned by analytic invariants of the
// reference's formulae (tests/test_oracle.py).  Against reference outputs the
// SPH operators are parity unpinned.
//
// Deliberate departures from the reference, all guarded situations where the
// reference reads undefined or stale data:
//   * ghost (tid 2) rows: the reference leaves the initial val(1)=1 at column
//     `pos` when the row's lowest-matid neighbour is a fluid particle
//     (isph.f90:125-128 with the tid-2 branch :274-296 writing only wall
//     entries); that slot-numbering artefact is not reproduced -- unwritten
//     entries are 0.
//   * a row whose diagonal sum is 0 (no neighbours) divides by zero in the
//     reference (isph.f90:434-441); here it becomes an identity row, b = 0.
//   * opt2_shift with delta = 0 gives 0/0 (part_shift.f90:90-91); here 0.
//   * opt2_shift applies a shift only to particles that computed one this
//     call; the reference adds stale xs (the pre-projection x) for a particle
//     with no neighbours (part_shift.f90:40,180).
//   * the PPE warm start is the particle's own previous pressure; the
//     reference reuses fsol indexed by the previous step's matid numbering.
//   * self-exclusion uses the particle index; the reference's (tid, matid)
//     test (search.f90:53-55) is the same thing because matids are unique.
#include "../include/bsc.h"

#include <omp.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

// Default-real (single precision) literals of the reference, promoted to FP64.
const double F_1EM5 = (double)1e-5f;   // functions.f90:75
const double F_1EM6 = (double)1e-6f;   // integrator.f90:497,582,625
const double C28_314 = (double)(28.0f * 3.14f);  // kernel.f90:52: 28.0*3.14
const double C3_314 = (double)(3.0f * 3.14f);    // kernel.f90:53: 3.0*3.14
const double ALP = 0.1;                          // kernel.f90:14

// state of the WCSPH calibration workload (orc_wcsph_*)
struct WcOrc {
    bool on = false;
    double rho0 = 0, B = 0, gam = 0, grav_c = 0, ys = 0, c2 = 0, nu = 0, alpha = 0, beta = 0;
    double gx0 = 0, gy0 = 0, gdx = 1, gdy = 1, R1 = 0, depth = 0, t0 = 0;
    int gnx = 0, gny = 0, np = 0;
    double xp[BSC_WCSPH_MAX_PROBES] = {};
    std::vector<double> theta, sw, mass, init;  // grid porosities, (1-phi) V_s, masses, x y vx vy rho
    std::vector<int> sg;                        // solid -> grid cell or -1
    // forward record: every state, list, porosity and pressure sum
    int nsteps = 0;
    std::vector<std::vector<double>> st, nn, PP;
    std::vector<std::vector<int64_t>> off, ids;
};

struct Orc {
    bsc_params P{};
    double t = 0.0, dt = 0.0, umax = 0.0, numax = 0.0, dtsol = 0.0;
    int solsteps = 1;
    int64_t n = 0;
    // particle records (plist, particle.f90:31-47)
    std::vector<double> x, y, vx, vy, xs, ys, vxs, vys, p, rho, oden, mass, xrest;
    std::vector<double> con, ovol, cdiff;  // salinity (plist%con, %ovol; pplist%cdiff)
    std::vector<int8_t> tid;
    std::vector<uint8_t> flags;
    std::vector<int64_t> matid;
    // derived properties (pplist, particle.f90:60-69)
    std::vector<double> por, gradvx, nut, tke, resist, varts, vel, coff;
    // cell grid (setup.f90:51-52,120-123): cells (i,j), i=1..celly, j=1..cellx
    double cw = 0, gx0 = 0, gy0 = 0;
    int cellx = 0, celly = 0;
    std::vector<int64_t> cell_off;   // CSR over cells, index (j-1)*celly+(i-1)
    std::vector<int64_t> cell_mem;
    std::vector<int> pci, pcj;       // cell of each particle
    // neighbour lists (verlet, interactions.f90:26-35)
    std::vector<int64_t> nb_off;
    std::vector<int64_t> nb_id;
    std::vector<double> nb_dist, nb_kx, nb_ky;
    bool have_lists = false;
    // porous solids (porlist) and their cells
    int64_t ns = 0;
    std::vector<double> sx, sy, sm, srho, spor;
    std::vector<int64_t> scell_off, scell_mem;
    // porosity field
    int pnx = 0, pny = 0;
    double px0 = 0, py0 = 0, pdx = 1, pdy = 1;
    std::vector<double> pgrid;
    // PPE (isph.f90:115-485), rows in matid order
    std::vector<int64_t> rowptr;
    std::vector<int64_t> col;
    std::vector<double> val, rhs, sol;
    bool have_csr = false;
    WcOrc wc;
    std::string err;
};

int fail(Orc* o, int code, const std::string& msg) {
    if (o) o->err = msg;
    return code;
}

inline bool has(uint8_t f, unsigned bit) { return (f & bit) != 0; }

// ---------------------------------------------------------------------------
// kernel.f90:34-162 (hybrid) and the Wendland C2 forms of kernel.f90:42-43,
// 102-103.  p1 = neighbour j, p2 = particle i: the result is grad_i W.
// ---------------------------------------------------------------------------
double Wab(const Orc* o, double r, double h) {
    if (o->P.kernel == BSC_KERNEL_WENDLAND_C2) {
        double a = 1.0 - (r / (2 * h));
        double a2 = a * a;
        return (7.0 / (4 * 3.140 * (h * h))) * (1 + (2 * r / h)) * (a2 * a2);
    }
    double t1, t2;
    if (r < h) {
        t1 = (4.0 - (6.0 * (r * r) / (h * h)) + (3.0 * (r * r * r) / (h * h * h)));
        double b = r / h;
        t2 = (b * b * b - (6.0 * r / h) + 6.0);
    } else {
        double a = 2.0 - r / h;
        t1 = a * a * a;
        t2 = a * a * a;
    }
    return ALP * t1 * (10.0 / (C28_314 * (h * h))) + (1.0 - ALP) * t2 * (1.0 / (C3_314 * (h * h)));
}

double Wo(const Orc* o, double h) {
    if (o->P.kernel == BSC_KERNEL_WENDLAND_C2) return (7.0 / (4 * 3.140 * (h * h)));
    double t1 = 4.0, t2 = 6.0;
    return ALP * t1 * (10.0 / (C28_314 * (h * h))) + (1.0 - ALP) * t2 * (1.0 / (C3_314 * (h * h)));
}

// Wabx/Waby with p1 = (xj,yj), p2 = (xi,yi); `di` = p2 - p1 component, i.e.
// (xi - xj) for Wabx.
double Wab_grad(const Orc* o, double di, double r, double h) {
    if (o->P.kernel == BSC_KERNEL_WENDLAND_C2) {
        double a = 1.0 - r / (2 * h);
        double dj = -di;  // p1 - p2 = xj - xi
        return (35.0 * dj * (a * a * a)) / (4.0 * 3.140 * ((h * h) * (h * h)));
    }
    double t1, t2;
    if (r < h) {
        t1 = ((9.0 * r / (h * h * h)) - (12.0 / (h * h))) * di;
        t2 = ((3.0 * r / (h * h * h)) - 6.0 / (r * h)) * di;
    } else {
        double a = 2.0 - r / h;
        t1 = ((3.0 / (r * h)) * (a * a)) * (-di);
        t2 = ((3.0 / (r * h)) * (a * a)) * (-di);
    }
    return ALP * t1 * (10.0 / (C28_314 * (h * h))) + (1.0 - ALP) * t2 * (1.0 / (C3_314 * (h * h)));
}

// functions.f90:28-42 dist(p1,p2), p1 = particle i
inline double dist(double xi, double yi, double xj, double yj) {
    double ddx = xi - xj, ddy = yi - yj;
    return std::sqrt((ddx * ddx) + (ddy * ddy));
}

// functions.f90:62-96 invertmat2D
void invertmat2D(double a[4]) {
    double det = a[0] * a[3] - a[1] * a[2];
    if ((std::fabs(det) >= F_1EM5) && !std::isnan(det) && std::isfinite(det)) {
        double r0 = a[3] / det, r1 = -a[1] / det, r2 = -a[2] / det, r3 = a[0] / det;
        a[0] = r0; a[1] = r1; a[2] = r2; a[3] = r3;
    } else {
        a[0] = 1.0; a[1] = 0.0; a[2] = 0.0; a[3] = 1.0;
    }
}

// porous.f90:12-30 and integrator.f90:12-30 vis(oden)
inline double vis(double oden) {
    double Sp = oden - 1000.0;
    return (1.002 + 0.001652 * Sp + 0.0000083 * (Sp * Sp)) * 0.001;
}

double porosity_at(const Orc* o, double px, double py) {
    if (o->pnx <= 0) return o->P.por;
    double fx = std::floor((px - o->px0) / o->pdx), fy = std::floor((py - o->py0) / o->pdy);
    if (!(fx >= 0 && fx < o->pnx && fy >= 0 && fy < o->pny)) return o->P.por;
    return o->pgrid[(int64_t)fy * o->pnx + (int64_t)fx];
}

// ---------------------------------------------------------------------------
// Cell grid: xleft=(j-2)*4h1, ybot=(celly-1-i)*4h1 (setup.f90:120-123),
// shifted by the grid origin so the tank's negative coordinates fit.
// ---------------------------------------------------------------------------
inline double xleft(const Orc* o, int j) { return o->gx0 + (j - 2) * o->cw; }
inline double xright(const Orc* o, int j) { return o->gx0 + (j - 1) * o->cw; }
inline double ybot(const Orc* o, int i) { return o->gy0 + (o->celly - 1 - i) * o->cw; }
inline double ytop(const Orc* o, int i) { return o->gy0 + (o->celly - i) * o->cw; }
inline int64_t cidx(const Orc* o, int i, int j) { return (int64_t)(j - 1) * o->celly + (i - 1); }

void locate(const Orc* o, double px, double py, int* ci, int* cj) {
    // the cell whose [xleft,xright) x [ybot,ytop) holds the point, clamped to
    // the interior range sx..ex, sy..ey (setup.f90:83-86)
    int j = 2, i = o->celly - 1;
    if (std::isfinite(px)) {
        double fj = std::floor((px - o->gx0) / o->cw);
        fj = std::min(std::max(fj, -1.0), (double)o->cellx);
        j = (int)fj + 2;
        while (j > 2 && px < xleft(o, j)) --j;
        while (j < o->cellx - 1 && px >= xright(o, j)) ++j;
    }
    if (std::isfinite(py)) {
        double fk = std::floor((py - o->gy0) / o->cw);
        fk = std::min(std::max(fk, -1.0), (double)o->celly);
        i = o->celly - 1 - (int)fk;
        while (i < o->celly - 1 && py < ybot(o, i)) ++i;
        while (i > 2 && py >= ytop(o, i)) --i;
    }
    j = std::min(std::max(j, 2), o->cellx - 1);
    i = std::min(std::max(i, 2), o->celly - 1);
    *ci = i;
    *cj = j;
}

// 2x2 quadrant block of search.f90:328-388: four cells in the order the
// reference visits them (ascending resetid numbering).
void quad_cells(const Orc* o, double px, double py, int i, int j, int ci[4], int cj[4]) {
    double midx = xleft(o, j) + std::fabs((xleft(o, j) - xright(o, j)) / 2);
    double midy = ybot(o, i) + std::fabs((ytop(o, i) - ybot(o, i)) / 2);
    if (px <= midx && py <= midy) {
        ci[0] = i; cj[0] = j - 1; ci[1] = i + 1; cj[1] = j - 1;
        ci[2] = i; cj[2] = j;     ci[3] = i + 1; cj[3] = j;
    } else if (px > midx && py <= midy) {
        ci[0] = i; cj[0] = j;     ci[1] = i + 1; cj[1] = j;
        ci[2] = i; cj[2] = j + 1; ci[3] = i + 1; cj[3] = j + 1;
    } else if (px > midx && py > midy) {
        ci[0] = i - 1; cj[0] = j;     ci[1] = i; cj[1] = j;
        ci[2] = i - 1; cj[2] = j + 1; ci[3] = i; cj[3] = j + 1;
    } else {
        ci[0] = i - 1; cj[0] = j - 1; ci[1] = i; cj[1] = j - 1;
        ci[2] = i - 1; cj[2] = j;     ci[3] = i; cj[3] = j;
    }
}

// bin every particle into its cell; members kept in ascending index order
void bin_particles(Orc* o) {
    const int64_t nc = (int64_t)o->cellx * o->celly;
    o->pci.assign(o->n, 0);
    o->pcj.assign(o->n, 0);
    std::vector<int64_t> cnt(nc + 1, 0);
    for (int64_t k = 0; k < o->n; ++k) {
        locate(o, o->x[k], o->y[k], &o->pci[k], &o->pcj[k]);
        cnt[cidx(o, o->pci[k], o->pcj[k]) + 1]++;
    }
    for (int64_t c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
    o->cell_off = cnt;
    o->cell_mem.assign(o->n, 0);
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int64_t k = 0; k < o->n; ++k) o->cell_mem[fill[cidx(o, o->pci[k], o->pcj[k])]++] = k;
}

void bin_solids(Orc* o) {
    const int64_t nc = (int64_t)o->cellx * o->celly;
    std::vector<int64_t> cnt(nc + 1, 0);
    std::vector<int64_t> sc(o->ns);
    for (int64_t k = 0; k < o->ns; ++k) {
        int i, j;
        locate(o, o->sx[k], o->sy[k], &i, &j);
        sc[k] = cidx(o, i, j);
        cnt[sc[k] + 1]++;
    }
    for (int64_t c = 0; c < nc; ++c) cnt[c + 1] += cnt[c];
    o->scell_off = cnt;
    o->scell_mem.assign(o->ns, 0);
    std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
    for (int64_t k = 0; k < o->ns; ++k) o->scell_mem[fill[sc[k]]++] = k;
}

// ---------------------------------------------------------------------------
// Deterministic reductions for the solvers: fixed 4096-element chunks summed
// in order, independent of the thread count.
// ---------------------------------------------------------------------------
double dot(const std::vector<double>& a, const std::vector<double>& b) {
    const int64_t n = (int64_t)a.size(), CH = 4096, nch = (n + CH - 1) / CH;
    std::vector<double> part(nch, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < nch; ++c) {
        double s = 0.0;
        for (int64_t k = c * CH; k < std::min(n, (c + 1) * CH); ++k) s = s + a[k] * b[k];
        part[c] = s;
    }
    double s = 0.0;
    for (int64_t c = 0; c < nch; ++c) s += part[c];
    return s;
}

void spmv(const std::vector<int64_t>& rp, const std::vector<int64_t>& cl, const std::vector<double>& vl,
          const std::vector<double>& in, std::vector<double>& out) {
    const int64_t n = (int64_t)rp.size() - 1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {  // solver.f90:99-111 spmv2
        double s = 0.0;
        for (int64_t k = rp[i]; k < rp[i + 1]; ++k) s = s + vl[k] * in[cl[k]];
        out[i] = s;
    }
}

bool tol_met(const bsc_params& P, double rn, double bn, double r0n) {
    double ref = (P.tol_mode == BSC_TOL_REL_R0) ? r0n : bn;
    return rn <= P.tol * ref;
}

// BiCGSTAB in the update order of solver.f90:163-213 (van der Vorst 1992),
// stopping on the recursively updated residual ||r|| <= tol * ||b|| (or
// ||r0||) instead of the reference's solution-change test (solver.f90:233-242).
int bicgstab(const bsc_params& P, const std::vector<int64_t>& rp, const std::vector<int64_t>& cl,
             const std::vector<double>& vl, const std::vector<double>& b, std::vector<double>& x,
             bsc_solve_info* info) {
    const int64_t n = (int64_t)b.size();
    std::vector<double> res(n), rs(n), p(n), mm1(n), mm2(n), si(n);
    spmv(rp, cl, vl, x, res);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) { rs[k] = b[k] - res[k]; p[k] = rs[k]; res[k] = rs[k]; }
    const double bn = std::sqrt(dot(b, b));
    const double r0n = std::sqrt(dot(rs, rs));
    info->b_norm = bn;
    info->r0_norm = r0n;
    int it = 0, status = BSC_OK, conv = tol_met(P, r0n, bn, r0n) ? 1 : 0, restarts = 0;
    while (!conv && it < P.maxit) {
        if (status == BSC_E_BREAKDOWN) {
            // rho or omega vanished: restart from x with a fresh shadow residual
            if (restarts == 8) break;
            ++restarts;
            status = BSC_OK;
            spmv(rp, cl, vl, x, mm1);
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < n; ++k) { rs[k] = b[k] - mm1[k]; p[k] = rs[k]; res[k] = rs[k]; }
            if (tol_met(P, std::sqrt(dot(rs, rs)), bn, r0n)) { conv = 1; break; }
        }
        ++it;
        spmv(rp, cl, vl, p, mm1);
        double prevr = dot(res, rs);
        double den = dot(mm1, res);
        if (prevr == 0.0 || den == 0.0) { status = BSC_E_BREAKDOWN; --it; continue; }
        double alpha = prevr / den;
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n; ++k) si[k] = rs[k] - alpha * mm1[k];
        spmv(rp, cl, vl, si, mm2);
        double tt = dot(mm2, mm2);
        double wi = (tt == 0.0) ? 0.0 : dot(mm2, si) / tt;
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n; ++k) {
            x[k] = x[k] + alpha * p[k] + wi * si[k];
            rs[k] = si[k] - wi * mm2[k];
        }
        double rn = std::sqrt(dot(rs, rs));
        if (tol_met(P, rn, bn, r0n)) { conv = 1; break; }
        if (wi == 0.0) { status = BSC_E_BREAKDOWN; continue; }
        double betas = (dot(rs, res) / prevr) * (alpha / wi);
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n; ++k) p[k] = rs[k] + betas * (p[k] - wi * mm1[k]);
    }
    spmv(rp, cl, vl, x, mm1);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) mm1[k] = b[k] - mm1[k];
    double tr = std::sqrt(dot(mm1, mm1));
    info->iterations = it;
    info->outer = 1;
    info->converged = conv;
    info->rel_residual = bn > 0 ? tr / bn : tr;
    if (!conv && status == BSC_OK) status = BSC_E_NOT_CONVERGED;
    info->status = status;
    return status;
}

// Restarted FGMRES(m) (Saad 1993) with modified Gram-Schmidt and Givens
// rotations, identity preconditioner: the public algorithm behind the MKL
// dfgmres call of solver.f90:319-343 (ipar(12)=1: stop on a zero Arnoldi
// vector).
int fgmres(const bsc_params& P, const std::vector<int64_t>& rp, const std::vector<int64_t>& cl,
           const std::vector<double>& vl, const std::vector<double>& b, std::vector<double>& x,
           bsc_solve_info* info) {
    const int64_t n = (int64_t)b.size();
    const int m = std::max(1, std::min<int>(P.restart, (int)std::max<int64_t>(n, 1)));
    std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
    std::vector<double> w(n), r(n);
    std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1);
    spmv(rp, cl, vl, x, r);
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < n; ++k) r[k] = b[k] - r[k];
    const double bn = std::sqrt(dot(b, b));
    double beta = std::sqrt(dot(r, r));
    const double r0n = beta;
    info->b_norm = bn;
    info->r0_norm = r0n;
    const double target = P.tol * ((P.tol_mode == BSC_TOL_REL_R0) ? r0n : bn);
    int it = 0, conv = (beta <= target) ? 1 : 0, status = BSC_OK;
    while (!conv && it < P.maxit && status == BSC_OK) {
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n; ++k) V[0][k] = r[k] / beta;
        std::fill(g.begin(), g.end(), 0.0);
        g[0] = beta;
        int j = 0;
        for (; j < m && it < P.maxit; ++j) {
            ++it;
            spmv(rp, cl, vl, V[j], w);
            for (int i = 0; i <= j; ++i) {
                double hij = dot(w, V[i]);
                H[(size_t)i * m + j] = hij;
#pragma omp parallel for schedule(static)
                for (int64_t k = 0; k < n; ++k) w[k] = w[k] - hij * V[i][k];
            }
            double hn = std::sqrt(dot(w, w));
            H[(size_t)(j + 1) * m + j] = hn;
            if (hn != 0.0) {
#pragma omp parallel for schedule(static)
                for (int64_t k = 0; k < n; ++k) V[j + 1][k] = w[k] / hn;
            }
            for (int i = 0; i < j; ++i) {
                double a = H[(size_t)i * m + j], c = H[(size_t)(i + 1) * m + j];
                H[(size_t)i * m + j] = cs[i] * a + sn[i] * c;
                H[(size_t)(i + 1) * m + j] = -sn[i] * a + cs[i] * c;
            }
            double a = H[(size_t)j * m + j], c = H[(size_t)(j + 1) * m + j];
            double den = std::sqrt(a * a + c * c);
            if (den == 0.0) { status = BSC_E_BREAKDOWN; ++j; break; }
            cs[j] = a / den;
            sn[j] = c / den;
            H[(size_t)j * m + j] = den;
            H[(size_t)(j + 1) * m + j] = 0.0;
            g[j + 1] = -sn[j] * g[j];
            g[j] = cs[j] * g[j];
            if (std::fabs(g[j + 1]) <= target || hn == 0.0) { ++j; break; }
        }
        // back substitution H(0:j,0:j) y = g, then x += V y
        std::vector<double> yv(j, 0.0);
        for (int i = j - 1; i >= 0; --i) {
            double s = g[i];
            for (int k = i + 1; k < j; ++k) s -= H[(size_t)i * m + k] * yv[k];
            yv[i] = s / H[(size_t)i * m + i];
        }
        for (int i = 0; i < j; ++i) {
#pragma omp parallel for schedule(static)
            for (int64_t k = 0; k < n; ++k) x[k] = x[k] + yv[i] * V[i][k];
        }
        spmv(rp, cl, vl, x, r);
#pragma omp parallel for schedule(static)
        for (int64_t k = 0; k < n; ++k) r[k] = b[k] - r[k];
        beta = std::sqrt(dot(r, r));
        if (beta <= target) conv = 1;
        if (status == BSC_E_BREAKDOWN && !conv) break;
        status = BSC_OK;
    }
    info->iterations = it;
    info->outer = 1;
    info->converged = conv;
    info->rel_residual = bn > 0 ? beta / bn : beta;
    if (!conv && status == BSC_OK) status = BSC_E_NOT_CONVERGED;
    info->status = conv ? BSC_OK : status;
    return info->status;
}

// x_p(t) = s0 + r(t) (s(t) - s0), s0 = s(0): the ramp takes the stroke from
// its starting value
double piston_x(const bsc_params& P, double tt, double* vel) {
    double s = 0, ds = 0, s0 = 0;
    for (int k = 0; k < P.piston_modes && k < BSC_MAX_PISTON_MODES; ++k) {
        double w = 2.0 * M_PI / P.piston_period[k];
        s += P.piston_amp[k] * std::sin(w * tt + P.piston_phase[k]);
        ds += P.piston_amp[k] * w * std::cos(w * tt + P.piston_phase[k]);
        s0 += P.piston_amp[k] * std::sin(P.piston_phase[k]);
    }
    double r = 1.0, dr = 0.0;
    if (P.piston_ramp > 0.0 && tt < P.piston_ramp) {
        r = 0.5 * (1.0 - std::cos(M_PI * tt / P.piston_ramp));
        dr = 0.5 * M_PI / P.piston_ramp * std::sin(M_PI * tt / P.piston_ramp);
    }
    if (vel) *vel = dr * (s - s0) + r * ds;
    return s0 + r * (s - s0);
}

}  // namespace

struct orc_ctx : Orc {};

extern "C" {

const char* orc_last_error(const orc_ctx* o) { return o ? o->err.c_str() : "null context"; }

int orc_create(const bsc_params* p, orc_ctx** out) {
    if (!p || !out) return BSC_E_INVALID;
    orc_ctx* o = new orc_ctx();
    o->P = *p;
    o->dt = p->dt;
    *out = o;
    return BSC_OK;
}

int orc_destroy(orc_ctx* o) {
    delete o;
    return BSC_OK;
}

int orc_set_time(orc_ctx* o, double t, double dt) {
    o->t = t;
    o->dt = dt;
    return BSC_OK;
}

int orc_get_time(const orc_ctx* o, double* t, double* dt) {
    if (t) *t = o->t;
    if (dt) *dt = o->dt;
    return BSC_OK;
}

int orc_upload_state(orc_ctx* o, const bsc_state_view* s) {
    if (!s || s->n <= 0 || !s->x || !s->y || !s->vx || !s->vy || !s->p || !s->rho || !s->oden ||
        !s->mass || !s->tid || !s->flags)
        return fail(o, BSC_E_INVALID, "upload_state: missing required field");
    const int64_t n = s->n;
    o->n = n;
    auto cp = [n](std::vector<double>& v, const double* src, double dflt) {
        v.assign(n, dflt);
        if (src) std::memcpy(v.data(), src, sizeof(double) * n);
    };
    cp(o->x, s->x, 0); cp(o->y, s->y, 0); cp(o->vx, s->vx, 0); cp(o->vy, s->vy, 0);
    cp(o->xs, s->xs, 0); cp(o->ys, s->ys, 0); cp(o->vxs, s->vxs, 0); cp(o->vys, s->vys, 0);
    cp(o->p, s->p, 0); cp(o->rho, s->rho, 0); cp(o->oden, s->oden, 0); cp(o->mass, s->mass, 0);
    cp(o->por, s->porosity, 1.0); cp(o->gradvx, s->gradvx, 0); cp(o->nut, s->nut, 0);
    cp(o->tke, s->tke, 0); cp(o->resist, s->resist, 0); cp(o->varts, s->varts, 0);
    cp(o->vel, s->vel, 0);
    cp(o->xrest, s->xrest ? s->xrest : s->x, 0);
    cp(o->con, s->con, 0);
    o->ovol.assign(n, 0.0);
    for (int64_t k = 0; k < n; ++k) o->ovol[k] = s->ovol ? s->ovol[k] : o->mass[k] / o->oden[k];  // internal.f90:103
    o->cdiff.assign(n, 0.0);
    o->coff.assign(4 * n, 0.0);
    if (s->L) std::memcpy(o->coff.data(), s->L, sizeof(double) * 4 * n);
    else for (int64_t k = 0; k < n; ++k) { o->coff[4 * k] = 1.0; o->coff[4 * k + 3] = 1.0; }
    o->tid.assign(s->tid, s->tid + n);
    o->flags.assign(s->flags, s->flags + n);
    o->matid.resize(n);
    for (int64_t k = 0; k < n; ++k) o->matid[k] = k;
    // grid (setup.f90:51-52 cellx/celly with the +4/+3 halo; origin = bounds)
    double xmin = o->P.xmin, xmax = o->P.xmax, ymin = o->P.ymin, ymax = o->P.ymax;
    if (!(xmax > xmin && ymax > ymin)) {
        xmin = *std::min_element(o->x.begin(), o->x.end()) - 4 * o->P.h;
        xmax = *std::max_element(o->x.begin(), o->x.end()) + 4 * o->P.h;
        ymin = *std::min_element(o->y.begin(), o->y.end()) - 4 * o->P.h;
        ymax = *std::max_element(o->y.begin(), o->y.end()) + 4 * o->P.h;
    }
    o->cw = 4 * o->P.h;  // incr*h1
    o->gx0 = xmin;
    o->gy0 = ymin;
    o->cellx = (int)std::ceil((xmax - xmin) / o->cw) + 4;
    o->celly = (int)std::ceil((ymax - ymin) / o->cw) + 3;
    o->sol = o->p;  // matrixid: fsol = fguess = pressure (memory.f90:117-144)
    o->have_lists = o->have_csr = false;
    bin_particles(o);
    if (o->ns > 0) bin_solids(o);
    return BSC_OK;
}

int orc_upload_porosity(orc_ctx* o, int32_t nx, int32_t ny, double x0, double y0, double dx, double dy,
                        const double* v) {
    if (nx <= 0 || ny <= 0 || !v || !(dx > 0) || !(dy > 0)) return fail(o, BSC_E_INVALID, "upload_porosity");
    o->pnx = nx; o->pny = ny; o->px0 = x0; o->py0 = y0; o->pdx = dx; o->pdy = dy;
    o->pgrid.assign(v, v + (int64_t)nx * ny);
    return BSC_OK;
}

int orc_upload_solids(orc_ctx* o, int64_t ns, const double* x, const double* y, const double* m,
                      const double* r, const double* por) {
    if (ns < 0 || (ns > 0 && (!x || !y || !m || !r))) return fail(o, BSC_E_INVALID, "upload_solids");
    o->ns = ns;
    o->sx.assign(x, x + ns); o->sy.assign(y, y + ns);
    o->sm.assign(m, m + ns); o->srho.assign(r, r + ns);
    o->spor.resize(ns);
    for (int64_t k = 0; k < ns; ++k) o->spor[k] = por ? por[k] : porosity_at(o, x[k], y[k]);
    if (o->cellx > 0 && ns > 0) bin_solids(o);
    return BSC_OK;
}

int orc_download_state(orc_ctx* o, bsc_state_view* s) {
    if (!s || s->n != o->n) return fail(o, BSC_E_INVALID, "download_state: size mismatch");
    const int64_t n = o->n;
    auto cp = [n](double* dst, const std::vector<double>& v) {
        if (dst) std::memcpy(dst, v.data(), sizeof(double) * n);
    };
    cp(s->x, o->x); cp(s->y, o->y); cp(s->vx, o->vx); cp(s->vy, o->vy);
    cp(s->xs, o->xs); cp(s->ys, o->ys); cp(s->vxs, o->vxs); cp(s->vys, o->vys);
    cp(s->p, o->p); cp(s->rho, o->rho); cp(s->oden, o->oden); cp(s->mass, o->mass);
    cp(s->porosity, o->por); cp(s->gradvx, o->gradvx); cp(s->nut, o->nut); cp(s->tke, o->tke);
    cp(s->resist, o->resist); cp(s->varts, o->varts); cp(s->vel, o->vel); cp(s->xrest, o->xrest);
    cp(s->con, o->con); cp(s->ovol, o->ovol);
    if (s->L) std::memcpy(s->L, o->coff.data(), sizeof(double) * 4 * n);
    if (s->tid) std::memcpy(s->tid, o->tid.data(), n);
    if (s->flags) std::memcpy(s->flags, o->flags.data(), n);
    return BSC_OK;
}

// greenfield wavemaker: piston particles at x_rest + x_p(t), velocity v_p(t)
int orc_piston(orc_ctx* o) {
    double vp = 0;
    double xp = piston_x(o->P, o->t, &vp);
    for (int64_t k = 0; k < o->n; ++k)
        if (has(o->flags[k], BSC_FLAG_PISTON)) {
            o->x[k] = o->xrest[k] + xp;
            o->vx[k] = vp; o->vxs[k] = vp;
            o->vy[k] = 0; o->vys[k] = 0;
        }
    return BSC_OK;
}

// isph.f90:16-47
int orc_projection(orc_ctx* o) {
    const double dt = o->dt;
#pragma omp parallel for schedule(static)
    for (int64_t k = 0; k < o->n; ++k) {
        if (o->tid[k] == BSC_TID_FLUID && !has(o->flags[k], BSC_FLAG_DEAD)) {
            o->xs[k] = o->x[k];
            o->x[k] = o->x[k] + (dt * o->vx[k] / o->por[k]);
            o->ys[k] = o->y[k];
            o->y[k] = o->y[k] + (dt * o->vy[k] / o->por[k]);
        }
    }
    return BSC_OK;
}

// integrator.f90:250-391 cellshift / :32-248 cellshiftalt: re-bin moved
// particles into their cells.  The outflow cut-offs of cellshiftalt
// (integrator.f90:60-61) apply to open-boundary runs only and are not part of
// this closed-tank path.
int orc_cellshift(orc_ctx* o, int32_t) {
    bin_particles(o);
    o->have_lists = false;
    return BSC_OK;
}

// isph.f90:88-113: matid numbering in (column j, row i, slot) order
int orc_resetid(orc_ctx* o) {
    int64_t c = 0;
    for (int j = 1; j <= o->cellx; ++j)
        for (int i = 1; i <= o->celly; ++i) {
            int64_t ci = cidx(o, i, j);
            for (int64_t k = o->cell_off[ci]; k < o->cell_off[ci + 1]; ++k) o->matid[o->cell_mem[k]] = c++;
        }
    return BSC_OK;
}

// search.f90:13-399 neighbour -> nsearch2
int orc_neighbour(orc_ctx* o) {
    const int64_t n = o->n;
    const double h = o->P.h;
    std::vector<std::vector<int64_t>> lid(n);
    std::vector<std::vector<double>> ld(n), lx(n), ly(n);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
        int ci[4], cj[4];
        quad_cells(o, o->x[i], o->y[i], o->pci[i], o->pcj[i], ci, cj);
        double res[4] = {0, 0, 0, 0};
        o->flags[i] &= (uint8_t)~BSC_FLAG_FREE;   // search.f90:41
        o->gradvx[i] = 0.0;                        // search.f90:42
        for (int q = 0; q < 4; ++q) {
            int64_t c = cidx(o, ci[q], cj[q]);
            for (int64_t s = o->cell_off[c]; s < o->cell_off[c + 1]; ++s) {
                int64_t j = o->cell_mem[s];
                if (j == i) continue;  // (tid,matid) self test, search.f90:53-55
                double radial = dist(o->x[i], o->y[i], o->x[j], o->y[j]);
                if (radial < (2 * h)) {
                    double res2 = Wab_grad(o, o->x[i] - o->x[j], radial, h);
                    double res4 = Wab_grad(o, o->y[i] - o->y[j], radial, h);
                    lid[i].push_back(j);
                    ld[i].push_back(radial);
                    lx[i].push_back(res2);
                    ly[i].push_back(res4);
                    double res1 = (o->mass[j]) * (o->x[j] - o->x[i]) / (o->rho[j]);
                    double res3 = (o->mass[j]) * (o->y[j] - o->y[i]) / (o->rho[j]);
                    res[0] = res[0] + res2 * res1;
                    res[1] = res[1] + res4 * res1;
                    res[2] = res[2] + res2 * res3;
                    res[3] = res[3] + res4 * res3;
                }
            }
        }
        if (o->tid[i] == BSC_TID_FLUID) {  // search.f90:268-306
            o->flags[i] &= (uint8_t)~(BSC_FLAG_FREE | BSC_FLAG_VICINITY);
            o->gradvx[i] = (res[0] + res[3]);
            invertmat2D(res);
            for (int q = 0; q < 4; ++q) o->coff[4 * i + q] = res[q];
            if ((o->gradvx[i] <= o->P.free_threshold) && !has(o->flags[i], BSC_FLAG_BUFFER))
                o->flags[i] |= BSC_FLAG_FREE;
        }
    }
    o->nb_off.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) o->nb_off[i + 1] = o->nb_off[i] + (int64_t)lid[i].size();
    const int64_t tot = o->nb_off[n];
    o->nb_id.resize(tot); o->nb_dist.resize(tot); o->nb_kx.resize(tot); o->nb_ky.resize(tot);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        std::copy(lid[i].begin(), lid[i].end(), o->nb_id.begin() + o->nb_off[i]);
        std::copy(ld[i].begin(), ld[i].end(), o->nb_dist.begin() + o->nb_off[i]);
        std::copy(lx[i].begin(), lx[i].end(), o->nb_kx.begin() + o->nb_off[i]);
        std::copy(ly[i].begin(), ly[i].end(), o->nb_ky.begin() + o->nb_off[i]);
    }
    o->have_lists = true;
    return BSC_OK;
}

// isph.f90:49-86 freesurf (serial scatter: no race)
int orc_freesurf(orc_ctx* o) {
    if (!o->have_lists) return fail(o, BSC_E_INVALID, "freesurf before neighbour");
    for (int64_t i = 0; i < o->n; ++i) {
        if (o->tid[i] == BSC_TID_FLUID && !has(o->flags[i], BSC_FLAG_BUFFER)) {
            if (o->gradvx[i] <= o->P.free_threshold)
                for (int64_t k = o->nb_off[i]; k < o->nb_off[i + 1]; ++k) o->flags[o->nb_id[k]] |= BSC_FLAG_VICINITY;
        }
    }
    return BSC_OK;
}

// porous.f90:107-224 effpor (porsearch :32-105, vis :12-30)
int orc_effpor(orc_ctx* o) {
    const double h = o->P.h;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->n; ++i) {
        double solidfrac = 0.0;
        o->resist[i] = 0.0;
        if (o->tid[i] != BSC_TID_FLUID) continue;
        o->por[i] = 1.0;
        int ci[4], cj[4];
        quad_cells(o, o->x[i], o->y[i], o->pci[i], o->pcj[i], ci, cj);
        // porsearch visits the particle's own cell first, then the other three
        int order[4], no = 0;
        for (int q = 0; q < 4; ++q)
            if (ci[q] == o->pci[i] && cj[q] == o->pcj[i]) order[no++] = q;
        for (int q = 0; q < 4; ++q)
            if (!(ci[q] == o->pci[i] && cj[q] == o->pcj[i])) order[no++] = q;
        if (o->ns > 0) {
            for (int qq = 0; qq < 4; ++qq) {
                int64_t c = cidx(o, ci[order[qq]], cj[order[qq]]);
                for (int64_t s = o->scell_off[c]; s < o->scell_off[c + 1]; ++s) {
                    int64_t k = o->scell_mem[s];
                    double radial = dist(o->x[i], o->y[i], o->sx[k], o->sy[k]);
                    if (radial < (2 * h))
                        solidfrac = solidfrac + (1.0 - o->spor[k]) * Wab(o, radial, h) * o->sm[k] / o->srho[k];
                }
            }
        }
        double cap = 1.0 - porosity_at(o, o->x[i], o->y[i]);
        if (solidfrac > cap) solidfrac = cap;
        double nn = 1.0 - solidfrac;
        o->por[i] = nn;
        o->rho[i] = nn * o->oden[i];
        // Ergun form of porous.f90:192,204-212 with Fch*sqrt(lamk) = beta/sqrt(n^3)
        double Fch = o->P.forch_beta / (std::sqrt(nn * nn * nn));
        double vmag = std::sqrt(o->vx[i] * o->vx[i] + o->vy[i] * o->vy[i]);
        double d = o->P.d50;
        o->resist[i] = -((vis(o->oden[i]) / o->oden[i]) * o->P.darcy_alpha * ((1.0 - nn) * (1.0 - nn)) /
                         ((nn * nn * nn) * (d * d))) -
                       ((Fch * vmag * (1.0 - nn)) / (std::sqrt(nn * nn * nn) * d));
    }
    return BSC_OK;
}

// turbulence.f90:12-110 eddyvis (slots btot+1..ptot = fluid particles)
int orc_eddyvis(orc_ctx* o) {
    if (!o->have_lists) return fail(o, BSC_E_INVALID, "eddyvis before neighbour");
    const double cs = o->P.eddy_cs, cv = o->P.eddy_cv, ce = o->P.eddy_ce, dl = o->P.dl;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->n; ++i) {
        if (o->tid[i] != BSC_TID_FLUID) continue;
        double t1 = 0, t2 = 0, t3 = 0;
        const double* L = &o->coff[4 * i];
        for (int64_t k = o->nb_off[i]; k < o->nb_off[i + 1]; ++k) {
            int64_t j = o->nb_id[k];
            double z1 = o->nb_kx[k], z2 = o->nb_ky[k];
            double du = o->vx[j] / o->por[j] - o->vx[i] / o->por[i];
            double dv = o->vy[j] / o->por[j] - o->vy[i] / o->por[i];
            t1 = t1 + (o->mass[j] * du * (L[0] * z1 + L[1] * z2)) / o->rho[j];
            t2 = t2 + (o->mass[j] * dv * (L[2] * z1 + L[3] * z2)) / o->rho[j];
            t3 = t3 + (0.50 * o->mass[j] * (du * (L[2] * z1 + L[3] * z2) + dv * (L[0] * z1 + L[1] * z2))) / o->rho[j];
        }
        double t4 = std::sqrt(2 * (t1 * t1 + t2 * t2) + (2 * t3) * (2 * t3));
        o->nut[i] = ((cs * dl) * (cs * dl)) * t4;
        o->tke[i] = (cv / ce) * ((dl * t4) * (dl * t4));
    }
    return BSC_OK;
}

// integrator.f90:458-713 int_vel
int orc_int_vel(orc_ctx* o) {
    if (!o->have_lists) return fail(o, BSC_E_INVALID, "int_vel before neighbour");
    const double dt = o->dt, dl = o->P.dl, h = o->P.h, lam = o->P.lam, g = o->P.g;
    // pass 1: free-surface artificial viscosity varts (:467-506)
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->n; ++i) {
        if (!has(o->flags[i], BSC_FLAG_FREE)) continue;
        double t1 = 0, t2 = 0;
        const double* L = &o->coff[4 * i];
        for (int64_t k = o->nb_off[i]; k < o->nb_off[i + 1]; ++k) {
            int64_t j = o->nb_id[k];
            double z1 = o->nb_kx[k], z2 = o->nb_ky[k];
            t1 = t1 + (o->vx[j] / o->por[j] - o->vx[i] / o->por[i]) * (L[0] * z1 + L[1] * z2) * (o->mass[j] / o->rho[j]);
            t2 = t2 + (o->vy[j] / o->por[j] - o->vy[i] / o->por[i]) * (L[2] * z1 + L[3] * z2) * (o->mass[j] / o->rho[j]);
        }
        o->varts[i] = o->P.varts_ps * (dl * dl) * std::sqrt(t1 * t1 + t2 * t2) *
                      std::sqrt(o->vx[i] * o->vx[i] + o->vy[i] * o->vy[i]) / ((o->umax + F_1EM6) * o->por[i]);
    }
    const double wo = Wo(o, h);
    // pass 2: viscous, SPS and drag predictor (:509-711)
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->n; ++i) {
        const uint8_t fi = o->flags[i];
        if (o->tid[i] == BSC_TID_FLUID && !has(fi, BSC_FLAG_BUFFER) && !has(fi, BSC_FLAG_DEAD)) {
            double vxs = 0.0, vys = 0.0;
            const double* L = &o->coff[4 * i];
            const double oi = o->oden[i], visi = vis(oi), ni = o->por[i], nuti = o->nut[i];
            for (int64_t k = o->nb_off[i]; k < o->nb_off[i + 1]; ++k) {
                int64_t j = o->nb_id[k];
                double z1 = o->nb_kx[k], z2 = o->nb_ky[k], r = o->nb_dist[k];
                double cmu;
                if (o->tid[j] == BSC_TID_FLUID) {
                    double oj = o->oden[j], visj = vis(oj);
                    cmu = 2 * visi * visj * ((1.0 / oi) * (1.0 / oj)) / ((visi / oi) + (visj / oj));
                } else {
                    cmu = visi * (1.0 / oi);
                }
                double vart;
                if (has(fi, BSC_FLAG_FREE)) vart = o->varts[i];
                else if (!has(fi, BSC_FLAG_FREE) && has(o->flags[j], BSC_FLAG_FREE) && !has(fi, BSC_FLAG_BUFFER))
                    vart = Wab(o, r, h) * o->varts[j] / wo;
                else vart = 0.0;
                double pvol = o->mass[j] / o->rho[j];
                double p_dist = 1.0 / (r * r + lam);
                double gx = (L[0] * z1 + L[1] * z2), gy = (L[2] * z1 + L[3] * z2);
                double dxij = o->x[i] - o->x[j], dyij = o->y[i] - o->y[j];
                for (int comp = 0; comp < 2; ++comp) {
                    double dvij = comp == 0 ? (o->vx[i] - o->vx[j]) : (o->vy[i] - o->vy[j]);
                    double t1 = (2 * pvol * dvij * dxij * gx) * p_dist;
                    double t2 = (2 * pvol * dvij * dyij * gy) * p_dist;
                    double& acc = (comp == 0) ? vxs : vys;
                    acc = acc + (t1 + t2) * (cmu + vart);
                    if (o->tid[j] > 2) {  // eddy viscosity of fluid pairs (:580-598)
                        double nutj = o->nut[j];
                        if ((nuti < F_1EM6) && (nutj < F_1EM6)) acc = acc + (t1 + t2) * (nuti + nutj) * 0.50;
                        else acc = acc + (t1 + t2) * ((2 * nuti * nutj) / (nuti + nutj));
                    }
                }
                // SPS turbulence term (:645-666)
                double tk1 = (pvol * (o->tke[j] - o->tke[i]) * gx);
                vxs = vxs - (tk1)*ni * 2.0 / 3;
                double tk2 = (pvol * (o->tke[j] - o->tke[i]) * gy);
                vys = vys - (tk2)*ni * 2.0 / 3;
            }
            o->vxs[i] = (o->vx[i] + (dt * vxs)) / (1.0 - dt * o->resist[i] * ni);
            o->vys[i] = (o->vy[i] + dt * (vys)) / (1.0 - dt * o->resist[i] * ni);
            o->vys[i] = o->vys[i] + g * ni * dt;
        }
        if (has(fi, BSC_FLAG_BUFFER)) {  // :691-698
            o->vxs[i] = o->vx[i];
            o->vys[i] = g * o->por[i] * dt;
        }
    }
    return BSC_OK;
}

// isph.f90:115-456 PPE assembly, then the solve and the scatter (:460-483)
int orc_ppesolve(orc_ctx* o, bsc_solve_info* info) {
    if (!o->have_lists) return fail(o, BSC_E_INVALID, "ppesolve before neighbour");
    const int64_t n = o->n, finmax = n;
    const double dt = o->dt, lam = o->P.lam, rho0 = o->P.rho0, rel_den = o->P.rel_den;
    // matid -> particle
    std::vector<int64_t> who(finmax, -1);
    for (int64_t k = 0; k < n; ++k) who[o->matid[k]] = k;
    o->rowptr.assign(finmax + 1, 0);
    for (int64_t pos = 0; pos < finmax; ++pos) {
        int64_t k = who[pos];
        int64_t sz = (k < 0) ? 1 : (o->nb_off[k + 1] - o->nb_off[k] + 1);
        o->rowptr[pos + 1] = o->rowptr[pos] + sz;
    }
    o->col.assign(o->rowptr[finmax], 0);
    o->val.assign(o->rowptr[finmax], 0.0);
    o->rhs.assign(finmax, 0.0);
    int bad_order = 0;
#pragma omp parallel for schedule(dynamic, 256) reduction(+ : bad_order)
    for (int64_t pos = 0; pos < finmax; ++pos) {
        const int64_t i = who[pos];
        const int64_t base = o->rowptr[pos];
        if (i < 0) {  // identity rows for unused matids (isph.f90:123-131)
            o->col[base] = pos; o->val[base] = 1.0; continue;
        }
        const int64_t b0 = o->nb_off[i], num = o->nb_off[i + 1] - b0;
        for (int64_t s = 0; s <= num; ++s) o->col[base + s] = pos;
        int64_t dia_pt = 0;
        double dia_term = 0.0, fv = 0.0;
        const double ni = o->por[i], rhoi = o->rho[i];
        const double rho_i = rhoi * (1.0 / ni);
        const double* Li = &o->coff[4 * i];
        int64_t prev = -1;
        for (int64_t m = 0; m < num; ++m) {
            const int64_t j = o->nb_id[b0 + m];
            const int64_t mj = o->matid[j];
            if (mj <= prev) bad_order++;
            prev = mj;
            int64_t ins_pt;
            if (pos > mj) { dia_pt = m + 1; ins_pt = m; }
            else ins_pt = m + 1;
            const double z1 = o->nb_kx[b0 + m], z2 = o->nb_ky[b0 + m];
            const double nj = o->por[j], rhoj = o->rho[j];
            double lamp = (has(o->flags[i], BSC_FLAG_FREE) && o->tid[j] == BSC_TID_FLUID)
                              ? (1.0 + o->oden[j] / (rho0 * rel_den)) : 1.0;
            const double rho_j = rhoj * (1.0 / nj);
            const double pvol = o->mass[j] * (1.0 / rhoj);
            const double r = dist(o->x[j], o->y[j], o->x[i], o->y[i]);
            const double p_dist = 1.0 / ((r * r) + lam);
            const double rho_ij = 2 * rhoj * rhoi * (1.0 / (nj * ni)) * (1.0 / ((rhoj * (1.0 / nj)) + (rhoi * (1.0 / ni))));
            const double dxij = o->x[i] - o->x[j], dyij = o->y[i] - o->y[j];
            if (o->tid[i] == BSC_TID_FLUID) {
                double gx = (Li[0] * z1 + Li[1] * z2), gy = (Li[2] * z1 + Li[3] * z2);
                double t1 = 2 * pvol * gx * dxij * (p_dist);
                double t2 = 2 * pvol * gy * dyij * (p_dist);
                o->val[base + ins_pt] = (-(t1 + t2));
                o->col[base + ins_pt] = mj;
                dia_term = dia_term + (t1 + t2) * lamp;
                if (o->tid[j] == BSC_TID_FLUID) {
                    t1 = (pvol * (o->vxs[j] * rho_ij / nj - o->vxs[i] * rho_ij / ni) * gx);
                    t2 = (pvol * (o->vys[j] * rho_ij / nj - o->vys[i] * rho_ij / ni) * gy);
                } else {
                    t1 = (pvol * (o->vxs[j] * rho_i / ni - o->vxs[i] * rho_i / ni) * gx);
                    t2 = (pvol * (o->vys[j] * rho_i / ni - o->vys[i] * rho_i / ni) * gy);
                }
                fv = fv + (t1 + t2) / dt;
            } else if (o->tid[i] == BSC_TID_GHOST) {
                double t1 = 2 * pvol * (z1) * dxij * (p_dist);
                double t2 = 2 * pvol * (z2) * dyij * (p_dist);
                if (o->tid[j] <= 2) {
                    o->val[base + ins_pt] = -(t1 + t2);
                    o->col[base + ins_pt] = mj;
                    dia_term = dia_term + (t1 + t2);
                }
            } else if (o->tid[i] == BSC_TID_WALL) {
                if (o->tid[j] == BSC_TID_FLUID) {
                    const double* Lj = &o->coff[4 * j];
                    double lamp2 = 1.0;
                    double gx = (Lj[0] * z1 + Lj[1] * z2), gy = (Lj[2] * z1 + Lj[3] * z2);
                    double t1 = 2 * o->mass[i] * gx * dxij * (p_dist) / (rhoi);
                    double t2 = 2 * o->mass[i] * gy * dyij * (p_dist) / (rhoi);
                    o->val[base + ins_pt] = -(t1 + t2) * lamp2;
                    o->col[base + ins_pt] = mj;
                    dia_term = dia_term + (t1 + t2);
                    t1 = (o->mass[i] * (o->vxs[j] * rho_j / nj - o->vxs[i] * rho_j / ni) * gx) / (rhoi);
                    t2 = (o->mass[i] * (o->vys[j] * rho_j / nj - o->vys[i] * rho_j / ni) * gy) / (rhoi);
                    fv = fv + (t1 + t2) / dt;
                } else if (o->tid[j] <= 2) {
                    double t1 = 2 * pvol * (z1) * dxij * (p_dist);
                    double t2 = 2 * pvol * (z2) * dyij * (p_dist);
                    o->val[base + ins_pt] = -(t1 + t2);
                    o->col[base + ins_pt] = mj;
                    dia_term = dia_term + (t1 + t2);
                }
            }
        }
        o->col[base + dia_pt] = pos;
        if (dia_term == 0.0 || !std::isfinite(dia_term)) {
            // guarded zero-neighbour row (the reference divides by zero)
            for (int64_t s = 0; s <= num; ++s) { o->val[base + s] = 0.0; }
            o->val[base + dia_pt] = 1.0;
            o->rhs[pos] = 0.0;
            continue;
        }
        o->val[base + dia_pt] = dia_term;
        const double t1 = o->val[base + dia_pt];
        o->rhs[pos] = fv / t1;  // Jacobi row scaling (isph.f90:434-442)
        for (int64_t s = 0; s <= num; ++s) o->val[base + s] = o->val[base + s] / t1;
    }
    if (bad_order) return fail(o, BSC_E_INVALID, "ppesolve: neighbour lists not in matid order (resetid missing)");
    // warm start from each particle's previous pressure
    o->sol.assign(finmax, 0.0);
    for (int64_t k = 0; k < n; ++k) o->sol[o->matid[k]] = o->p[k];
    bsc_solve_info loc{};
    bsc_solve_info* si = info ? info : &loc;
    int st = (o->P.solver == BSC_SOLVER_FGMRES) ? fgmres(o->P, o->rowptr, o->col, o->val, o->rhs, o->sol, si)
                                                : bicgstab(o->P, o->rowptr, o->col, o->val, o->rhs, o->sol, si);
    for (int64_t k = 0; k < n; ++k) o->p[k] = o->sol[o->matid[k]];
    o->have_csr = true;
    if (st != BSC_OK) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "ppesolve: solver status %d after %d iterations, rel res %.3e", st,
                      si->iterations, si->rel_residual);
        o->err = buf;
    }
    return st;
}

// integrator.f90:715-865 comp_vel
int orc_comp_vel(orc_ctx* o) {
    if (!o->have_lists) return fail(o, BSC_E_INVALID, "comp_vel before neighbour");
    const double dt = o->dt;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->n; ++i) {
        const uint8_t fi = o->flags[i];
        if (o->tid[i] == BSC_TID_FLUID && !has(fi, BSC_FLAG_BUFFER) && !has(fi, BSC_FLAG_DEAD)) {
            double vx = 0.0, vy = 0.0;
            const double* L = &o->coff[4 * i];
            const double ni = o->por[i], rhoi = o->rho[i], pi = o->p[i];
            for (int64_t k = o->nb_off[i]; k < o->nb_off[i + 1]; ++k) {
                int64_t j = o->nb_id[k];
                double z1 = o->nb_kx[k], z2 = o->nb_ky[k];
                double nj = o->por[j], rhoj = o->rho[j], pj = o->p[j];
                double gx = (L[0] * z1 + L[1] * z2), gy = (L[2] * z1 + L[3] * z2);
                double t1;
                if (o->tid[j] == BSC_TID_FLUID)
                    t1 = 2 * ((o->mass[j] / rhoj) * (ni * ni) * ((pj * rhoi / ni) + (pi * rhoj / nj)) * gx) /
                         ((rhoi) * ((rhoi / ni) + (rhoj / nj)));
                else
                    t1 = ((o->mass[j] / rhoj) * (ni * ni) * (pj + pi) * gx) / rhoi;
                vx = vx - t1 * dt;
                if (o->tid[j] == BSC_TID_FLUID)
                    t1 = 2 * ((o->mass[j] / rhoj) * (ni * ni) * ((pj * rhoi / ni) + (pi * rhoj / nj)) * gy) /
                         ((rhoi) * ((rhoi / ni) + (rhoj / nj)));
                else
                    t1 = ((o->mass[j] / rhoj) * (ni * ni) * (pj + pi) * gy) / rhoi;
                vy = vy - t1 * dt;
            }
            o->vx[i] = o->vxs[i] + vx;
            o->vy[i] = o->vys[i] + vy;
            o->vel[i] = std::sqrt(o->vx[i] * o->vx[i] + o->vy[i] * o->vy[i]) / ni;
        }
        if (has(fi, BSC_FLAG_BUFFER)) { o->vx[i] = o->vxs[i]; o->vy[i] = 0.0; }
        if (has(fi, BSC_FLAG_DEAD) && !has(fi, BSC_FLAG_BUFFER)) {
            o->vx[i] = 0.0; o->vy[i] = 0.0; o->vxs[i] = 0.0; o->vys[i] = 0.0;
        }
    }
    return BSC_OK;
}

// integrator.f90:867-906 comp_pos
int orc_comp_pos(orc_ctx* o) {
    const double dt = o->dt;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < o->n; ++i) {
        if (o->tid[i] == BSC_TID_FLUID && !has(o->flags[i], BSC_FLAG_DEAD)) {
            o->x[i] = (o->x[i] + o->xs[i] + dt * o->vx[i] / o->por[i]) / 2.0;
            o->y[i] = (o->y[i] + o->ys[i] + dt * o->vy[i] / o->por[i]) / 2.0;
            if (has(o->flags[i], BSC_FLAG_BUFFER) && (o->x[i] > o->P.buffer_release_xmin) &&
                (o->x[i] < o->P.buffer_release_xmax))
                o->flags[i] &= (uint8_t)~BSC_FLAG_BUFFER;
        }
    }
    return BSC_OK;
}

// part_shift.f90:12-192 opt2_shift
int orc_opt2_shift(orc_ctx* o) {
    if (!o->have_lists) return fail(o, BSC_E_INVALID, "opt2_shift before neighbour");
    const double h = o->P.h, csh = o->P.csh, lim = o->P.maxshift * o->P.dl;
    std::vector<uint8_t> done(o->n, 0);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->n; ++i) {
        const uint8_t fi = o->flags[i];
        if (!(o->tid[i] == BSC_TID_FLUID && !has(fi, BSC_FLAG_BUFFER) && !has(fi, BSC_FLAG_DEAD))) continue;
        const int64_t b0 = o->nb_off[i], b1 = o->nb_off[i + 1];
        if (b1 == b0) continue;
        // the surface normal is computed and then forced to zero, as is pint
        // (part_shift.f90:51-70): the shift uses the uncorrected gradient.
        const double frac = has(fi, BSC_FLAG_FREE) ? 0.01 : 1.0;
        double xs = 0.0, ys = 0.0;
        for (int64_t k = b0; k < b1; ++k) {
            int64_t j = o->nb_id[k];
            xs = xs - csh * (h * h) * frac * (o->nb_kx[k]) * (o->mass[j] / o->rho[j]);
        }
        double sxs = (xs == 0.0) ? 0.0 : std::min(std::fabs(xs), lim) * xs / std::fabs(xs);
        for (int64_t k = b0; k < b1; ++k) {
            int64_t j = o->nb_id[k];
            ys = ys - csh * (h * h) * frac * (o->nb_ky[k]) * (o->mass[j] / o->rho[j]);
        }
        double sys = (ys == 0.0) ? 0.0 : std::min(std::fabs(ys), lim) * ys / std::fabs(ys);
        const double* L = &o->coff[4 * i];
        double t1 = 0, t2 = 0;
        for (int64_t k = b0; k < b1; ++k) {
            int64_t j = o->nb_id[k];
            double z1 = o->nb_kx[k], z2 = o->nb_ky[k];
            t1 = t1 + ((L[0] * z1 + L[1] * z2) * (o->vx[j] - o->vx[i])) * (o->mass[j] / o->rho[j]);
            t2 = t2 + ((L[2] * z1 + L[3] * z2) * (o->vx[j] - o->vx[i])) * (o->mass[j] / o->rho[j]);
        }
        double svx = t1 * xs + t2 * ys;
        t1 = 0; t2 = 0;
        for (int64_t k = b0; k < b1; ++k) {
            int64_t j = o->nb_id[k];
            double z1 = o->nb_kx[k], z2 = o->nb_ky[k];
            t1 = t1 + ((L[0] * z1 + L[1] * z2) * (o->vy[j] - o->vy[i])) * (o->mass[j] / o->rho[j]);
            t2 = t2 + ((L[2] * z1 + L[3] * z2) * (o->vy[j] - o->vy[i])) * (o->mass[j] / o->rho[j]);
        }
        double svy = t1 * xs + t2 * ys;
        o->xs[i] = sxs; o->ys[i] = sys; o->vxs[i] = svx; o->vys[i] = svy;
        done[i] = 1;
    }
    // part_shift.f90:173-190
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < o->n; ++i) {
        if (done[i]) {
            o->x[i] = o->x[i] + o->xs[i];
            o->y[i] = o->y[i] + o->ys[i];
            o->vx[i] = o->vx[i] + o->vxs[i];
            o->vy[i] = o->vy[i] + o->vys[i];
        }
    }
    return BSC_OK;
}

// integrator.f90:908-976 timestep (maxvel/maxeddy of comp_vel :853-861)
int orc_timestep(orc_ctx* o, double* dt_inout) {
    double umax = 0.0, numax = 0.0;
    for (int64_t i = 0; i < o->n; ++i) {
        umax = std::max(umax, std::fabs(o->vel[i]));
        numax = std::max(numax, std::fabs(o->nut[i]));
    }
    o->umax = umax;
    o->numax = numax;
    const double sig1 = o->P.sig1, dl = o->P.dl, mu = o->P.mu, rho = o->P.rho0, t = o->t;
    double dt;
    if (t <= 1.0)
        dt = std::min(std::min(sig1 * (dl) / umax, sig1 * ((dl) * (dl)) / ((mu / rho) + numax)), 0.0010);
    else if (t > 1.0 && t <= 2.50)
        dt = (double)std::min(std::min((float)(sig1 * (dl) / umax), (float)(sig1 * ((dl) * (dl)) * rho / mu)), 0.002f);
    else if (t > 3.0 && t <= 4.0)
        dt = (double)std::min(std::min((float)(sig1 * (dl) / umax), (float)(sig1 * ((dl) * (dl)) * rho / mu)), 0.004f);
    else
        dt = std::min(std::min(sig1 * (dl) / umax, sig1 * ((dl) * (dl)) / ((mu / rho) + numax)), 0.0050);
    if (!std::isfinite(numax)) numax = 0.0;
    // integrator.f90:964-972; the sub-steps cover the next step's dt (the
    // rule's, or the fixed dt of the benchmark mode)
    const double dtn = o->P.dt_mode == BSC_DT_ADAPTIVE ? dt : o->dt;
    double dtsol = sig1 * (dl * dl) / (o->P.diffusivity + numax / o->P.tschmidt);
    int solsteps = 1;
    if (dtsol < dtn) {
        solsteps = (int)std::ceil(dtn / dtsol);
        dtsol = dtn / solsteps;
    }
    dtsol = (dtsol < dtn) ? dtsol : dtn;
    o->dtsol = dtsol;
    o->solsteps = solsteps;
    if (o->P.dt_mode == BSC_DT_ADAPTIVE) o->dt = dt;
    if (dt_inout) *dt_inout = (o->P.dt_mode == BSC_DT_ADAPTIVE) ? dt : o->dt;
    return BSC_OK;
}

int orc_get_dt_rule(orc_ctx* o, double* umax, double* numax, double* dtsol, int32_t* solsteps) {
    if (umax) *umax = o->umax;
    if (numax) *numax = o->numax;
    if (dtsol) *dtsol = o->dtsol;
    if (solsteps) *solsteps = o->solsteps;
    return BSC_OK;
}

// scalar.f90:114-240 scalart: the dispersion flux of every fluid particle.
// The kernel gradient takes the distance stored by the neighbour search and
// the current positions, as hWabx(x, plist(k), dist(m), h1) does.
int orc_scalart(orc_ctx* o) {
    if (!o->have_lists) return fail(o, BSC_E_INVALID, "scalart before neighbour");
    const double al = o->P.disp_long, at = o->P.disp_trans, Dm = o->P.diffusivity, tor = 1.0;
    const double tsc = o->P.tschmidt, h = o->P.h, lam = o->P.lam;
    const double cap = 0.12 * (o->P.dl * o->P.dl) / o->dt;
    const double nut_min = (double)1e-6f;  // `nut < 1e-6`, a default-real literal
    auto live = [o](int64_t k) { return o->tid[k] == BSC_TID_FLUID && !has(o->flags[k], BSC_FLAG_DEAD); };
    auto clampD = [Dm, cap](double D) {
        D = (D > 0.0) ? D : Dm;      // merge(D, Dm, D > 0): a NaN gives Dm
        return (D <= cap) ? D : cap;  // merge(D, cap, D <= cap)
    };
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < o->n; ++i) {
        if (!live(i)) continue;
        o->cdiff[i] = 0.0;
        const double con1 = o->con[i];
        const double vi = std::sqrt(o->vx[i] * o->vx[i] + o->vy[i] * o->vy[i]);
        const double ni = o->por[i];
        const double Dxi = clampD(Dm + ((al * (o->vx[i] * o->vx[i])) + (at * (o->vy[i] * o->vy[i])) +
                                        ((al - at) * o->vx[i] * o->vy[i])) / (vi * ni));
        const double Dyi = clampD(Dm + ((at * (o->vx[i] * o->vx[i])) + (al * (o->vy[i] * o->vy[i])) +
                                        ((al - at) * o->vx[i] * o->vy[i])) / (vi * ni));
        double cd = 0.0;
        for (int64_t e = o->nb_off[i]; e < o->nb_off[i + 1]; ++e) {
            const int64_t j = o->nb_id[e];
            if (!live(j)) continue;
            const double con2 = o->con[j];
            const double vj = std::sqrt(o->vx[j] * o->vx[j] + o->vy[j] * o->vy[j]);
            const double nj = o->por[j];
            const double Dxj = clampD(Dm + ((al * (o->vx[j] * o->vx[j])) + (at * (o->vy[j] * o->vy[j])) +
                                            ((al - at) * o->vx[j] * o->vy[j])) / (vj * nj));
            const double Dyj = clampD(Dm + ((at * (o->vx[j] * o->vx[j])) + (al * (o->vy[j] * o->vy[j])) +
                                            ((al - at) * o->vx[j] * o->vy[j])) / (vj * nj));
            double t1x, t1y;
            if ((ni >= 0.8) || (nj >= 0.8)) {
                if ((o->nut[i] < nut_min) && (o->nut[j] < nut_min)) {
                    t1x = Dm + (o->nut[i] + o->nut[j]) * 0.50 / tsc;
                } else {
                    t1x = 2 * (((Dm + o->nut[i] / tsc) * (Dm + o->nut[j] / tsc)) /
                               ((Dm + o->nut[i] / tsc) + (Dm + o->nut[j] / tsc)));
                }
                t1y = t1x;
            } else {
                t1x = 2.0 * tor * Dxi * Dxj / (Dxi + Dxj);
                t1y = 2.0 * tor * Dyi * Dyj / (Dyi + Dyj);
            }
            const double t3 = (o->ovol[i]) * (ni + nj) / (ni * nj);
            const double r = o->nb_dist[e];
            const double gx = Wab_grad(o, o->x[i] - o->x[j], r, h), gy = Wab_grad(o, o->y[i] - o->y[j], r, h);
            cd = cd + (t1x * t3 * (con1 - con2) * (o->x[i] - o->x[j]) * gx / (r * r + lam)) +
                 (t1y * t3 * (con1 - con2) * (o->y[i] - o->y[j]) * gy / (r * r + lam));
        }
        o->cdiff[i] = cd;
    }
    return BSC_OK;
}

// scalar.f90:242-275
int orc_scalarupdate(orc_ctx* o, double stime) {
    for (int64_t i = 0; i < o->n; ++i) {
        if (o->tid[i] != BSC_TID_FLUID || has(o->flags[i], BSC_FLAG_DEAD)) continue;
        o->con[i] = o->con[i] + o->cdiff[i] * stime;
        if (has(o->flags[i], BSC_FLAG_BUFFER) && o->x[i] < o->P.buffer_con_xmax) o->con[i] = o->P.buffer_con;
    }
    return BSC_OK;
}

// scalar.f90:277-305, with rhomin = rho (initialize.f90:22) and
// rhomax = rho rel_den (setup.f90:19)
int orc_densityupdate(orc_ctx* o) {
    const double rhomin = o->P.rho0, rhomax = o->P.rho0 * o->P.rel_den;
    for (int64_t i = 0; i < o->n; ++i) {
        if (o->tid[i] != BSC_TID_FLUID || has(o->flags[i], BSC_FLAG_DEAD)) continue;
        o->oden[i] = 0.5 * (rhomax + rhomin) + o->con[i] * (rhomax - rhomin);
        o->mass[i] = o->oden[i] * o->ovol[i];
        o->rho[i] = o->oden[i] * o->por[i];
    }
    return BSC_OK;
}

int orc_remove_particles(orc_ctx* o, int32_t rule, double a, double b, int64_t* removed_out);

// main.f90:41-65; with salinity, the phase-3 loop of main.f90:198-260
// (without its open-boundary buffers)
int orc_step(orc_ctx* o, int32_t nsteps, bsc_solve_info* last) {
    for (int s = 0; s < nsteps; ++s) {
        o->t = o->t + o->dt;
        int st;
        if (o->P.salinity) {
            if (!o->have_lists) {
                orc_cellshift(o, 0);
                orc_neighbour(o);
            }
            if (!(o->dtsol > 0.0)) orc_timestep(o, nullptr);
            for (int k = 0; k < o->solsteps; ++k) {  // main.f90:210-215
                orc_scalart(o);
                orc_scalarupdate(o, o->dtsol);
            }
        }
        orc_piston(o);
        orc_projection(o);
        orc_cellshift(o, 0);
        orc_resetid(o);
        orc_neighbour(o);
        orc_effpor(o);
        orc_eddyvis(o);
        orc_int_vel(o);
        st = orc_ppesolve(o, last);
        if (st != BSC_OK) return st;
        orc_comp_vel(o);
        orc_comp_pos(o);
        orc_cellshift(o, 1);
        if (o->P.outflow) {  // cellshiftalt's outflow cut-off (integrator.f90:60-61)
            int64_t gone = 0;
            st = orc_remove_particles(o, BSC_REMOVE_OUTFLOW, o->P.outflow_xcut, o->P.outflow_ycut, &gone);
            if (st != BSC_OK) return st;
        }
        orc_neighbour(o);
        orc_freesurf(o);
        orc_effpor(o);
        orc_opt2_shift(o);
        if (o->P.salinity) orc_densityupdate(o);
        orc_timestep(o, nullptr);
        if (o->P.salinity) orc_eddyvis(o);
    }
    return BSC_OK;
}

int orc_get_neighbors(orc_ctx* o, int64_t* offsets, int32_t* ids) {
    if (!o->have_lists) return fail(o, BSC_E_INVALID, "get_neighbors before neighbour");
    if (offsets) std::memcpy(offsets, o->nb_off.data(), sizeof(int64_t) * (o->n + 1));
    if (ids) {
        for (int64_t i = 0; i < o->n; ++i) {
            std::vector<int32_t> v;
            for (int64_t k = o->nb_off[i]; k < o->nb_off[i + 1]; ++k) v.push_back((int32_t)o->nb_id[k]);
            std::sort(v.begin(), v.end());
            std::copy(v.begin(), v.end(), ids + o->nb_off[i]);
        }
    }
    return BSC_OK;
}

// CSR in id space, columns sorted, rows in id order
int orc_export_csr(orc_ctx* o, int64_t* rowptr, int32_t* col, double* val, double* rhs) {
    if (!o->have_csr) return fail(o, BSC_E_INVALID, "export_csr before ppesolve");
    const int64_t n = o->n;
    std::vector<int64_t> who(n);
    for (int64_t k = 0; k < n; ++k) who[o->matid[k]] = k;
    std::vector<int64_t> rp(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        int64_t pos = o->matid[i];
        rp[i + 1] = rp[i] + (o->rowptr[pos + 1] - o->rowptr[pos]);
    }
    if (rowptr) std::memcpy(rowptr, rp.data(), sizeof(int64_t) * (n + 1));
    if (rhs) for (int64_t i = 0; i < n; ++i) rhs[i] = o->rhs[o->matid[i]];
    if (col || val) {
        for (int64_t i = 0; i < n; ++i) {
            int64_t pos = o->matid[i];
            std::vector<std::pair<int32_t, double>> e;
            for (int64_t k = o->rowptr[pos]; k < o->rowptr[pos + 1]; ++k) e.push_back({(int32_t)who[o->col[k]], o->val[k]});
            std::stable_sort(e.begin(), e.end(), [](auto& a, auto& b) { return a.first < b.first; });
            for (size_t s = 0; s < e.size(); ++s) {
                if (col) col[rp[i] + s] = e[s].first;
                if (val) val[rp[i] + s] = e[s].second;
            }
        }
    }
    return BSC_OK;
}

// standalone CSR solve (solver.f90:129 bicgstab(...) / :306 fgmres)
int orc_csr_solve(const bsc_params* p, int32_t n, const int32_t* rowptr, const int32_t* col, const double* val,
                  const double* b, double* x, bsc_solve_info* info) {
    if (!p || n <= 0 || !rowptr || !col || !val || !b || !x || !info) return BSC_E_INVALID;
    std::vector<int64_t> rp(rowptr, rowptr + n + 1), cl(col, col + rowptr[n]);
    std::vector<double> vl(val, val + rowptr[n]), bb(b, b + n), xx(x, x + n);
    int st = (p->solver == BSC_SOLVER_FGMRES) ? fgmres(*p, rp, cl, vl, bb, xx, info) : bicgstab(*p, rp, cl, vl, bb, xx, info);
    std::memcpy(x, xx.data(), sizeof(double) * n);
    return st;
}

// free-surface elevation at probes: sum_i V_i w1(x_i - xp) - depth over fluid,
// w1 the 1-D Wendland C2 kernel with radius 2h (greenfield: the reference's
// probe.f90:86-125 interpolates pressure only)
int orc_probe_eta(orc_ctx* o, int32_t np, const double* xp, double depth, double* eta) {
    const double h = o->P.h, R = 2 * h;
    for (int k = 0; k < np; ++k) {
        double s = 0.0;
        for (int64_t i = 0; i < o->n; ++i) {
            if (o->tid[i] != BSC_TID_FLUID) continue;
            double q = std::fabs(o->x[i] - xp[k]) / R;
            if (q < 1.0) {
                double a = 1.0 - q;
                s += (o->mass[i] / o->rho[i]) * (1.25 / R) * (a * a * a) * (1.0 + 3.0 * q);
            }
        }
        eta[k] = s - depth;
    }
    return BSC_OK;
}

int orc_num_threads(void) { return omp_get_max_threads(); }
void orc_set_threads(int32_t nt) { if (nt > 0) omp_set_num_threads(nt); }

}  // extern "C"

extern "C" {
// test hook: W(r), grad factor F(r) (grad_i W = F (x_i - x_j)) and Wo of the
// selected kernel, evaluated with the restated kernel.f90 formulae
int orc_eval_kernel(const bsc_params* p, double r, double* w, double* f, double* w0) {
    if (!p) return BSC_E_INVALID;
    Orc o;
    o.P = *p;
    if (w) *w = Wab(&o, r, p->h);
    if (f) *f = (r > 0) ? Wab_grad(&o, 1.0, r, p->h) : 0.0;
    if (w0) *w0 = Wo(&o, p->h);
    return BSC_OK;
}
}

// ---------------------------------------------------------------------------
// WCSPH calibration workload: forward map and its adjoint, restated on the
// CPU.  The forward step follows the formulae of wcsph.f90 (Tait EOS with the
// negative-pressure reset of dentopress :36-62, continuity with the delta term
// and hydrostatic correction of calmasscons :66-129), a pressure gradient and
// laminar viscosity in the symmetric SPH forms, the Ergun drag of porous.f90:
// 192-212, and the implicit-drag velocity update with x' = x + dt v'/n.  It
// runs on the model's own masses m = rho_init dl^2.  The adjoint is written in
// scatter form: each pair term of particle i's sums sends its derivatives to
// both i and j.  It is not organised like the gather-form CUDA adjoint, which
// makes it an independent check of that bookkeeping.  No checkpointing: every
// state of the run is kept.
// ---------------------------------------------------------------------------
namespace {

struct WcPre {
    std::vector<double> rt, pp, rh, drh;
};

double wc_wendF(const Orc* o) { const double h = o->P.h; return 35.0 / (4.0 * 3.140 * ((h * h) * (h * h))); }
double wc_wendW(const Orc* o) { const double h = o->P.h; return 7.0 / (4.0 * 3.140 * (h * h)); }
// Wendland C2: W(r), F(r) with grad_i W = F (x_i - x_j), dF/dr
double wc_W(const Orc* o, double r) {
    const double q = r / o->P.h, a = 1.0 - 0.5 * q;
    return wc_wendW(o) * (1.0 + 2.0 * q) * a * a * a * a;
}
double wc_F(const Orc* o, double r) { const double a = 1.0 - 0.5 * r / o->P.h; return -wc_wendF(o) * a * a * a; }
double wc_dF(const Orc* o, double r) {
    const double a = 1.0 - 0.5 * r / o->P.h;
    return 1.5 * wc_wendF(o) * a * a / o->P.h;
}
// the probes' 1-D Wendland C2 kernel of radius R1 and its q-derivative
double wc_w1(double q, double R1) { const double a = 1.0 - q; return (1.25 / R1) * a * a * a * (1.0 + 3.0 * q); }
double wc_w1q(double q, double R1) { const double a = 1.0 - q; return -(15.0 / R1) * q * a * a; }

bool fluid(const Orc* o, int64_t i) { return o->tid[i] == BSC_TID_FLUID; }

void wc_pre(const Orc* o, const double* y, const double* rho, WcPre& q) {
    const WcOrc& w = o->wc;
    const int64_t n = o->n;
    q.rt.resize(n); q.pp.resize(n); q.rh.resize(n); q.drh.resize(n);
    for (int64_t i = 0; i < n; ++i) {
        const double r = fluid(o, i) ? std::max(rho[i], w.rho0) : rho[i];
        double p = w.B * (std::pow(r / w.rho0, w.gam) - 1.0);
        if (p < 0.0) p = 0.0;  // wcsph.f90:49-52
        q.rt[i] = r;
        q.pp[i] = p;
        const double s = 1.0 + w.grav_c * (w.ys - y[i]);
        q.rh[i] = w.rho0 * std::pow(s, 1.0 / w.gam);       // wcsph.f90:82-86
        q.drh[i] = -w.rho0 * w.grav_c / w.gam * std::pow(s, 1.0 / w.gam) / s;
    }
}

void wc_solids(Orc* o) {
    WcOrc& w = o->wc;
    w.sw.resize(o->ns);
    w.sg.resize(o->ns);
    for (int64_t s = 0; s < o->ns; ++s) {
        const double fx = std::floor((o->sx[s] - w.gx0) / w.gdx), fy = std::floor((o->sy[s] - w.gy0) / w.gdy);
        int g = -1;
        if (fx >= 0 && fx < w.gnx && fy >= 0 && fy < w.gny) g = (int)fy * w.gnx + (int)fx;
        const double phi = g >= 0 ? w.theta[g] : o->P.por;
        w.sw[s] = (1.0 - phi) * (o->sm[s] / o->srho[s]);
        w.sg[s] = g;
    }
}

double wc_porosity(const Orc* o, int64_t i) {
    const double H2 = 4.0 * o->P.h * o->P.h;
    double f = 0.0;
    for (int64_t s = 0; s < o->ns; ++s) {
        const double dx = o->x[i] - o->sx[s], dy = o->y[i] - o->sy[s], d2 = dx * dx + dy * dy;
        if (d2 < H2) f += o->wc.sw[s] * wc_W(o, std::sqrt(d2));
    }
    return 1.0 - f;
}

void wc_eta(const Orc* o, const double* x, const double* rho, double* eta) {
    const WcOrc& w = o->wc;
    for (int p = 0; p < w.np; ++p) {
        double s = 0.0;
        for (int64_t i = 0; i < o->n; ++i) {
            if (!fluid(o, i)) continue;
            const double q = std::fabs(x[i] - w.xp[p]) / w.R1;
            if (q < 1.0) s += (w.mass[i] / rho[i]) * wc_w1(q, w.R1);
        }
        eta[p] = s - w.depth;
    }
}

// one forward step of the state in o->x, y, vx, vy, rho
void wc_step(Orc* o, std::vector<double>& nbuf, std::vector<double>& Pbuf) {
    WcOrc& w = o->wc;
    const int64_t n = o->n;
    const double dt = o->dt, lam = o->P.lam, g = o->P.g, d = o->P.d50;
    o->t += dt;
    orc_piston(static_cast<orc_ctx*>(o));
    bin_particles(o);
    orc_neighbour(static_cast<orc_ctx*>(o));
    WcPre q;
    wc_pre(o, o->y.data(), o->rho.data(), q);
    nbuf.assign(n, 1.0);
    Pbuf.assign(2 * n, 0.0);
    std::vector<double> nx(n), ny(n), nvx(n), nvy(n), nr(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        nx[i] = o->x[i]; ny[i] = o->y[i]; nvx[i] = o->vx[i]; nvy[i] = o->vy[i]; nr[i] = o->rho[i];
        if (!fluid(o, i)) continue;
        const double ni = wc_porosity(o, i);
        nbuf[i] = ni;
        const double rti = q.rt[i], pri = q.pp[i] / (rti * rti);
        double Dr = 0, Px = 0, Py = 0, Vx = 0, Vy = 0;
        for (int64_t e = o->nb_off[i]; e < o->nb_off[i + 1]; ++e) {
            const int64_t j = o->nb_id[e];
            const double dx = o->x[i] - o->x[j], dy = o->y[i] - o->y[j];
            const double r2 = dx * dx + dy * dy, r = std::sqrt(r2);
            const double F = wc_F(o, r), G = F * r2 / (r2 + lam);
            const double mj = w.mass[j], Vj = mj / q.rt[j];
            const double dvx = o->vx[i] - o->vx[j], dvy = o->vy[i] - o->vy[j];
            Dr += mj * (rti / q.rt[j]) * F * (dvx * dx + dvy * dy);
            Dr += w.c2 * (q.rt[j] - rti - q.rh[j] + q.rh[i]) * (-G) * Vj;
            const double pc = mj * (pri + q.pp[j] / (q.rt[j] * q.rt[j])) * F;
            Px += pc * dx;
            Py += pc * dy;
            Vx += 2.0 * w.nu * Vj * G * dvx;
            Vy += 2.0 * w.nu * Vj * G * dvy;
        }
        const double ax = -ni * Px + Vx, ay = -ni * Py + Vy + ni * g;
        const double vxi = o->vx[i], vyi = o->vy[i];
        const double vm = std::sqrt(vxi * vxi + vyi * vyi), on = 1.0 - ni, n3 = ni * ni * ni;
        const double R = -w.nu * w.alpha * on * on / (n3 * d * d) - w.beta * vm * on / (n3 * d);
        const double D = 1.0 - dt * R * ni;
        nvx[i] = (vxi + dt * ax) / D;
        nvy[i] = (vyi + dt * ay) / D;
        nx[i] = o->x[i] + dt * nvx[i] / ni;
        ny[i] = o->y[i] + dt * nvy[i] / ni;
        nr[i] = rti + dt * Dr;
        Pbuf[i] = Px;
        Pbuf[n + i] = Py;
    }
    o->x.swap(nx); o->y.swap(ny); o->vx.swap(nvx); o->vy.swap(nvy); o->rho.swap(nr);
}

void wc_store(const Orc* o, std::vector<double>& dst) {
    const int64_t n = o->n;
    dst.resize(5 * n);
    std::copy(o->x.begin(), o->x.end(), dst.begin());
    std::copy(o->y.begin(), o->y.end(), dst.begin() + n);
    std::copy(o->vx.begin(), o->vx.end(), dst.begin() + 2 * n);
    std::copy(o->vy.begin(), o->vy.end(), dst.begin() + 3 * n);
    std::copy(o->rho.begin(), o->rho.end(), dst.begin() + 4 * n);
}

void wc_restore(Orc* o, const std::vector<double>& src) {
    const int64_t n = o->n;
    std::copy(src.begin(), src.begin() + n, o->x.begin());
    std::copy(src.begin() + n, src.begin() + 2 * n, o->y.begin());
    std::copy(src.begin() + 2 * n, src.begin() + 3 * n, o->vx.begin());
    std::copy(src.begin() + 3 * n, src.begin() + 4 * n, o->vy.begin());
    std::copy(src.begin() + 4 * n, src.begin() + 5 * n, o->rho.begin());
}

}  // namespace

extern "C" {

int orc_wcsph_setup(orc_ctx* o, const bsc_wcsph_params* p) {
    if (!o || !p) return BSC_E_INVALID;
    const int G = p->grid_nx * p->grid_ny;
    if (p->grid_nx < 1 || p->grid_ny < 1 || G > BSC_WCSPH_MAX_GRID || !p->grid_por || !(p->grid_dx > 0) ||
        !(p->grid_dy > 0) || p->nprobe < 1 || p->nprobe > BSC_WCSPH_MAX_PROBES || !(p->c0 > 0) || !(p->gamma > 0))
        return fail(o, BSC_E_INVALID, "wcsph_setup: bad parameters");
    WcOrc& w = o->wc;
    w = WcOrc();
    w.on = true;
    w.rho0 = o->P.rho0;
    w.gam = p->gamma;
    w.B = o->P.rho0 * p->c0 * p->c0 / p->gamma;
    w.grav_c = std::fabs(o->P.g) * p->gamma / (p->c0 * p->c0);
    w.ys = p->surface_y;
    w.c2 = p->delta * 2.0 * o->P.h * p->c0;
    w.nu = p->nu;
    w.alpha = p->alpha;
    w.beta = p->beta;
    w.gx0 = p->grid_x0; w.gy0 = p->grid_y0; w.gdx = p->grid_dx; w.gdy = p->grid_dy;
    w.gnx = p->grid_nx; w.gny = p->grid_ny;
    w.np = p->nprobe;
    for (int k = 0; k < w.np; ++k) w.xp[k] = p->probe_x[k];
    w.R1 = 2.0 * o->P.h;
    w.depth = p->probe_depth;
    w.theta.assign(p->grid_por, p->grid_por + G);
    const int64_t n = o->n;
    w.mass.resize(n);
    for (int64_t i = 0; i < n; ++i) {
        const double s = 1.0 + w.grav_c * (w.ys - o->y[i]);
        const double r = o->y[i] < w.ys ? w.rho0 * std::pow(s, 1.0 / w.gam) : w.rho0;
        o->rho[i] = r;
        w.mass[i] = r * o->P.dl * o->P.dl;
    }
    wc_store(o, w.init);
    w.t0 = o->t;
    wc_solids(o);
    return BSC_OK;
}

int orc_wcsph_set_params(orc_ctx* o, double alpha, double beta, const double* grid) {
    if (!o || !o->wc.on) return o ? fail(o, BSC_E_INVALID, "wcsph_set_params before wcsph_setup") : BSC_E_INVALID;
    o->wc.alpha = alpha;
    o->wc.beta = beta;
    if (grid) std::copy(grid, grid + o->wc.gnx * o->wc.gny, o->wc.theta.begin());
    wc_solids(o);
    return BSC_OK;
}

int orc_wcsph_forward(orc_ctx* o, int32_t nsteps, int32_t every, double* eta) {
    if (!o || !o->wc.on) return o ? fail(o, BSC_E_INVALID, "wcsph_forward before wcsph_setup") : BSC_E_INVALID;
    if (nsteps < 1 || every < 1 || !eta) return fail(o, BSC_E_INVALID, "wcsph_forward: bad arguments");
    WcOrc& w = o->wc;
    wc_restore(o, w.init);
    o->t = w.t0;
    w.nsteps = nsteps;
    w.st.assign(nsteps + 1, {});
    w.nn.assign(nsteps, {});
    w.PP.assign(nsteps, {});
    w.off.assign(nsteps, {});
    w.ids.assign(nsteps, {});
    for (int s = 0; s < nsteps; ++s) {
        wc_store(o, w.st[s]);
        wc_step(o, w.nn[s], w.PP[s]);
        w.off[s] = o->nb_off;
        w.ids[s] = o->nb_id;
        wc_eta(o, o->x.data(), o->rho.data(), eta + (int64_t)s * w.np);
    }
    wc_store(o, w.st[nsteps]);
    return BSC_OK;
}

int orc_wcsph_adjoint(orc_ctx* o, const double* dJ, double* grad) {
    if (!o || !o->wc.on) return o ? fail(o, BSC_E_INVALID, "wcsph_adjoint before wcsph_setup") : BSC_E_INVALID;
    WcOrc& w = o->wc;
    if (w.nsteps < 1 || !dJ || !grad) return fail(o, BSC_E_INVALID, "wcsph_adjoint: run wcsph_forward first");
    const int64_t n = o->n;
    const int G = w.gnx * w.gny;
    const double dt = o->dt, lam = o->P.lam, g = o->P.g, d = o->P.d50, H2 = 4.0 * o->P.h * o->P.h;
    std::fill(grad, grad + 2 + G, 0.0);
    // adjoint of the state after the current step: x y vx vy rho
    std::vector<double> L(5 * n, 0.0), Ln(5 * n);
    std::vector<double> lax(n), lay(n), lD(n), ln(n), ort(n), op(n);
    for (int s = w.nsteps - 1; s >= 0; --s) {
        const double* S0 = w.st[s].data();
        const double* S1 = w.st[s + 1].data();
        const double *x = S0, *y = S0 + n, *vx = S0 + 2 * n, *vy = S0 + 3 * n, *rho = S0 + 4 * n;
        // the loss term of the state after step s
        for (int64_t i = 0; i < n; ++i) {
            if (!fluid(o, i)) continue;
            const double V = w.mass[i] / S1[4 * n + i];
            for (int p = 0; p < w.np; ++p) {
                const double dd = S1[i] - w.xp[p], q = std::fabs(dd) / w.R1;
                if (q >= 1.0) continue;
                L[i] += dJ[(int64_t)s * w.np + p] * V * wc_w1q(q, w.R1) * (dd >= 0 ? 1.0 : -1.0) / w.R1;
                L[4 * n + i] += dJ[(int64_t)s * w.np + p] * (-V / S1[4 * n + i]) * wc_w1(q, w.R1);
            }
        }
        WcPre q;
        wc_pre(o, y, rho, q);
        const double* nb = w.nn[s].data();
        const double* P = w.PP[s].data();
        // per-particle part: position update, drag, the porosity's direct roles
        for (int64_t i = 0; i < n; ++i) {
            Ln[i] = Ln[n + i] = Ln[2 * n + i] = Ln[3 * n + i] = 0.0;
            lax[i] = lay[i] = lD[i] = ln[i] = ort[i] = op[i] = 0.0;
            if (!fluid(o, i)) continue;
            const double ni = nb[i], vxn = S1[2 * n + i], vyn = S1[3 * n + i];
            const double vm = std::sqrt(vx[i] * vx[i] + vy[i] * vy[i]), on = 1.0 - ni, n3 = ni * ni * ni;
            const double R = -w.nu * w.alpha * on * on / (n3 * d * d) - w.beta * vm * on / (n3 * d);
            const double D = 1.0 - dt * R * ni;
            // x' = x + dt v'/n
            Ln[i] = L[i];
            Ln[n + i] = L[n + i];
            const double lvx1 = L[2 * n + i] + dt * L[i] / ni, lvy1 = L[3 * n + i] + dt * L[n + i] / ni;
            double lni = -dt * (L[i] * vxn + L[n + i] * vyn) / (ni * ni);
            // v' = (v + dt a) / D
            lax[i] = dt * lvx1 / D;
            lay[i] = dt * lvy1 / D;
            const double lDD = -(lvx1 * vxn + lvy1 * vyn) / D;
            // D = 1 - dt R n
            const double lR = -dt * ni * lDD;
            lni += -dt * R * lDD;
            const double dRdn = -w.nu * w.alpha / (d * d) * (-2.0 * on / n3 - 3.0 * on * on / (n3 * ni)) -
                                w.beta * vm / d * (-1.0 / n3 - 3.0 * on / (n3 * ni));
            lni += lR * dRdn;
            Ln[2 * n + i] = lvx1 / D;
            Ln[3 * n + i] = lvy1 / D;
            if (vm > 0.0) {
                const double c = lR * (-w.beta * on / (n3 * d)) / vm;
                Ln[2 * n + i] += c * vx[i];
                Ln[3 * n + i] += c * vy[i];
            }
            grad[0] += lR * (-w.nu * on * on / (n3 * d * d));
            grad[1] += lR * (-vm * on / (n3 * d));
            // a = -n P + visc + n g
            lni += lax[i] * (-P[i]) + lay[i] * (-P[n + i] + g);
            ln[i] = lni;
            // rho' = rt + dt Drho
            lD[i] = dt * L[4 * n + i];
            ort[i] = L[4 * n + i];
        }
        // pair terms of particle i's sums, scattered to both ends
        const std::vector<int64_t>& off = w.off[s];
        const std::vector<int64_t>& ids = w.ids[s];
        for (int64_t i = 0; i < n; ++i) {
            if (!fluid(o, i)) continue;
            const double rti = q.rt[i], pi_ = q.pp[i], ni = nb[i];
            for (int64_t e = off[i]; e < off[i + 1]; ++e) {
                const int64_t j = ids[e];
                const bool fj = fluid(o, j);
                const double dx = x[i] - x[j], dy = y[i] - y[j];
                const double r2 = dx * dx + dy * dy, r = std::sqrt(r2);
                const double F = wc_F(o, r), dF = wc_dF(o, r), den = r2 + lam;
                const double G_ = F * r2 / den, dG = dF * r2 / den + F * 2.0 * r * lam / (den * den);
                const double rtj = q.rt[j], pj = q.pp[j], mj = w.mass[j], Vj = mj / rtj;
                const double dvx = vx[i] - vx[j], dvy = vy[i] - vy[j], dvd = dvx * dx + dvy * dy;
                double gx = 0, gy = 0;  // adjoint of d = x_i - x_j
                // continuity: m_j (rt_i / rt_j) F (v_ij . d)
                {
                    const double c = mj * rti / rtj, l = lD[i];
                    ort[i] += l * (mj / rtj) * F * dvd;
                    if (fj) ort[j] += l * (-mj * rti / (rtj * rtj)) * F * dvd;
                    Ln[2 * n + i] += l * c * F * dx;
                    Ln[3 * n + i] += l * c * F * dy;
                    if (fj) {
                        Ln[2 * n + j] -= l * c * F * dx;
                        Ln[3 * n + j] -= l * c * F * dy;
                    }
                    gx += l * c * (F * dvx + dF / r * dvd * dx);
                    gy += l * c * (F * dvy + dF / r * dvd * dy);
                }
                // delta term: c2 (rt_j - rt_i - rh_j + rh_i) (-G) V_j
                {
                    const double l = lD[i], del = rtj - rti - q.rh[j] + q.rh[i];
                    ort[i] += l * w.c2 * G_ * Vj;
                    if (fj) ort[j] += l * w.c2 * (-G_) * Vj * (1.0 - del / rtj);
                    Ln[n + i] += l * w.c2 * q.drh[i] * (-G_) * Vj;
                    if (fj) Ln[n + j] += l * w.c2 * q.drh[j] * G_ * Vj;
                    gx += l * w.c2 * del * (-dG / r) * Vj * dx;
                    gy += l * w.c2 * del * (-dG / r) * Vj * dy;
                }
                // pressure: -n_i m_j (p_i / rt_i^2 + p_j / rt_j^2) F d
                {
                    const double lad = lax[i] * dx + lay[i] * dy;
                    const double pc = mj * (pi_ / (rti * rti) + pj / (rtj * rtj));
                    gx += -ni * pc * (F * lax[i] + dF / r * lad * dx);
                    gy += -ni * pc * (F * lay[i] + dF / r * lad * dy);
                    op[i] += -ni * mj / (rti * rti) * F * lad;
                    ort[i] += -ni * mj * (-2.0 * pi_ / (rti * rti * rti)) * F * lad;
                    if (fj) {
                        op[j] += -ni * mj / (rtj * rtj) * F * lad;
                        ort[j] += -ni * mj * (-2.0 * pj / (rtj * rtj * rtj)) * F * lad;
                    }
                }
                // viscosity: 2 nu V_j G (v_i - v_j)
                {
                    const double c = 2.0 * w.nu * Vj * G_, ldv = lax[i] * dvx + lay[i] * dvy;
                    Ln[2 * n + i] += c * lax[i];
                    Ln[3 * n + i] += c * lay[i];
                    if (fj) {
                        Ln[2 * n + j] -= c * lax[i];
                        Ln[3 * n + j] -= c * lay[i];
                        ort[j] += 2.0 * w.nu * (-mj / (rtj * rtj)) * G_ * ldv;
                    }
                    gx += 2.0 * w.nu * Vj * ldv * dG / r * dx;
                    gy += 2.0 * w.nu * Vj * ldv * dG / r * dy;
                }
                Ln[i] += gx;
                Ln[n + i] += gy;
                if (fj) {
                    Ln[j] -= gx;
                    Ln[n + j] -= gy;
                }
            }
            // porosity n_i = 1 - sum_s (1 - phi_s) V_s W(r_is)
            for (int64_t sd = 0; sd < o->ns; ++sd) {
                const double dx = x[i] - o->sx[sd], dy = y[i] - o->sy[sd], d2 = dx * dx + dy * dy;
                if (!(d2 < H2)) continue;
                const double r = std::sqrt(d2), F = wc_F(o, r);
                Ln[i] += ln[i] * (-w.sw[sd] * F * dx);
                Ln[n + i] += ln[i] * (-w.sw[sd] * F * dy);
                if (w.sg[sd] >= 0) grad[2 + w.sg[sd]] += ln[i] * (o->sm[sd] / o->srho[sd]) * wc_W(o, r);
            }
        }
        // pressure of the EOS, then the clamp rt = max(rho, rho0)
        for (int64_t i = 0; i < n; ++i) {
            if (!fluid(o, i)) {
                Ln[4 * n + i] = 0.0;
                continue;
            }
            const double rt = q.rt[i];
            ort[i] += op[i] * w.B * w.gam * std::pow(rt / w.rho0, w.gam - 1.0) / w.rho0;
            Ln[4 * n + i] = rho[i] >= w.rho0 ? ort[i] : 0.0;
        }
        L.swap(Ln);
    }
    return BSC_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// particles leaving and entering: internal.f90:544-614 remove_buffer1/2, the
// outflow cut-off of cellshiftalt (integrator.f90:55-110) and the appends of
// insert_buffer1/2 (internal.f90:475-542).  The state is rebuilt through
// download and upload, which keeps the survivors' order.
// ---------------------------------------------------------------------------
namespace {

struct OrcHost {
    std::vector<std::vector<double>> f;
    std::vector<double> L;
    std::vector<int8_t> tid;
    std::vector<uint8_t> fl;
    bsc_state_view v{};
};

double* bsc_state_view::*const ORC_DBL[] = {
    &bsc_state_view::x,       &bsc_state_view::y,      &bsc_state_view::vx,    &bsc_state_view::vy,
    &bsc_state_view::xs,      &bsc_state_view::ys,     &bsc_state_view::vxs,   &bsc_state_view::vys,
    &bsc_state_view::p,       &bsc_state_view::rho,    &bsc_state_view::oden,  &bsc_state_view::mass,
    &bsc_state_view::porosity, &bsc_state_view::gradvx, &bsc_state_view::nut,  &bsc_state_view::tke,
    &bsc_state_view::resist,  &bsc_state_view::varts,  &bsc_state_view::vel,   &bsc_state_view::xrest,
    &bsc_state_view::con,     &bsc_state_view::ovol};
constexpr int ORC_ND = sizeof(ORC_DBL) / sizeof(ORC_DBL[0]);

void host_resize(OrcHost& h, int64_t n) {
    h.f.assign(ORC_ND, std::vector<double>(n));
    h.L.assign(4 * n, 0.0);
    h.tid.assign(n, 0);
    h.fl.assign(n, 0);
    h.v = bsc_state_view{};
    h.v.n = n;
    for (int k = 0; k < ORC_ND; ++k) h.v.*ORC_DBL[k] = h.f[k].data();
    h.v.L = h.L.data();
    h.v.tid = h.tid.data();
    h.v.flags = h.fl.data();
}

}  // namespace

extern "C" {

int orc_remove_particles(orc_ctx* o, int32_t rule, double a, double b, int64_t* removed_out) {
    if (!o) return BSC_E_INVALID;
    if (rule < BSC_REMOVE_BUFFER_RIGHT || rule > BSC_REMOVE_OUTFLOW)
        return fail(o, BSC_E_INVALID, "remove_particles: unknown rule");
    const int64_t n = o->n;
    std::vector<char> keep(n);
    int64_t kept = 0;
    for (int64_t i = 0; i < n; ++i) {
        const bool buf = has(o->flags[i], BSC_FLAG_BUFFER);
        bool rm = false;
        if (rule == BSC_REMOVE_BUFFER_RIGHT) rm = buf && o->x[i] >= a;   // internal.f90:559-560
        if (rule == BSC_REMOVE_BUFFER_LEFT) rm = buf && o->x[i] <= a;    // internal.f90:595-596
        if (rule == BSC_REMOVE_OUTFLOW)                                 // integrator.f90:60-61
            rm = o->tid[i] == BSC_TID_FLUID && !buf && o->x[i] <= a && o->y[i] > b;
        keep[i] = !rm;
        kept += !rm;
    }
    if (removed_out) *removed_out = n - kept;
    if (kept == 0) return fail(o, BSC_E_INVALID, "remove_particles: the rule removes every particle");
    if (kept == n) {
        o->have_lists = o->have_csr = false;
        return BSC_OK;
    }
    OrcHost all, out;
    host_resize(all, n);
    orc_download_state(o, &all.v);
    host_resize(out, kept);
    for (int64_t i = 0, d = 0; i < n; ++i) {
        if (!keep[i]) continue;
        for (int k = 0; k < ORC_ND; ++k) out.f[k][d] = all.f[k][i];
        for (int q = 0; q < 4; ++q) out.L[4 * d + q] = all.L[4 * i + q];
        out.tid[d] = all.tid[i];
        out.fl[d] = all.fl[i];
        ++d;
    }
    return orc_upload_state(o, &out.v);
}

int orc_particle_count(const orc_ctx* o, int64_t* n) {
    if (!o || !n) return BSC_E_INVALID;
    *n = o->n;
    return BSC_OK;
}

int orc_insert_particles(orc_ctx* o, const bsc_state_view* a) {
    if (!o || !a || a->n <= 0) return BSC_E_INVALID;
    const int64_t n = o->n, m = a->n, t = n + m;
    OrcHost all;
    host_resize(all, t);
    all.v.n = n;
    orc_download_state(o, &all.v);
    for (int k = 0; k < ORC_ND; ++k) {
        const double* src = a->*ORC_DBL[k];
        for (int64_t q = 0; q < m; ++q) {
            double v = 0.0;
            if (src) v = src[q];
            else if (ORC_DBL[k] == &bsc_state_view::porosity) v = 1.0;
            else if (ORC_DBL[k] == &bsc_state_view::xrest) v = a->x[q];
            else if (ORC_DBL[k] == &bsc_state_view::ovol) v = a->mass[q] / a->oden[q];
            all.f[k][n + q] = v;
        }
    }
    for (int64_t q = 0; q < m; ++q) {
        for (int r = 0; r < 4; ++r) all.L[4 * (n + q) + r] = a->L ? a->L[4 * q + r] : (r == 0 || r == 3 ? 1.0 : 0.0);
        all.tid[n + q] = a->tid[q];
        all.fl[n + q] = a->flags[q];
    }
    all.v.n = t;
    return orc_upload_state(o, &all.v);
}

}  // extern "C"
