// buffers.cu -- particles leaving and entering the state: the open-boundary
// buffers (internal.f90:475-614) and the outflow cut-off of cellshiftalt
// (integrator.f90:55-110).
//
// Removal is a device compaction: keep flags per row and per id, two
// exclusive scans, one gather of every field into the reorder buffer.  Rows
// keep their order and ids stay dense and in upload order (the survivors'
// ids are renumbered 0..n'-1 in their old order), so a download still
// returns the host's arrays minus the removed particles.
//
// Insertion appends particles with the ids after the last.  It is a timed
// event of the reference (every ins_1 / ins_2 of simulated time), so the
// state goes down to the host and back up with the new particles, into
// arrays with a quarter of headroom.
#include <cstring>
#include <vector>

#include "bsc_internal.cuh"

struct bsc_ctx : bsc::Ctx {};  // the same definition as in api.cu

namespace bsc {
namespace {

// which particles a rule removes
__device__ __forceinline__ bool removed(int rule, double a, double b, int8_t tid, uint8_t fl, double x, double y) {
    const bool buf = fl & BSC_FLAG_BUFFER;
    switch (rule) {
        case BSC_REMOVE_BUFFER_RIGHT:  // remove_buffer1 keeps buffer particles with x < rv_buf_r
            return buf && x >= a;
        case BSC_REMOVE_BUFFER_LEFT:  // remove_buffer2 keeps buffer particles with x > rv_buf_l
            return buf && x <= a;
        case BSC_REMOVE_OUTFLOW:  // cellshiftalt keeps x > xlcutoff, buffers, and y <= ytcutoff
            return tid == BSC_TID_FLUID && !buf && x <= a && y > b;
        default:
            return false;
    }
}

__global__ void k_keep(int64_t n, State S, int rule, double a, double b, int32_t* __restrict__ keep_row,
                       int32_t* __restrict__ keep_id) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t k = removed(rule, a, b, S.tid[i], S.flags[i], S.x[i], S.y[i]) ? 0 : 1;
    keep_row[i] = k;
    keep_id[S.id[i]] = k;
}

__global__ void k_compact(int64_t n, FieldPtrs src, FieldPtrs dst, State S, State D,
                          const int32_t* __restrict__ keep_row, const int32_t* __restrict__ pos_row,
                          const int32_t* __restrict__ pos_id) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n || !keep_row[i]) return;
    const int32_t d = pos_row[i];
    for (int f = 0; f < N_DBL_FIELDS; ++f) dst.d[f][d] = src.d[f][i];
    D.tid[d] = S.tid[i];
    D.flags[d] = S.flags[i];
    D.id[d] = pos_id[S.id[i]];
}

}  // namespace
}  // namespace bsc

using namespace bsc;

extern "C" {

int bsc_remove_particles(bsc_ctx* c, int32_t rule, double a, double b, int64_t* removed_out) {
    if (!c) return BSC_E_INVALID;
    if (!c->have_state) return set_err(c, BSC_E_INVALID, "remove_particles before upload_state");
    if (rule < BSC_REMOVE_BUFFER_RIGHT || rule > BSC_REMOVE_OUTFLOW)
        return set_err(c, BSC_E_INVALID, "remove_particles: unknown rule");
    const int64_t n = c->n;
    // scratch: the cell-list arrays (rebuilt below) and the L staging buffer
    int32_t *keep_row = c->pcell, *pos_row = c->pslot, *keep_id = c->sorted, *pos_id = (int32_t*)c->lstage;
    const unsigned g = blocks_for(n, 256);
    k_keep<<<g, 256, 0, c->stream>>>(n, c->S, rule, a, b, keep_row, keep_id);
    BSC_LAUNCH(c);
    int rc;
    if ((rc = scan_exclusive(c, keep_row, pos_row, (int)n)) || (rc = scan_exclusive(c, keep_id, pos_id, (int)n)))
        return rc;
    int32_t h[2];
    BSC_CUDA(c, cudaMemcpyAsync(&h[0], pos_row + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaMemcpyAsync(&h[1], keep_row + n - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaStreamSynchronize(c->stream));
    const int64_t kept = (int64_t)h[0] + h[1];
    if (removed_out) *removed_out = n - kept;
    if (kept == 0) return set_err(c, BSC_E_INVALID, "remove_particles: the rule removes every particle");
    if (kept < n) {
        k_compact<<<g, 256, 0, c->stream>>>(n, fields_of(c->S), fields_of(c->S2), c->S, c->S2, keep_row, pos_row,
                                            pos_id);
        BSC_LAUNCH(c);
        std::swap(c->S, c->S2);
        c->n = kept;
        drop_graphs(c);  // captured for the old row count
        wc_free(c);      // the WCSPH record is per particle
        // the neighbour lists index the old rows: empty until the next search
        BSC_CUDA(c, cudaMemsetAsync(c->cnt, 0, sizeof(int32_t) * kept, c->stream));
        c->have_lists = c->have_csr = false;
    }
    // the cell lists held the scratch: rebuild them for the current rows
    return cells_build(c, false);
}

int bsc_particle_count(const bsc_ctx* c, int64_t* n) {
    if (!c || !n) return BSC_E_INVALID;
    *n = c->n;
    return BSC_OK;
}

int bsc_insert_particles(bsc_ctx* c, const bsc_state_view* a) {
    if (!c || !a) return BSC_E_INVALID;
    if (!c->have_state) return set_err(c, BSC_E_INVALID, "insert_particles before upload_state");
    if (a->n <= 0 || !a->x || !a->y || !a->vx || !a->vy || !a->p || !a->rho || !a->oden || !a->mass || !a->tid ||
        !a->flags)
        return set_err(c, BSC_E_INVALID, "insert_particles: missing required field or bad n");
    const int64_t n = c->n, m = a->n, t = n + m;
    // every field of the view, the current state then the new particles
    double* bsc_state_view::*dbl[] = {&bsc_state_view::x,      &bsc_state_view::y,       &bsc_state_view::vx,
                                      &bsc_state_view::vy,     &bsc_state_view::xs,      &bsc_state_view::ys,
                                      &bsc_state_view::vxs,    &bsc_state_view::vys,     &bsc_state_view::p,
                                      &bsc_state_view::rho,    &bsc_state_view::oden,    &bsc_state_view::mass,
                                      &bsc_state_view::porosity, &bsc_state_view::gradvx, &bsc_state_view::nut,
                                      &bsc_state_view::tke,    &bsc_state_view::resist,  &bsc_state_view::varts,
                                      &bsc_state_view::vel,    &bsc_state_view::xrest,   &bsc_state_view::con,
                                      &bsc_state_view::ovol};
    constexpr int ND = sizeof(dbl) / sizeof(dbl[0]);
    std::vector<std::vector<double>> f(ND, std::vector<double>(t));
    std::vector<double> L(4 * t);
    std::vector<int8_t> tid(t);
    std::vector<uint8_t> fl(t);
    bsc_state_view v{};
    v.n = n;
    for (int k = 0; k < ND; ++k) v.*dbl[k] = f[k].data();
    v.L = L.data();
    v.tid = tid.data();
    v.flags = fl.data();
    int rc = bsc_download_state(c, &v);
    if (rc) return rc;
    for (int k = 0; k < ND; ++k) {
        double* dst = f[k].data() + n;
        const double* src = a->*dbl[k];
        if (src) {
            std::memcpy(dst, src, sizeof(double) * m);
        } else if (dbl[k] == &bsc_state_view::porosity) {
            for (int64_t q = 0; q < m; ++q) dst[q] = 1.0;
        } else if (dbl[k] == &bsc_state_view::xrest) {
            std::memcpy(dst, a->x, sizeof(double) * m);
        } else if (dbl[k] == &bsc_state_view::ovol) {
            for (int64_t q = 0; q < m; ++q) dst[q] = a->mass[q] / a->oden[q];  // internal.f90:498: ovol = fmass / rho
        } else {
            std::memset(dst, 0, sizeof(double) * m);
        }
    }
    if (a->L) {
        std::memcpy(L.data() + 4 * n, a->L, sizeof(double) * 4 * m);
    } else {
        for (int64_t q = n; q < t; ++q) {
            L[4 * q] = 1.0;
            L[4 * q + 1] = L[4 * q + 2] = 0.0;
            L[4 * q + 3] = 1.0;
        }
    }
    std::memcpy(tid.data() + n, a->tid, m);
    std::memcpy(fl.data() + n, a->flags, m);
    v.n = t;
    if (c->cap < t) c->cap_hint = t + t / 4;  // room for the next insertions
    return bsc_upload_state(c, &v);
}

}  // extern "C"
