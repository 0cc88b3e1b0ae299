// snapshot.cu -- the reference's text snapshots (output.f90:188-234
// `combined`): fluid/fluid_<k>.txt, buffer/buffer_<k>.txt and
// fluid/dead_<k>.txt, one line per fluid particle,
//   x, y, p (F10.3), vx, vy (ES10.3), con + 0.5 (F10.5), single spaces.
//
// Asynchronous: the fields are gathered into id order on the device and
// copied into pinned host buffers on the context stream, so later steps are
// ordered after the copy; a host thread waits for the copy, formats the
// lines in parallel chunks and writes the files while the GPU steps on.
// Lines are in id (upload) order; the reference's order is its cell-slot
// history, which no other code reads.
#include <sys/stat.h>

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "bsc_internal.cuh"

struct bsc_ctx : bsc::Ctx {};  // the same definition as in api.cu

namespace bsc {

struct SnapState {
    std::thread worker;
    bool busy = false;
    int rc = BSC_OK;
    std::string err;
    int64_t cap = 0;
    double *h = nullptr, *d = nullptr;     // pinned / device: x y p vx vy con+0.5 (6 n), id order
    uint8_t *hf = nullptr, *df = nullptr;  // pinned / device: tid, flags (2 n)
    cudaEvent_t ev = nullptr;
};

namespace {

constexpr int NSF = 6;

__global__ void k_snap_gather(int64_t n, State S, const int32_t* __restrict__ id, double* __restrict__ out,
                              uint8_t* __restrict__ outf) {
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int64_t d = id[k];
    out[d] = S.x[k];
    out[n + d] = S.y[k];
    out[2 * n + d] = S.p[k];
    out[3 * n + d] = S.vx[k];
    out[4 * n + d] = S.vy[k];
    out[5 * n + d] = S.con[k] + 0.50;
    outf[d] = (uint8_t)S.tid[k];
    outf[n + d] = S.flags[k];
}

// Fortran Fw.d: fixed point, right-justified; asterisks when it does not fit
void fmt_F(char* dst, double v, int w, int d) {
    char buf[64];
    int len = std::snprintf(buf, sizeof buf, "%*.*f", w, d, v);
    if (len > w || !std::isfinite(v)) {
        if (!std::isfinite(v)) {
            len = std::snprintf(buf, sizeof buf, "%*s", w, std::isnan(v) ? "NaN" : (v > 0 ? "Infinity" : "-Infinity"));
            if (len <= w) {
                std::memcpy(dst, buf, w);
                return;
            }
        }
        std::memset(dst, '*', w);
        return;
    }
    std::memcpy(dst, buf, w);
}

// Fortran ESw.d: one nonzero digit before the point, exponent E+dd, or +ddd
// without the E for exponents of three digits
void fmt_ES(char* dst, double v, int w, int d) {
    if (!std::isfinite(v)) {
        fmt_F(dst, v, w, d);
        return;
    }
    char buf[64];
    std::snprintf(buf, sizeof buf, "%.*E", d, v);
    char* e = std::strchr(buf, 'E');
    const int ex = std::atoi(e + 1);
    *e = '\0';
    char out[64];
    if (std::abs(ex) <= 99)
        std::snprintf(out, sizeof out, "%sE%c%02d", buf, ex < 0 ? '-' : '+', std::abs(ex));
    else
        std::snprintf(out, sizeof out, "%s%c%03d", buf, ex < 0 ? '-' : '+', std::abs(ex));
    const int len = (int)std::strlen(out);
    if (len > w) {
        std::memset(dst, '*', w);
        return;
    }
    std::memset(dst, ' ', w - len);
    std::memcpy(dst + (w - len), out, len);
}

constexpr int LINE = 10 * 6 + 5 + 1;  // six fields, five 1X spaces, newline

void fmt_line(char* p, const double* f) {
    fmt_F(p, f[0], 10, 3);
    p[10] = ' ';
    fmt_F(p + 11, f[1], 10, 3);
    p[21] = ' ';
    fmt_F(p + 22, f[2], 10, 3);
    p[32] = ' ';
    fmt_ES(p + 33, f[3], 10, 3);
    p[43] = ' ';
    fmt_ES(p + 44, f[4], 10, 3);
    p[54] = ' ';
    fmt_F(p + 55, f[5], 10, 5);
    p[65] = '\n';
}

// which file a particle goes to (output.f90:201-224): 0 fluid, 1 buffer, 2 dead, -1 none
int file_of(uint8_t tid, uint8_t fl) {
    if (tid != BSC_TID_FLUID) return -1;
    const bool buf = fl & BSC_FLAG_BUFFER, dead = fl & BSC_FLAG_DEAD;
    if (!buf && !dead) return 0;
    if (buf && !dead) return 1;
    if (dead && !buf) return 2;
    return -1;
}

int make_dir(const std::string& d) {
    if (mkdir(d.c_str(), 0777) == 0 || errno == EEXIST) return 0;
    return -1;
}

void write_files(SnapState* s, int64_t n, std::string dir, int64_t index) {
    const double* h = s->h;
    const uint8_t *tid = s->hf, *fl = s->hf + n;
    const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    std::vector<std::string> chunk[3];
    for (auto& c : chunk) c.assign(nt, std::string());
    std::vector<std::thread> ts;
    for (unsigned t = 0; t < nt; ++t) {
        ts.emplace_back([&, t]() {
            const int64_t a = n * t / nt, b = n * (t + 1) / nt;
            char line[LINE];
            double f[NSF];
            for (int64_t i = a; i < b; ++i) {
                const int k = file_of(tid[i], fl[i]);
                if (k < 0) continue;
                for (int q = 0; q < NSF; ++q) f[q] = h[q * n + i];
                fmt_line(line, f);
                chunk[k][t].append(line, LINE);
            }
        });
    }
    for (auto& t : ts) t.join();
    const std::string sub[3] = {dir + "/fluid", dir + "/buffer", dir + "/fluid"};
    const std::string name[3] = {"fluid_", "buffer_", "dead_"};
    if (make_dir(dir) || make_dir(sub[0]) || make_dir(sub[1])) {
        s->rc = BSC_E_INVALID;
        s->err = "snapshot: cannot create " + dir + "/fluid or " + dir + "/buffer";
        return;
    }
    for (int k = 0; k < 3; ++k) {
        const std::string path = sub[k] + "/" + name[k] + std::to_string(index) + ".txt";
        FILE* fp = std::fopen(path.c_str(), "wb");
        if (!fp) {
            s->rc = BSC_E_INVALID;
            s->err = "snapshot: cannot write " + path;
            return;
        }
        bool ok = true;
        for (const std::string& c : chunk[k]) ok = ok && std::fwrite(c.data(), 1, c.size(), fp) == c.size();
        ok = (std::fclose(fp) == 0) && ok;
        if (!ok) {
            s->rc = BSC_E_INVALID;
            s->err = "snapshot: short write to " + path;
            return;
        }
    }
}

int snap_wait(Ctx* c) {
    SnapState* s = c->snap;
    if (!s || !s->busy) return BSC_OK;
    s->worker.join();
    s->busy = false;
    if (s->rc) {
        const int rc = s->rc;
        s->rc = BSC_OK;
        return set_err(c, rc, s->err);
    }
    return BSC_OK;
}

}  // namespace

void snap_free(Ctx* c) {
    SnapState* s = c->snap;
    if (!s) return;
    if (s->busy) s->worker.join();
    if (s->h) cudaFreeHost(s->h);
    if (s->hf) cudaFreeHost(s->hf);
    if (s->d) cudaFree(s->d);
    if (s->df) cudaFree(s->df);
    if (s->ev) cudaEventDestroy(s->ev);
    delete s;
    c->snap = nullptr;
}

}  // namespace bsc

using namespace bsc;

extern "C" {

int bsc_snapshot_begin(bsc_ctx* c, const char* dir, int64_t index) {
    if (!c || !dir) return BSC_E_INVALID;
    if (!c->have_state) return set_err(c, BSC_E_INVALID, "snapshot before upload_state");
    int rc = snap_wait(c);  // one snapshot in flight: the buffers are reused
    if (rc) return rc;
    if (!c->snap) {
        c->snap = new (std::nothrow) SnapState();
        if (!c->snap) return BSC_E_NOMEM;
        BSC_CUDA(c, cudaEventCreateWithFlags(&c->snap->ev, cudaEventDisableTiming));
    }
    SnapState* s = c->snap;
    const int64_t n = c->n;
    if (s->cap < n) {
        if (s->h) cudaFreeHost(s->h);
        if (s->hf) cudaFreeHost(s->hf);
        if (s->d) cudaFree(s->d);
        if (s->df) cudaFree(s->df);
        s->h = s->d = nullptr;
        s->hf = s->df = nullptr;
        s->cap = 0;
        BSC_CUDA(c, cudaMallocHost((void**)&s->h, sizeof(double) * NSF * n));
        BSC_CUDA(c, cudaMallocHost((void**)&s->hf, 2 * n));
        BSC_CUDA(c, cudaMalloc((void**)&s->d, sizeof(double) * NSF * n));
        BSC_CUDA(c, cudaMalloc((void**)&s->df, 2 * n));
        s->cap = n;
    }
    // gather into id order and copy out, in stream order: the steps queued
    // after this call run after the copy
    k_snap_gather<<<blocks_for(n, 256), 256, 0, c->stream>>>(n, c->S, c->S.id, s->d, s->df);
    BSC_LAUNCH(c);
    BSC_CUDA(c, cudaMemcpyAsync(s->h, s->d, sizeof(double) * NSF * n, cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaMemcpyAsync(s->hf, s->df, 2 * n, cudaMemcpyDeviceToHost, c->stream));
    BSC_CUDA(c, cudaEventRecord(s->ev, c->stream));
    s->rc = BSC_OK;
    s->busy = true;
    const std::string d(dir);
    cudaEvent_t ev = s->ev;
    s->worker = std::thread([s, n, d, index, ev]() {
        if (cudaEventSynchronize(ev) != cudaSuccess) {
            s->rc = BSC_E_CUDA;
            s->err = "snapshot: copy failed";
            return;
        }
        write_files(s, n, d, index);
    });
    return BSC_OK;
}

int bsc_snapshot_wait(bsc_ctx* c) {
    if (!c) return BSC_E_INVALID;
    return snap_wait(c);
}

}  // extern "C"
