// ellop.cuh -- the PPE operator in the neighbour-list (ELL) layout, shared by
// the Krylov solvers (ppe.cu) and the multigrid preconditioner (mg.cu).
#pragma once
#include "bsc_internal.cuh"

namespace bsc {

// grid-stride loop over [0, n)
#define GRID_LOOP(i, n) \
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// The Jacobi-scaled PPE matrix I + N: unit diagonal (not stored), the
// off-diagonals N in the slots of the neighbour lists.
template <typename T>
struct EllOp {
    const T* aval;
    const int32_t* nbr;
    const int32_t* cnt;
    int kmax;
    int unroll = 0;  // 1: eight, then four entries per round (that many gathers in flight)
    const void* key() const { return aval; }
    // the column stride of the ELL layout is 32 slots
    template <typename X, typename A>
    __device__ __forceinline__ A row(int64_t i, const X* __restrict__ x) const {
        A s = (A)x[i];
        const int m = cnt[i];
        const int64_t e0 = ell(i, 0, kmax);
        int k = 0;
        for (; unroll && k + 8 <= m; k += 8) {
            const int64_t e = e0 + (int64_t)k * 32;
            int j[8];
            T a[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                j[u] = nbr[e + 32 * u];
                a[u] = aval[e + 32 * u];
            }
            X xv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) xv[u] = x[j[u]];
#pragma unroll
            for (int u = 0; u < 8; ++u) s += (A)a[u] * (A)xv[u];
        }
        for (; unroll && k + 4 <= m; k += 4) {
            const int64_t e = e0 + (int64_t)k * 32;
            const int j0 = nbr[e], j1 = nbr[e + 32], j2 = nbr[e + 64], j3 = nbr[e + 96];
            const T a0 = aval[e], a1 = aval[e + 32], a2 = aval[e + 64], a3 = aval[e + 96];
            const X x0 = x[j0], x1 = x[j1], x2 = x[j2], x3 = x[j3];
            s += (A)a0 * (A)x0;
            s += (A)a1 * (A)x1;
            s += (A)a2 * (A)x2;
            s += (A)a3 * (A)x3;
        }
        for (; k < m; ++k) {
            const int64_t e = e0 + (int64_t)k * 32;
            s += (A)aval[e] * (A)x[nbr[e]];
        }
        return s;
    }
};

// The V-cycle's FP16 copy of I + N, four bytes an entry: the column as a
// 16-bit offset from the first row of its 32-row slice and the FP16 value,
// one load.  A slice with an offset outside 16 bits (ok == 0; rare under
// Morton order) reads the separate column and FP16 value arrays.  A warp
// covers one slice, so the branch is warp-uniform.
struct EllPack16 {
    const uint32_t* ent;
    const uint8_t* ok;
    const int32_t* nbr;
    const __half* aval;
    const int32_t* cnt;
    int kmax;
    const void* key() const { return ent; }
    template <typename X, typename A>
    __device__ __forceinline__ A row(int64_t i, const X* __restrict__ x) const {
        A s = (A)x[i];
        const int m = cnt[i];
        const int64_t e0 = ell(i, 0, kmax);
        if (ok[i >> 5]) {
            const int64_t b = i & ~(int64_t)31;
            int k = 0;
            for (; k + 8 <= m; k += 8) {
                uint32_t p[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) p[u] = ent[e0 + (int64_t)(k + u) * 32];
                X xv[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) xv[u] = x[b + (int16_t)(p[u] & 0xffffu)];
#pragma unroll
                for (int u = 0; u < 8; ++u) s += (A)__half2float(__ushort_as_half((unsigned short)(p[u] >> 16))) * (A)xv[u];
            }
            for (; k < m; ++k) {
                const uint32_t p = ent[e0 + (int64_t)k * 32];
                s += (A)__half2float(__ushort_as_half((unsigned short)(p >> 16))) * (A)x[b + (int16_t)(p & 0xffffu)];
            }
        } else {
            for (int k = 0; k < m; ++k) {
                const int64_t e = e0 + (int64_t)k * 32;
                s += (A)__half2float(aval[e]) * (A)x[nbr[e]];
            }
        }
        return s;
    }
};

// The mixed path's FP32 copy of I + N: each stored entry's column and value
// packed in one 8-byte word, so an entry is one load (the same 8 bytes per
// entry as separate column and value arrays, half the load instructions).
struct EllPackF {
    const int2* ent;
    const int32_t* cnt;
    int kmax;
    const void* key() const { return ent; }
    template <typename X, typename A>
    __device__ __forceinline__ A row(int64_t i, const X* __restrict__ x) const {
        A s = (A)x[i];
        const int m = cnt[i];
        const int64_t e0 = ell(i, 0, kmax);
        int k = 0;
        for (; k + 8 <= m; k += 8) {
            int2 p[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) p[u] = ent[e0 + (int64_t)(k + u) * 32];
            X xv[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) xv[u] = x[p[u].x];
#pragma unroll
            for (int u = 0; u < 8; ++u) s += (A)__int_as_float(p[u].y) * (A)xv[u];
        }
        for (; k + 4 <= m; k += 4) {
            int2 p[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) p[u] = ent[e0 + (int64_t)(k + u) * 32];
            X xv[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) xv[u] = x[p[u].x];
#pragma unroll
            for (int u = 0; u < 4; ++u) s += (A)__int_as_float(p[u].y) * (A)xv[u];
        }
        for (; k < m; ++k) {
            const int2 p = ent[e0 + (int64_t)k * 32];
            s += (A)__int_as_float(p.y) * (A)x[p.x];
        }
        return s;
    }
};

}  // namespace bsc
