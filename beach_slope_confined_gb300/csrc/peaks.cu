// peaks.cu -- measured FMA throughput and copy bandwidth of the current GPU.
//
// The pair kernels of the FP64 path are bounded by the FP64 FMA rate, which
// is far below the FP32 rate on this part, so the roofline of each kernel is
// min(HBM, FP64 FMA) and both denominators are measured here rather than
// taken from a data sheet.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "bsc_internal.cuh"

namespace {

constexpr int CHAINS = 8;
constexpr int ITERS = 2048;

template <typename T>
__global__ void k_fma(T* out, T a, T b) {
    T acc[CHAINS];
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) acc[k] = (T)(threadIdx.x + k);
    for (int it = 0; it < ITERS; ++it) {
#pragma unroll
        for (int k = 0; k < CHAINS; ++k) acc[k] = fma(acc[k], a, b);
    }
    T s = 0;
#pragma unroll
    for (int k = 0; k < CHAINS; ++k) s += acc[k];
    if (s == (T)-1.2345) out[blockIdx.x] = s;  // keep the chain alive
}

template <typename T>
double fma_gflops(int sms) {
    const int threads = 256, blocks = sms * 16;
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T) * blocks) != cudaSuccess) return -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma<T><<<blocks, threads>>>(out, (T)0.999999, (T)1e-7);
    cudaDeviceSynchronize();
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(e0);
        k_fma<T><<<blocks, threads>>>(out, (T)0.999999, (T)1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double flops = 2.0 * CHAINS * ITERS * (double)threads * blocks;
    return flops / (best * 1e-3) / 1e9;
}

__global__ void k_copy(const double2* __restrict__ a, double2* __restrict__ b, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

double copy_gbs(int sms) {
    const size_t bytes = (size_t)1 << 30, n = bytes / sizeof(double2);
    double2 *a = nullptr, *b = nullptr;
    if (cudaMalloc(&a, bytes) != cudaSuccess) return -1.0;
    if (cudaMalloc(&b, bytes) != cudaSuccess) {
        cudaFree(a);
        return -1.0;
    }
    cudaMemset(a, 0, bytes);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_copy<<<sms * 8, 512>>>(a, b, n);
    cudaDeviceSynchronize();
    float best = 1e30f;
    for (int r = 0; r < 5; ++r) {
        cudaEventRecord(e0);
        k_copy<<<sms * 8, 512>>>(a, b, n);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        best = std::min(best, ms);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(a);
    cudaFree(b);
    return 2.0 * bytes / (best * 1e-3) / 1e9;
}

}  // namespace

extern "C" int bsc_measure_peaks(double* fp64_gflops, double* fp32_gflops, double* copy_bw) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return BSC_E_NOT_BUILT;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (fp64_gflops) *fp64_gflops = fma_gflops<double>(sms);
    if (fp32_gflops) *fp32_gflops = fma_gflops<float>(sms);
    if (copy_bw) *copy_bw = copy_gbs(sms);
    return cudaGetLastError() == cudaSuccess ? BSC_OK : BSC_E_CUDA;
}

// ---- self-test of the device arithmetic helpers -----------------------------------
namespace {

// deterministic inputs: sign, mantissa in [1, 2) and exponent in [-100, 100]
// from a hash of the index
__device__ double selftest_value(unsigned long long k) {
    unsigned long long h = k * 0x9E3779B97F4A7C15ull;
    h ^= h >> 31;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 29;
    const double m = 1.0 + (double)(h >> 11) * (1.0 / 9007199254740992.0);
    const int e = (int)((h >> 3) % 201) - 100;
    return ((h & 1) ? -m : m) * exp2((double)e);
}

__global__ void k_selftest(long long n, unsigned long long* res) {
    unsigned long long mism = 0, ulp = 0, rel = 0, srel = 0;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n;
         k += (long long)gridDim.x * blockDim.x) {
        const double x = selftest_value((unsigned long long)k);
        const float a = bsc::f32_of(x), b = __double2float_rn(x);
        const int d = abs((int)(__float_as_uint(a) & 0x7fffffffu) - (int)(__float_as_uint(b) & 0x7fffffffu));
        if (__float_as_uint(a) != __float_as_uint(b)) ++mism;
        ulp = max(ulp, (unsigned long long)d);
        const double r = fabs(fma(bsc::rcp_nr(x), x, -1.0));  // relative error of 1/x
        rel = max(rel, (unsigned long long)__double_as_longlong(r));
        const double ax = fabs(x), sx = sqrt(ax);                 // relative error of sqrt_nr
        const double sr = fabs(bsc::sqrt_nr(ax) - sx) / sx;
        srel = max(srel, (unsigned long long)__double_as_longlong(sr));
    }
    atomicAdd(&res[0], mism);
    atomicMax(&res[1], ulp);
    atomicMax(&res[2], rel);
    atomicMax(&res[3], srel);
}

}  // namespace

extern "C" int bsc_selftest(int64_t n, int64_t* f32_mismatches, int64_t* f32_max_ulp, double* rcp_max_rel,
                            double* sqrt_max_rel) {
    if (n <= 0 || !f32_mismatches || !f32_max_ulp || !rcp_max_rel || !sqrt_max_rel) return BSC_E_INVALID;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return BSC_E_NOT_BUILT;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    unsigned long long* res = nullptr;
    if (cudaMalloc(&res, 4 * sizeof(unsigned long long)) != cudaSuccess) return BSC_E_NOMEM;
    unsigned long long h[4] = {0, 0, 0, 0};
    cudaMemcpy(res, h, sizeof h, cudaMemcpyHostToDevice);
    k_selftest<<<sms * 8, 256>>>((long long)n, res);
    cudaMemcpy(h, res, sizeof h, cudaMemcpyDeviceToHost);
    cudaFree(res);
    if (cudaGetLastError() != cudaSuccess) return BSC_E_CUDA;
    *f32_mismatches = (int64_t)h[0];
    *f32_max_ulp = (int64_t)h[1];
    double r;
    std::memcpy(&r, &h[2], sizeof r);
    *rcp_max_rel = r;
    std::memcpy(&r, &h[3], sizeof r);
    *sqrt_max_rel = r;
    return BSC_OK;
}
