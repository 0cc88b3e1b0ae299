// peaks.cu -- measured FMA throughput and copy bandwidth of the current GPU.
//
// The pair kernels of the FP64 path are bounded by the FP64 FMA rate, which
// is far below the FP32 rate on this part, so the roofline of each kernel is
// min(HBM, FP64 FMA) and both denominators are measured here rather than
// taken from a data sheet.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/bsc.h"

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
