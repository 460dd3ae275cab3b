// hfx_peaks.cu -- FP64 / FP32 FMA-loop throughput of the device: the
// denominators of the roofline fractions reported for the Fock-build
// kernels (the measured peaks cover only HBM copy and bf16 GEMM);
// and the FP64 tensor-core (DMMA, mma.sync m8n8k4 f64) throughput, the rate
// a tensor-core Hermite->Cartesian transform could at best reach.
#include <cuda_runtime.h>

#include "hfx_engine.hpp"

namespace hfx {

template <typename T>
__global__ void k_fma_loop(T* out, int iters, T a, T b)
{
    T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3;
    T x4 = x0 + (T)4, x5 = x0 + (T)5, x6 = x0 + (T)6, x7 = x0 + (T)7;
    for (int i = 0; i < iters; ++i) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
    if (s == (T)-12345.0) out[blockIdx.x * blockDim.x + threadIdx.x] = s;  // keeps the loop live
}

template <typename T>
static double measure(int nsm, int iters)
{
    T* out = nullptr;
    int threads = 256, blocks = nsm * 8;
    cuda_check(cudaMalloc(&out, sizeof(T) * threads * blocks), "peaks malloc");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_fma_loop<T><<<blocks, threads>>>(out, iters / 10, (T)0.999, (T)0.001);  // warm-up
    cudaEventRecord(e0);
    k_fma_loop<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
    cudaEventRecord(e1);
    cuda_check(cudaEventSynchronize(e1), "peaks kernel");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    double flops = 2.0 * 8.0 * iters * (double)threads * blocks;
    return flops / (ms * 1e-3) / 1e9;
}

// 8 independent m8n8k4 FP64 MMA chains per warp: 8 x 512 flops per iteration
__global__ void k_dmma_loop(double* out, int iters)
{
    const double a = 1e-3 * (double)(threadIdx.x + 1), b = 0.999;
    double c[8][2];
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = (double)k;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                         : "+d"(c[k][0]), "+d"(c[k][1])
                         : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
    if (s == -12345.0) out[blockIdx.x * blockDim.x + threadIdx.x] = s;   // keeps the loop live
}

static double measure_dmma(int nsm, int iters)
{
    double* out = nullptr;
    int threads = 256, blocks = nsm * 8;
    cuda_check(cudaMalloc(&out, sizeof(double) * threads * blocks), "peaks malloc");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_dmma_loop<<<blocks, threads>>>(out, iters / 10);   // warm-up
    cudaEventRecord(e0);
    k_dmma_loop<<<blocks, threads>>>(out, iters);
    cudaEventRecord(e1);
    cuda_check(cudaEventSynchronize(e1), "dmma peak kernel");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    const double warps = (double)threads / 32 * blocks;
    return 512.0 * 8.0 * iters * warps / (ms * 1e-3) / 1e9;
}

}  // namespace hfx

extern "C" hfx_status hfx_measure_dmma_peak(int device, double* gflops)
{
    try {
        if (!gflops) throw hfx::Error(HFX_ERR_INVALID, "null argument");
        hfx::cuda_check(cudaSetDevice(device), "cudaSetDevice");
        int nsm = 1;
        hfx::cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device), "SM count");
        *gflops = hfx::measure_dmma(nsm, 1 << 11);
        return HFX_OK;
    } catch (const hfx::Error& e) {
        hfx::set_last_error(e.what());
        return e.code;
    }
}

extern "C" hfx_status hfx_measure_peaks(int device, double* fp64_gflops, double* fp32_gflops)
{
    try {
        hfx::cuda_check(cudaSetDevice(device), "cudaSetDevice");
        int nsm = 1;
        hfx::cuda_check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device), "SM count");
        if (fp64_gflops) *fp64_gflops = hfx::measure<double>(nsm, 1 << 13);
        if (fp32_gflops) *fp32_gflops = hfx::measure<float>(nsm, 1 << 16);
        return HFX_OK;
    } catch (const hfx::Error& e) {
        hfx::set_last_error(e.what());
        return e.code;
    }
}
