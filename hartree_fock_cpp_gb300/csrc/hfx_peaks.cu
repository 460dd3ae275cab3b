// hfx_peaks.cu -- FP64 / FP32 FMA-loop throughput of the device: the
// denominators of the roofline fractions reported for the Fock-build
// kernels (the measured peaks cover only HBM copy and bf16 GEMM).
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

}  // namespace hfx

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
