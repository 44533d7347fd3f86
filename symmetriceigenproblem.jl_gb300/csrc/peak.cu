// peak.cu -- FMA- and FP64-tensor-throughput calibration of the device the library runs on.
//
// The Givens kernels are bound by the FP64 (or FP32) FMA pipe, not by HBM or tensor cores,
// so their roofline needs the FMA issue rate of the GPU as it runs now (clocks, power cap).
// This kernel issues independent FMA chains from every thread of a full grid and reports
// flops / time (an FMA counts 2 flops).  It runs for a few milliseconds, has no memory
// traffic beyond one store per thread, and ends by itself.
#include <cuda_runtime.h>

#include "symeig.h"

namespace symeig {
namespace {

template <typename T>
__global__ void __launch_bounds__(256) fma_peak_kernel(T* out, int iters, T b, T c)
{
    T a0 = (T)threadIdx.x * (T)1e-3, a1 = a0 + (T)1, a2 = a0 + (T)2, a3 = a0 + (T)3;
    T a4 = a0 + (T)4, a5 = a0 + (T)5, a6 = a0 + (T)6, a7 = a0 + (T)7;
    for (int i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
        a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
    }
    const T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (s == (T)1234.5678) out[0] = s;  // never true; keeps the chains alive
}

// FP64 tensor-core rate: independent mma.sync.m8n8k4 .f64 chains (the instruction the dense
// kernels use), 2*8*8*4 = 512 flops each.
__global__ void __launch_bounds__(256) dmma_peak_kernel(double* out, int iters)
{
    double c[8][2];
#pragma unroll
    for (int q = 0; q < 8; ++q) c[q][0] = c[q][1] = 0.0;
    const double a = 1e-3 * (threadIdx.x & 31), b = 0.5;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int q = 0; q < 8; ++q)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};"
                         : "+d"(c[q][0]), "+d"(c[q][1]) : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += c[q][0] + c[q][1];
    if (s == 1234.5678) out[0] = s;
}

int measure_dmma(int sm_count, int iters, double* tflops)
{
    double* out = nullptr;
    if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return SYMEIG_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const dim3 grid(sm_count * 4), block(256);
    dmma_peak_kernel<<<grid, block>>>(out, iters / 4);  // warm-up
    cudaEventRecord(e0);
    dmma_peak_kernel<<<grid, block>>>(out, iters);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return SYMEIG_ERR_CUDA;
    const double flops = 512.0 * 8.0 * iters * (double)grid.x * (block.x / 32);
    *tflops = flops / (ms * 1e-3) / 1e12;
    return SYMEIG_OK;
}

template <typename T>
int measure(int sm_count, int iters, double* tflops)
{
    T* out = nullptr;
    if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return SYMEIG_ERR_NOMEM;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const dim3 grid(sm_count * 8), block(256);
    fma_peak_kernel<T><<<grid, block>>>(out, iters / 4, (T)0.999, (T)1e-3);  // warm-up
    cudaEventRecord(e0);
    fma_peak_kernel<T><<<grid, block>>>(out, iters, (T)0.999, (T)1e-3);
    cudaEventRecord(e1);
    cudaError_t err = cudaEventSynchronize(e1);
    float ms = 0.f;
    if (err == cudaSuccess) err = cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess || ms <= 0.f) return SYMEIG_ERR_CUDA;
    const double flops = 2.0 * 8.0 * iters * (double)grid.x * block.x;
    *tflops = flops / (ms * 1e-3) / 1e12;
    return SYMEIG_OK;
}

}  // namespace
}  // namespace symeig

extern "C" int symeig_measure_fma_peak(int device, int32_t fp64, double* tflops)
{
    if (!tflops) return SYMEIG_ERR_NULL;
    if (cudaSetDevice(device) != cudaSuccess) return SYMEIG_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return SYMEIG_ERR_CUDA;
    // about 8 ms of work at the GB300 rates (1.2 TFLOP/s FP64, 70 TFLOP/s FP32)
    return fp64 ? symeig::measure<double>(sms, 2000, tflops)
                : symeig::measure<float>(sms, 100000, tflops);
}

extern "C" int symeig_measure_dmma_peak(int device, double* tflops)
{
    if (!tflops) return SYMEIG_ERR_NULL;
    if (cudaSetDevice(device) != cudaSuccess) return SYMEIG_ERR_CUDA;
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess)
        return SYMEIG_ERR_CUDA;
    // a few ms of work at ~1.2 TFLOP/s
    return symeig::measure_dmma(sms, 2000, tflops);
}
