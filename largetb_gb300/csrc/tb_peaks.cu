// tb_peaks.cu -- a measurement helper beside the library (libtb_peaks.so),
// not part of the drop-in C-ABI: the FP64 FMA rate of the CUDA cores, the
// roofline of the plain FP64 recurrence and of the stochastic path, which
// are bound by it on GB300.
//
// Every thread runs eight independent FMA chains held in registers (no
// memory traffic), with enough CTAs for eight per SM; the best of three
// CUDA-event-timed launches after a warm-up gives 2 flop per FMA / time.
#include <cuda_runtime.h>

#include <cstdint>

namespace {

__global__ void __launch_bounds__(256) k_fp64_fma_chains(int iters, double seed, double *out)
{
    double a[8];
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = seed + 1e-3 * (threadIdx.x + 32 * j);
    const double b = 0.9999999999, c = 1e-12;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 8; j++) a[j] = fma(a[j], b, c);
    }
    double s = 0.0;
#pragma unroll
    for (int j = 0; j < 8; j++) s += a[j];
    if (s == -1.0) out[blockIdx.x] = s;  // never true: keeps the chains live
}

}  // namespace

// FP64 FMA rate of `device` in TFLOP/s (2 flop per FMA), on the legacy
// default stream; makes `device` current for the calling thread.  Returns 0,
// or the CUDA error code.
extern "C" int tb_peak_fp64_fma(int device, double *tflops)
{
    if (!tflops) return (int)cudaErrorInvalidValue;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return (int)e;
    int nsm = 0;
    if ((e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess) return (int)e;
    const int blocks = nsm * 8, threads = 256, iters = 8192;
    double *out = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    if ((e = cudaMalloc(&out, sizeof(double) * blocks)) != cudaSuccess) return (int)e;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    float best = 0.f;
    for (int rep = 0; rep < 4 && e == cudaSuccess; rep++) {
        cudaEventRecord(t0);
        k_fp64_fma_chains<<<blocks, threads>>>(iters, 1.0 + rep, out);
        cudaEventRecord(t1);
        if ((e = cudaEventSynchronize(t1)) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, t0, t1);
        if (rep > 0 && (best == 0.f || ms < best)) best = ms;  // launch 0 is the warm-up
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaFree(out);
    if (e != cudaSuccess) return (int)e;
    const double flop = 2.0 * 8.0 * (double)iters * (double)blocks * threads;
    *tflops = best > 0.f ? flop / (best * 1e-3) / 1e12 : 0.0;
    return 0;
}
