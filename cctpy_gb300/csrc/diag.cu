// Pipe-peak probes: the roofline denominators of the Biot-Savart kernels, which are bound
// by the FP32 (FP32c form) or FP64 (plain form) CUDA-core pipe, not by HBM or tensor cores.
// Each thread runs 8 independent fused multiply-add chains; flops = 2 per FMA.
#include "cctgpu_internal.cuh"

namespace cctgpu {

template <typename T>
__global__ void __launch_bounds__(256) fma_chain_kernel(T *out, int iters, T a, T b) {
    T x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = (T)(threadIdx.x + i) * (T)1e-3;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = fma(x[i], a, b);
    }
    T s = 0;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += x[i];
    if (s == (T)12345.678) out[0] = s;   // keeps the chains live; never true for these inputs
}

// Packed FP32x2 chains (two FP32 FMAs per instruction).
__global__ void __launch_bounds__(256) fma2_chain_kernel(float *out, int iters, float a, float b) {
    uint64_t x[8], av, bv;
    asm("mov.b64 %0, {%1, %1};" : "=l"(av) : "f"(a));
    asm("mov.b64 %0, {%1, %1};" : "=l"(bv) : "f"(b));
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float v = (float)(threadIdx.x + i) * 1e-3f;
        asm("mov.b64 %0, {%1, %2};" : "=l"(x[i]) : "f"(v), "f"(v + 0.5f));
    }
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) asm("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[i]) : "l"(av), "l"(bv));
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(x[i]));
        s += lo + hi;
    }
    if (s == 12345.678f) out[0] = s;
}

template <typename T>
static int probe(double *flops_per_s, int iters, bool packed = false) {
    int dev = 0, sms = 0;
    CCT_TRY_CUDA(cudaGetDevice(&dev));
    CCT_TRY_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    T *out = nullptr;
    CCT_TRY_CUDA(cudaMalloc(&out, sizeof(T)));
    cudaEvent_t e0, e1;
    CCT_TRY_CUDA(cudaEventCreate(&e0));
    CCT_TRY_CUDA(cudaEventCreate(&e1));
    const int grid = sms * 8;
    auto launch = [&](int n) {
        if (packed)
            fma2_chain_kernel<<<grid, 256>>>(reinterpret_cast<float *>(out), n, 0.999999f, 1e-7f);
        else
            fma_chain_kernel<T><<<grid, 256>>>(out, n, (T)0.999999, (T)1e-7);
    };
    launch(iters / 8);   // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
        CCT_TRY_CUDA(cudaEventRecord(e0));
        launch(iters);
        CCT_TRY_CUDA(cudaEventRecord(e1));
        CCT_TRY_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        CCT_TRY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    *flops_per_s = (packed ? 2.0 : 1.0) * 2.0 * 8.0 * (double)iters * (double)grid * 256.0 / (best * 1e-3);
    return CCT_OK;
}

}  // namespace cctgpu

extern "C" int cct_probe_fma_peak(int kind, double *flops_per_s) {
    cctgpu::clear_error();
    if (!flops_per_s) return cctgpu::set_error(CCT_ERR_ARG, "null output");
    if (kind == 1) return cctgpu::probe<double>(flops_per_s, 1 << 12);
    if (kind == 2) return cctgpu::probe<float>(flops_per_s, 1 << 15, true);
    return cctgpu::probe<float>(flops_per_s, 1 << 16);
}
