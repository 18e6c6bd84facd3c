// Arithmetic-pipe probe: the FMA throughput this GPU sustains in FP64, FP32 and packed FP32x2, the
// denominators of the FP64 and FP32 pipe fractions the EAM passes are measured against (the peak file
// of the GPU pool holds only HBM and tensor-core figures). Each thread runs kChains independent FMA
// chains of kIters steps; the grid fills every SM several times over. Timed with CUDA events on a
// private stream, after one warm-up launch.

#include <cuda_runtime.h>

#include "../../include/misa_gb300.h"

namespace mg {
void set_global_error(const char *msg);
}

namespace {

constexpr int kChains = 8;
constexpr int kIters = 4096;
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_fma_f64(double a, double b, double *out) {
    double x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = (double) (threadIdx.x + c);
    for (int i = 0; i < kIters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    if (s == 1.2345) out[0] = s;  // keeps the chains live; never true for the probe's inputs
}

__global__ void __launch_bounds__(kThreads) k_fma_f32(float a, float b, float *out) {
    float x[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) x[c] = (float) (threadIdx.x + c);
    for (int i = 0; i < kIters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += x[c];
    if (s == 1.2345f) out[0] = s;
}

// packed pairs: one fma.rn.f32x2 performs two FP32 FMAs
__global__ void __launch_bounds__(kThreads) k_fma_f32x2(float a, float b, float *out) {
    unsigned long long x[kChains], av, bv;
    asm("mov.b64 %0, {%1, %1};" : "=l"(av) : "f"(a));
    asm("mov.b64 %0, {%1, %1};" : "=l"(bv) : "f"(b));
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        const float lo = (float) (threadIdx.x + c), hi = lo + 0.5f;
        asm("mov.b64 %0, {%1, %2};" : "=l"(x[c]) : "f"(lo), "f"(hi));
    }
    for (int i = 0; i < kIters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) asm("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[c]) : "l"(av), "l"(bv));
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < kChains; c++) {
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(x[c]));
        s += lo + hi;
    }
    if (s == 1.2345f) out[0] = s;
}

}  // namespace

extern "C" mg_status mg_probe_fma(int32_t kind, double *flops_per_s) {
    if (!flops_per_s || kind < 0 || kind > 2) {
        mg::set_global_error("mg_probe_fma: kind is 0 (FP64), 1 (FP32) or 2 (FP32x2), and the output must not be NULL");
        return MG_ERR_ARG;
    }
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    void *out = nullptr;
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e == cudaSuccess) e = cudaMalloc(&out, 16);
    float ms = 0.f;
    const int blocks = sms * 16;
    // a and b keep every chain finite: x -> x * a + b converges to b / (1 - a)
    for (int rep = 0; rep < 2 && e == cudaSuccess; rep++) {
        if (rep == 1) e = cudaEventRecord(e0, st);
        if (kind == 0) k_fma_f64<<<blocks, kThreads, 0, st>>>(0.999, 0.001, static_cast<double *>(out));
        else if (kind == 1) k_fma_f32<<<blocks, kThreads, 0, st>>>(0.999f, 0.001f, static_cast<float *>(out));
        else k_fma_f32x2<<<blocks, kThreads, 0, st>>>(0.999f, 0.001f, static_cast<float *>(out));
        if (e == cudaSuccess) e = cudaGetLastError();
        if (rep == 1 && e == cudaSuccess) e = cudaEventRecord(e1, st);
    }
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    if (out) cudaFree(out);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    if (e != cudaSuccess) {
        mg::set_global_error(cudaGetErrorString(e));
        return MG_ERR_CUDA;
    }
    const double fmas = (double) blocks * kThreads * kChains * kIters * (kind == 2 ? 2.0 : 1.0);
    *flops_per_s = 2.0 * fmas / (ms * 1e-3);
    return MG_OK;
}
