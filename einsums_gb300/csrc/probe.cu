// FP64 throughput probes: the roofline denominator of the plain form.  The
// measured-peaks file of the GPU pool has no FP64 figure, so the benchmark
// measures it on the box it runs on: a DFMA loop (CUDA cores) and a DMMA loop
// (mma.sync m8n8k4 f64 tensor instructions), each with independent chains so
// that issue rate, not latency, bounds it.
#include "common.cuh"

namespace eg {
namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_probe_dfma(double *out, int iters, double seed) {
    double a[kChains];
#pragma unroll
    for (int c = 0; c < kChains; c++) a[c] = seed + threadIdx.x * 1e-7 + c;
    const double x = 1.0 - 1e-9, y = 1e-9;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++) a[c] = fma(a[c], x, y);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += a[c];
    if (s == 1234.5) out[0] = s; // keeps the loop alive
}

__global__ void __launch_bounds__(256) k_probe_dmma(double *out, int iters, double seed) {
    double acc[kChains][2];
#pragma unroll
    for (int c = 0; c < kChains; c++) acc[c][0] = acc[c][1] = 0.0;
    const double a = seed + threadIdx.x * 1e-9, b = 1.0 - 1e-12;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int c = 0; c < kChains; c++)
            asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0, %1}, {%2}, {%3}, {%0, %1};\n"
                         : "+d"(acc[c][0]), "+d"(acc[c][1])
                         : "d"(a), "d"(b));
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < kChains; c++) s += acc[c][0] + acc[c][1];
    if (s == 1234.5) out[0] = s;
}

} // namespace
} // namespace eg

// flops: DFMA counts 2 per thread-FMA; m8n8k4 DMMA counts 2*8*8*4 per warp-instruction.
extern "C" eg_status eg_measure_fp64_peak(double *dfma_tflops, double *dmma_tflops) {
    using namespace eg;
    if (!dfma_tflops || !dmma_tflops) return fail(EG_ERROR_INVALID_ARGUMENT, "NULL output");
    double *d = nullptr;
    EG_CUDA(cudaMalloc(&d, sizeof(double)));
    cudaEvent_t e0, e1;
    EG_CUDA(cudaEventCreate(&e0));
    EG_CUDA(cudaEventCreate(&e1));
    const int blocks = num_sms() * 8, threads = 256, iters = 4096;
    float ms = 0.f;
    // warm-up
    k_probe_dfma<<<blocks, threads>>>(d, 64, 1.0);
    k_probe_dmma<<<blocks, threads>>>(d, 64, 1.0);
    EG_CUDA(cudaDeviceSynchronize());
    EG_CUDA(cudaEventRecord(e0));
    k_probe_dfma<<<blocks, threads>>>(d, iters, 1.0);
    EG_CUDA(cudaEventRecord(e1));
    EG_CUDA(cudaEventSynchronize(e1));
    EG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    *dfma_tflops = 2.0 * kChains * (double)iters * blocks * threads / (ms * 1e-3) / 1e12;
    EG_CUDA(cudaEventRecord(e0));
    k_probe_dmma<<<blocks, threads>>>(d, iters, 1.0);
    EG_CUDA(cudaEventRecord(e1));
    EG_CUDA(cudaEventSynchronize(e1));
    EG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    *dmma_tflops = 2.0 * 8 * 8 * 4 * kChains * (double)iters * blocks * (threads / 32) / (ms * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    return EG_SUCCESS;
}
