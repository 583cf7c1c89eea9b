// FP64 throughput probes: the roofline denominator of the plain form.  The
// measured-peaks file of the GPU pool has no FP64 figure, so the benchmark
// measures it on the box it runs on: a DFMA loop (CUDA cores) and a DMMA loop
// (mma.sync m8n8k4 f64 tensor instructions), each with independent chains so
// that issue rate, not latency, bounds it.
#include <algorithm>
#include <vector>

#include "common.cuh"

namespace eg {
namespace {

constexpr int kChains = 8;

__global__ void __launch_bounds__(256) k_probe_dfma(double *out, int iters, double seed, long long *cycles) {
    const long long t0 = clock64();
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
    __syncthreads();
    if (threadIdx.x == 0) cycles[blockIdx.x] = clock64() - t0;
}

__global__ void __launch_bounds__(256) k_probe_dmma(double *out, int iters, double seed, long long *cycles) {
    const long long t0 = clock64();
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
    __syncthreads();
    if (threadIdx.x == 0) cycles[blockIdx.x] = clock64() - t0;
}

} // namespace
} // namespace eg

// flops: DFMA counts 2 per thread-FMA; m8n8k4 DMMA counts 2*8*8*4 per warp-instruction.
// Best of three runs after a warm-up run.  Each block of the single resident
// wave records its SM cycles; *probe_mhz (may be NULL) receives the clock the
// DFMA loop ran at (its cycles over its event time) -- the dense FP64 loops run
// well below the maximum SM clock on this GPU, so kernels that mix FP64 with
// other work can exceed these rates.
extern "C" eg_status eg_measure_fp64_peak(double *dfma_tflops, double *dmma_tflops) {
    return eg_measure_fp64_peak_clock(dfma_tflops, dmma_tflops, nullptr);
}

extern "C" eg_status eg_measure_fp64_peak_clock(double *dfma_tflops, double *dmma_tflops, double *probe_mhz) {
    using namespace eg;
    if (!dfma_tflops || !dmma_tflops) return fail(EG_ERROR_INVALID_ARGUMENT, "NULL output");
    const int blocks = num_sms() * 8, threads = 256, iters = 4096;
    int dev = 0, khz = 0;
    EG_CUDA(cudaGetDevice(&dev));
    EG_CUDA(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev));
    double *d = nullptr;
    long long *cyc = nullptr;
    EG_CUDA(cudaMalloc(&d, sizeof(double)));
    if (cudaMalloc(&cyc, blocks * sizeof(long long)) != cudaSuccess) {
        cudaFree(d);
        return fail(EG_ERROR_OUT_OF_MEMORY, "eg_measure_fp64_peak: cudaMalloc");
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<long long> hc(blocks);
    // best of three runs after a warm-up run; returns the run's ms and its SM clock in MHz
    auto timed = [&](auto launch, double &mhz) -> float {
        float best = 1e30f;
        for (int rep = 0; rep < 4; rep++) {
            float ms = 0.f;
            if (cudaEventRecord(e0) != cudaSuccess) return -1.f;
            launch();
            if (cudaEventRecord(e1) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) return -1.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && ms < best) {
                best = ms;
                if (cudaMemcpy(hc.data(), cyc, blocks * sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess)
                    return -1.f;
                std::vector<long long> sorted(hc);
                std::sort(sorted.begin(), sorted.end());
                mhz = (double)sorted[blocks / 2] / (ms * 1e3);
            }
        }
        return best;
    };
    double mhz_fma = 0.0, mhz_mma = 0.0;
    const float ms_fma = timed([&] { k_probe_dfma<<<blocks, threads>>>(d, iters, 1.0, cyc); }, mhz_fma);
    const float ms_mma = timed([&] { k_probe_dmma<<<blocks, threads>>>(d, iters, 1.0, cyc); }, mhz_mma);
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    cudaFree(cyc);
    if (err != cudaSuccess) return cuda_fail(err, "eg_measure_fp64_peak");
    if (ms_fma <= 0.f || ms_mma <= 0.f || mhz_fma <= 0.0 || mhz_mma <= 0.0)
        return fail(EG_ERROR_CUDA, "eg_measure_fp64_peak: timing failed");
    (void)khz;
    *dfma_tflops = 2.0 * kChains * (double)iters * blocks * threads / (ms_fma * 1e-3) / 1e12;
    *dmma_tflops = 2.0 * 8 * 8 * 4 * kChains * (double)iters * blocks * (threads / 32) / (ms_mma * 1e-3) / 1e12;
    if (probe_mhz) *probe_mhz = mhz_fma;
    return EG_SUCCESS;
}
