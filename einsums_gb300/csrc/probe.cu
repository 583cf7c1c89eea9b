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

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__global__ void __launch_bounds__(256) k_probe_dfma(double *out, int iters, double seed, long long *cycles,
                                                    unsigned long long *ns) {
    const long long t0 = clock64();
    const unsigned long long g0 = global_ns();
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
    if (threadIdx.x == 0) {
        cycles[blockIdx.x] = clock64() - t0;
        ns[blockIdx.x] = global_ns() - g0;
    }
}

__global__ void __launch_bounds__(256) k_probe_dmma(double *out, int iters, double seed, long long *cycles,
                                                    unsigned long long *ns) {
    const long long t0 = clock64();
    const unsigned long long g0 = global_ns();
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
    if (threadIdx.x == 0) {
        cycles[blockIdx.x] = clock64() - t0;
        ns[blockIdx.x] = global_ns() - g0;
    }
}

} // namespace
} // namespace eg

// flops: DFMA counts 2 per thread-FMA; m8n8k4 DMMA counts 2*8*8*4 per warp-instruction.
// Best of three runs after a warm-up run.  Each block records its SM cycles and
// its own duration (global timer); *probe_mhz (may be NULL) receives the median
// block's cycles over its duration, the SM clock the DFMA loop ran at.  Blocks
// of one launch share the FP64 pipe unevenly and finish at different times, so
// a block's cycles over the whole launch's time would understate the clock.
// On GB300 both loops stay below the FP64 pipe's rate: ncu counts the DMMA
// instructions on the FP64 pipe (none on the tensor pipe), at 97 % of its
// active cycles, and the DFMA loop keeps the pipe 84 % busy, while the
// register-tiled contraction kernel keeps it 96 % busy and runs faster.
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
    unsigned long long *bns = nullptr;
    EG_CUDA(cudaMalloc(&d, sizeof(double)));
    if (cudaMalloc(&cyc, blocks * sizeof(long long)) != cudaSuccess) {
        cudaFree(d);
        return fail(EG_ERROR_OUT_OF_MEMORY, "eg_measure_fp64_peak: cudaMalloc");
    }
    if (cudaMalloc(&bns, blocks * sizeof(unsigned long long)) != cudaSuccess) {
        cudaFree(d);
        cudaFree(cyc);
        return fail(EG_ERROR_OUT_OF_MEMORY, "eg_measure_fp64_peak: cudaMalloc");
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<long long> hc(blocks);
    std::vector<unsigned long long> hn(blocks);
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
                if (cudaMemcpy(hc.data(), cyc, blocks * sizeof(long long), cudaMemcpyDeviceToHost) != cudaSuccess ||
                    cudaMemcpy(hn.data(), bns, blocks * sizeof(unsigned long long), cudaMemcpyDeviceToHost) !=
                        cudaSuccess)
                    return -1.f;
                std::vector<double> clk;
                clk.reserve(blocks);
                for (int b = 0; b < blocks; b++)
                    if (hn[b] > 0) clk.push_back((double)hc[b] * 1e3 / (double)hn[b]); // cycles per ns -> MHz
                if (clk.empty()) return -1.f;
                std::sort(clk.begin(), clk.end());
                mhz = clk[clk.size() / 2];
            }
        }
        return best;
    };
    double mhz_fma = 0.0, mhz_mma = 0.0;
    const float ms_fma = timed([&] { k_probe_dfma<<<blocks, threads>>>(d, iters, 1.0, cyc, bns); }, mhz_fma);
    const float ms_mma = timed([&] { k_probe_dmma<<<blocks, threads>>>(d, iters, 1.0, cyc, bns); }, mhz_mma);
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    cudaFree(cyc);
    cudaFree(bns);
    if (err != cudaSuccess) return cuda_fail(err, "eg_measure_fp64_peak");
    if (ms_fma <= 0.f || ms_mma <= 0.f || mhz_fma <= 0.0 || mhz_mma <= 0.0)
        return fail(EG_ERROR_CUDA, "eg_measure_fp64_peak: timing failed");
    (void)khz;
    *dfma_tflops = 2.0 * kChains * (double)iters * blocks * threads / (ms_fma * 1e-3) / 1e12;
    *dmma_tflops = 2.0 * 8 * 8 * 4 * kChains * (double)iters * blocks * (threads / 32) / (ms_mma * 1e-3) / 1e12;
    if (probe_mhz) *probe_mhz = mhz_fma;
    return EG_SUCCESS;
}
