// Allocation-free dot product: eg_dot_noalloc.
//
// Some callers cannot let a library call cudaMalloc: applications whose
// device memory is entirely owned by another allocator (a framework's caching
// allocator, or an arena reserved at start-up), and latency-critical loops
// that must not pay for an allocation.  For them this entry point runs the
// two-pass dot reduction with its partial sums kept in a fixed scratch array
// that is part of the library image on every GPU that loads it, instead of
// the per-stream workspace the other entry points grow with cudaMalloc.
//
// Limits and sharing:
//  * the scratch holds kNoAllocParts partial sums, one per block of
//    kNoAllocChunk elements, so a call takes at most
//    kNoAllocParts * kNoAllocChunk = 2^28 elements; longer inputs are
//    rejected with EG_ERROR_NOT_SUPPORTED;
//  * every call on a device uses the same array; each block overwrites its
//    own partial before the final pass reads it, so nothing carries over
//    between calls, but two calls whose kernels overlap on the GPU (different
//    streams, or host threads) race on the array;
//  * every call looks up the array's device address on the current device
//    (cudaGetSymbolAddress, which allocates nothing), so the address stays
//    right after a device reset or a new primary context; the first call on a
//    device also loads the library's device code there, so make that first
//    call before any stream capture;
//  * C is C_prefactor * C + AB_prefactor * sum, as the reference's C++ DOT
//    choice computes it: with C_prefactor == 0 a NaN or infinity already in C
//    stays in the result (eg_einsum with C++ semantics does the same).
#include "common.cuh"

namespace eg {

namespace {

constexpr int kNoAllocParts = 4096;
constexpr int64_t kNoAllocChunk = 65536;
constexpr int kNoAllocThreads = 256;

// The scratch: kNoAllocParts doubles (32 KB) on every device that loads the library.
static __device__ __align__(256) double g_noalloc_partials[kNoAllocParts];

// The array's address on the current device.  In host code the symbol
// g_noalloc_partials is only a host-side stand-in, never a device address.
eg_status scratch_on_current_device(double **out) {
    void *p = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (err != cudaSuccess) return cuda_fail(err, "cudaGetSymbolAddress(g_noalloc_partials)");
    *out = (double *)p;
    return EG_SUCCESS;
}

__global__ void __launch_bounds__(kNoAllocThreads) k_dot_noalloc_partial(const double *__restrict__ A,
                                                                         const double *__restrict__ B, int64_t n,
                                                                         double *partial) {
    __shared__ double warp_sums[kNoAllocThreads / 32];
    const int64_t begin = (int64_t)blockIdx.x * kNoAllocChunk;
    const int64_t end = min(begin + kNoAllocChunk, n);
    double acc0 = 0.0, acc1 = 0.0;
    int64_t i = begin + threadIdx.x;
    for (; i + kNoAllocThreads < end; i += 2 * kNoAllocThreads) {
        acc0 = fma(__ldg(A + i), __ldg(B + i), acc0);
        acc1 = fma(__ldg(A + i + kNoAllocThreads), __ldg(B + i + kNoAllocThreads), acc1);
    }
    if (i < end) acc0 = fma(__ldg(A + i), __ldg(B + i), acc0);
    double v = acc0 + acc1;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < kNoAllocThreads / 32; w++) s += warp_sums[w];
        partial[blockIdx.x] = s;
    }
}

// One block: sums the partials in a fixed order (Neumaier within a thread, a
// compensated tree across the block), then
// C = C_prefactor * C + AB_prefactor * sum, as the reference's DOT choice does.
__global__ void __launch_bounds__(kNoAllocThreads) k_dot_noalloc_final(const double *partial, int nparts, double *C,
                                                                       double cp, double ab) {
    __shared__ double sh_s[kNoAllocThreads / 32], sh_c[kNoAllocThreads / 32];
    double s = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < nparts; i += kNoAllocThreads) {
        const double x = partial[i];
        const double t = s + x;
        c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    const double sum = block_sum_compensated<kNoAllocThreads>(s, c, sh_s, sh_c);
    if (threadIdx.x == 0) *C = cp * (*C) + ab * sum;
}

} // namespace

} // namespace eg

extern "C" eg_status eg_dot_noalloc(double C_prefactor, double *C, double AB_prefactor, const double *A,
                                    const double *B, int64_t n, void *stream) {
    using namespace eg;
    set_error("");
    if (!C) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_dot_noalloc: C is NULL");
    if (n < 0) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_dot_noalloc: negative length");
    if (n > 0 && (!A || !B)) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_dot_noalloc: A or B is NULL");
    if (n > (int64_t)kNoAllocParts * kNoAllocChunk)
        return fail(EG_ERROR_NOT_SUPPORTED, "eg_dot_noalloc: length " + std::to_string(n) + " exceeds the maximum of " +
                                                std::to_string((int64_t)kNoAllocParts * kNoAllocChunk) +
                                                " elements (fixed scratch of " + std::to_string(kNoAllocParts) +
                                                " partial sums)");
    double *scratch = nullptr;
    eg_status st = scratch_on_current_device(&scratch);
    if (st != EG_SUCCESS) return st;
    cudaStream_t s = (cudaStream_t)stream;
    const int nparts = (int)((n + kNoAllocChunk - 1) / kNoAllocChunk);
    if (nparts > 0) {
        LaunchScope ls_("k_dot_noalloc_partial", s);
        k_dot_noalloc_partial<<<nparts, kNoAllocThreads, 0, s>>>(A, B, n, scratch);
    }
    EG_CHECK_LAUNCH("k_dot_noalloc_partial");
    {
        LaunchScope ls_("k_dot_noalloc_final", s);
        k_dot_noalloc_final<<<1, kNoAllocThreads, 0, s>>>(scratch, nparts, C, C_prefactor, AB_prefactor);
    }
    EG_CHECK_LAUNCH("k_dot_noalloc_final");
    return EG_SUCCESS;
}
