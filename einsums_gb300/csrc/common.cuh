// Shared definitions of the einsums_gb300 CUDA library: status plumbing,
// the canonical contraction descriptor that every pattern is lowered to, and
// the per-stream scratch workspace.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/einsums_gb300.h"

namespace eg {

// ---------------------------------------------------------------- errors --
void set_error(const std::string &msg);
eg_status fail(eg_status st, const std::string &msg);
eg_status cuda_fail(cudaError_t err, const char *what);

#define EG_CUDA(call)                                                                                                  \
    do {                                                                                                               \
        cudaError_t eg_err_ = (call);                                                                                  \
        if (eg_err_ != cudaSuccess) return ::eg::cuda_fail(eg_err_, #call);                                           \
    } while (0)

#define EG_CHECK_LAUNCH(name)                                                                                          \
    do {                                                                                                               \
        cudaError_t eg_err_ = cudaGetLastError();                                                                      \
        if (eg_err_ != cudaSuccess) return ::eg::cuda_fail(eg_err_, name);                                            \
    } while (0)

// ------------------------------------------------------------ index maps --
// A group of modes walked as one linear index.  Mode 0 is the slowest; the
// linear index is decomposed from the last mode.  s[t][d] is the element
// stride of operand t (0 = A, 1 = B, 2 = C) along mode d.
constexpr int kMaxModes = 8;

struct ModeGroup {
    int n = 0;
    int64_t total = 1;
    int64_t ext[kMaxModes] = {};
    int64_t s[3][kMaxModes] = {};
};

// Offsets of linear index `i` in the three operands.
__host__ __device__ inline void group_offsets(const ModeGroup &g, int64_t i, int64_t &oa, int64_t &ob, int64_t &oc) {
    oa = ob = oc = 0;
    for (int d = g.n - 1; d >= 0; d--) {
        const int64_t e = g.ext[d];
        const int64_t q = i / e;
        const int64_t r = i - q * e;
        i = q;
        oa += r * g.s[0][d];
        ob += r * g.s[1][d];
        oc += r * g.s[2][d];
    }
}

// 32-bit variant for groups whose total fits in int32 (checked on the host).
__host__ __device__ inline void group_offsets32(const ModeGroup &g, uint32_t i, int64_t &oa, int64_t &ob, int64_t &oc) {
    oa = ob = oc = 0;
    for (int d = g.n - 1; d >= 0; d--) {
        const uint32_t e = (uint32_t)g.ext[d];
        const uint32_t q = i / e;
        const uint32_t r = i - q * e;
        i = q;
        oa += (int64_t)r * g.s[0][d];
        ob += (int64_t)r * g.s[1][d];
        oc += (int64_t)r * g.s[2][d];
    }
}

// Compensated sum of one value pair (s, c) per thread over a block of NT
// threads (NT a multiple of 32, at most 1024), in a fixed tree order: pairs are
// merged with Knuth's TwoSum, the rounding error of each merge going to c.  The
// depth is log2(NT) dependent merges, so the FP64 latency stays small (a serial
// loop over the threads' sums would take NT of them).  Returns s + c in thread 0.
template <int NT>
__device__ __forceinline__ double block_sum_compensated(double s, double c, double *sh_s, double *sh_c) {
    auto merge = [](double &a, double &ca, double b, double cb) {
        const double t = a + b, bb = t - a;
        const double e = (a - (t - bb)) + (b - bb);
        a = t;
        ca = (ca + cb) + e;
    };
    for (int o = 16; o > 0; o >>= 1) {
        const double s2 = __shfl_down_sync(0xffffffffu, s, o), c2 = __shfl_down_sync(0xffffffffu, c, o);
        merge(s, c, s2, c2);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        sh_s[w] = s;
        sh_c[w] = c;
    }
    __syncthreads();
    if (w == 0) {
        s = lane < NT / 32 ? sh_s[lane] : 0.0;
        c = lane < NT / 32 ? sh_c[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            const double s2 = __shfl_down_sync(0xffffffffu, s, o), c2 = __shfl_down_sync(0xffffffffu, c, o);
            merge(s, c, s2, c2);
        }
    }
    return s + c;
}

// Canonical contraction:  C[b,m,n] = cp*C + ab * sum_k A[b,m,k] B[b,n,k]
//   batch: modes in A, B and C      m: modes in A and C (and C-only modes)
//   n:     modes in B and C         k: summed modes (links; free modes under
//                                       the Python semantics)
struct Contraction {
    ModeGroup batch, m, n, k;
    const double *A = nullptr;
    const double *B = nullptr;
    double *C = nullptr;
    double cp = 0.0, ab = 1.0;
    bool zero_when_cp_zero = true; // false reproduces the reference's "C *= C_prefactor" paths
    int64_t c_elems = 0;           // number of C positions written (product of all C modes)
};

// ------------------------------------------------------------- workspace --
// Grow-only device scratch, one per (device, stream); never shrinks while the
// library is loaded.  Calls that share a stream are ordered, so reuse is safe.
eg_status workspace(cudaStream_t stream, size_t bytes, void **ptr);

// Device-side error word of kernels with bounded waits, one per (device,
// stream); kernels set it with atomicCAS(ptr, 0, code) and eg_stream_status
// reads and clears it.
eg_status status_word(cudaStream_t stream, int **ptr);

// Device memory accounting used by eg_device_alloc and the workspace.
eg_status tracked_malloc(size_t bytes, void **ptr);
eg_status tracked_free(void *ptr);

inline int num_sms() {
    static int sms = [] {
        int dev = 0, v = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        return v > 0 ? v : 148;
    }();
    return sms;
}

// ------------------------------------------------------- launch records --
// Counts every kernel launch; with profiling on, brackets it with events.
class LaunchScope {
  public:
    LaunchScope(const char *name, cudaStream_t s);
    ~LaunchScope();

  private:
    const char *name_;
    cudaStream_t s_;
    cudaEvent_t e0_ = nullptr, e1_ = nullptr;
};

// ------------------------------------------------------------- launchers --
eg_status launch_elementwise(const Contraction &c, cudaStream_t s);
eg_status launch_scale(const ModeGroup &g, double *C, double cp, cudaStream_t s);
eg_status launch_dot(const Contraction &c, cudaStream_t s);
eg_status launch_gemv(const Contraction &c, cudaStream_t s);
eg_status launch_contract_f64(const Contraction &c, cudaStream_t s);
eg_status launch_split_contract(const Contraction &c, int slices, cudaStream_t s, eg_split_report *rep);

struct PermuteDesc {
    int rank = 0;
    int64_t ext[kMaxModes] = {};
    int64_t sA[kMaxModes] = {}; // A stride along each C-ordered mode
    int64_t sC[kMaxModes] = {};
    const double *A = nullptr;
    double *C = nullptr;
    double cp = 0.0, ap = 1.0;
};
eg_status launch_permute(const PermuteDesc &p, cudaStream_t s);

} // namespace eg
