// Self-test of the failure path of the bounded device waits.
//
// One CTA takes the same steps as the tensor kernel when a pipeline barrier is
// never satisfied: warp 0 allocates tensor memory, thread 0 waits on an
// mbarrier that nothing arrives on until `limit_ns` passes, records the code in
// the stream's status word and raises the CTA's abort flag; warp 1 waits on the
// same barrier and leaves on seeing the flag; then tensor memory is freed and
// the kernel returns.  eg_stream_status reports EG_ERROR_TIMEOUT afterwards and
// the context stays usable.  The wait is bounded by the limit (at most 2 s).
#include "ptx.cuh"
#include "common.cuh"

#include <cuda_runtime.h>

namespace eg {
namespace {

constexpr int kSelftestCode = 6;

__global__ void __launch_bounds__(64, 1) k_selftest_wait(int *status, unsigned long long limit_ns) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        ptx::mbar_init(&bar, 1);
        abort_flag = 0;
        ptx::fence_mbar_init();
    }
    if (warp == 0) {
        ptx::tmem_alloc(&tmem_slot, 32);
        ptx::tmem_relinquish();
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    const uint32_t tmem = tmem_slot;
    if (threadIdx.x == 0) {
        if (!ptx::mbar_wait(&bar, 0, limit_ns, nullptr)) {
            atomicCAS(status, 0, kSelftestCode);
            *(volatile int *)&abort_flag = 1;
        }
    } else if (threadIdx.x == 32) {
        // a second role: gives up when the first one raises the flag (or at the limit)
        ptx::mbar_wait(&bar, 0, limit_ns + 100000000ull, (volatile int *)&abort_flag);
    }
    ptx::tc_fence_before();
    __syncthreads();
    ptx::tc_fence_after();
    if (warp == 0) ptx::tmem_dealloc(tmem, 32);
}

} // namespace
} // namespace eg

extern "C" eg_status eg_selftest_wait_timeout(uint64_t limit_ns, void *stream) {
    eg::set_error("");
    if (limit_ns == 0 || limit_ns > 2000000000ull)
        return eg::fail(EG_ERROR_INVALID_ARGUMENT, "eg_selftest_wait_timeout: limit must be in (0, 2 s]");
    int *status = nullptr;
    eg_status st = eg::status_word((cudaStream_t)stream, &status);
    if (st != EG_SUCCESS) return st;
    {
        eg::LaunchScope ls_("k_selftest_wait", (cudaStream_t)stream);
        eg::k_selftest_wait<<<1, 64, 0, (cudaStream_t)stream>>>(status, (unsigned long long)limit_ns);
    }
    EG_CHECK_LAUNCH("k_selftest_wait");
    return EG_SUCCESS;
}
