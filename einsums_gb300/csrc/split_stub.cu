#include "common.cuh"
namespace eg {
eg_status launch_split_contract(const Contraction &, int, cudaStream_t, eg_split_report *) {
    return fail(EG_ERROR_NOT_SUPPORTED, "split-BF16 form not built");
}
} // namespace eg
