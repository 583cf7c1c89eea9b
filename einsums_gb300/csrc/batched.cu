// List einsum over many (C, A, B) triples sharing one index pattern.
#include <vector>

#include "common.cuh"

namespace eg {
eg_status einsum_impl(double cp, const int32_t *Cl, const eg_tensor *C, double ab, const int32_t *Al, const eg_tensor *A,
                      const int32_t *Bl, const eg_tensor *B, const eg_options *opt_in, cudaStream_t stream,
                      int32_t *alg_out);
} // namespace eg

extern "C" eg_status eg_einsum_batched(double C_prefactor, const int32_t *C_labels, const eg_tensor *C_list,
                                       double AB_prefactor, const int32_t *A_labels, const eg_tensor *A_list,
                                       const int32_t *B_labels, const eg_tensor *B_list, int64_t count,
                                       const eg_options *opt, void *stream, int32_t *algorithm_choice) {
    eg::set_error("");
    if (count < 0) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "negative count");
    if (count == 0) return EG_SUCCESS; // the reference returns before dispatching an empty list
    if (!C_list || !A_list || !B_list) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "NULL list");
    for (int64_t i = 0; i < count; i++) {
        int32_t alg = 0;
        eg_status st = eg::einsum_impl(C_prefactor, C_labels, &C_list[i], AB_prefactor, A_labels, &A_list[i], B_labels,
                                       &B_list[i], opt, (cudaStream_t)stream, &alg);
        if (st != EG_SUCCESS) return st;
        if (i == 0 && algorithm_choice) *algorithm_choice = alg;
    }
    return EG_SUCCESS;
}
