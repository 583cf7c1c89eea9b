// C entry point over the reference's own HPTT transposer, used only to pin the
// oracle's permute (test infrastructure; see oracle/hptt_ref.py).  Calls
// hptt::create_plan exactly as compile_permute does for row-major tensors
// (libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Permute.hpp:37-171).
#include <Einsums/HPTT/HPTT.hpp>

#include <cstddef>
#include <vector>

extern "C" int hptt_ref_permute(int rank, const int *perm, const size_t *sizeA, double alpha, const double *A,
                                double beta, double *B, int threads) {
    auto plan = hptt::create_plan(perm, rank, alpha, A, sizeA, nullptr, beta, B, nullptr, hptt::ESTIMATE, threads,
                                  nullptr, true);
    if (!plan) return 1;
    plan->execute();
    return 0;
}
