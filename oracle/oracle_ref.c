/*
 * CPU oracle: C restatement of the reference's scalar einsum loops.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load this library, and only to check
 * results.  The product (einsums_gb300/) never links or calls it.
 *
 * Functions here follow, loop for loop:
 *   oracle_generic_cpp  -- einsum_generic_algorithm / einsums_generic_target_loop /
 *                          einsums_generic_link_loop,
 *                          libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Backends/BaseAlgebra.hpp:24-139
 *                          (C already scaled or zeroed by the caller, as at :129-133).
 *                          OpenMP parallelises the outermost target loop only
 *                          (EINSUMS_OMP_PARALLEL_FOR with nested parallelism off),
 *                          so every link sum is computed by one thread, in order.
 *   oracle_generic_py   -- PyEinsumGenericPlan::execute_generic,
 *                          libs/EinsumsPy/TensorAlgebra/include/EinsumsPy/TensorAlgebra/PyTensorAlgebra.hpp:565-601
 *                          (serial walk over the full unique-index space).
 *   oracle_permute      -- element loop of permute(),
 *                          libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Permute.hpp:389-405.
 *
 * All strides and extents are in elements.  Rank is at most ORACLE_MAX_RANK.
 */
#include <stddef.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORACLE_MAX_RANK 16

typedef struct {
    int n_link;
    const int64_t *dims;
    const int64_t *sA;
    const int64_t *sB;
} link_space;

/* einsums_generic_link_loop (BaseAlgebra.hpp:24-55): recursive nested sum,
 * each level accumulating the sums of the level below. */
static double link_loop(const link_space *L, int level, int64_t ia, int64_t ib,
                        const double *A, const double *B) {
    if (level == L->n_link) return A[ia] * B[ib];
    const int64_t n = L->dims[level], sa = L->sA[level], sb = L->sB[level];
    double sum = 0.0;
    if (level == L->n_link - 1) {
        for (int64_t i = 0; i < n; i++) sum += A[ia + i * sa] * B[ib + i * sb];
    } else {
        for (int64_t i = 0; i < n; i++) sum += link_loop(L, level + 1, ia + i * sa, ib + i * sb, A, B);
    }
    return sum;
}

/* einsums_generic_target_loop (BaseAlgebra.hpp:57-83) below the outermost level. */
static void target_loop(int level, int n_target, const int64_t *tdims, const int64_t *sC,
                        const int64_t *sA, const int64_t *sB, const link_space *L,
                        int64_t ic, int64_t ia, int64_t ib, double ab_pref, double *C,
                        const double *A, const double *B) {
    if (level == n_target) {
        C[ic] += ab_pref * link_loop(L, 0, ia, ib, A, B);
        return;
    }
    for (int64_t i = 0; i < tdims[level]; i++)
        target_loop(level + 1, n_target, tdims, sC, sA, sB, L, ic + i * sC[level], ia + i * sA[level],
                    ib + i * sB[level], ab_pref, C, A, B);
}

void oracle_generic_cpp(int n_target, const int64_t *tdims, const int64_t *sC, const int64_t *tA,
                        const int64_t *tB, int n_link, const int64_t *ldims, const int64_t *lA,
                        const int64_t *lB, double ab_pref, double *C, const double *A, const double *B,
                        int nthreads) {
    link_space L = {n_link, ldims, lA, lB};
    if (n_target == 0) {
        /* Rank-0 C with links (BaseAlgebra.hpp:122-128). */
        C[0] += ab_pref * link_loop(&L, 0, 0, 0, A, B);
        return;
    }
    const int64_t n0 = tdims[0];
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
    for (int64_t i = 0; i < n0; i++)
        target_loop(1, n_target, tdims, sC, tA, tB, &L, i * sC[0], i * tA[0], i * tB[0], ab_pref, C, A, B);
    (void)nthreads;
}

/* PyEinsumGenericPlan::execute_generic (PyTensorAlgebra.hpp:585-601):
 * C[c] += AB_prefactor * A[a] * B[b] over every point of the unique-index
 * space, in row-major order of that space, serially. */
void oracle_generic_py(int n_unique, const int64_t *udims, const int64_t *sC, const int64_t *sA,
                       const int64_t *sB, double ab_pref, double *C, const double *A, const double *B) {
    int64_t idx[ORACLE_MAX_RANK] = {0};
    int64_t total = 1;
    for (int u = 0; u < n_unique; u++) total *= udims[u];
    int64_t ic = 0, ia = 0, ib = 0;
    for (int64_t s = 0; s < total; s++) {
        C[ic] += ab_pref * A[ia] * B[ib];
        /* odometer increment, last index fastest */
        for (int u = n_unique - 1; u >= 0; u--) {
            idx[u]++;
            ic += sC[u];
            ia += sA[u];
            ib += sB[u];
            if (idx[u] < udims[u]) break;
            ic -= sC[u] * udims[u];
            ia -= sA[u] * udims[u];
            ib -= sB[u] * udims[u];
            idx[u] = 0;
        }
    }
}

/* Element loop of permute (Permute.hpp:389-405): for every C index,
 * C[idx] = beta * C[idx] + alpha * A[perm(idx)].  Basic tensors go through
 * HPTT (Permute.hpp:375-378), whose beta == 0 path stores alpha * A without
 * reading C; that is reproduced here, so -0.0 keeps its sign.  sA_c[d] is the
 * stride of A along the A mode that carries C's d-th index. */
void oracle_permute(int rank, const int64_t *cdims, const int64_t *sC, const int64_t *sA_c,
                    double beta, double *C, double alpha, const double *A) {
    int64_t idx[ORACLE_MAX_RANK] = {0};
    int64_t total = 1;
    for (int d = 0; d < rank; d++) total *= cdims[d];
    int64_t ic = 0, ia = 0;
    for (int64_t s = 0; s < total; s++) {
        double a = A[ia];
        /* HPTT's beta == 0 kernels write alpha * A without reading B. */
        C[ic] = (beta == 0.0) ? alpha * a : beta * C[ic] + alpha * a;
        for (int d = rank - 1; d >= 0; d--) {
            idx[d]++;
            ic += sC[d];
            ia += sA_c[d];
            if (idx[d] < cdims[d]) break;
            ic -= sC[d] * cdims[d];
            ia -= sA_c[d] * cdims[d];
            idx[d] = 0;
        }
    }
}

/* Straight copy used by permute's bit-exact path: C = A[perm] with alpha == 1
 * and beta == 0, i.e. a pure data movement (HPTT's alpha=1, beta=0 case). */
void oracle_permute_copy(int rank, const int64_t *cdims, const int64_t *sC, const int64_t *sA_c,
                         double *C, const double *A) {
    int64_t idx[ORACLE_MAX_RANK] = {0};
    int64_t total = 1;
    for (int d = 0; d < rank; d++) total *= cdims[d];
    int64_t ic = 0, ia = 0;
    for (int64_t s = 0; s < total; s++) {
        C[ic] = A[ia];
        for (int d = rank - 1; d >= 0; d--) {
            idx[d]++;
            ic += sC[d];
            ia += sA_c[d];
            if (idx[d] < cdims[d]) break;
            ic -= sC[d] * cdims[d];
            ia -= sA_c[d] * cdims[d];
            idx[d] = 0;
        }
    }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
