// Fock two-electron build for integrals with 8-fold permutational symmetry:
// eg_fock_jk_symmetric.
//
//   F = F_prefactor * F + J_prefactor * J + K_prefactor * K
//   J[p,q] = sum_rs g[p,q,r,s] D[r,s]      (einsum pq <- pqrs, rs: GEMV)
//   K[p,q] = sum_rs g[p,r,q,s] D[r,s]      (einsum pq <- prqs, rs: GENERIC)
//
// The reference computes F += 2 J and F -= K as two general einsum calls over
// the whole of g (libs/Einsums/TensorAlgebra/tests/unit/QChemTests.cpp:300-303,
// dispatched by Backends/Dispatch.hpp:444-560 and BaseAlgebra.hpp:85-139).
// With g[p,q,r,s] = g[q,p,r,s] = g[p,q,s,r] = g[r,s,p,q] and D symmetric, only
// the canonical quartets p >= q, r >= s, pair(p,q) >= pair(r,s) -- an eighth
// of g -- need to be read.  Each canonical element g, scaled by its degeneracy
// f (1/2 for each of p == q, r == s and pair(p,q) == pair(r,s)), makes six
// contributions to two non-symmetric accumulators, with J = 2 (YJ + YJ^T) and
// K = XK + XK^T:
//
//   T1 YJ[p,q] += f g D[r,s]   T2 YJ[r,s] += f g D[p,q]   T3 XK[p,r] += f g D[q,s]
//   T4 XK[q,r] += f g D[p,s]   T5 XK[p,s] += f g D[q,r]   T6 XK[q,s] += f g D[p,r]
//
// Six FP64 multiply-adds per canonical element, 0.75 n^4 in all, against
// 2 n^4 for the two general contractions.  On this GPU those multiply-adds,
// not HBM, bound the build: the FP64 pipe retires about one warp-wide FMA
// per 64 cycles per SM sub-partition, so every kernel here keeps the FP64
// instructions to the multiply-adds themselves and does its index arithmetic,
// degeneracy scaling (exponent decrements) and loads on the other pipes.
//
// Kernels (no atomics: every partial has one home and the last pass sums
// them in a fixed order, so the result is deterministic):
//   k_fock_pair_blocks      one CTA per (p, r, chunk of 64 q): the block
//                           B[q,s] = g[p,q,r,s] is staged in shared memory;
//                           row sums give T1 and T4, column sums T2, T5 and
//                           the block total T3.
//   k_fock_exchange_blocks  one CTA per (q, s): the weighted total T6 of the
//                           block g[q,p,s,r] (= g[p,q,r,s]) over (p, r).
//   k_fock_reduce           one CTA per output row: sums the partials of
//                           YJ and XK.
//   k_fock_combine          applies J = 2 (YJ + YJ^T), K = XK + XK^T and the
//                           prefactors.
#include <algorithm>
#include <cmath>

#include "common.cuh"

namespace eg {

namespace {

constexpr int kFockThreads = 128;
constexpr int kFockChunk = 64; // rows q of a pair block staged per CTA

// x / 2, exactly: an exponent decrement for normal numbers, else a multiply.
__device__ __forceinline__ double half_exact(double x) {
    const long long b = __double_as_longlong(x);
    if (((b >> 52) & 0x7ff) > 1) return __longlong_as_double(b - (1ll << 52));
    return x * 0.5;
}

struct FockScratch {
    double *S1;  // [p][r][q]      T1 row sums
    double *S4;  // [q][p][r]      T4 row sums
    double *S2;  // [r][p][c][s]   T2 column sums of chunk c
    double *S5;  // [p][r][c][s]   T5 column sums of chunk c
    double *X3;  // [p][r][c]      T3 totals of chunk c
    double *X6;  // [q][s]         T6 totals
    double *YJ;  // [i][j], i >= j  combined T1 + T2
    double *XK;  // [i][j]          combined T3..T6
};

// Pair block (p, r), p >= r, rows q in chunk c.  Unit index x runs the pairs
// from the largest p down so that the big blocks start first.
__global__ void __launch_bounds__(kFockThreads) k_fock_pair_blocks(const double *__restrict__ g,
                                                                   const double *__restrict__ D, int n, int nc,
                                                                   FockScratch sc) {
    extern __shared__ double sm[];
    const int npairs = n * (n + 1) / 2;
    const int x = npairs - 1 - (int)blockIdx.x;
    int p = (int)((sqrtf(8.0f * (float)x + 1.0f) - 1.0f) * 0.5f);
    while ((p + 1) * (p + 2) / 2 <= x) p++;
    while (p * (p + 1) / 2 > x) p--;
    const int r = x - p * (p + 1) / 2;
    const int c = blockIdx.y;
    const int q0 = c * kFockChunk;
    if (q0 > p) return;
    const int nq = min(kFockChunk, p + 1 - q0);
    const int ns = r + 1;
    const int ld = ns | 1; // odd row stride: rows of the column walk fall in different banks
    double *T = sm;                      // [nq][ld]
    double *Dr = T + kFockChunk * ld;    // D[r][0..n)
    double *Dp = Dr + n;                 // D[p][0..n)
    const int tid = threadIdx.x;
    for (int i = tid; i < n; i += kFockThreads) {
        Dr[i] = __ldg(D + (size_t)r * n + i);
        Dp[i] = __ldg(D + (size_t)p * n + i);
    }
    // Stage the block with its degeneracy factors.  Row q, columns s <= r (s <= q
    // when p == r, the rest of the row zero).
    const bool diag = p == r;
    for (int e = tid; e < nq * ns; e += kFockThreads) {
        const int ql = e / ns, s = e - ql * ns;
        const int q = q0 + ql;
        double v = 0.0;
        if (!diag || s <= q) {
            v = __ldcs(g + (((size_t)p * n + q) * n + r) * n + s);
            if (q == p) v = half_exact(v);
            if (s == r) v = half_exact(v);
            if (diag && s == q) v = half_exact(v);
        }
        T[ql * ld + s] = v;
    }
    __syncthreads();
    // Rows: two threads per row split the columns; T1 with D[r][s], T4 with D[p][s].
    {
        const int ql = tid >> 1, h = tid & 1;
        double a1 = 0.0, a4 = 0.0;
        if (ql < nq) {
            const double *row = T + ql * ld;
            for (int s = h; s < ns; s += 2) {
                const double v = row[s];
                a1 = fma(v, Dr[s], a1);
                a4 = fma(v, Dp[s], a4);
            }
        }
        a1 += __shfl_xor_sync(0xffffffffu, a1, 1);
        a4 += __shfl_xor_sync(0xffffffffu, a4, 1);
        if (ql < nq && h == 0) {
            const int q = q0 + ql;
            sc.S1[((size_t)p * n + r) * n + q] = a1;
            sc.S4[((size_t)q * n + p) * n + r] = a4;
        }
    }
    // Columns: T2 with D[p][q], T5 with D[q][r] = D[r][q], T3 with D[q][s].
    double a3 = 0.0;
    for (int s = tid; s < ns; s += kFockThreads) {
        double a2 = 0.0, a5 = 0.0;
        for (int ql = 0; ql < nq; ql++) {
            const double v = T[ql * ld + s];
            const int q = q0 + ql;
            a2 = fma(v, Dp[q], a2);
            a5 = fma(v, Dr[q], a5);
            a3 = fma(v, __ldg(D + (size_t)q * n + s), a3);
        }
        sc.S2[(((size_t)r * n + p) * nc + c) * n + s] = a2;
        sc.S5[(((size_t)p * n + r) * nc + c) * n + s] = a5;
    }
    __shared__ double red[kFockThreads / 32];
    for (int o = 16; o > 0; o >>= 1) a3 += __shfl_down_sync(0xffffffffu, a3, o);
    if ((tid & 31) == 0) red[tid >> 5] = a3;
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        for (int w = 0; w < kFockThreads / 32; w++) t += red[w];
        sc.X3[((size_t)p * n + r) * nc + c] = t;
    }
}

// Exchange block (q, s): T6 = sum over canonical (p, r) with p >= q, r >= s of
// f g[q,p,s,r] D[p,r].  Rows p in [max(q, s), n); row p holds r in [s, p],
// without r = p when q < s (then pair(p,q) < pair(p,s)).  The rows are walked
// as one flattened index so that short rows leave no lanes idle.
__global__ void __launch_bounds__(kFockThreads) k_fock_exchange_blocks(const double *__restrict__ g,
                                                                       const double *__restrict__ D, int n,
                                                                       double *__restrict__ X6) {
    const int u = n * n - 1 - (int)blockIdx.x; // small (q, s) -- the big blocks -- first
    const int q = u / n, s = u - q * n;
    const int p0 = max(q, s);
    const int drop = q < s ? 1 : 0;
    const int L0 = p0 - s + 1 - drop; // length of row p0; row p0 + i has L0 + i elements
    const int rows = n - p0;
    const long long total = (long long)rows * L0 + (long long)rows * (rows - 1) / 2;
    const double *gq = g + ((size_t)q * n) * n * n;
    double acc = 0.0;
    // (i, off): row and position of flattened index k; rows are walked forward
    // as k advances (integer work only: the FP64 pipe is kept for the sums)
    long long k = threadIdx.x, off = k;
    int i = 0;
    while (i < rows && off >= L0 + i) {
        off -= L0 + i;
        i++;
    }
    for (; k < total; k += kFockThreads) {
        const int p = p0 + i;
        const int rr = s + (int)off;
        double v = __ldcs(gq + ((size_t)p * n + s) * n + rr);
        if (p == q) v = half_exact(v);
        if (rr == s) v = half_exact(v);
        if (p == rr && q == s) v = half_exact(v);
        acc = fma(v, __ldg(D + (size_t)p * n + rr), acc);
        off += kFockThreads;
        while (i < rows && off >= L0 + i) {
            off -= L0 + i;
            i++;
        }
    }
    __shared__ double red[kFockThreads / 32];
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < kFockThreads / 32; w++) t += red[w];
        X6[(size_t)q * n + s] = t;
    }
}

// Row i of YJ (j <= i) and XK from the partials: one thread per j, so that
// every partial row is read contiguously; each sum runs in a fixed order.
__global__ void __launch_bounds__(kFockThreads) k_fock_reduce(int n, int nc, FockScratch sc) {
    const int i = blockIdx.x;
    for (int j = threadIdx.x; j < n; j += kFockThreads) {
        // XK[i][j]: T6, then T4 over pair blocks (p, r = j) with p >= max(i, j)
        double xa = sc.X6[(size_t)i * n + j], xb = 0.0;
        for (int p = max(i, j); p < n; p++) xb += sc.S4[((size_t)i * n + p) * n + j];
        if (i >= j) {
            // T3 over the chunks of pair block (i, j); T5 over pair blocks (i, r), j <= r <= i
            for (int c = 0; c * kFockChunk <= i; c++) xa += sc.X3[((size_t)i * n + j) * nc + c];
            for (int r = j; r <= i; r++)
                for (int c = 0; c * kFockChunk <= i; c++) xb += sc.S5[(((size_t)i * n + r) * nc + c) * n + j];
            // YJ[i][j]: T1 over pair blocks (i, r), r <= i; T2 over pair blocks (p, i), p >= i
            double ya = 0.0, yb = 0.0;
            for (int r = 0; r <= i; r++) ya += sc.S1[((size_t)i * n + r) * n + j];
            for (int p = i; p < n; p++)
                for (int c = 0; c * kFockChunk <= p; c++) yb += sc.S2[(((size_t)i * n + p) * nc + c) * n + j];
            sc.YJ[(size_t)i * n + j] = ya + yb;
        }
        sc.XK[(size_t)i * n + j] = xa + xb;
    }
}

// F = fp F + jp J + kp K with J = 2 (YJ + YJ^T) and K = XK + XK^T.
__global__ void __launch_bounds__(kFockThreads) k_fock_combine(double *F, int n, FockScratch sc, double fp, double jp,
                                                               double kp, int zero_f) {
    const int i = blockIdx.x;
    for (int j = threadIdx.x; j < n; j += kFockThreads) {
        const double yj = sc.YJ[(size_t)max(i, j) * n + min(i, j)];
        const double J = (i == j ? 4.0 : 2.0) * yj;
        const double K = sc.XK[(size_t)i * n + j] + sc.XK[(size_t)j * n + i];
        double *f = F + (size_t)i * n + j;
        const double add = jp * J + kp * K;
        *f = zero_f ? add : fma(fp, *f, add);
    }
}

} // namespace

} // namespace eg

extern "C" eg_status eg_fock_jk_symmetric(double F_prefactor, double *F, double J_prefactor, double K_prefactor,
                                          const double *g, const double *D, int64_t n, void *stream) {
    using namespace eg;
    set_error("");
    if (n < 0) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_fock_jk_symmetric: negative n");
    if (n == 0) return EG_SUCCESS;
    if (!F || !g || !D) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_fock_jk_symmetric: NULL pointer");
    // pair-block shared memory: 64 staged rows of up to n doubles plus two rows of D
    const size_t smem = ((size_t)kFockChunk * (size_t)(n | 1) + 2 * (size_t)n) * sizeof(double);
    if (n > 46340 / 2 || smem > 220 * 1024)
        return fail(EG_ERROR_NOT_SUPPORTED, "eg_fock_jk_symmetric: n = " + std::to_string(n) +
                                                " exceeds the largest supported (" +
                                                std::to_string((220 * 1024 / 8 - 0) / (kFockChunk + 2)) + ")");
    const int nn = (int)n;
    const int nc = (nn + kFockChunk - 1) / kFockChunk;
    const size_t n3 = (size_t)nn * nn * nn;
    const size_t elems = 2 * n3 + 2 * n3 * nc + (size_t)nn * nn * nc + 3 * (size_t)nn * nn;
    cudaStream_t s = (cudaStream_t)stream;
    void *ws = nullptr;
    eg_status st = workspace(s, elems * sizeof(double), &ws);
    if (st != EG_SUCCESS) return st;
    FockScratch sc;
    sc.S1 = (double *)ws;
    sc.S4 = sc.S1 + n3;
    sc.S2 = sc.S4 + n3;
    sc.S5 = sc.S2 + n3 * nc;
    sc.X3 = sc.S5 + n3 * nc;
    sc.X6 = sc.X3 + (size_t)nn * nn * nc;
    sc.YJ = sc.X6 + (size_t)nn * nn;
    sc.XK = sc.YJ + (size_t)nn * nn;
    static bool attr_set = false;
    if (!attr_set) {
        EG_CUDA(cudaFuncSetAttribute(k_fock_pair_blocks, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024));
        attr_set = true;
    }
    {
        LaunchScope ls_("k_fock_pair_blocks", s);
        k_fock_pair_blocks<<<dim3((unsigned)(nn * (nn + 1) / 2), (unsigned)nc), kFockThreads, smem, s>>>(g, D, nn, nc,
                                                                                                        sc);
    }
    EG_CHECK_LAUNCH("k_fock_pair_blocks");
    {
        LaunchScope ls_("k_fock_exchange_blocks", s);
        k_fock_exchange_blocks<<<(unsigned)(nn * nn), kFockThreads, 0, s>>>(g, D, nn, sc.X6);
    }
    EG_CHECK_LAUNCH("k_fock_exchange_blocks");
    {
        LaunchScope ls_("k_fock_reduce", s);
        k_fock_reduce<<<(unsigned)nn, kFockThreads, 0, s>>>(nn, nc, sc);
    }
    EG_CHECK_LAUNCH("k_fock_reduce");
    {
        LaunchScope ls_("k_fock_combine", s);
        k_fock_combine<<<(unsigned)nn, kFockThreads, 0, s>>>(F, nn, sc, F_prefactor, J_prefactor, K_prefactor,
                                                            F_prefactor == 0.0 ? 1 : 0);
    }
    EG_CHECK_LAUNCH("k_fock_combine");
    return EG_SUCCESS;
}
