// Plain FP64 kernels of the canonical contraction
//   C[b,m,n] = cp*C + ab * sum_k A[b,m,k] B[b,n,k]
// with every operand addressed through folded index maps, so permuted and
// strided operands are read in place (nothing is materialised).
//
//   k_elementwise   no summed modes: DIRECT / GER / broadcasts
//                   (replaces hipBLASVendor/src/direct_prod.hip:20-200, ger, and
//                    GPUTensorAlgebra.hpp:87-140)
//   k_dot_*         rank-0 C: deterministic two-pass reduction, no atomics
//                   (replaces GPULinearAlgebra.hpp:35-101 and GPUTensorAlgebra.hpp:146-198)
//   k_gemv          one of the M/N groups empty: one CTA or warp per output
//                   (replaces hipblasDgemv at GPULinearAlgebra.hpp:346-386)
//   k_contract_f64  general case: 64x64 register-tiled DFMA contraction
//                   (replaces hipblasDgemm_64 and the atomicAdd generic kernel
//                    GPUTensorAlgebra.hpp:28-82)
#include <algorithm>
#include <utility>

#include "common.cuh"

namespace eg {

namespace {

__device__ __forceinline__ double epilogue(double acc, double *cptr, double cp, double ab, bool zero) {
    const double v = ab * acc;
    if (zero && cp == 0.0) return v;
    return cp * (*cptr) + v;
}

// ----------------------------------------------------------- elementwise --
template <bool Wide>
__global__ void k_elementwise(ModeGroup g, const double *__restrict__ A, const double *__restrict__ B, double *C,
                              double cp, double ab, bool zero) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.total; i += stride) {
        int64_t oa, ob, oc;
        if (Wide)
            group_offsets(g, i, oa, ob, oc);
        else
            group_offsets32(g, (uint32_t)i, oa, ob, oc);
        C[oc] = epilogue(A[oa] * B[ob], C + oc, cp, ab, zero);
    }
}

// C = cp*C over every element of C (or C = 0 when cp == 0), walking C's own
// modes; the prologue the reference applies to the whole output before a
// generic contraction (BaseAlgebra.hpp:129-133), needed when C has repeated
// labels and the contraction itself visits only its diagonal.
template <bool Wide>
__global__ void k_scale(ModeGroup g, double *C, double cp) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < g.total; i += stride) {
        int64_t oa, ob, oc;
        if (Wide)
            group_offsets(g, i, oa, ob, oc);
        else
            group_offsets32(g, (uint32_t)i, oa, ob, oc);
        C[oc] = cp == 0.0 ? 0.0 : cp * C[oc];
    }
}

// ------------------------------------------------------ block reductions --
template <int THREADS>
__device__ __forceinline__ double block_sum(double v, double *smem) {
    // Fixed shuffle tree, then the warp sums in warp order: deterministic.
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    constexpr int W = THREADS / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (W == 1) return v;
    __syncthreads();
    if (lane == 0) smem[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (warp == 0) {
        t = lane < W ? smem[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t; // valid in warp 0
}

// -------------------------------------------------------------------- dot --
constexpr int kDotThreads = 256;

template <bool Contig>
__global__ void __launch_bounds__(kDotThreads) k_dot_partial(ModeGroup k, const double *__restrict__ A,
                                                             const double *__restrict__ B, double *partial,
                                                             int64_t chunk) {
    __shared__ double smem[32];
    const int64_t begin = (int64_t)blockIdx.x * chunk;
    const int64_t end = min(begin + chunk, k.total);
    double acc0 = 0.0, acc1 = 0.0;
    if (Contig) {
        int64_t i = begin + threadIdx.x;
        for (; i + kDotThreads < end; i += 2 * kDotThreads) {
            acc0 = fma(__ldg(A + i), __ldg(B + i), acc0);
            acc1 = fma(__ldg(A + i + kDotThreads), __ldg(B + i + kDotThreads), acc1);
        }
        if (i < end) acc0 = fma(__ldg(A + i), __ldg(B + i), acc0);
    } else {
        for (int64_t i = begin + threadIdx.x; i < end; i += kDotThreads) {
            int64_t oa, ob, oc;
            group_offsets(k, i, oa, ob, oc);
            acc0 = fma(__ldg(A + oa), __ldg(B + ob), acc0);
        }
    }
    const double s = block_sum<kDotThreads>(acc0 + acc1, smem);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// Sums the per-block partials in a fixed order: Neumaier compensation within a
// thread, then a compensated tree across the block.
__global__ void __launch_bounds__(kDotThreads) k_dot_final(const double *partial, int nparts, double *C, double cp,
                                                           double ab, bool zero) {
    __shared__ double sh_s[kDotThreads / 32], sh_c[kDotThreads / 32];
    double s = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < nparts; i += kDotThreads) {
        const double x = partial[i];
        const double t = s + x;
        c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    const double sum = block_sum_compensated<kDotThreads>(s, c, sh_s, sh_c);
    if (threadIdx.x == 0) *C = epilogue(sum, C, cp, ab, zero);
}

// ------------------------------------------------------------------- gemv --
// Output positions are walked through `rows` (batch and the non-empty M or N
// group, offsets in A/B/C); every output sums over `k`.
// KContig: k is one mode of stride 1 in A and B.  Otherwise the offsets of
// every k in A and B come from tables (offk[0..K) for A, offk[K..2K) for B),
// or, when offk is null, from the mode decomposition.  Four independent
// accumulators keep four loads of each operand in flight per thread.
template <int TPR, bool KContig>
__global__ void __launch_bounds__(256) k_gemv(ModeGroup rows, ModeGroup k, const double *__restrict__ A,
                                              const double *__restrict__ B, double *C, double cp, double ab,
                                              bool zero, const int64_t *__restrict__ offk) {
    __shared__ double smem[32];
    constexpr int RPB = 256 / TPR; // rows per block
    const int sub = threadIdx.x / TPR, lane = threadIdx.x % TPR;
    const int64_t K = k.total;
    for (int64_t r = (int64_t)blockIdx.x * RPB + sub; r < rows.total; r += (int64_t)gridDim.x * RPB) {
        int64_t ra, rb, rc;
        group_offsets(rows, r, ra, rb, rc);
        const double *a = A + ra;
        const double *b = B + rb;
        double acc[4] = {0.0, 0.0, 0.0, 0.0};
        int64_t i = lane;
        if (KContig && ((((uintptr_t)a) | ((uintptr_t)b)) & 15) == 0) {
            // 16-byte pairs: eight values of each operand in flight per thread
            const double2 *a2 = (const double2 *)a, *b2 = (const double2 *)b;
            const int64_t K2 = K / 2;
            int64_t j = lane;
            for (; j + 3 * TPR < K2; j += 4 * TPR) {
#pragma unroll
                for (int u = 0; u < 4; u++) {
                    const double2 x = __ldg(a2 + j + u * TPR), y = __ldg(b2 + j + u * TPR);
                    acc[u] = fma(x.x, y.x, acc[u]);
                    acc[u] = fma(x.y, y.y, acc[u]);
                }
            }
            for (; j < K2; j += TPR) {
                const double2 x = __ldg(a2 + j), y = __ldg(b2 + j);
                acc[0] = fma(x.x, y.x, acc[0]);
                acc[0] = fma(x.y, y.y, acc[0]);
            }
            if ((K & 1) && lane == 0) acc[1] = fma(__ldg(a + K - 1), __ldg(b + K - 1), acc[1]);
        } else if (KContig) {
            for (; i + 3 * TPR < K; i += 4 * TPR) {
#pragma unroll
                for (int u = 0; u < 4; u++) acc[u] = fma(__ldg(a + i + u * TPR), __ldg(b + i + u * TPR), acc[u]);
            }
            for (; i < K; i += TPR) acc[0] = fma(__ldg(a + i), __ldg(b + i), acc[0]);
        } else if (offk) {
            for (; i + 3 * TPR < K; i += 4 * TPR) {
#pragma unroll
                for (int u = 0; u < 4; u++)
                    acc[u] = fma(__ldg(a + __ldg(offk + i + u * TPR)), __ldg(b + __ldg(offk + K + i + u * TPR)), acc[u]);
            }
            for (; i < K; i += TPR) acc[0] = fma(__ldg(a + __ldg(offk + i)), __ldg(b + __ldg(offk + K + i)), acc[0]);
        } else {
            for (; i < K; i += TPR) {
                int64_t oa, ob, oc;
                group_offsets32(k, (uint32_t)i, oa, ob, oc);
                acc[0] = fma(__ldg(a + oa), __ldg(b + ob), acc[0]);
            }
        }
        double s = (acc[0] + acc[1]) + (acc[2] + acc[3]);
        if (TPR == 32) {
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        } else {
            s = block_sum<TPR>(s, smem);
        }
        if (lane == 0) C[rc] = epilogue(s, C + rc, cp, ab, zero);
        if (TPR != 32) __syncthreads();
    }
}

// Long k: one CTA takes RB outputs at a time, each k of B (the vector, shared
// by every output) and each pair of table offsets is loaded once and used for
// RB rows of A, so the vector's L1 traffic and the reductions are divided by
// RB.  Contig: k is one mode of stride 1 in A and B (with 16-byte pairs when
// aligned); otherwise offk[0..K) / offk[K..2K) hold the offsets of every k in A
// and B.
template <int RB, bool Contig>
__global__ void __launch_bounds__(256) k_gemv_rows(ModeGroup rows, ModeGroup k, const double *__restrict__ A,
                                                   const double *__restrict__ B, double *C, double cp, double ab,
                                                   bool zero, const int64_t *__restrict__ offk) {
    __shared__ double red[8][RB];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t K = k.total;
    for (int64_t r0 = (int64_t)blockIdx.x * RB; r0 < rows.total; r0 += (int64_t)gridDim.x * RB) {
        const double *a[RB];
        const double *b = B;
        bool aligned = true;
#pragma unroll
        for (int q = 0; q < RB; q++) {
            const int64_t r = r0 + q < rows.total ? r0 + q : rows.total - 1; // tail rows repeat the last one
            int64_t ra, rb, oc;
            group_offsets(rows, r, ra, rb, oc);
            a[q] = A + ra;
            b = B + rb; // the same for every row: the rows run over A's modes only
            aligned &= (((uintptr_t)a[q]) & 15) == 0;
        }
        aligned &= (((uintptr_t)b) & 15) == 0;
        double acc[RB];
#pragma unroll
        for (int q = 0; q < RB; q++) acc[q] = 0.0;
        if (Contig && aligned) {
            const int64_t K2 = K / 2;
            // CTAs start at different points of k so that concurrently read rows
            // (a fixed stride apart) do not hit the same memory channels in step
            const int64_t start = K2 > 4096 ? ((r0 / RB) * 1031 % (K2 / 256)) * 256 : 0;
            auto body = [&](int64_t j) {
                const double2 y = __ldg((const double2 *)b + j);
#pragma unroll
                for (int q = 0; q < RB; q++) {
                    const double2 x = __ldg((const double2 *)a[q] + j);
                    acc[q] = fma(x.x, y.x, acc[q]);
                    acc[q] = fma(x.y, y.y, acc[q]);
                }
            };
            for (int64_t j = start + tid; j < K2; j += 256) body(j);
            for (int64_t j = tid; j < start; j += 256) body(j);
            if ((K & 1) && tid == 0) {
                const double y = __ldg(b + K - 1);
#pragma unroll
                for (int q = 0; q < RB; q++) acc[q] = fma(__ldg(a[q] + K - 1), y, acc[q]);
            }
        } else if (Contig) {
            for (int64_t i = tid; i < K; i += 256) {
                const double y = __ldg(b + i);
#pragma unroll
                for (int q = 0; q < RB; q++) acc[q] = fma(__ldg(a[q] + i), y, acc[q]);
            }
        } else {
            for (int64_t i = tid; i < K; i += 256) {
                const int64_t oa = __ldg(offk + i);
                const double y = __ldg(b + __ldg(offk + K + i));
#pragma unroll
                for (int q = 0; q < RB; q++) acc[q] = fma(__ldg(a[q] + oa), y, acc[q]);
            }
        }
        // fixed-order reduction: warp trees, then the warps in order
#pragma unroll
        for (int q = 0; q < RB; q++) {
            double v = acc[q];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) red[warp][q] = v;
        }
        __syncthreads();
        if (tid < RB && r0 + tid < rows.total) {
            double v = 0.0;
            for (int w = 0; w < 8; w++) v += red[w][tid];
            int64_t ra, rb, oc;
            group_offsets(rows, r0 + tid, ra, rb, oc);
            C[oc] = epilogue(v, C + oc, cp, ab, zero);
        }
        __syncthreads();
    }
}

// Offsets of every k of a mode group in A (out[0..K)) and in B (out[K..2K)).
__global__ void k_k_offsets(ModeGroup k, int64_t *out) {
    const int64_t K = k.total;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < K; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t oa, ob, oc;
        group_offsets32(k, (uint32_t)i, oa, ob, oc);
        out[i] = oa;
        out[K + i] = ob;
    }
}

// ------------------------------------------------------ tiled contraction --
constexpr int BM = 64, BN = 64, BK = 16, kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_contract_f64(ModeGroup bg, ModeGroup mg, ModeGroup ng, ModeGroup kg,
                                                           const double *__restrict__ A, const double *__restrict__ B,
                                                           double *C, double cp, double ab, bool zero, int a_kfast,
                                                           int b_kfast) {
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t m0 = (int64_t)blockIdx.y * BM, n0 = (int64_t)blockIdx.x * BN;
    const int64_t M = mg.total, N = ng.total, K = kg.total;

    // Load assignment: element e = tid + 256*i of the 64x16 tile.  When the
    // operand is contiguous along k, consecutive threads walk k; otherwise m.
    int lm[4], lk[4], ln[4], lkb[4];
    int64_t offA[4], offB[4];
    bool okA[4], okB[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int e = tid + kThreads * i;
        lm[i] = a_kfast ? e / BK : e % BM;
        lk[i] = a_kfast ? e % BK : e / BM;
        ln[i] = b_kfast ? e / BK : e % BN;
        lkb[i] = b_kfast ? e % BK : e / BN;
        int64_t oa, ob, oc;
        okA[i] = m0 + lm[i] < M;
        group_offsets32(mg, (uint32_t)(okA[i] ? m0 + lm[i] : 0), oa, ob, oc);
        offA[i] = oa;
        okB[i] = n0 + ln[i] < N;
        group_offsets32(ng, (uint32_t)(okB[i] ? n0 + ln[i] : 0), oa, ob, oc);
        offB[i] = ob;
    }

    for (int64_t b = blockIdx.z; b < bg.total; b += gridDim.z) {
        int64_t ba, bb, bc;
        group_offsets(bg, b, ba, bb, bc);
        double acc[4][4];
#pragma unroll
        for (int i = 0; i < 4; i++)
#pragma unroll
            for (int j = 0; j < 4; j++) acc[i][j] = 0.0;

        for (int64_t k0 = 0; k0 < K; k0 += BK) {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                const int64_t ka = k0 + lk[i];
                double va = 0.0;
                if (okA[i] && ka < K) {
                    int64_t oa, ob, oc;
                    group_offsets32(kg, (uint32_t)ka, oa, ob, oc);
                    va = __ldg(A + ba + offA[i] + oa);
                }
                As[lk[i]][lm[i]] = va;
                const int64_t kb = k0 + lkb[i];
                double vb = 0.0;
                if (okB[i] && kb < K) {
                    int64_t oa, ob, oc;
                    group_offsets32(kg, (uint32_t)kb, oa, ob, oc);
                    vb = __ldg(B + bb + offB[i] + ob);
                }
                Bs[lkb[i]][ln[i]] = vb;
            }
            __syncthreads();
#pragma unroll
            for (int kk = 0; kk < BK; kk++) {
                double a[4], bv[4];
#pragma unroll
                for (int i = 0; i < 4; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
                for (int j = 0; j < 4; j++) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int j = 0; j < 4; j++) acc[i][j] = fma(a[i], bv[j], acc[i][j]);
            }
            __syncthreads();
        }

#pragma unroll
        for (int i = 0; i < 4; i++) {
            const int64_t m = m0 + ty + 16 * i;
            if (m >= M) continue;
            int64_t ma, mb, mc;
            group_offsets32(mg, (uint32_t)m, ma, mb, mc);
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int64_t n = n0 + tx + 16 * j;
                if (n >= N) continue;
                int64_t na, nb, nc;
                group_offsets32(ng, (uint32_t)n, na, nb, nc);
                double *cptr = C + bc + mc + nc;
                *cptr = epilogue(acc[i][j], cptr, cp, ab, zero);
            }
        }
    }
}

ModeGroup concat(std::initializer_list<const ModeGroup *> groups) {
    ModeGroup g;
    g.total = 1;
    for (const ModeGroup *x : groups)
        for (int d = 0; d < x->n; d++) {
            g.ext[g.n] = x->ext[d];
            for (int t = 0; t < 3; t++) g.s[t][g.n] = x->s[t][d];
            g.total *= x->ext[d];
            g.n++;
        }
    return g;
}

bool fits32(const ModeGroup &g) { return g.total < (int64_t(1) << 31); }

int grid_for(int64_t work, int per_block) {
    int64_t blocks = (work + per_block - 1) / per_block;
    const int64_t cap = (int64_t)num_sms() * 32;
    if (blocks > cap) blocks = cap;
    return (int)(blocks < 1 ? 1 : blocks);
}

} // namespace

eg_status launch_elementwise(const Contraction &c, cudaStream_t s) {
    ModeGroup g = concat({&c.batch, &c.m, &c.n});
    if (g.total == 0) return EG_SUCCESS;
    const int grid = grid_for(g.total, 256);
    if (fits32(g))
        { LaunchScope ls_("k_elementwise", s);
        k_elementwise<false><<<grid, 256, 0, s>>>(g, c.A, c.B, c.C, c.cp, c.ab, c.zero_when_cp_zero);
        }
    else
        { LaunchScope ls_("k_elementwise", s);
        k_elementwise<true><<<grid, 256, 0, s>>>(g, c.A, c.B, c.C, c.cp, c.ab, c.zero_when_cp_zero);
        }
    EG_CHECK_LAUNCH("k_elementwise");
    return EG_SUCCESS;
}

eg_status launch_scale(const ModeGroup &g, double *C, double cp, cudaStream_t s) {
    if (g.total == 0) return EG_SUCCESS;
    const int grid = grid_for(g.total, 256);
    {
        LaunchScope ls_("k_scale", s);
        if (fits32(g))
            k_scale<false><<<grid, 256, 0, s>>>(g, C, cp);
        else
            k_scale<true><<<grid, 256, 0, s>>>(g, C, cp);
    }
    EG_CHECK_LAUNCH("k_scale");
    return EG_SUCCESS;
}

eg_status launch_dot(const Contraction &c, cudaStream_t s) {
    const ModeGroup &k = c.k;
    const int64_t per_block_min = 4096;
    int64_t nblocks = (k.total + per_block_min - 1) / per_block_min;
    const int64_t cap = (int64_t)num_sms() * 8;
    if (nblocks > cap) nblocks = cap;
    if (nblocks < 1) nblocks = 1;
    const int64_t chunk = (k.total + nblocks - 1) / nblocks;
    void *ws = nullptr;
    eg_status st = workspace(s, (size_t)nblocks * sizeof(double), &ws);
    if (st != EG_SUCCESS) return st;
    double *partial = (double *)ws;
    const bool contig = k.n == 1 && k.s[0][0] == 1 && k.s[1][0] == 1;
    if (contig)
        { LaunchScope ls_("k_dot_partial", s);
        k_dot_partial<true><<<(int)nblocks, kDotThreads, 0, s>>>(k, c.A, c.B, partial, chunk);
        }
    else
        { LaunchScope ls_("k_dot_partial", s);
        k_dot_partial<false><<<(int)nblocks, kDotThreads, 0, s>>>(k, c.A, c.B, partial, chunk);
        }
    EG_CHECK_LAUNCH("k_dot_partial");
    { LaunchScope ls_("k_dot_final", s);
    k_dot_final<<<1, kDotThreads, 0, s>>>(partial, (int)nblocks, c.C, c.cp, c.ab, c.zero_when_cp_zero);
    }
    EG_CHECK_LAUNCH("k_dot_final");
    return EG_SUCCESS;
}

eg_status launch_gemv(const Contraction &c, cudaStream_t s) {
    ModeGroup rows = concat({&c.batch, &c.m, &c.n});
    ModeGroup k = c.k;
    if (!fits32(k)) return fail(EG_ERROR_NOT_SUPPORTED, "gemv: summed extent exceeds 2^31");
    const bool contig = k.n == 1 && k.s[0][0] == 1 && k.s[1][0] == 1;
    // Long k, unbatched, one free group: the operand without free modes is a
    // vector shared by every output, and k_gemv_rows reuses it for RB rows.  It
    // takes the rows from its first operand, so when they run over B's modes
    // (M empty) the operands and their stride components are swapped.
    const bool rows_kernel = k.total >= 2048 && c.batch.n == 0 && (c.m.n == 0) != (c.n.n == 0);
    const double *X = c.A, *Y = c.B;
    if (rows_kernel && c.m.n == 0) {
        for (int d = 0; d < rows.n; d++) std::swap(rows.s[0][d], rows.s[1][d]);
        for (int d = 0; d < k.n; d++) std::swap(k.s[0][d], k.s[1][d]);
        std::swap(X, Y);
    }
    // offset tables for a strided k, built once and shared by every output
    int64_t *offk = nullptr;
    if (!contig && k.total <= (int64_t(1) << 24) && rows.total > 1) {
        void *ws = nullptr;
        eg_status st = workspace(s, (size_t)k.total * 2 * sizeof(int64_t), &ws);
        if (st != EG_SUCCESS) return st;
        offk = (int64_t *)ws;
        {
            LaunchScope ls_("k_k_offsets", s);
            k_k_offsets<<<(int)std::min<int64_t>((k.total + 255) / 256, (int64_t)num_sms() * 8), 256, 0, s>>>(k, offk);
        }
        EG_CHECK_LAUNCH("k_k_offsets");
    }
    if (rows_kernel && (contig || offk)) {
        constexpr int RB = 4;
        const int grid = grid_for(rows.total, RB);
        LaunchScope ls_("k_gemv", s);
        if (contig)
            k_gemv_rows<RB, true><<<grid, 256, 0, s>>>(rows, k, X, Y, c.C, c.cp, c.ab, c.zero_when_cp_zero, nullptr);
        else
            k_gemv_rows<RB, false><<<grid, 256, 0, s>>>(rows, k, X, Y, c.C, c.cp, c.ab, c.zero_when_cp_zero, offk);
    } else if (k.total >= 2048) {
        const int grid = grid_for(rows.total, 1);
        LaunchScope ls_("k_gemv", s);
        if (contig)
            k_gemv<256, true><<<grid, 256, 0, s>>>(rows, k, X, Y, c.C, c.cp, c.ab, c.zero_when_cp_zero, nullptr);
        else
            k_gemv<256, false><<<grid, 256, 0, s>>>(rows, k, X, Y, c.C, c.cp, c.ab, c.zero_when_cp_zero, offk);
    } else {
        const int grid = grid_for(rows.total, 8);
        LaunchScope ls_("k_gemv", s);
        if (contig)
            k_gemv<32, true><<<grid, 256, 0, s>>>(rows, k, X, Y, c.C, c.cp, c.ab, c.zero_when_cp_zero, nullptr);
        else
            k_gemv<32, false><<<grid, 256, 0, s>>>(rows, k, X, Y, c.C, c.cp, c.ab, c.zero_when_cp_zero, offk);
    }
    EG_CHECK_LAUNCH("k_gemv");
    return EG_SUCCESS;
}

eg_status launch_contract_f64(const Contraction &c, cudaStream_t s) {
    if (!fits32(c.m) || !fits32(c.n) || !fits32(c.k))
        return fail(EG_ERROR_NOT_SUPPORTED, "contraction: a mode group exceeds 2^31 elements");
    const int64_t gx = (c.n.total + BN - 1) / BN, gy = (c.m.total + BM - 1) / BM;
    if (gy > 65535) return fail(EG_ERROR_NOT_SUPPORTED, "contraction: too many row tiles");
    const int64_t gz = c.batch.total < 65535 ? c.batch.total : 65535;
    const int a_kfast = c.k.n > 0 && c.k.s[0][c.k.n - 1] == 1 && !(c.m.n > 0 && c.m.s[0][c.m.n - 1] == 1);
    const int b_kfast = c.k.n > 0 && c.k.s[1][c.k.n - 1] == 1 && !(c.n.n > 0 && c.n.s[1][c.n.n - 1] == 1);
    dim3 grid((unsigned)gx, (unsigned)gy, (unsigned)(gz < 1 ? 1 : gz));
    { LaunchScope ls_("k_contract_f64", s);
    k_contract_f64<<<grid, kThreads, 0, s>>>(c.batch, c.m, c.n, c.k, c.A, c.B, c.C, c.cp, c.ab, c.zero_when_cp_zero,
                                             a_kfast, b_kfast);
    }
    EG_CHECK_LAUNCH("k_contract_f64");
    return EG_SUCCESS;
}

} // namespace eg
