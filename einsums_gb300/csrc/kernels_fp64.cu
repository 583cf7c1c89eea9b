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

// Sums the per-block partials in a fixed order with Neumaier compensation.
__global__ void __launch_bounds__(kDotThreads) k_dot_final(const double *partial, int nparts, double *C, double cp,
                                                           double ab, bool zero) {
    __shared__ double hi[kDotThreads], lo[kDotThreads];
    double s = 0.0, c = 0.0;
    for (int i = threadIdx.x; i < nparts; i += kDotThreads) {
        const double x = partial[i];
        const double t = s + x;
        c += (fabs(s) >= fabs(x)) ? (s - t) + x : (x - t) + s;
        s = t;
    }
    hi[threadIdx.x] = s;
    lo[threadIdx.x] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        double S = 0.0, Cc = 0.0;
        for (int i = 0; i < kDotThreads; i++) {
            const double x = hi[i];
            const double t = S + x;
            Cc += (fabs(S) >= fabs(x)) ? (S - t) + x : (x - t) + S;
            S = t;
            Cc += lo[i];
        }
        *C = epilogue(S + Cc, C, cp, ab, zero);
    }
}

// ------------------------------------------------------------------- gemv --
// Output positions are walked through `rows` (batch and the non-empty M or N
// group, offsets in A/B/C); every output sums over `k`.
template <int TPR, bool KContig>
__global__ void __launch_bounds__(256) k_gemv(ModeGroup rows, ModeGroup k, const double *__restrict__ A,
                                              const double *__restrict__ B, double *C, double cp, double ab,
                                              bool zero) {
    __shared__ double smem[32];
    constexpr int RPB = 256 / TPR; // rows per block
    const int sub = threadIdx.x / TPR, lane = threadIdx.x % TPR;
    for (int64_t r = (int64_t)blockIdx.x * RPB + sub; r < rows.total; r += (int64_t)gridDim.x * RPB) {
        int64_t ra, rb, rc;
        group_offsets(rows, r, ra, rb, rc);
        const double *a = A + ra;
        const double *b = B + rb;
        double acc0 = 0.0, acc1 = 0.0;
        if (KContig) {
            int64_t i = lane;
            for (; i + TPR < k.total; i += 2 * TPR) {
                acc0 = fma(__ldg(a + i), __ldg(b + i), acc0);
                acc1 = fma(__ldg(a + i + TPR), __ldg(b + i + TPR), acc1);
            }
            if (i < k.total) acc0 = fma(__ldg(a + i), __ldg(b + i), acc0);
        } else {
            for (int64_t i = lane; i < k.total; i += TPR) {
                int64_t oa, ob, oc;
                group_offsets32(k, (uint32_t)i, oa, ob, oc);
                acc0 = fma(__ldg(a + oa), __ldg(b + ob), acc0);
            }
        }
        double s = acc0 + acc1;
        if (TPR == 32) {
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        } else {
            s = block_sum<TPR>(s, smem);
        }
        if (lane == 0) C[rc] = epilogue(s, C + rc, cp, ab, zero);
        if (TPR != 32) __syncthreads();
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
    const ModeGroup &k = c.k;
    if (!fits32(k)) return fail(EG_ERROR_NOT_SUPPORTED, "gemv: summed extent exceeds 2^31");
    const bool contig = k.n == 1 && k.s[0][0] == 1 && k.s[1][0] == 1;
    if (k.total >= 2048) {
        const int grid = grid_for(rows.total, 1);
        if (contig)
            { LaunchScope ls_("k_gemv", s);
            k_gemv<256, true><<<grid, 256, 0, s>>>(rows, k, c.A, c.B, c.C, c.cp, c.ab, c.zero_when_cp_zero);
            }
        else
            { LaunchScope ls_("k_gemv", s);
            k_gemv<256, false><<<grid, 256, 0, s>>>(rows, k, c.A, c.B, c.C, c.cp, c.ab, c.zero_when_cp_zero);
            }
    } else {
        const int grid = grid_for(rows.total, 8);
        if (contig)
            { LaunchScope ls_("k_gemv", s);
            k_gemv<32, true><<<grid, 256, 0, s>>>(rows, k, c.A, c.B, c.C, c.cp, c.ab, c.zero_when_cp_zero);
            }
        else
            { LaunchScope ls_("k_gemv", s);
            k_gemv<32, false><<<grid, 256, 0, s>>>(rows, k, c.A, c.B, c.C, c.cp, c.ab, c.zero_when_cp_zero);
            }
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
