// Grouped execution of many independent contractions that share one index
// pattern but not their extents (the reference's list einsum,
// Backends/Dispatch.hpp:1264-1286, and block-sparse blocks).
//
// A plan lowers every item to the canonical contraction, builds a device-side
// work list of output tiles (largest first), and captures the whole batch as
// a CUDA graph that later calls replay:
//   * FP64: one persistent launch of k_grouped_f64 over the work list; each
//     entry computes a 32x32 or 64x64 tile with the DFMA core, the tile size
//     chosen per shape bucket by the autotuner (autotune.cpp);
//   * split-BF16: three digit-splitting launches per operand covering every
//     item (grouped variants of split.cu's kernels, unit -> item by binary
//     search over a prefix table), then one persistent launch of the
//     tcgen05 GEMM over the work list (k_tc_split_gemm<true>).
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "grouped.cuh"
#include "split.cuh"

namespace eg {
eg_status lower_for_group(double cp, const int32_t *Cl, const eg_tensor *C, double ab, const int32_t *Al,
                          const eg_tensor *A, const int32_t *Bl, const eg_tensor *B, const eg_options &opt,
                          Contraction &out, int32_t *alg_out, bool &gemm_shaped);
eg_status encode_planes_public(CUtensorMap *map, void *base, int64_t Kp, int64_t rows, int64_t planes);
int64_t mode_group_affine_stride(const ModeGroup &g, int comp);
eg_status encode_planes_extent(CUtensorMap *map, void *base, int64_t K, int64_t rows, int64_t planes, int64_t Kp,
                               int64_t Rp);
void set_capture_mode(bool on);
void count_launches(uint64_t n);
} // namespace eg

namespace eg::grouped {

namespace {

// ------------------------------------------------------------ FP64 tiles --
struct F64Item {
    const double *A, *B;
    double *C;
    ModeGroup b, m, n, k;
    int a_kfast, b_kfast;
};

constexpr int BK = 16, THREADS = 256, LD = 65;

template <int T>
__device__ __forceinline__ void f64_tile(const F64Item &it, int64_t bidx, int mt, int nt, double cp, double ab,
                                         bool zero, double (*As)[LD], double (*Bs)[LD]) {
    constexpr int R = T / 16; // outputs per thread per dimension, and loads per thread per operand
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t m0 = (int64_t)mt * T, n0 = (int64_t)nt * T;
    const int64_t M = it.m.total, N = it.n.total, K = it.k.total;
    int64_t ba, bb, bc;
    group_offsets(it.b, bidx, ba, bb, bc);
    int lm[R], lk[R], ln[R], lkb[R];
    int64_t offA[R], offB[R];
    bool okA[R], okB[R];
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int e = tid + THREADS * i;
        lm[i] = it.a_kfast ? e / BK : e % T;
        lk[i] = it.a_kfast ? e % BK : e / T;
        ln[i] = it.b_kfast ? e / BK : e % T;
        lkb[i] = it.b_kfast ? e % BK : e / T;
        int64_t oa, ob, oc;
        okA[i] = m0 + lm[i] < M;
        group_offsets32(it.m, (uint32_t)(okA[i] ? m0 + lm[i] : 0), oa, ob, oc);
        offA[i] = ba + oa;
        okB[i] = n0 + ln[i] < N;
        group_offsets32(it.n, (uint32_t)(okB[i] ? n0 + ln[i] : 0), oa, ob, oc);
        offB[i] = bb + ob;
    }
    double acc[R][R];
#pragma unroll
    for (int i = 0; i < R; i++)
#pragma unroll
        for (int j = 0; j < R; j++) acc[i][j] = 0.0;
    for (int64_t k0 = 0; k0 < K; k0 += BK) {
#pragma unroll
        for (int i = 0; i < R; i++) {
            const int64_t ka = k0 + lk[i];
            double va = 0.0;
            if (okA[i] && ka < K) {
                int64_t oa, ob, oc;
                group_offsets32(it.k, (uint32_t)ka, oa, ob, oc);
                va = __ldg(it.A + offA[i] + oa);
            }
            As[lk[i]][lm[i]] = va;
            const int64_t kb = k0 + lkb[i];
            double vb = 0.0;
            if (okB[i] && kb < K) {
                int64_t oa, ob, oc;
                group_offsets32(it.k, (uint32_t)kb, oa, ob, oc);
                vb = __ldg(it.B + offB[i] + ob);
            }
            Bs[lkb[i]][ln[i]] = vb;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; kk++) {
            double a[R], b[R];
#pragma unroll
            for (int i = 0; i < R; i++) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < R; j++) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < R; i++)
#pragma unroll
                for (int j = 0; j < R; j++) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int64_t m = m0 + ty + 16 * i;
        if (m >= M) continue;
        int64_t ma, mb, mc;
        group_offsets32(it.m, (uint32_t)m, ma, mb, mc);
#pragma unroll
        for (int j = 0; j < R; j++) {
            const int64_t n = n0 + tx + 16 * j;
            if (n >= N) continue;
            int64_t na, nb, nc;
            group_offsets32(it.n, (uint32_t)n, na, nb, nc);
            double *cptr = it.C + bc + mc + nc;
            const double v = ab * acc[i][j];
            *cptr = (zero && cp == 0.0) ? v : cp * (*cptr) + v;
        }
    }
}

// Work entry: {item, batch index, mt, nt}; tile size per item in `tiles`.
__global__ void __launch_bounds__(THREADS) k_grouped_f64(const F64Item *items, const int *tiles, const int4 *work,
                                                          int nwork, double cp, double ab, int zero) {
    __shared__ double As[BK][LD];
    __shared__ double Bs[BK][LD];
    for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
        const int4 e = work[w];
        const F64Item &it = items[e.x];
        if (tiles[e.x] == 64)
            f64_tile<64>(it, e.y, e.z, e.w, cp, ab, zero != 0, As, Bs);
        else
            f64_tile<32>(it, e.y, e.z, e.w, cp, ab, zero != 0, As, Bs);
    }
}

// --------------------------------------------------- grouped digit split --
struct GOp {
    const double *X;
    ModeGroup bg, rg, kg;
    int comp;             // 0: A, 1: B
    int row_fast;         // operand contiguous along rows
    int nbatch;
    int64_t rows, Rp, K, Kp;
    int64_t rowbase;      // first entry in the row-max / exponent arrays
    int64_t zbase;        // first digit plane
    int64_t rtab, ktab;   // first entries of this operand's row and K offsets in the plan's offset table
    int64_t sr, sk;       // the single element stride of the rows / of K when the modes nest (else 0: tables)
};

__device__ __forceinline__ int64_t pick(int comp, int64_t oa, int64_t ob) { return comp == 0 ? oa : ob; }

// One work unit = 32 rows of one operand of one item (and batch index): the
// rows' maxima (the operand is read once along its contiguous direction), their
// exponents, then the digit planes of those rows, written K-major in BF16 pairs
// through a 32 x 64 shared tile when the operand is contiguous along its rows.
// Only the real rows and K are written: the planes and exponents of padded rows
// and of K beyond the item's extent are zeroed once when the plan is built and
// never written after.
constexpr int kGU = 32, kGK = 64, kGThreads = 256, kGWarps = kGThreads / 32;

template <int S>
__global__ void __launch_bounds__(kGThreads, 4) k_grouped_split(const GOp *ops, const int4 *units, int nunits,
                                                             const long long *__restrict__ offs, int *rexpA,
                                                             int *rexpB, __nv_bfloat16 *planesA,
                                                             __nv_bfloat16 *planesB, int64_t Rmax, int64_t Kmaxp) {
    __shared__ double tile[kGU][kGK + 1];
    __shared__ unsigned long long red[kGWarps][kGU];
    __shared__ int ex[kGU];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int u = blockIdx.x; u < nunits; u += gridDim.x) {
        const int4 un = units[u];
        const GOp &g = ops[un.x];
        const int64_t b = un.y, r0 = un.z;
        const int64_t K = g.K;
        const int nr = (int)(g.rows - r0 < kGU ? g.rows - r0 : kGU);
        const long long *koff = offs + g.ktab; // element offset of each k in this operand
        const int64_t sk = g.sk;
        auto kofs = [&](int64_t k) -> int64_t { return sk ? k * sk : (int64_t)__ldg(koff + k); };
        const double *X = g.X;
        int64_t oa, ob, oc;
        group_offsets(g.bg, b, oa, ob, oc);
        const int64_t obase = pick(g.comp, oa, ob);
        const bool row_fast = g.row_fast != 0;
        // row offsets: the lane's row (rows contiguous) or the warp's rows w + 8j (K contiguous)
        int64_t orow[kGU / kGWarps];
#pragma unroll
        for (int j = 0; j < kGU / kGWarps; j++) {
            const int rr = row_fast ? lane : w + kGWarps * j;
            orow[j] = (rr < nr && (j == 0 || !row_fast))
                          ? obase + (g.sr ? (r0 + rr) * g.sr : (int64_t)__ldg(offs + g.rtab + r0 + rr))
                          : 0;
        }
        // phase 1: row maxima of |x| as IEEE bit patterns
        if (row_fast) {
            unsigned long long mx = 0;
            if (lane < nr) {
#pragma unroll 8
                for (int64_t k = w; k < K; k += kGWarps)
                    mx = max(mx, split::abs_bits(__ldg(X + orow[0] + kofs(k))));
            }
            red[w][lane] = mx;
        } else {
#pragma unroll
            for (int j = 0; j < kGU / kGWarps; j++) {
                const int rr = w + kGWarps * j;
                unsigned long long mx = 0;
                if (rr < nr) {
#pragma unroll 4
                    for (int64_t k = lane; k < K; k += 32)
                        mx = max(mx, split::abs_bits(__ldg(X + orow[j] + kofs(k))));
                }
                for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
                if (lane == 0) {
                    red[0][rr] = mx;
                    for (int q = 1; q < kGWarps; q++) red[q][rr] = 0;
                }
            }
        }
        __syncthreads();
        if (w == 0) {
            unsigned long long mx = red[0][lane];
            for (int q = 1; q < kGWarps; q++) mx = max(mx, red[q][lane]);
            const double m = __longlong_as_double((long long)mx);
            int e = 0;
            if (!isfinite(m))
                e = INT_MIN;
            else if (m > 0.0)
                frexp(m, &e);
            ex[lane] = e;
            if (lane < nr) (g.comp ? rexpB : rexpA)[g.rowbase + b * g.Rp + r0 + lane] = e;
        }
        __syncthreads();
        // phase 2: digit planes, 64 K at a time
        __nv_bfloat16 *planes = g.comp ? planesB : planesA;
        const int64_t z0 = g.zbase + b * S;
        for (int64_t k0 = 0; k0 < K; k0 += kGK) {
            if (row_fast) {
#pragma unroll
                for (int kk = w; kk < kGK; kk += kGWarps) {
                    const int64_t k = k0 + kk;
                    tile[lane][kk] = (k < K && lane < nr) ? __ldg(X + orow[0] + kofs(k)) : 0.0;
                }
            } else {
#pragma unroll
                for (int j = 0; j < kGU / kGWarps; j++) {
                    const int rr = w + kGWarps * j;
#pragma unroll
                    for (int h = 0; h < kGK / 32; h++) {
                        const int64_t k = k0 + lane + 32 * h;
                        tile[rr][lane + 32 * h] = (rr < nr && k < K) ? __ldg(X + orow[j] + kofs(k)) : 0.0;
                    }
                }
            }
            __syncthreads();
            const int64_t k = k0 + 2 * lane;
#pragma unroll
            for (int j = 0; j < kGU / kGWarps; j++) {
                const int rr = w + kGWarps * j;
                if (rr < nr && k < K) {
                    uint32_t pk[S];
                    const int e = ex[rr];
                    if (e == INT_MIN) {
#pragma unroll
                        for (int q = 0; q < S; q++) pk[q] = 0u;
                    } else {
                        split::digits_bf16x2<S>(tile[rr][2 * lane], tile[rr][2 * lane + 1], e, pk);
                    }
#pragma unroll
                    for (int q = 0; q < S; q++)
                        *reinterpret_cast<uint32_t *>(planes + ((z0 + q) * Rmax + r0 + rr) * Kmaxp + k) = pk[q];
                }
            }
            __syncthreads();
        }
    }
}

template <int S>
void launch_grouped_split_s(const GOp *ops, const int4 *units, int nunits, const long long *offs, int *eA, int *eB,
                            __nv_bfloat16 *pA, __nv_bfloat16 *pB, int64_t Rmax, int64_t Kmaxp, cudaStream_t s) {
    const int grid = (int)std::min<int64_t>(std::max(nunits, 1), (int64_t)num_sms() * 8);
    k_grouped_split<S><<<grid, kGThreads, 0, s>>>(ops, units, nunits, offs, eA, eB, pA, pB, Rmax, Kmaxp);
}

void launch_grouped_split(int S, const GOp *ops, const int4 *units, int nunits, const long long *offs, int *eA,
                          int *eB, __nv_bfloat16 *pA, __nv_bfloat16 *pB, int64_t Rmax, int64_t Kmaxp, cudaStream_t s) {
    switch (S) {
    case 2: launch_grouped_split_s<2>(ops, units, nunits, offs, eA, eB, pA, pB, Rmax, Kmaxp, s); break;
    case 3: launch_grouped_split_s<3>(ops, units, nunits, offs, eA, eB, pA, pB, Rmax, Kmaxp, s); break;
    case 4: launch_grouped_split_s<4>(ops, units, nunits, offs, eA, eB, pA, pB, Rmax, Kmaxp, s); break;
    case 5: launch_grouped_split_s<5>(ops, units, nunits, offs, eA, eB, pA, pB, Rmax, Kmaxp, s); break;
    default: launch_grouped_split_s<6>(ops, units, nunits, offs, eA, eB, pA, pB, Rmax, Kmaxp, s); break;
    }
}

int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

bool fast_along(const ModeGroup &g, int comp) { return g.n > 0 && g.s[comp][g.n - 1] == 1; }

} // namespace

// ------------------------------------------------------------------ plan --

namespace {

eg_status dev_copy(Plan &plan, const void *host, size_t bytes, void **dev) {
    void *p = nullptr;
    eg_status st = tracked_malloc(bytes ? bytes : 16, &p);
    if (st != EG_SUCCESS) return st;
    plan.owned.push_back(p);
    if (bytes) EG_CUDA(cudaMemcpy(p, host, bytes, cudaMemcpyHostToDevice));
    *dev = p;
    return EG_SUCCESS;
}

eg_status dev_alloc(Plan &plan, size_t bytes, void **dev) {
    void *p = nullptr;
    eg_status st = tracked_malloc(bytes ? bytes : 16, &p);
    if (st != EG_SUCCESS) return st;
    plan.owned.push_back(p);
    *dev = p;
    return EG_SUCCESS;
}

struct CaptureGuard {
    CaptureGuard() { set_capture_mode(true); }
    ~CaptureGuard() { set_capture_mode(false); }
};

// Issues the FP64 grouped launch on `s` (captured by the caller).
eg_status issue_f64(const F64Item *items, const int *tiles, const int4 *work, int nwork, double cp, double ab,
                    int zero, cudaStream_t s) {
    if (nwork <= 0) return EG_SUCCESS;
    const int grid = std::min(nwork, num_sms() * 8);
    {
        LaunchScope ls_("k_grouped_f64", s);
        k_grouped_f64<<<grid, THREADS, 0, s>>>(items, tiles, work, nwork, cp, ab, zero);
    }
    EG_CHECK_LAUNCH("k_grouped_f64");
    return EG_SUCCESS;
}

// Cost-ordered work list (largest K first) of tiles of size tile[item].
std::vector<int4> f64_work(const std::vector<Contraction> &cs, const std::vector<int> &tiles) {
    std::vector<std::pair<int64_t, int4>> w;
    for (size_t i = 0; i < cs.size(); i++) {
        const int T = tiles[i];
        const int64_t mt = (cs[i].m.total + T - 1) / T, nt = (cs[i].n.total + T - 1) / T;
        for (int64_t b = 0; b < cs[i].batch.total; b++)
            for (int64_t x = 0; x < mt; x++)
                for (int64_t y = 0; y < nt; y++)
                    w.push_back({cs[i].k.total * T * T, make_int4((int)i, (int)b, (int)x, (int)y)});
    }
    std::stable_sort(w.begin(), w.end(), [](auto &a, auto &b) { return a.first > b.first; });
    std::vector<int4> out;
    out.reserve(w.size());
    for (auto &e : w) out.push_back(e.second);
    return out;
}

F64Item f64_item(const Contraction &c) {
    F64Item it;
    it.A = c.A;
    it.B = c.B;
    it.C = c.C;
    it.b = c.batch;
    it.m = c.m;
    it.n = c.n;
    it.k = c.k;
    it.a_kfast = c.k.n > 0 && c.k.s[0][c.k.n - 1] == 1 && !(c.m.n > 0 && c.m.s[0][c.m.n - 1] == 1);
    it.b_kfast = c.k.n > 0 && c.k.s[1][c.k.n - 1] == 1 && !(c.n.n > 0 && c.n.s[1][c.n.n - 1] == 1);
    return it;
}

// Times a FP64 grouped launch of `items` with tile size T into scratch outputs.
eg_status time_f64(const std::vector<Contraction> &bucket, int T, cudaStream_t s, float *ms) {
    // outputs redirected to compact scratch so user data is untouched
    std::vector<Contraction> cs = bucket;
    size_t total = 0;
    for (auto &c : cs) total += (size_t)(c.batch.total * c.m.total * c.n.total);
    Plan tmp;
    void *scratch = nullptr;
    eg_status st = dev_alloc(tmp, total * sizeof(double), &scratch);
    if (st != EG_SUCCESS) return st;
    size_t off = 0;
    std::vector<F64Item> items;
    for (auto &c : cs) {
        c.C = (double *)scratch + off;
        // compact C strides: batch, m, n row-major
        int64_t stride = 1;
        for (int d = c.n.n - 1; d >= 0; d--) {
            c.n.s[2][d] = stride;
            stride *= c.n.ext[d];
        }
        for (int d = c.m.n - 1; d >= 0; d--) {
            c.m.s[2][d] = stride;
            stride *= c.m.ext[d];
        }
        for (int d = c.batch.n - 1; d >= 0; d--) {
            c.batch.s[2][d] = stride;
            stride *= c.batch.ext[d];
        }
        off += (size_t)(c.batch.total * c.m.total * c.n.total);
        items.push_back(f64_item(c));
    }
    std::vector<int> tiles(cs.size(), T);
    auto work = f64_work(cs, tiles);
    void *d_items, *d_tiles, *d_work;
    if ((st = dev_copy(tmp, items.data(), items.size() * sizeof(F64Item), &d_items)) != EG_SUCCESS) return st;
    if ((st = dev_copy(tmp, tiles.data(), tiles.size() * sizeof(int), &d_tiles)) != EG_SUCCESS) return st;
    if ((st = dev_copy(tmp, work.data(), work.size() * sizeof(int4), &d_work)) != EG_SUCCESS) return st;
    cudaEvent_t e0, e1;
    EG_CUDA(cudaEventCreate(&e0));
    EG_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int rep = 0; rep < 3; rep++) {
        EG_CUDA(cudaEventRecord(e0, s));
        st = issue_f64((F64Item *)d_items, (int *)d_tiles, (int4 *)d_work, (int)work.size(), 0.0, 1.0, 1, s);
        if (st != EG_SUCCESS) break;
        EG_CUDA(cudaEventRecord(e1, s));
        EG_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        EG_CUDA(cudaEventElapsedTime(&t, e0, e1));
        if (rep > 0) best = std::min(best, t);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = best;
    return st;
}

} // namespace

// Chooses the FP64 tile size of every item: per shape bucket from the tuning
// cache, timing both sizes on the bucket's items when the cache has no entry.
eg_status choose_f64_tiles(const std::vector<Contraction> &cs, cudaStream_t s, std::vector<int> &tiles) {
    tiles.assign(cs.size(), 64);
    std::map<std::string, std::vector<size_t>> buckets;
    for (size_t i = 0; i < cs.size(); i++)
        buckets[autotune::bucket_key("f64", cs[i].m.total, cs[i].n.total, cs[i].k.total)].push_back(i);
    for (auto &kv : buckets) {
        int choice = 0;
        if (!autotune::lookup(kv.first, &choice)) {
            if (autotune::enabled()) {
                std::vector<Contraction> sample;
                for (size_t j = 0; j < kv.second.size() && j < 256; j++) sample.push_back(cs[kv.second[j]]);
                float t32 = 0, t64 = 0;
                eg_status st = time_f64(sample, 32, s, &t32);
                if (st != EG_SUCCESS) return st;
                if ((st = time_f64(sample, 64, s, &t64)) != EG_SUCCESS) return st;
                choice = t32 < t64 ? 32 : 64;
                autotune::store(kv.first, choice);
            } else {
                const Contraction &c = cs[kv.second[0]];
                choice = (c.m.total <= 48 || c.n.total <= 48) ? 32 : 64;
            }
        }
        for (size_t i : kv.second) tiles[i] = choice;
    }
    return EG_SUCCESS;
}

// Builds and captures the FP64 plan.
eg_status build_f64_plan(Plan &plan, const std::vector<Contraction> &cs, cudaStream_t s) {
    std::vector<int> tiles;
    eg_status st = choose_f64_tiles(cs, s, tiles);
    if (st != EG_SUCCESS) return st;
    std::vector<F64Item> items;
    for (auto &c : cs) items.push_back(f64_item(c));
    auto work = f64_work(cs, tiles);
    void *d_items, *d_tiles, *d_work;
    if ((st = dev_copy(plan, items.data(), items.size() * sizeof(F64Item), &d_items)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, tiles.data(), tiles.size() * sizeof(int), &d_tiles)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, work.data(), work.size() * sizeof(int4), &d_work)) != EG_SUCCESS) return st;
    const Contraction &c0 = cs[0];
    EG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    {
        CaptureGuard g;
        st = issue_f64((F64Item *)d_items, (int *)d_tiles, (int4 *)d_work, (int)work.size(), c0.cp, c0.ab,
                       c0.zero_when_cp_zero ? 1 : 0, s);
    }
    cudaGraph_t graph = nullptr;
    cudaError_t err = cudaStreamEndCapture(s, &graph);
    if (st != EG_SUCCESS) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (err != cudaSuccess) return cuda_fail(err, "cudaStreamEndCapture");
    plan.graph = graph;
    EG_CUDA(cudaGraphInstantiate(&plan.exec, graph, 0));
    plan.kernels = work.empty() ? 0 : 1;
    return EG_SUCCESS;
}

// Builds and captures the split-BF16 plan; returns EG_ERROR_NOT_SUPPORTED when
// an item's K needs more than one exact pass (the caller then runs items one by one).
eg_status build_split_plan(Plan &plan, const std::vector<Contraction> &cs, int slices, cudaStream_t s) {
    using namespace split;
    const int S = slices ? slices : 5;
    if (S < 2 || S > kMaxSlices) return fail(EG_ERROR_INVALID_ARGUMENT, "split form: slices must be in 2..6");
    const int64_t kmax = max_k_per_pass(S);
    int64_t Rmax = kBM, Kmaxp = kKStep, zA = 0, zB = 0, rowsA = 0, rowsB = 0;
    for (auto &c : cs) {
        if (c.k.total > kmax) return fail(EG_ERROR_NOT_SUPPORTED, "grouped split: K above one exact pass");
        if (c.k.total <= 0) return fail(EG_ERROR_NOT_SUPPORTED, "grouped split: an item sums over no index");
        if (c.m.total >= (1ll << 31) || c.n.total >= (1ll << 31) || c.k.total >= (1ll << 31))
            return fail(EG_ERROR_NOT_SUPPORTED, "grouped split: extent above 2^31");
        Rmax = std::max({Rmax, round_up(c.m.total, kBM), round_up(c.n.total, kBN)});
        Kmaxp = std::max(Kmaxp, round_up(c.k.total, kKStep));
    }
    std::vector<GOp> opsA, opsB;
    std::vector<TcItem> items;
    std::vector<std::pair<int64_t, int4>> work;
    std::vector<int4> units; // (operand, batch index, first row); operands A then B of every item
    for (size_t i = 0; i < cs.size(); i++) {
        const Contraction &c = cs[i];
        const int64_t nb = c.batch.total, M = c.m.total, N = c.n.total, K = c.k.total;
        const int64_t Kp = round_up(K, kKStep), Mp = round_up(M, kBM), Np = round_up(N, kBN);
        GOp a{};
        a.X = c.A;
        a.bg = c.batch;
        a.rg = c.m;
        a.kg = c.k;
        a.comp = 0;
        a.row_fast = !fast_along(c.k, 0) && fast_along(c.m, 0);
        a.nbatch = (int)nb;
        a.rows = M;
        a.Rp = Mp;
        a.K = K;
        a.Kp = Kp;
        a.rowbase = rowsA;
        a.zbase = zA;
        a.sr = mode_group_affine_stride(c.m, 0);
        a.sk = mode_group_affine_stride(c.k, 0);
        GOp b = a;
        b.X = c.B;
        b.rg = c.n;
        b.comp = 1;
        b.row_fast = !fast_along(c.k, 1) && fast_along(c.n, 1);
        b.rows = N;
        b.Rp = Np;
        b.rowbase = rowsB;
        b.zbase = zB;
        b.sr = mode_group_affine_stride(c.n, 1);
        b.sk = mode_group_affine_stride(c.k, 1);
        opsA.push_back(a);
        opsB.push_back(b);
        TcItem it{};
        it.C = c.C;
        it.M = M;
        it.N = N;
        it.nkb = (int)(Kp / kBK);
        it.zA = (int)zA;
        it.zB = (int)zB;
        it.eAoff = (int)rowsA;
        it.eBoff = (int)rowsB;
        it.Mp = (int)Mp;
        it.Np = (int)Np;
        it.bg = c.batch;
        it.mg = c.m;
        it.ng = c.n;
        items.push_back(it);
        for (int64_t bb = 0; bb < nb; bb++)
            for (int64_t x = 0; x < Mp / kBM; x++)
                for (int64_t y = 0; y < Np / kBN; y++)
                    work.push_back({Kp, make_int4((int)i, (int)bb, (int)x, (int)y)});
        rowsA += nb * Mp;
        rowsB += nb * Np;
        zA += nb * S;
        zB += nb * S;
    }
    if (zA >= (1ll << 31) || rowsA >= (1ll << 31) || rowsB >= (1ll << 31))
        return fail(EG_ERROR_NOT_SUPPORTED, "grouped split: batch too large");
    std::stable_sort(work.begin(), work.end(), [](auto &x, auto &y) { return x.first > y.first; });
    std::vector<int4> wl;
    for (auto &w : work) wl.push_back(w.second);
    // one splitting unit per 32 real rows of every operand (and batch index)
    std::vector<GOp> ops(opsA);
    ops.insert(ops.end(), opsB.begin(), opsB.end());
    // row and K element offsets of every operand, fixed by the strides: built once here
    std::vector<long long> offs;
    for (auto &op : ops) {
        int64_t oa, ob, oc;
        op.rtab = (int64_t)offs.size();
        for (int64_t r = 0; r < op.rows; r++) {
            group_offsets(op.rg, r, oa, ob, oc);
            offs.push_back(op.comp ? ob : oa);
        }
        op.ktab = (int64_t)offs.size();
        for (int64_t k = 0; k < op.K; k++) {
            group_offsets(op.kg, k, oa, ob, oc);
            offs.push_back(op.comp ? ob : oa);
        }
    }
    for (size_t i = 0; i < ops.size(); i++)
        for (int64_t bb = 0; bb < ops[i].nbatch; bb++)
            for (int64_t r0 = 0; r0 < ops[i].rows; r0 += 32) units.push_back(make_int4((int)i, (int)bb, (int)r0, 0));
    if (units.size() >= (size_t)INT_MAX) return fail(EG_ERROR_NOT_SUPPORTED, "grouped split: batch too large");

    void *planesA, *planesB, *eA, *eB, *d_ops, *d_units, *d_offs, *d_items, *d_work, *rbuf;
    eg_status st;
    if ((st = dev_alloc(plan, rbuf_bytes(), &rbuf)) != EG_SUCCESS) return st;
    const size_t pbytesA = (size_t)zA * Rmax * Kmaxp * 2, pbytesB = (size_t)zB * Rmax * Kmaxp * 2;
    if ((st = dev_alloc(plan, pbytesA, &planesA)) != EG_SUCCESS) return st;
    if ((st = dev_alloc(plan, pbytesB, &planesB)) != EG_SUCCESS) return st;
    if ((st = dev_alloc(plan, (size_t)rowsA * 4, &eA)) != EG_SUCCESS) return st;
    if ((st = dev_alloc(plan, (size_t)rowsB * 4, &eB)) != EG_SUCCESS) return st;
    // padded rows and K are never written by the splitting kernel: zero them once
    EG_CUDA(cudaMemsetAsync(planesA, 0, pbytesA, s));
    EG_CUDA(cudaMemsetAsync(planesB, 0, pbytesB, s));
    EG_CUDA(cudaMemsetAsync(eA, 0, (size_t)rowsA * 4, s));
    EG_CUDA(cudaMemsetAsync(eB, 0, (size_t)rowsB * 4, s));
    if ((st = dev_copy(plan, ops.data(), ops.size() * sizeof(GOp), &d_ops)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, units.data(), units.size() * sizeof(int4), &d_units)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, offs.data(), offs.size() * sizeof(long long), &d_offs)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, items.data(), items.size() * sizeof(TcItem), &d_items)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, wl.data(), wl.size() * sizeof(int4), &d_work)) != EG_SUCCESS) return st;

    CUtensorMap tmA, tmB;
    if ((st = encode_planes_public(&tmA, planesA, Kmaxp, Rmax, zA)) != EG_SUCCESS) return st;
    if ((st = encode_planes_public(&tmB, planesB, Kmaxp, Rmax, zB)) != EG_SUCCESS) return st;
    // per-item maps: each item's planes with its own M (N) and K as the extents
    std::vector<CUtensorMap> maps(2 * items.size());
    for (size_t i = 0; i < items.size(); i++) {
        const TcItem &it = items[i];
        const Contraction &c = cs[i];
        if (it.M == 0 || it.N == 0 || c.batch.total == 0) continue; // no tiles: the maps are never used
        const int64_t planes = c.batch.total * S, K = c.k.total;
        const size_t plane = (size_t)Rmax * Kmaxp;
        if ((st = encode_planes_extent(&maps[2 * i], (__nv_bfloat16 *)planesA + (size_t)it.zA * plane, K, it.M, planes,
                                       Kmaxp, Rmax)) != EG_SUCCESS)
            return st;
        if ((st = encode_planes_extent(&maps[2 * i + 1], (__nv_bfloat16 *)planesB + (size_t)it.zB * plane, K, it.N,
                                       planes, Kmaxp, Rmax)) != EG_SUCCESS)
            return st;
    }
    void *d_maps = nullptr;
    if ((st = dev_copy(plan, maps.data(), maps.size() * sizeof(CUtensorMap), &d_maps)) != EG_SUCCESS) return st;
    int *status = nullptr;
    if ((st = status_word(s, &status)) != EG_SUCCESS) return st;

    const Contraction &c0 = cs[0];
    TcGemmParams p{};
    p.S = S;
    p.nbatch = 1;
    p.cp = c0.cp;
    p.ab = c0.ab;
    p.zero = c0.zero_when_cp_zero ? 1 : 0;
    p.eA = (int *)eA;
    p.eB = (int *)eB;
    p.shift_const = -2 * kTopBits - kBits * (S - 1);
    {
        int k = 0;
        const double f = std::frexp(std::fabs(c0.ab), &k);
        p.ab_pow2 = (f == 0.5) ? 1 : 0;
        p.ab_neg = (p.ab_pow2 && c0.ab < 0) ? 1 : 0;
        if (p.ab_pow2) p.shift_const += k - 1;
    }
    p.status = status;
    p.timeout_ns = 2000ull * 1000 * 1000;
    p.d0 = 0; // every slice group in one launch (K fits one exact pass)
    p.d1 = S;
    p.ksplit = 1; // no K slicing in grouped launches
    p.kslice = 0;
    p.item_maps = (const CUtensorMap *)d_maps;
    p.rbuf = (long long *)rbuf;
    static const bool prof_on = std::getenv("EINSUMS_GB300_TC_PROFILE") != nullptr;
    if (prof_on) {
        // per-role cycle counters summed over the plan's replays, printed when it is destroyed
        void *prof = nullptr;
        const size_t pbytes = (size_t)num_sms() * 8 * sizeof(unsigned long long);
        if ((st = dev_alloc(plan, pbytes, &prof)) != EG_SUCCESS) return st;
        EG_CUDA(cudaMemsetAsync(prof, 0, pbytes, s));
        p.prof = (unsigned long long *)prof;
        plan.prof = p.prof;
    }

    if ((st = ensure_tc_attributes()) != EG_SUCCESS) return st;
    EG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    {
        CaptureGuard g;
        auto issue = [&]() -> eg_status {
            launch_grouped_split(S, (const GOp *)d_ops, (const int4 *)d_units, (int)units.size(),
                                 (const long long *)d_offs, (int *)eA, (int *)eB,
                                 (__nv_bfloat16 *)planesA, (__nv_bfloat16 *)planesB, Rmax, Kmaxp, s);
            EG_CHECK_LAUNCH("grouped digit splitting");
            return launch_tc_gemm_grouped(tmA, tmB, p, (TcItem *)d_items, (int4 *)d_work, (int)wl.size(), s);
        };
        st = issue();
    }
    cudaGraph_t graph = nullptr;
    cudaError_t err = cudaStreamEndCapture(s, &graph);
    if (st != EG_SUCCESS) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (err != cudaSuccess) return cuda_fail(err, "cudaStreamEndCapture");
    plan.graph = graph;
    EG_CUDA(cudaGraphInstantiate(&plan.exec, graph, 0));
    plan.kernels = 2;
    plan.report = eg_split_report{S, S * (S + 1) / 2, kBits, error_bound(S)};
    return EG_SUCCESS;
}

} // namespace eg::grouped
