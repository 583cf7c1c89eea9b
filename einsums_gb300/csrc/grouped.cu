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
    int64_t units_before; // prefix of units (rowmax units for the rowmax table, digit units for the digits table)
};

constexpr int TT = 32, TR = 8;

__device__ __forceinline__ int find_item(const GOp *ops, int nops, int64_t u) {
    int lo = 0, hi = nops - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (ops[mid].units_before <= u)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ int64_t pick(int comp, int64_t oa, int64_t ob) { return comp == 0 ? oa : ob; }

__global__ void __launch_bounds__(TT *TR) k_grouped_rowmax(const GOp *ops, int nops, int64_t total_units,
                                                           unsigned long long *rowmax) {
    __shared__ unsigned long long red[TR][TT];
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int64_t u = blockIdx.x; u < total_units; u += gridDim.x) {
        const GOp &g = ops[find_item(ops, nops, u)];
        const int64_t local = u - g.units_before;
        const int64_t rt = (g.rows + TT - 1) / TT, kt = (g.K + TT - 1) / TT;
        const int64_t ktile = local % kt, rtile = (local / kt) % rt, b = local / (kt * rt);
        int64_t oa, ob, oc;
        group_offsets(g.bg, b, oa, ob, oc);
        const int64_t obase = pick(g.comp, oa, ob);
        const int64_t r0 = rtile * TT, k0 = ktile * TT;
        unsigned long long *rm = rowmax + g.rowbase + b * g.Rp;
        if (g.row_fast) {
            const int64_t r = r0 + tx;
            unsigned long long mx = 0;
            if (r < g.rows) {
                group_offsets32(g.rg, (uint32_t)r, oa, ob, oc);
                const int64_t orow = obase + pick(g.comp, oa, ob);
                for (int j = ty; j < TT; j += TR) {
                    const int64_t k = k0 + j;
                    if (k < g.K) {
                        group_offsets32(g.kg, (uint32_t)k, oa, ob, oc);
                        mx = max(mx, (unsigned long long)__double_as_longlong(fabs(__ldg(g.X + orow + pick(g.comp, oa, ob)))));
                    }
                }
            }
            red[ty][tx] = mx;
            __syncthreads();
            if (ty == 0) {
                for (int j = 1; j < TR; j++) mx = max(mx, red[j][tx]);
                if (r < g.rows && mx) atomicMax(rm + r, mx);
            }
            __syncthreads();
        } else {
            const int64_t k = k0 + tx;
            int64_t okk = 0;
            if (k < g.K) {
                group_offsets32(g.kg, (uint32_t)k, oa, ob, oc);
                okk = pick(g.comp, oa, ob);
            }
            for (int j = ty; j < TT; j += TR) {
                const int64_t r = r0 + j;
                unsigned long long v = 0;
                if (r < g.rows && k < g.K) {
                    group_offsets32(g.rg, (uint32_t)r, oa, ob, oc);
                    v = (unsigned long long)__double_as_longlong(fabs(__ldg(g.X + obase + pick(g.comp, oa, ob) + okk)));
                }
                for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
                if (tx == 0 && r < g.rows && v) atomicMax(rm + r, v);
            }
        }
    }
}

__global__ void __launch_bounds__(TT *TR) k_grouped_digits(const GOp *ops, int nops, int64_t total_units,
                                                           const int *rexp, __nv_bfloat16 *planes, int64_t Rmax,
                                                           int64_t Kmaxp, int S) {
    __shared__ double tile[TT][TT + 1];
    __shared__ int ex[TT];
    const int tx = threadIdx.x, ty = threadIdx.y;
    for (int64_t u = blockIdx.x; u < total_units; u += gridDim.x) {
        const GOp &g = ops[find_item(ops, nops, u)];
        const int64_t local = u - g.units_before;
        const int64_t rt = g.Rp / TT, kt = g.Kp / TT;
        const int64_t ktile = local % kt, rtile = (local / kt) % rt, b = local / (kt * rt);
        int64_t oa, ob, oc;
        group_offsets(g.bg, b, oa, ob, oc);
        const int64_t obase = pick(g.comp, oa, ob);
        const int64_t r0 = rtile * TT, k0 = ktile * TT;
        if (ty == 0) ex[tx] = (r0 + tx < g.rows) ? rexp[g.rowbase + b * g.Rp + r0 + tx] : 0;
        if (g.row_fast) {
            const int64_t r = r0 + tx;
            int64_t orow = 0;
            if (r < g.rows) {
                group_offsets32(g.rg, (uint32_t)r, oa, ob, oc);
                orow = obase + pick(g.comp, oa, ob);
            }
            for (int j = ty; j < TT; j += TR) {
                const int64_t k = k0 + j;
                double v = 0.0;
                if (r < g.rows && k < g.K) {
                    group_offsets32(g.kg, (uint32_t)k, oa, ob, oc);
                    v = __ldg(g.X + orow + pick(g.comp, oa, ob));
                }
                tile[tx][j] = v;
            }
        } else {
            const int64_t k = k0 + tx;
            int64_t okk = 0;
            if (k < g.K) {
                group_offsets32(g.kg, (uint32_t)k, oa, ob, oc);
                okk = pick(g.comp, oa, ob);
            }
            for (int j = ty; j < TT; j += TR) {
                const int64_t r = r0 + j;
                double v = 0.0;
                if (r < g.rows && k < g.K) {
                    group_offsets32(g.rg, (uint32_t)r, oa, ob, oc);
                    v = __ldg(g.X + obase + pick(g.comp, oa, ob) + okk);
                }
                tile[j][tx] = v;
            }
        }
        __syncthreads();
        for (int j = ty; j < TT; j += TR) {
            const int64_t r = r0 + j;
            int dig[split::kMaxSlices];
            const int e = ex[j];
            if (e == INT_MIN) {
                for (int s = 0; s < S; s++) dig[s] = 0;
            } else {
                split::to_digits(tile[j][tx], e, S, dig);
            }
            const int64_t z0 = g.zbase + b * S;
            for (int s = 0; s < S; s++)
                planes[((z0 + s) * Rmax + r) * Kmaxp + k0 + tx] = __float2bfloat16_rn((float)dig[s]);
        }
        __syncthreads();
    }
}

__global__ void k_grouped_exponent(const unsigned long long *rowmax, int *e, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double mx = __longlong_as_double((long long)rowmax[i]);
        int ex = 0;
        if (!isfinite(mx))
            ex = INT_MIN;
        else if (mx > 0.0)
            frexp(mx, &ex);
        e[i] = ex;
    }
}

int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

bool fast_along(const ModeGroup &g, int comp) { return g.n > 0 && g.s[comp][g.n - 1] == 1; }

} // namespace

// ------------------------------------------------------------------ plan --
struct Plan {
    int device = 0;
    int precision = EG_PRECISION_FP64;
    int slices = 0;
    int64_t count = 0;
    int32_t algorithm = 0;
    std::vector<void *> owned; // device buffers owned by the plan
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint64_t kernels = 0; // kernels in one replay
    eg_split_report report{};
    ~Plan();
};

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
    int64_t unitsA = 0, unitsB = 0, dunitsA = 0, dunitsB = 0;
    std::vector<int64_t> dprefA, dprefB;
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
        a.units_before = unitsA;
        GOp b = a;
        b.X = c.B;
        b.rg = c.n;
        b.comp = 1;
        b.row_fast = !fast_along(c.k, 1) && fast_along(c.n, 1);
        b.rows = N;
        b.Rp = Np;
        b.rowbase = rowsB;
        b.zbase = zB;
        b.units_before = unitsB;
        opsA.push_back(a);
        opsB.push_back(b);
        dprefA.push_back(dunitsA);
        dprefB.push_back(dunitsB);
        unitsA += nb * ((M + 31) / 32) * ((K + 31) / 32);
        unitsB += nb * ((N + 31) / 32) * ((K + 31) / 32);
        dunitsA += nb * (Mp / 32) * (Kp / 32);
        dunitsB += nb * (Np / 32) * (Kp / 32);
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
    // digit-unit prefixes replace the rowmax prefixes in the digit tables
    std::vector<GOp> dopsA = opsA, dopsB = opsB;
    for (size_t i = 0; i < cs.size(); i++) {
        dopsA[i].units_before = dprefA[i];
        dopsB[i].units_before = dprefB[i];
    }

    void *planesA, *planesB, *maxA, *maxB, *eA, *eB, *d_opsA, *d_opsB, *d_dopsA, *d_dopsB, *d_items, *d_work, *rbuf;
    eg_status st;
    if ((st = dev_alloc(plan, rbuf_bytes(), &rbuf)) != EG_SUCCESS) return st;
    if ((st = dev_alloc(plan, (size_t)zA * Rmax * Kmaxp * 2, &planesA)) != EG_SUCCESS) return st;
    if ((st = dev_alloc(plan, (size_t)zB * Rmax * Kmaxp * 2, &planesB)) != EG_SUCCESS) return st;
    if ((st = dev_alloc(plan, (size_t)rowsA * 8, &maxA)) != EG_SUCCESS) return st;
    if ((st = dev_alloc(plan, (size_t)rowsB * 8, &maxB)) != EG_SUCCESS) return st;
    if ((st = dev_alloc(plan, (size_t)rowsA * 4, &eA)) != EG_SUCCESS) return st;
    if ((st = dev_alloc(plan, (size_t)rowsB * 4, &eB)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, opsA.data(), opsA.size() * sizeof(GOp), &d_opsA)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, opsB.data(), opsB.size() * sizeof(GOp), &d_opsB)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, dopsA.data(), dopsA.size() * sizeof(GOp), &d_dopsA)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, dopsB.data(), dopsB.size() * sizeof(GOp), &d_dopsB)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, items.data(), items.size() * sizeof(TcItem), &d_items)) != EG_SUCCESS) return st;
    if ((st = dev_copy(plan, wl.data(), wl.size() * sizeof(int4), &d_work)) != EG_SUCCESS) return st;

    CUtensorMap tmA, tmB;
    if ((st = encode_planes_public(&tmA, planesA, Kmaxp, Rmax, zA)) != EG_SUCCESS) return st;
    if ((st = encode_planes_public(&tmB, planesB, Kmaxp, Rmax, zB)) != EG_SUCCESS) return st;
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
    p.ksplit = 1; // no K slicing in grouped launches
    p.kslice = 0;
    p.rbuf = (long long *)rbuf;

    const int cap = num_sms() * 16;
    if ((st = ensure_tc_attributes()) != EG_SUCCESS) return st;
    EG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
    {
        CaptureGuard g;
        auto issue = [&]() -> eg_status {
            EG_CUDA(cudaMemsetAsync(maxA, 0, (size_t)rowsA * 8, s));
            EG_CUDA(cudaMemsetAsync(maxB, 0, (size_t)rowsB * 8, s));
            k_grouped_rowmax<<<(int)std::min<int64_t>(std::max<int64_t>(unitsA, 1), cap), dim3(TT, TR), 0, s>>>(
                (GOp *)d_opsA, (int)cs.size(), unitsA, (unsigned long long *)maxA);
            k_grouped_rowmax<<<(int)std::min<int64_t>(std::max<int64_t>(unitsB, 1), cap), dim3(TT, TR), 0, s>>>(
                (GOp *)d_opsB, (int)cs.size(), unitsB, (unsigned long long *)maxB);
            k_grouped_exponent<<<(int)std::min<int64_t>((rowsA + 255) / 256 + 1, cap), 256, 0, s>>>(
                (unsigned long long *)maxA, (int *)eA, rowsA);
            k_grouped_exponent<<<(int)std::min<int64_t>((rowsB + 255) / 256 + 1, cap), 256, 0, s>>>(
                (unsigned long long *)maxB, (int *)eB, rowsB);
            k_grouped_digits<<<(int)std::min<int64_t>(std::max<int64_t>(dunitsA, 1), cap), dim3(TT, TR), 0, s>>>(
                (GOp *)d_dopsA, (int)cs.size(), dunitsA, (int *)eA, (__nv_bfloat16 *)planesA, Rmax, Kmaxp, S);
            k_grouped_digits<<<(int)std::min<int64_t>(std::max<int64_t>(dunitsB, 1), cap), dim3(TT, TR), 0, s>>>(
                (GOp *)d_dopsB, (int)cs.size(), dunitsB, (int *)eB, (__nv_bfloat16 *)planesB, Rmax, Kmaxp, S);
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
    plan.kernels = 7;
    plan.report = eg_split_report{S, S * (S + 1) / 2, kBits, error_bound(S)};
    return EG_SUCCESS;
}

} // namespace eg::grouped
