// Permute: C[idx] = cp*C[idx] + ap*A[perm(idx)], coalesced on both sides.
//
// Replaces the scalar grid-stride permute_kernel and the LibreTT call of the
// reference's device permute (libs/Einsums/TensorAlgebra/include/Einsums/
// TensorAlgebra/Backends/DevicePermute.hpp:34-73, :134-207, and
// src/DevicePermute.hip:20-60), whose writes are uncoalesced.
//
// After folding modes that stay contiguous in both tensors, two cases remain:
//  * the fastest mode of A is also the fastest mode of C: a row copy, each
//    warp streaming consecutive elements of both tensors;
//  * otherwise: 32x32 tiles staged through shared memory -- a warp reads 32
//    consecutive elements of A along A's fastest mode and, after the tile is
//    transposed in shared memory, writes 32 consecutive elements of C along
//    C's fastest mode.
// Arithmetic follows HPTT, the reference's host transposer: cp == 0 stores
// ap*A without reading C (a plain copy when ap == 1, so the copy is bit-exact),
// otherwise ap*A + cp*C without fused multiply-adds.
#include <mutex>
#include <vector>

#include "common.cuh"
#include "ptx.cuh"

namespace eg {
eg_status build_permute_desc(double cp, const int32_t *Cl, const eg_tensor *C, double ap, const int32_t *Al,
                             const eg_tensor *A, PermuteDesc &p);

namespace {

struct PermuteMap {
    int n = 0; // "rest" modes (every mode but the tiled ones)
    int64_t total = 1;
    int64_t ext[kMaxModes] = {};
    int64_t sA[kMaxModes] = {};
    int64_t sC[kMaxModes] = {};
};

__device__ __forceinline__ void rest_offsets(const PermuteMap &r, int64_t i, int64_t &oa, int64_t &oc) {
    oa = oc = 0;
    for (int d = r.n - 1; d >= 0; d--) {
        const int64_t q = i / r.ext[d];
        const int64_t x = i - q * r.ext[d];
        i = q;
        oa += x * r.sA[d];
        oc += x * r.sC[d];
    }
}

template <int MODE> // 0: copy, 1: ap*a (cp == 0), 2: ap*a + cp*c
__device__ __forceinline__ double combine(double a, const double *c, double ap, double cp) {
    if (MODE == 0) return a;
    if (MODE == 1) return __dmul_rn(ap, a);
    return __dadd_rn(__dmul_rn(ap, a), __dmul_rn(cp, *c));
}

// Fastest modes shared: rows of length L with strides sa/sc along the row.  A
// warp takes a chunk of up to kRowChunk elements of one row (the decomposition
// of the row index is paid once per chunk) and keeps four loads in flight.
constexpr int64_t kRowChunk = 2048;
template <int MODE>
__global__ void __launch_bounds__(256) k_permute_rows(PermuteMap rest, int64_t L, int64_t sa, int64_t sc,
                                                      const double *__restrict__ A, double *C, double ap, double cp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t chunks = (L + kRowChunk - 1) / kRowChunk;
    const int64_t units = rest.total * chunks;
    for (int64_t u = (int64_t)blockIdx.x * 8 + warp; u < units; u += (int64_t)gridDim.x * 8) {
        const int64_t row = u / chunks, ch = u - row * chunks;
        int64_t oa, oc;
        rest_offsets(rest, row, oa, oc);
        const double *a = A + oa;
        double *c = C + oc;
        const int64_t x0 = ch * kRowChunk, x1 = min(L, x0 + kRowChunk);
        int64_t x = x0 + lane;
        for (; x + 96 < x1; x += 128) {
            double v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) v[q] = __ldg(a + (x + 32 * q) * sa);
#pragma unroll
            for (int q = 0; q < 4; q++) {
                double *cptr = c + (x + 32 * q) * sc;
                *cptr = combine<MODE>(v[q], cptr, ap, cp);
            }
        }
        for (; x < x1; x += 32) {
            double *cptr = c + x * sc;
            *cptr = combine<MODE>(__ldg(a + x * sa), cptr, ap, cp);
        }
    }
}

constexpr int TILE = 32, ROWS = 8;
constexpr int64_t kStrip = 8; // tiles along C's fastest mode per work unit

// ia runs along A's fastest mode (extent EA, strides saA in A / scA in C);
// ic runs along C's fastest mode (extent EC, strides saC in A / scC in C).
template <int MODE>
__global__ void __launch_bounds__(TILE *ROWS) k_permute_tiles(PermuteMap rest, int64_t EA, int64_t EC, int64_t saA,
                                                              int64_t scA, int64_t saC, int64_t scC,
                                                              const double *__restrict__ A, double *C, double ap,
                                                              double cp) {
    __shared__ double tile[TILE][TILE + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t tilesA = (EA + TILE - 1) / TILE, tilesC = (EC + TILE - 1) / TILE;
    // a work unit is a strip: one index of the rest modes, one tile row along A's
    // fastest mode and up to kStrip tiles along C's fastest mode, so that the
    // decomposition of the unit is paid once per strip rather than per tile
    const int64_t segs = (tilesC + kStrip - 1) / kStrip;
    const int64_t units = rest.total * tilesA * segs;
    for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
        const int64_t sg = u % segs, ta = (u / segs) % tilesA, r = u / (segs * tilesA);
        int64_t oa, oc;
        rest_offsets(rest, r, oa, oc);
        const int64_t a0 = ta * TILE;
        const double *Ar = A + oa + (a0 + tx) * saA;       // this thread's reads: ia = a0 + tx
        const bool a_in = a0 + tx < EA;
        const int64_t cbeg = sg * kStrip * TILE, cend = min(EC, cbeg + kStrip * TILE);
        for (int64_t c0 = cbeg; c0 < cend; c0 += TILE) {
            // read: consecutive threads walk A's fastest mode
#pragma unroll
            for (int j = 0; j < TILE; j += ROWS) {
                const int64_t ic = c0 + ty + j;
                if (a_in && ic < cend) tile[ty + j][tx] = __ldg(Ar + ic * saC);
            }
            __syncthreads();
            // write: consecutive threads walk C's fastest mode
            const int64_t ic = c0 + tx;
            if (ic < cend) {
                double *Cc = C + oc + ic * scC;
#pragma unroll
                for (int j = 0; j < TILE; j += ROWS) {
                    const int64_t ia = a0 + ty + j;
                    if (ia < EA) {
                        double *cptr = Cc + ia * scA;
                        *cptr = combine<MODE>(tile[tx][ty + j], cptr, ap, cp);
                    }
                }
            }
            __syncthreads();
        }
    }
}

// ---------------------------------------------------------------- TMA tiles --
// The transposing case through the tensor-memory accelerator: a 32x32 box of A
// (A's fastest mode x C's fastest mode, plus one index of every other mode) is
// loaded into shared memory, transposed there, and the 32x32 box of C is
// stored back with one bulk tensor store.  Tiles at the edges are clipped by
// the hardware (zero fill on load, bounds on store).  A ring of kTmaStages
// slots keeps the loads of later tiles in flight while a tile is transposed;
// a slot's output buffer is reused only after its store has read it.
constexpr int kTmaTile = 32, kTmaStages = 4, kTmaThreads = 256;
constexpr int kTmaBoxBytes = kTmaTile * kTmaTile * 8;
constexpr int kTmaSmem = 2 * kTmaStages * kTmaBoxBytes + 128 + 1024;
constexpr unsigned long long kTmaWaitNs = 2000ull * 1000 * 1000;
constexpr unsigned long long kTmaDrainNs = 200ull * 1000 * 1000;

struct TmaPermute {
    int rank = 0;                  // tensor-map rank: 2 + rest modes (at most 5)
    uint32_t tilesA = 0, tilesC = 0, total = 0; // total < 2^31
    uint32_t rext[3] = {1, 1, 1};  // extents of the rest modes (slowest first)
};

template <int R>
__device__ __forceinline__ void tma_load(void *dst, const CUtensorMap *m, uint64_t *bar, const int (&c)[5]) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst), b = (uint32_t)__cvta_generic_to_shared(bar);
    const uint64_t mp = reinterpret_cast<uint64_t>(m);
    if constexpr (R == 2)
        asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
                     "%4}], [%2];" ::"r"(d), "l"(mp), "r"(b), "r"(c[0]), "r"(c[1])
                     : "memory");
    else if constexpr (R == 3)
        asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
                     "%4, %5}], [%2];" ::"r"(d), "l"(mp), "r"(b), "r"(c[0]), "r"(c[1]), "r"(c[2])
                     : "memory");
    else if constexpr (R == 4)
        asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
                     "%4, %5, %6}], [%2];" ::"r"(d), "l"(mp), "r"(b), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3])
                     : "memory");
    else
        asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, "
                     "%4, %5, %6, %7}], [%2];" ::"r"(d), "l"(mp), "r"(b), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]),
                     "r"(c[4])
                     : "memory");
}

template <int R>
__device__ __forceinline__ void tma_store(const CUtensorMap *m, const void *src, const int (&c)[5]) {
    const uint32_t sp = (uint32_t)__cvta_generic_to_shared(src);
    const uint64_t mp = reinterpret_cast<uint64_t>(m);
    if constexpr (R == 2)
        asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(mp), "r"(sp),
                     "r"(c[0]), "r"(c[1])
                     : "memory");
    else if constexpr (R == 3)
        asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(mp),
                     "r"(sp), "r"(c[0]), "r"(c[1]), "r"(c[2])
                     : "memory");
    else if constexpr (R == 4)
        asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%2, %3, %4, %5}], [%1];" ::"l"(mp),
                     "r"(sp), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3])
                     : "memory");
    else
        asm volatile("cp.async.bulk.tensor.5d.global.shared::cta.bulk_group [%0, {%2, %3, %4, %5, %6}], [%1];" ::"l"(
                         mp),
                     "r"(sp), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4])
                     : "memory");
}

// Box coordinates of tile t: {A-fast, C-fast, rest...} for the load and
// {C-fast, A-fast, rest...} for the store (32-bit arithmetic: one thread issues
// every copy of the CTA, so this sits on its critical path).
__device__ __forceinline__ void tma_tile_coords(const TmaPermute &tp, uint32_t t, int (&ca)[5], int (&cc)[5]) {
    uint32_t q = t / tp.tilesC;
    const uint32_t tc = t - q * tp.tilesC;
    t = q;
    q = t / tp.tilesA;
    const uint32_t ta = t - q * tp.tilesA;
    t = q;
    ca[0] = cc[1] = (int)(ta * kTmaTile);
    ca[1] = cc[0] = (int)(tc * kTmaTile);
#pragma unroll
    for (int d = 2; d >= 0; d--) { // rest modes, fastest last; map dims 2.. hold them slowest last
        q = tp.rext[d] == 1 ? t : t / tp.rext[d];
        ca[2 + d] = cc[2 + d] = (int)(t - q * tp.rext[d]);
        t = q;
    }
}

template <int R, int MODE>
__global__ void __launch_bounds__(kTmaThreads) k_permute_tma(const __grid_constant__ CUtensorMap mapA,
                                                             const __grid_constant__ CUtensorMap mapC, TmaPermute tp,
                                                             double ap, int *status) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    double *in = (double *)smem;                                  // [stage][C-fast j][A-fast i]
    double *out = (double *)(smem + kTmaStages * kTmaBoxBytes);   // [stage][A-fast i][C-fast j]
    uint64_t *full = (uint64_t *)(smem + 2 * kTmaStages * kTmaBoxBytes);
    volatile int *abort_flag = (volatile int *)(full + kTmaStages);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        for (int i = 0; i < kTmaStages; i++) ptx::mbar_init(&full[i], 1);
        *abort_flag = 0;
        ptx::fence_mbar_init();
        ptx::tma_prefetch_desc(&mapA);
        ptx::tma_prefetch_desc(&mapC);
    }
    __syncthreads();
    const uint32_t first = blockIdx.x, step = gridDim.x;
    auto issue_load = [&](uint32_t k) { // local tile k of this CTA into slot k % stages
        const uint32_t t = first + k * step;
        if (t >= tp.total) return;
        int ca[5], cc[5];
        tma_tile_coords(tp, t, ca, cc);
        uint64_t *bar = &full[k % kTmaStages];
        ptx::mbar_arrive_expect_tx(bar, (uint32_t)kTmaBoxBytes);
        tma_load<R>(in + (k % kTmaStages) * kTmaTile * kTmaTile, &mapA, bar, ca);
    };
    if (tid == 0)
        for (uint32_t k = 0; k < kTmaStages; k++) issue_load(k);
    int st_c[5] = {0, 0, 0, 0, 0}; // thread 0: the store coordinates of the current tile
    uint32_t k = 0;
    for (; first + k * step < tp.total; k++) {
        const int slot = (int)(k % kTmaStages);
        const uint32_t parity = (k / kTmaStages) & 1u;
        if (tid == 0) {
            int ca[5];
            tma_tile_coords(tp, first + k * step, ca, st_c);
        }
        if (!ptx::mbar_wait(&full[slot], parity, kTmaWaitNs, abort_flag)) {
            *abort_flag = 1;
            atomicCAS(status, 0, 6);
        }
        if (tid == 0) // the store that last read this slot's output buffer has finished reading
            asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(kTmaStages - 1) : "memory");
        __syncthreads();
        if (*abort_flag) break;
        const double *src = in + slot * kTmaTile * kTmaTile;
        double *dst = out + slot * kTmaTile * kTmaTile;
        // lane l moves element (j = l, i = (l + c) mod 32): both the read of row j
        // and the write of row i touch 16 distinct 8-byte bank pairs per half-warp
#pragma unroll
        for (int c = warp; c < kTmaTile; c += kTmaThreads / 32) {
            const int j = lane, i = (lane + c) & (kTmaTile - 1);
            const double v = src[j * kTmaTile + i];
            dst[i * kTmaTile + j] = MODE == 0 ? v : __dmul_rn(ap, v);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            tma_store<R>(&mapC, dst, st_c);
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
        } else if (tid == 32) {
            issue_load(k + kTmaStages); // this slot's input buffer was read by every thread above
        }
    }
    if (tid == 0) asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
    if (*abort_flag && tid == 0) {
        // a wait gave up at tile k: the loads of tiles k .. k + stages - 1 may still be
        // in flight into this CTA's shared memory; give each a bounded wait to land
        for (uint32_t kk = k; kk < k + kTmaStages && first + kk * step < tp.total; kk++)
            ptx::mbar_wait(&full[kk % kTmaStages], (kk / kTmaStages) & 1u, kTmaDrainNs, nullptr);
    }
    __syncthreads();
}

} // namespace

eg_status encode_tiled_f64(CUtensorMap *map, const void *base, int rank, const uint64_t *dims,
                           const uint64_t *strides_bytes, const uint32_t *box);

// What a permute launch needs, fixed by the shapes and strides alone: a
// compiled plan keeps it and runs it on new pointers.
struct PermuteLaunch {
    bool empty = false;
    bool rows = false; // fastest modes shared: row copies, else tiles
    int mode = 0;      // 0: copy, 1: ap*a, 2: ap*a + cp*c
    int grid = 0;
    PermuteMap rest;
    int64_t L = 0, sa = 0, sc = 0;                                 // rows
    int64_t EA = 0, EC = 0, saA = 0, scA = 0, saC = 0, scC = 0; // tiles
    double ap = 1.0, cp = 0.0;
    // TMA form of the tiled case (cp == 0, fastest strides 1, other strides
    // multiples of 16 bytes, at most three other modes); maps are encoded per run
    bool tma = false;
    TmaPermute tp;
    int64_t rsA[3] = {}, rsC[3] = {}; // strides of the other modes (elements)
};

PermuteLaunch prepare_permute(const PermuteDesc &p) {
    PermuteLaunch pl;
    pl.ap = p.ap;
    pl.cp = p.cp;
    // Fold modes (in C order) that are contiguous in both tensors; drop extent-1 modes.
    std::vector<int64_t> ext, sA, sC;
    int64_t total = 1;
    for (int d = 0; d < p.rank; d++) {
        total *= p.ext[d];
        if (p.ext[d] == 1) continue;
        if (!ext.empty() && sA.back() == p.sA[d] * p.ext[d] && sC.back() == p.sC[d] * p.ext[d]) {
            ext.back() *= p.ext[d];
            sA.back() = p.sA[d];
            sC.back() = p.sC[d];
            continue;
        }
        ext.push_back(p.ext[d]);
        sA.push_back(p.sA[d]);
        sC.push_back(p.sC[d]);
    }
    if (total == 0) {
        pl.empty = true;
        return pl;
    }
    if (ext.empty()) { // a single element
        ext.push_back(1);
        sA.push_back(1);
        sC.push_back(1);
    }
    const int n = (int)ext.size();
    auto argmin = [&](const std::vector<int64_t> &st) {
        int best = 0;
        for (int d = 1; d < n; d++)
            if (st[d] < st[best] || (st[d] == st[best] && ext[d] > ext[best])) best = d;
        return best;
    };
    const int fa = argmin(sA), fc = argmin(sC);
    pl.mode = (p.cp == 0.0) ? (p.ap == 1.0 ? 0 : 1) : 2;
    const int cap = num_sms() * 16;
    for (int d = 0; d < n; d++) {
        if (d == fa || d == fc) continue;
        pl.rest.ext[pl.rest.n] = ext[d];
        pl.rest.sA[pl.rest.n] = sA[d];
        pl.rest.sC[pl.rest.n] = sC[d];
        pl.rest.total *= ext[d];
        pl.rest.n++;
    }
    if (fa == fc) {
        pl.rows = true;
        pl.L = ext[fc];
        pl.sa = sA[fc];
        pl.sc = sC[fc];
        const int64_t work = (pl.rest.total * ((pl.L + kRowChunk - 1) / kRowChunk) + 7) / 8;
        pl.grid = (int)(work < cap ? work : cap);
        return pl;
    }
    pl.EA = ext[fa];
    pl.EC = ext[fc];
    pl.saA = sA[fa];
    pl.scA = sC[fa];
    pl.saC = sA[fc];
    pl.scC = sC[fc];
    const int64_t work =
        pl.rest.total * ((pl.EA + TILE - 1) / TILE) * (((pl.EC + TILE - 1) / TILE + kStrip - 1) / kStrip);
    pl.grid = (int)(work < cap ? work : cap);
    // the TMA form: a plain or scaled copy of whole 32x32 boxes along two
    // contiguous fastest modes, the other strides 16-byte multiples
    bool ok = pl.mode <= 1 && pl.rest.n <= 3 && pl.saA == 1 && pl.scC == 1 && pl.EA >= kTmaTile &&
              pl.EC >= kTmaTile && pl.EA < (1ll << 31) && pl.EC < (1ll << 31) && pl.saC % 2 == 0 && pl.scA % 2 == 0;
    for (int d = 0; d < pl.rest.n && ok; d++)
        ok = pl.rest.sA[d] % 2 == 0 && pl.rest.sC[d] % 2 == 0 && pl.rest.ext[d] < (1ll << 31);
    if (ok) {
        pl.tma = true;
        pl.tp.rank = 2 + pl.rest.n;
        pl.tp.tilesA = (uint32_t)((pl.EA + kTmaTile - 1) / kTmaTile);
        pl.tp.tilesC = (uint32_t)((pl.EC + kTmaTile - 1) / kTmaTile);
        const int64_t total = pl.rest.total * (int64_t)pl.tp.tilesA * pl.tp.tilesC;
        pl.tma = total < (1ll << 31);
        pl.tp.total = (uint32_t)total;
        for (int d = 0; d < pl.rest.n; d++) {
            pl.tp.rext[d] = (uint32_t)pl.rest.ext[d];
            pl.rsA[d] = pl.rest.sA[d];
            pl.rsC[d] = pl.rest.sC[d];
        }
    }
    return pl;
}

namespace {
template <int MODE>
eg_status launch_tma(const PermuteLaunch &pl, int grid, const CUtensorMap &mA, const CUtensorMap &mC, int *status,
                     cudaStream_t s) {
    switch (pl.tp.rank) {
    case 2: k_permute_tma<2, MODE><<<grid, kTmaThreads, kTmaSmem, s>>>(mA, mC, pl.tp, pl.ap, status); break;
    case 3: k_permute_tma<3, MODE><<<grid, kTmaThreads, kTmaSmem, s>>>(mA, mC, pl.tp, pl.ap, status); break;
    case 4: k_permute_tma<4, MODE><<<grid, kTmaThreads, kTmaSmem, s>>>(mA, mC, pl.tp, pl.ap, status); break;
    default: k_permute_tma<5, MODE><<<grid, kTmaThreads, kTmaSmem, s>>>(mA, mC, pl.tp, pl.ap, status); break;
    }
    return EG_SUCCESS;
}

eg_status ensure_tma_attributes() {
    static std::once_flag once;
    static cudaError_t err = cudaSuccess;
    std::call_once(once, [] {
        auto set = [&](const void *f) {
            if (err == cudaSuccess) err = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, kTmaSmem);
        };
        set((const void *)k_permute_tma<2, 0>);
        set((const void *)k_permute_tma<3, 0>);
        set((const void *)k_permute_tma<4, 0>);
        set((const void *)k_permute_tma<5, 0>);
        set((const void *)k_permute_tma<2, 1>);
        set((const void *)k_permute_tma<3, 1>);
        set((const void *)k_permute_tma<4, 1>);
        set((const void *)k_permute_tma<5, 1>);
    });
    if (err != cudaSuccess) return cuda_fail(err, "cudaFuncSetAttribute(k_permute_tma)");
    return EG_SUCCESS;
}

// Resident CTAs of the TMA permute per SM (its ring takes 65 KB of shared memory).
int tma_blocks_per_sm() {
    static std::once_flag once;
    static int per_sm = 1;
    std::call_once(once, [] {
        int n = 0;
        if (ensure_tma_attributes() == EG_SUCCESS &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_permute_tma<4, 0>, kTmaThreads, kTmaSmem) ==
                cudaSuccess &&
            n > 0)
            per_sm = n;
        cudaGetLastError();
    });
    return per_sm;
}

// Encodes the two maps for these pointers and launches; EG_ERROR_NOT_SUPPORTED
// (nothing launched) when the pointers or the driver reject the TMA form.
eg_status run_permute_tma(const PermuteLaunch &pl, const double *A, double *C, cudaStream_t s) {
    if (((uintptr_t)A & 15) || ((uintptr_t)C & 15)) return EG_ERROR_NOT_SUPPORTED;
    const int R = pl.tp.rank;
    uint64_t dA[5], dC[5], sA[4], sC[4];
    uint32_t box[5] = {kTmaTile, kTmaTile, 1, 1, 1};
    dA[0] = (uint64_t)pl.EA;
    dA[1] = (uint64_t)pl.EC;
    sA[0] = (uint64_t)pl.saC * 8;
    dC[0] = (uint64_t)pl.EC;
    dC[1] = (uint64_t)pl.EA;
    sC[0] = (uint64_t)pl.scA * 8;
    for (int d = 0; d + 2 < R; d++) {
        dA[2 + d] = dC[2 + d] = (uint64_t)pl.tp.rext[d];
        sA[1 + d] = (uint64_t)pl.rsA[d] * 8;
        sC[1 + d] = (uint64_t)pl.rsC[d] * 8;
    }
    CUtensorMap mA, mC;
    if (encode_tiled_f64(&mA, A, R, dA, sA, box) != EG_SUCCESS) return EG_ERROR_NOT_SUPPORTED;
    if (encode_tiled_f64(&mC, C, R, dC, sC, box) != EG_SUCCESS) return EG_ERROR_NOT_SUPPORTED;
    set_error("");
    eg_status st = ensure_tma_attributes();
    if (st != EG_SUCCESS) return st;
    int *status = nullptr;
    if ((st = status_word(s, &status)) != EG_SUCCESS) return st;
    const int64_t slots = (int64_t)tma_blocks_per_sm() * num_sms();
    const int grid = (int)(pl.tp.total < slots ? pl.tp.total : slots);
    {
        LaunchScope ls_("k_permute_tma", s);
        st = pl.mode == 0 ? launch_tma<0>(pl, grid, mA, mC, status, s) : launch_tma<1>(pl, grid, mA, mC, status, s);
    }
    if (st != EG_SUCCESS) return st;
    EG_CHECK_LAUNCH("k_permute_tma");
    return EG_SUCCESS;
}
} // namespace

eg_status run_permute(const PermuteLaunch &pl, const double *A, double *C, cudaStream_t s) {
    if (pl.empty) return EG_SUCCESS;
    if (pl.tma) {
        const eg_status st = run_permute_tma(pl, A, C, s);
        if (st != EG_ERROR_NOT_SUPPORTED) return st;
        set_error(""); // the tile kernel below takes the case the TMA form declined
    }
    if (pl.rows) {
        {
            LaunchScope ls_("k_permute_rows", s);
            if (pl.mode == 0)
                k_permute_rows<0><<<pl.grid, 256, 0, s>>>(pl.rest, pl.L, pl.sa, pl.sc, A, C, pl.ap, pl.cp);
            else if (pl.mode == 1)
                k_permute_rows<1><<<pl.grid, 256, 0, s>>>(pl.rest, pl.L, pl.sa, pl.sc, A, C, pl.ap, pl.cp);
            else
                k_permute_rows<2><<<pl.grid, 256, 0, s>>>(pl.rest, pl.L, pl.sa, pl.sc, A, C, pl.ap, pl.cp);
        }
        EG_CHECK_LAUNCH("k_permute_rows");
        return EG_SUCCESS;
    }
    const dim3 block(TILE, ROWS);
    {
        LaunchScope ls_("k_permute_tiles", s);
        if (pl.mode == 0)
            k_permute_tiles<0><<<pl.grid, block, 0, s>>>(pl.rest, pl.EA, pl.EC, pl.saA, pl.scA, pl.saC, pl.scC, A, C,
                                                        pl.ap, pl.cp);
        else if (pl.mode == 1)
            k_permute_tiles<1><<<pl.grid, block, 0, s>>>(pl.rest, pl.EA, pl.EC, pl.saA, pl.scA, pl.saC, pl.scC, A, C,
                                                        pl.ap, pl.cp);
        else
            k_permute_tiles<2><<<pl.grid, block, 0, s>>>(pl.rest, pl.EA, pl.EC, pl.saA, pl.scA, pl.saC, pl.scC, A, C,
                                                        pl.ap, pl.cp);
    }
    EG_CHECK_LAUNCH("k_permute_tiles");
    return EG_SUCCESS;
}

eg_status launch_permute(const PermuteDesc &p, cudaStream_t s) { return run_permute(prepare_permute(p), p.A, p.C, s); }

} // namespace eg

struct eg_permute_plan {
    eg::PermuteLaunch launch;
};

extern "C" {

eg_status eg_permute_plan_create(double C_prefactor, const int32_t *C_labels, const eg_tensor *C, double A_prefactor,
                                 const int32_t *A_labels, const eg_tensor *A, eg_permute_plan **plan) {
    eg::set_error("");
    if (!plan) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "plan is NULL");
    *plan = nullptr;
    try {
        eg::PermuteDesc d;
        const eg_status st = eg::build_permute_desc(C_prefactor, C_labels, C, A_prefactor, A_labels, A, d);
        if (st != EG_SUCCESS) return st;
        *plan = new eg_permute_plan{eg::prepare_permute(d)};
        return EG_SUCCESS;
    } catch (...) {
        return eg::fail(EG_ERROR_OUT_OF_MEMORY, "eg_permute_plan_create: allocation failed");
    }
}

eg_status eg_permute_plan_execute(const eg_permute_plan *plan, double *C, const double *A, void *stream) {
    eg::set_error("");
    if (!plan) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "plan is NULL");
    if (!plan->launch.empty && (!C || !A)) return eg::fail(EG_ERROR_INVALID_ARGUMENT, "C or A is NULL");
    return eg::run_permute(plan->launch, A, C, (cudaStream_t)stream);
}

eg_status eg_permute_plan_destroy(eg_permute_plan *plan) {
    delete plan;
    return EG_SUCCESS;
}

} // extern "C"
