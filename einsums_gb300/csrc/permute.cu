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
#include <vector>

#include "common.cuh"

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

} // namespace

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
    return pl;
}

eg_status run_permute(const PermuteLaunch &pl, const double *A, double *C, cudaStream_t s) {
    if (pl.empty) return EG_SUCCESS;
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
