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

eg_status launch_permute(const PermuteDesc &p, cudaStream_t s) {
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
    if (total == 0) return EG_SUCCESS;
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
    const int mode = (p.cp == 0.0) ? (p.ap == 1.0 ? 0 : 1) : 2;
    const int cap = num_sms() * 16;

    PermuteMap rest;
    for (int d = 0; d < n; d++) {
        if (d == fa || d == fc) continue;
        rest.ext[rest.n] = ext[d];
        rest.sA[rest.n] = sA[d];
        rest.sC[rest.n] = sC[d];
        rest.total *= ext[d];
        rest.n++;
    }
    if (fa == fc) {
        const int64_t L = ext[fc];
        const int64_t work = (rest.total * ((L + kRowChunk - 1) / kRowChunk) + 7) / 8;
        const int grid = (int)(work < cap ? work : cap);
        if (mode == 0)
            { LaunchScope ls_("k_permute_rows", s);
            k_permute_rows<0><<<grid, 256, 0, s>>>(rest, L, sA[fc], sC[fc], p.A, p.C, p.ap, p.cp);
            }
        else if (mode == 1)
            { LaunchScope ls_("k_permute_rows", s);
            k_permute_rows<1><<<grid, 256, 0, s>>>(rest, L, sA[fc], sC[fc], p.A, p.C, p.ap, p.cp);
            }
        else
            { LaunchScope ls_("k_permute_rows", s);
            k_permute_rows<2><<<grid, 256, 0, s>>>(rest, L, sA[fc], sC[fc], p.A, p.C, p.ap, p.cp);
            }
        EG_CHECK_LAUNCH("k_permute_rows");
        return EG_SUCCESS;
    }
    const int64_t EA = ext[fa], EC = ext[fc];
    const int64_t work = rest.total * ((EA + TILE - 1) / TILE) * (((EC + TILE - 1) / TILE + kStrip - 1) / kStrip);
    const int grid = (int)(work < cap ? work : cap);
    dim3 block(TILE, ROWS);
    if (mode == 0)
        { LaunchScope ls_("k_permute_tiles", s);
        k_permute_tiles<0><<<grid, block, 0, s>>>(rest, EA, EC, sA[fa], sC[fa], sA[fc], sC[fc], p.A, p.C, p.ap, p.cp);
        }
    else if (mode == 1)
        { LaunchScope ls_("k_permute_tiles", s);
        k_permute_tiles<1><<<grid, block, 0, s>>>(rest, EA, EC, sA[fa], sC[fa], sA[fc], sC[fc], p.A, p.C, p.ap, p.cp);
        }
    else
        { LaunchScope ls_("k_permute_tiles", s);
        k_permute_tiles<2><<<grid, block, 0, s>>>(rest, EA, EC, sA[fa], sC[fa], sA[fc], sC[fc], p.A, p.C, p.ap, p.cp);
        }
    EG_CHECK_LAUNCH("k_permute_tiles");
    return EG_SUCCESS;
}

} // namespace eg
