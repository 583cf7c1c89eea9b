// Host orchestration of the split-BF16 form and its digit-splitting kernels.
//
//   k_split_rowmax   max |x| of every operand row (atomicMax on the bit
//                    pattern of |x|, which orders like the value; deterministic)
//   k_split_exponent row exponent e with |x| < 2^e (INT_MIN for a row holding
//                    Inf/NaN, whose outputs are written as NaN)
//   k_split_digits   32x64 tiles staged through shared memory (double-buffered
//                    asynchronous copies) so the operand is read along its
//                    contiguous mode and the digit planes are written along k;
//                    padding rows/columns are written as 0
// then the tcgen05 GEMM (tc_gemm.cu) over the digit planes.  The operands'
// index permutation is folded into the address maps of these kernels and of
// the GEMM epilogue: nothing but the BF16 digit planes is materialised.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>

#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "split.cuh"

namespace eg {
void set_split_report(const eg_split_report &r);
}

namespace eg::split {

namespace {

// Operand view for the splitting kernels: rows (batch x row group) and k.
struct OperandMap {
    ModeGroup bg, rg, kg;
    int comp;          // stride component: 0 for A, 1 for B
    int64_t rows, Rp;  // logical and padded rows per batch
    int64_t K, Kp;
    int nbatch;
    // Element offsets of every row and every k (filled by k_operand_offsets),
    // or null: then each offset is decomposed mode by mode, which costs integer
    // divisions per element and made these kernels ALU-bound.
    const int64_t *offr = nullptr, *offk = nullptr;
    // When a group walks memory with a single stride (the usual case: its modes
    // are nested like a row-major block), that stride; the offset is then
    // index * stride, with no table load in the dependency chain.  0 otherwise.
    int64_t sr = 0, sk = 0;
};

__device__ __forceinline__ int64_t comp_of(int comp, int64_t oa, int64_t ob) { return comp == 0 ? oa : ob; }

__device__ __forceinline__ int64_t off_b(const OperandMap &m, int64_t b) {
    if (m.bg.n == 0) return 0;
    int64_t oa, ob, oc;
    group_offsets(m.bg, b, oa, ob, oc);
    return comp_of(m.comp, oa, ob);
}
__device__ __forceinline__ int64_t decompose_r(const OperandMap &m, int64_t r) {
    int64_t oa, ob, oc;
    group_offsets32(m.rg, (uint32_t)r, oa, ob, oc);
    return comp_of(m.comp, oa, ob);
}
__device__ __forceinline__ int64_t decompose_k(const OperandMap &m, int64_t k) {
    int64_t oa, ob, oc;
    group_offsets32(m.kg, (uint32_t)k, oa, ob, oc);
    return comp_of(m.comp, oa, ob);
}
__device__ __forceinline__ int64_t off_r(const OperandMap &m, int64_t r) {
    if (m.sr) return r * m.sr;
    return m.offr ? __ldg(m.offr + r) : decompose_r(m, r);
}
__device__ __forceinline__ int64_t off_k(const OperandMap &m, int64_t k) {
    if (m.sk) return k * m.sk;
    return m.offk ? __ldg(m.offk + k) : decompose_k(m, k);
}

// Fills the row and k offset tables of an operand.
__global__ void k_operand_offsets(OperandMap m, int64_t *offr, int64_t *offk) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.rows; i += stride) offr[i] = decompose_r(m, i);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < m.K; i += stride) offk[i] = decompose_k(m, i);
}

constexpr int T = 32, TR = 8;

// Splits a work index w = (b * n1 + i1) * n0 + i0 into its parts, in 32-bit
// arithmetic when the work count fits (`narrow`): a 64-bit division is a long
// subroutine, and the splitting kernels pay this once per work unit.
__device__ __forceinline__ void split_unit(int64_t w, int64_t n0, int64_t n1, bool narrow, int64_t &i0, int64_t &i1,
                                           int64_t &b) {
    if (narrow) {
        const uint32_t x = (uint32_t)w, a = (uint32_t)n0, c = (uint32_t)n1;
        const uint32_t q = x / a, q2 = q / c;
        i0 = x - q * a;
        i1 = q - q2 * c;
        b = q2;
    } else {
        const int64_t q = w / n0, q2 = q / n1;
        i0 = w - q * n0;
        i1 = q - q2 * n1;
        b = q2;
    }
}

// Row maxima over work units of rows x kchunk k (kchunk a multiple of T), the
// k loop inside the unit so that the unit's decomposition, batch offset and
// row offsets are paid once per unit; one atomicMax per row per unit.
//
// row_fast (the operand is contiguous along rows): a unit is 256 rows, one per
// thread, each thread walking all k of the chunk for its row with 8 loads in
// flight.  A CTA's eight warps read 2 KB contiguous at each k, and consecutive
// units are consecutive row blocks at the same k range; no reduction between
// threads is needed.  Otherwise (contiguous along k): a unit is 32 rows, lanes
// walk k and each warp reduces its 4 rows with shuffles at the unit's end.
constexpr int kRowFastBatch = 8;   // loads a thread keeps in flight when it walks one row
constexpr int kRowFastRows = T * TR; // rows of a unit when the operand is contiguous along rows
__global__ void __launch_bounds__(T *TR, 5) k_split_rowmax(OperandMap m, const double *__restrict__ X,
                                                        unsigned long long *rowmax, int row_fast, int kchunk) {
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t rows_per_unit = row_fast ? kRowFastRows : T;
    const int64_t rt = (m.rows + rows_per_unit - 1) / rows_per_unit, kcs = (m.K + kchunk - 1) / kchunk;
    const int64_t units = (int64_t)m.nbatch * rt * kcs;
    const bool narrow = units < INT_MAX;
    for (int64_t u = blockIdx.x; u < units; u += gridDim.x) {
        int64_t i0, i1, b;
        split_unit(u, row_fast ? rt : kcs, row_fast ? kcs : rt, narrow, i0, i1, b);
        const int64_t kc = row_fast ? i1 : i0, rtile = row_fast ? i0 : i1;
        const int64_t ob = off_b(m, b);
        const int64_t r0 = rtile * rows_per_unit;
        const int64_t kbeg = kc * kchunk, kend = min(m.K, kbeg + kchunk);
        if (row_fast) {
            const int64_t r = r0 + ty * T + tx;
            if (r < m.rows) {
                const double *xr = X + ob + off_r(m, r);
                unsigned long long mx = 0;
                int64_t k = kbeg;
                for (; k + kRowFastBatch <= kend; k += kRowFastBatch) {
                    unsigned long long v[kRowFastBatch];
#pragma unroll
                    for (int i = 0; i < kRowFastBatch; i++) v[i] = abs_bits(__ldg(xr + off_k(m, k + i)));
#pragma unroll
                    for (int i = 0; i < kRowFastBatch; i++) mx = max(mx, v[i]);
                }
                for (; k < kend; k++) mx = max(mx, abs_bits(__ldg(xr + off_k(m, k))));
                if (mx) atomicMax(rowmax + b * m.Rp + r, mx);
            }
        } else {
            // thread (tx, ty): rows r0+ty, +8, ...; k = kbeg+tx, +32, ...; warp reduce along k
            constexpr int RPT = T / TR;
            const double *xr[RPT];
            unsigned long long mx[RPT];
#pragma unroll
            for (int j = 0; j < RPT; j++) {
                const int64_t r = r0 + ty + TR * j;
                xr[j] = r < m.rows ? X + ob + off_r(m, r) : nullptr;
                mx[j] = 0;
            }
#pragma unroll 2
            for (int64_t k = kbeg + tx; k < kend; k += T) {
                const int64_t okk = off_k(m, k);
#pragma unroll
                for (int j = 0; j < RPT; j++)
                    if (xr[j]) mx[j] = max(mx[j], abs_bits(__ldg(xr[j] + okk)));
            }
#pragma unroll
            for (int j = 0; j < RPT; j++) {
                unsigned long long v = mx[j];
                for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
                const int64_t r = r0 + ty + TR * j;
                if (tx == 0 && r < m.rows && v) atomicMax(rowmax + b * m.Rp + r, v);
            }
        }
    }
}

__global__ void k_split_exponent(const unsigned long long *rowmax, int *e, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double mx = __longlong_as_double((long long)rowmax[i]);
        int ex = 0;
        if (!isfinite(mx))
            ex = INT_MIN;
        else if (mx > 0.0)
            frexp(mx, &ex); // mx = f 2^ex with f in [0.5, 1): |x| <= mx < 2^ex
        e[i] = ex;
    }
}

// Tiles of 32 rows x 64 k staged through shared memory so that the operand is
// read along its contiguous mode; each thread then converts two consecutive k
// of a row and writes them as one BF16 pair per digit plane (a warp stores 128
// contiguous bytes per plane).  Padding rows and columns are written as 0.
//
// A work unit is a strip of up to kDigitStrip k tiles of one 32-row tile, so
// that the unit's decomposition, exponents and row offsets are paid per strip.
// Consecutive units walk the operand's contiguous mode: k strips of one row
// tile, or (row_fast) row tiles of one k strip.  Within a strip the tiles are
// double-buffered: asynchronous copies (cp.async, zero-filled outside the
// operand) bring tile t+1 into shared memory while tile t is converted.
constexpr int TK = 2 * T;
constexpr int64_t kDigitStrip = 8; // k tiles per work unit
__device__ __forceinline__ void cp_async8(double *dst, const double *src, bool valid) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(d), "l"(src), "r"(valid ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <int S>
__global__ void __launch_bounds__(T *TR) k_split_digits(OperandMap m, const double *__restrict__ X, const int *rexp,
                                                        __nv_bfloat16 *planes, int row_fast) {
    __shared__ double tile[2][T][TK + 1];
    __shared__ int ex[T];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int64_t rt = m.Rp / T, kt = m.Kp / TK, segs = (kt + kDigitStrip - 1) / kDigitStrip;
    const int64_t work = (int64_t)m.nbatch * rt * segs;
    const bool narrow = work < INT_MAX;
    const int64_t plane = m.Rp * m.Kp;
    constexpr int RPT = T / TR;
    for (int64_t w = blockIdx.x; w < work; w += gridDim.x) {
        int64_t i0, i1, b;
        split_unit(w, row_fast ? rt : segs, row_fast ? segs : rt, narrow, i0, i1, b);
        const int64_t sg = row_fast ? i1 : i0, rtile = row_fast ? i0 : i1;
        const int64_t ob = off_b(m, b);
        const int64_t r0 = rtile * T;
        __syncthreads(); // the previous strip's last reads of ex[] and of the tiles are done
        if (ty == 0) ex[tx] = (r0 + tx < m.rows) ? rexp[b * m.Rp + r0 + tx] : 0;
        const double *xr[RPT]; // row_fast: row r0+tx in xr[0]; else rows r0+ty+8j
#pragma unroll
        for (int j = 0; j < RPT; j++) {
            const int64_t r = row_fast ? (j == 0 ? r0 + tx : m.rows) : r0 + ty + TR * j;
            xr[j] = r < m.rows ? X + ob + off_r(m, r) : nullptr;
        }
        auto load_tile = [&](int buf, int64_t k0) {
            if (row_fast) {
#pragma unroll
                for (int j = ty; j < TK; j += TR) {
                    const int64_t k = k0 + j;
                    const bool ok = xr[0] && k < m.K;
                    cp_async8(&tile[buf][tx][j], ok ? xr[0] + off_k(m, k) : X, ok);
                }
            } else {
#pragma unroll
                for (int h = 0; h < 2; h++) {
                    const int64_t k = k0 + h * T + tx;
                    const bool kin = k < m.K;
                    const int64_t okk = kin ? off_k(m, k) : 0;
#pragma unroll
                    for (int j = 0; j < RPT; j++) {
                        const bool ok = xr[j] && kin;
                        cp_async8(&tile[buf][ty + TR * j][h * T + tx], ok ? xr[j] + okk : X, ok);
                    }
                }
            }
            cp_async_commit();
        };
        const int64_t kt_beg = sg * kDigitStrip, kt_end = min(kt, (sg + 1) * kDigitStrip);
        load_tile(0, kt_beg * TK);
        for (int64_t ktile = kt_beg; ktile < kt_end; ktile++) {
            const int cur = (int)((ktile - kt_beg) & 1);
            const int64_t k0 = ktile * TK;
            if (ktile + 1 < kt_end) {
                load_tile(cur ^ 1, k0 + TK);
                cp_async_wait<1>();
            } else {
                cp_async_wait<0>();
            }
            __syncthreads();
            // write: thread tx converts k0 + 2tx and k0 + 2tx + 1 of each of its rows
#pragma unroll
            for (int j = ty; j < T; j += TR) {
                const int64_t r = r0 + j;
                uint32_t pk[S];
                const int e = ex[j];
                if (e == INT_MIN) {
#pragma unroll
                    for (int s = 0; s < S; s++) pk[s] = 0u;
                } else {
                    digits_bf16x2<S>(tile[cur][j][2 * tx], tile[cur][j][2 * tx + 1], e, pk);
                }
                uint32_t *out = (uint32_t *)(planes + ((int64_t)b * S) * plane + r * m.Kp + k0) + tx;
#pragma unroll
                for (int s = 0; s < S; s++) out[(int64_t)s * (plane / 2)] = pk[s];
            }
            __syncthreads();
        }
    }
}

// CTAs of `kernel` (256 threads, static shared memory) that fit on the GPU at
// once: the splitting kernels launch exactly one wave of them and loop over
// their work units, so no partial second wave trails the launch.
template <typename F>
int resident_grid(F kernel) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, T * TR, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
    return per_sm * num_sms();
}

// K chunk (a multiple of `gran`) for `row_units` row blocks: among splits into
// about one to four units per resident CTA, the one whose last wave of units is
// fullest (the fewest units when two are about as full).
int balanced_chunk(int64_t row_units, int64_t K, int64_t resident, int gran) {
    const int64_t ktiles = std::max<int64_t>(1, (K + gran - 1) / gran);
    row_units = std::max<int64_t>(1, row_units);
    int64_t best_tiles = ktiles;
    double best_eff = -1.0;
    for (int per = 1; per <= 4; per++) {
        const int64_t want = std::min(ktiles, std::max<int64_t>(1, resident * per / row_units));
        const int64_t tiles = (ktiles + want - 1) / want; // tiles of `gran` k per chunk
        const int64_t units = row_units * ((ktiles + tiles - 1) / tiles);
        const int64_t waves = (units + resident - 1) / resident;
        const double eff = (double)units / (double)(waves * resident);
        if (eff > best_eff + 0.02) {
            best_eff = eff;
            best_tiles = tiles;
        }
    }
    return (int)(best_tiles * gran);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    });
    return fn;
}

// 3-D map over [planes][rows][Kp] BF16, box 64 (k) x box_rows rows x 1, 128-byte swizzle.
eg_status encode_planes(CUtensorMap *map, void *base, int64_t Kp, int64_t rows, int64_t planes, int box_rows = kBM) {
    auto fn = encode_fn();
    if (!fn) return fail(EG_ERROR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    cuuint64_t dims[3] = {(cuuint64_t)Kp, (cuuint64_t)rows, (cuuint64_t)planes};
    cuuint64_t strides[2] = {(cuuint64_t)(Kp * 2), (cuuint64_t)(Kp * 2 * rows)};
    cuuint32_t box[3] = {(cuuint32_t)kBK, (cuuint32_t)box_rows, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(EG_ERROR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return EG_SUCCESS;
}

int64_t round_up(int64_t x, int64_t m) { return (x + m - 1) / m * m; }

bool is_fast(const ModeGroup &g, int comp) { return g.n > 0 && g.s[comp][g.n - 1] == 1; }

// The single stride of a group whose modes (extent-1 modes ignored) nest like a
// row-major block in operand `comp`, else 0.
int64_t affine_stride(const ModeGroup &g, int comp) {
    int64_t stride = 0, span = 0; // stride of the fastest mode seen, and stride * extents so far
    for (int d = g.n - 1; d >= 0; d--) {
        if (g.ext[d] == 1) continue;
        const int64_t sd = g.s[comp][d];
        if (stride == 0) {
            if (sd == 0) return 0;
            stride = sd;
            span = sd * g.ext[d];
        } else {
            if (sd != span) return 0;
            span = sd * g.ext[d];
        }
    }
    return stride == 0 ? 1 : stride; // no mode of extent > 1: the group has one index, offset 0
}

eg_status split_operand(OperandMap om, const double *X, unsigned long long *rowmax, int *rexp,
                        __nv_bfloat16 *planes, int S, cudaStream_t s, int64_t *offr, int64_t *offk) {
    const bool k_fast = is_fast(om.kg, om.comp);
    om.sr = affine_stride(om.rg, om.comp);
    om.sk = affine_stride(om.kg, om.comp);
    if (om.sr && om.sk) offr = offk = nullptr; // no tables needed
    if (offr && offk) {
        const int64_t n = std::max(om.rows, om.K);
        {
            LaunchScope ls_("k_operand_offsets", s);
            k_operand_offsets<<<(int)std::min<int64_t>((n + 255) / 256, (int64_t)num_sms() * 8), 256, 0, s>>>(om, offr,
                                                                                                            offk);
        }
        EG_CHECK_LAUNCH("k_operand_offsets");
        om.offr = offr;
        om.offk = offk;
    }
    const bool r_fast = !k_fast && is_fast(om.rg, om.comp);
    EG_CUDA(cudaMemsetAsync(rowmax, 0, (size_t)om.nbatch * om.Rp * sizeof(unsigned long long), s));
    const int cap = num_sms() * 8;
    {
        static const int resident = resident_grid(k_split_rowmax);
        const int64_t unit_rows = r_fast ? kRowFastRows : T;
        const int64_t rows_units = (int64_t)om.nbatch * ((om.rows + unit_rows - 1) / unit_rows);
        const int kchunk = balanced_chunk(rows_units, om.K, resident, r_fast ? kRowFastBatch : T);
        const int64_t work = rows_units * ((om.K + kchunk - 1) / kchunk);
        const int grid = (int)(work < resident ? (work < 1 ? 1 : work) : resident);
        LaunchScope ls_("k_split_rowmax", s);
        k_split_rowmax<<<grid, dim3(T, TR), 0, s>>>(om, X, rowmax, r_fast ? 1 : 0, kchunk);
    }
    EG_CHECK_LAUNCH("k_split_rowmax");
    {
        const int64_t n = (int64_t)om.nbatch * om.Rp;
        LaunchScope ls_("k_split_exponent", s);
        k_split_exponent<<<(int)std::min<int64_t>((n + 255) / 256, cap), 256, 0, s>>>(rowmax, rexp, n);
    }
    EG_CHECK_LAUNCH("k_split_exponent");
    {
        const int64_t work = (int64_t)om.nbatch * (om.Rp / T) * ((om.Kp / TK + kDigitStrip - 1) / kDigitStrip);
        static const int resident = resident_grid(k_split_digits<5>); // the S variants share a register budget
        const int grid = (int)(work < resident ? work : resident);
        LaunchScope ls_("k_split_digits", s);
        const int rf = r_fast ? 1 : 0;
        switch (S) {
        case 2: k_split_digits<2><<<grid, dim3(T, TR), 0, s>>>(om, X, rexp, planes, rf); break;
        case 3: k_split_digits<3><<<grid, dim3(T, TR), 0, s>>>(om, X, rexp, planes, rf); break;
        case 4: k_split_digits<4><<<grid, dim3(T, TR), 0, s>>>(om, X, rexp, planes, rf); break;
        case 5: k_split_digits<5><<<grid, dim3(T, TR), 0, s>>>(om, X, rexp, planes, rf); break;
        default: k_split_digits<6><<<grid, dim3(T, TR), 0, s>>>(om, X, rexp, planes, rf); break;
        }
    }
    EG_CHECK_LAUNCH("k_split_digits");
    return EG_SUCCESS;
}

} // namespace

} // namespace eg::split

namespace eg {

eg_status encode_planes_public(CUtensorMap *map, void *base, int64_t Kp, int64_t rows, int64_t planes) {
    return split::encode_planes(map, base, Kp, rows, planes);
}

int64_t mode_group_affine_stride(const ModeGroup &g, int comp) { return split::affine_stride(g, comp); }

// A tiled map over an FP64 tensor of rank 2..5: dims[0] is the contiguous mode,
// strides_bytes[i] the byte stride of mode i + 1, no swizzle, zero fill.
eg_status encode_tiled_f64(CUtensorMap *map, const void *base, int rank, const uint64_t *dims,
                           const uint64_t *strides_bytes, const uint32_t *box) {
    auto fn = split::encode_fn();
    if (!fn) return fail(EG_ERROR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    cuuint64_t d[5], st[4];
    cuuint32_t b[5], es[5];
    for (int i = 0; i < rank; i++) {
        d[i] = dims[i];
        b[i] = box[i];
        es[i] = 1;
        if (i + 1 < rank) st[i] = strides_bytes[i];
    }
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, (cuuint32_t)rank, const_cast<void *>(base), d, st, b, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(EG_ERROR_NOT_SUPPORTED, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return EG_SUCCESS;
}

// A map over `planes` planes of `rows` x `K` BF16 digits laid out with row
// stride Kp and plane stride Rp * Kp elements (the extents may be below the
// padded layout: TMA then fills the rest of a box with zeros).
eg_status encode_planes_extent(CUtensorMap *map, void *base, int64_t K, int64_t rows, int64_t planes, int64_t Kp,
                               int64_t Rp) {
    auto fn = split::encode_fn();
    if (!fn) return fail(EG_ERROR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)planes};
    cuuint64_t strides[2] = {(cuuint64_t)(Kp * 2), (cuuint64_t)(Kp * 2 * Rp)};
    cuuint32_t box[3] = {(cuuint32_t)split::kBK, (cuuint32_t)split::kBM, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, base, dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(EG_ERROR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return EG_SUCCESS;
}

eg_status launch_split_contract(const Contraction &c, int slices, cudaStream_t s, eg_split_report *rep) {
    using namespace split;
    const int S = slices ? slices : 5;
    if (S < 2 || S > kMaxSlices) return fail(EG_ERROR_INVALID_ARGUMENT, "split form: slices must be in 2..6");
    const int64_t nb = c.batch.total, M = c.m.total, N = c.n.total, K = c.k.total;
    if (M >= (int64_t(1) << 31) || N >= (int64_t(1) << 31) || K >= (int64_t(1) << 31) || nb * S >= (int64_t(1) << 31))
        return fail(EG_ERROR_NOT_SUPPORTED, "split form: a mode group exceeds 2^31 elements");
    const int64_t Kp = round_up(K, kKStep), Mp = round_up(M, kBM), Np = round_up(N, kBN);

    // workspace: digit planes of A and B, row maxima, exponents, status word
    const size_t bytesA = (size_t)nb * S * Mp * Kp * 2, bytesB = (size_t)nb * S * Np * Kp * 2;
    const size_t offB = round_up((int64_t)bytesA, 1024);
    const size_t offMaxA = offB + round_up((int64_t)bytesB, 1024);
    const size_t offMaxB = offMaxA + round_up(nb * Mp * 8, 256);
    const size_t offEA = offMaxB + round_up(nb * Np * 8, 256);
    const size_t offEB = offEA + round_up(nb * Mp * 4, 256);
    const size_t offR = offEB + round_up(nb * Np * 4, 256);
    // offset tables (rows and k of each operand) unless they would be large
    const bool tables = M + K <= (int64_t(1) << 25) && N + K <= (int64_t(1) << 25);
    const size_t offTab = offR + rbuf_bytes();
    const size_t tabBytes = tables ? (size_t)(M + N + 2 * K) * 8 : 0;
    // K slices in parallel when the output has fewer tiles than half the SMs
    const int64_t tiles = nb * (Mp / kBM) * (Np / kBN);
    const bool kslicing = tiles < num_sms() / 2;
    // CTA pairs (256x128 tiles) whenever the output has two or more row tiles
    const int clusters = Mp / kBM >= 2 ? tc_pair_clusters() : 0;
    const bool pair = clusters > 0;
    const size_t offRacc = round_up((int64_t)(offTab + tabBytes), 256);
    const size_t raccBytes = kslicing ? (size_t)tiles * kBM * kBN * 8 : 0;
    const size_t offRcnt = offRacc + raccBytes;
    const size_t rcntBytes = kslicing ? (size_t)tiles * 8 * sizeof(int) : 0;
    const size_t total = offRcnt + rcntBytes;
    void *ws = nullptr;
    eg_status st = workspace(s, total, &ws);
    if (st != EG_SUCCESS) return st;
    char *base = (char *)ws;
    __nv_bfloat16 *planesA = (__nv_bfloat16 *)base, *planesB = (__nv_bfloat16 *)(base + offB);
    unsigned long long *maxA = (unsigned long long *)(base + offMaxA), *maxB = (unsigned long long *)(base + offMaxB);
    int *eA = (int *)(base + offEA), *eB = (int *)(base + offEB);
    int *status = nullptr;
    if ((st = status_word(s, &status)) != EG_SUCCESS) return st;

    OperandMap oa{c.batch, c.m, c.k, 0, M, Mp, K, Kp, (int)nb};
    OperandMap ob{c.batch, c.n, c.k, 1, N, Np, K, Kp, (int)nb};
    int64_t *tab = tables ? (int64_t *)(base + offTab) : nullptr;
    if ((st = split_operand(oa, c.A, maxA, eA, planesA, S, s, tab, tables ? tab + M : nullptr)) != EG_SUCCESS) return st;
    if ((st = split_operand(ob, c.B, maxB, eB, planesB, S, s, tables ? tab + M + K : nullptr,
                            tables ? tab + M + K + N : nullptr)) != EG_SUCCESS)
        return st;

    CUtensorMap tmA, tmB;
    if ((st = encode_planes(&tmA, planesA, Kp, Mp, nb * S)) != EG_SUCCESS) return st;
    if ((st = encode_planes(&tmB, planesB, Kp, Np, nb * S, pair ? kBN / 2 : kBN)) != EG_SUCCESS) return st;

    TcGemmParams p{};
    p.pair = pair ? 1 : 0;
    p.S = S;
    p.mtiles = (int)(Mp / kBM);
    p.ntiles = (int)(Np / kBN);
    p.nbatch = (int)nb;
    p.M = M;
    p.N = N;
    p.Mp = (int)Mp;
    p.Np = (int)Np;
    p.bg = c.batch;
    p.mg = c.m;
    p.ng = c.n;
    p.C = c.C;
    p.ab = c.ab;
    p.eA = eA;
    p.eB = eB;
    p.shift_const = -2 * kTopBits - kBits * (S - 1);
    {
        int k = 0;
        const double f = std::frexp(std::fabs(c.ab), &k); // |ab| = f 2^k
        p.ab_pow2 = (f == 0.5) ? 1 : 0;
        p.ab_neg = (p.ab_pow2 && c.ab < 0) ? 1 : 0;
        if (p.ab_pow2) p.shift_const += k - 1;
    }
    p.status = status;
    p.timeout_ns = 2000ull * 1000 * 1000;
    p.rbuf = (long long *)(base + offR);
    p.racc = kslicing ? (long long *)(base + offRacc) : nullptr;
    p.rcnt = kslicing ? (int *)(base + offRcnt) : nullptr;

    // Launches: when all slice groups' exact sum fits int64 over the whole K (up to
    // 65024 for S = 5), one.  Otherwise the slice groups are cut into ranges whose
    // own exact sums fit (S = 6 with K = 16384: groups 0-4 and 5), each range added
    // into C in FP64 by its own launch -- one extra rounding per range instead of a
    // launch (and a read and write of C) per 128 of K; a range that still cannot
    // take the whole K runs K passes.
    const int64_t nkb_total = Kp / kBK;
    std::vector<std::pair<int, int>> ranges;
    for (int d0 = 0; d0 < S;) {
        int d1 = d0 + 1;
        while (d1 < S && max_k_per_pass_groups(d0, d1 + 1) >= Kp) d1++;
        ranges.push_back({d0, d1});
        d0 = d1;
    }
    const int shift_base = p.shift_const;
    bool first_launch = true;
    for (const auto &range : ranges) {
        p.d0 = range.first;
        p.d1 = range.second;
        p.shift_const = shift_base + kBits * (S - p.d1);
        const int64_t kb_per_pass = max_k_per_pass_groups(p.d0, p.d1) / kBK;
        if (kb_per_pass < 1) return fail(EG_ERROR_NOT_SUPPORTED, "split form: slice count too large for exact accumulation");
        for (int64_t kb0 = 0; kb0 < nkb_total || kb0 == 0; kb0 += kb_per_pass) {
            p.kb0 = (int)kb0;
            p.nkb = (int)std::min<int64_t>(kb_per_pass, nkb_total - kb0);
            // slices of at least 16 K blocks (one exact chunk); the count minimises the
            // estimated makespan: rounds of work entries over the SMs times the K blocks
            // of one entry, plus about four blocks' worth of per-entry epilogue work
            p.ksplit = 1;
            p.kslice = p.nkb;
            if (kslicing && p.nkb >= 32) {
                // schedule units: tiles over SMs, or pair tiles over CTA pairs
                const int64_t units = pair ? nb * ((Mp / kBM + 1) / 2) * (Np / kBN) : tiles;
                const int64_t workers = pair ? clusters : num_sms();
                int64_t best = -1;
                for (int ks = 1; ks <= p.nkb / 16; ks++) {
                    const int64_t slice = round_up((p.nkb + ks - 1) / ks, kKStep / kBK);
                    const int64_t n = (p.nkb + slice - 1) / slice; // slices actually used
                    const int64_t rounds = (units * n + workers - 1) / workers;
                    const int64_t cost = rounds * (slice + 4);
                    if (best < 0 || cost < best) {
                        best = cost;
                        p.kslice = (int)slice;
                        p.ksplit = (int)n;
                    }
                }
            }
            if (p.ksplit > 1) {
                EG_CUDA(cudaMemsetAsync(p.racc, 0, raccBytes, s));
                EG_CUDA(cudaMemsetAsync(p.rcnt, 0, rcntBytes, s));
            }
            const bool first = first_launch;
            first_launch = false;
            p.cp = first ? c.cp : 1.0;
            p.zero = first ? (c.zero_when_cp_zero ? 1 : 0) : 0;
            if (p.nkb <= 0) break;
            static const bool prof_on = std::getenv("EINSUMS_GB300_TC_PROFILE") != nullptr;
            unsigned long long *prof = nullptr;
            if (prof_on) {
                EG_CUDA(cudaMalloc(&prof, (size_t)num_sms() * 8 * sizeof(unsigned long long)));
                EG_CUDA(cudaMemsetAsync(prof, 0, (size_t)num_sms() * 8 * sizeof(unsigned long long), s));
            }
            p.prof = prof;
            if ((st = launch_tc_gemm(tmA, tmB, p, s)) != EG_SUCCESS) return st;
            if (prof) {
                // Per-role wait/busy cycles summed over CTAs (a tracing aid, off by default).
                std::vector<unsigned long long> h((size_t)num_sms() * 8);
                EG_CUDA(cudaMemcpyAsync(h.data(), prof, h.size() * 8, cudaMemcpyDeviceToHost, s));
                EG_CUDA(cudaStreamSynchronize(s));
                cudaFree(prof);
                double tot[8] = {0};
                int ran = 0; // CTAs of the launch (its grid may be below the SM count)
                for (size_t i = 0; i < h.size(); i++) tot[i % 8] += (double)h[i];
                for (size_t i = 6; i < h.size(); i += 8) ran += h[i] > 0 ? 1 : 0;
                std::fprintf(stderr,
                             "[tc profile] M=%lld N=%lld K=%lld tiles=%d: total %.3g cyc/CTA | producer wait empty %.1f%% | "
                             "mma wait full %.1f%% | mma wait acc %.1f%% | epi wait acc %.1f%% | epi flush %.1f%% | "
                             "epi final %.1f%%\n",
                             (long long)M, (long long)N, (long long)K, p.mtiles * p.ntiles * p.nbatch,
                             tot[6] / (ran > 0 ? ran : 1), 100 * tot[0] / tot[6], 100 * tot[1] / tot[6], 100 * tot[2] / tot[6],
                             100 * tot[3] / tot[6], 100 * tot[4] / tot[6], 100 * tot[5] / tot[6]);
            }
        }
    }
    if (rep) {
        rep->slices = S;
        rep->slice_pairs = S * (S + 1) / 2;
        rep->bits_per_slice = kBits;
        rep->error_bound = error_bound(S);
    }
    return EG_SUCCESS;
}

} // namespace eg
