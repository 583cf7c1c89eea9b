// Split-BF16 ("Ozaki") form of the canonical contraction.
//
// Every FP64 operand row (a fixed (batch, m) of A, or (batch, n) of B, over
// all summed modes k) is scaled by its own power of two 2^e, |x| < 2^e, and
// cut into S balanced base-256 digits:
//     x = 2^(e-7) * sum_{s<S} a_s 2^(-8 s),   a_s integer in [-128, 128]
// so each digit ("slice") is exact in BF16 and a slice product is an integer
// below 2^14.  The product of two rows is
//     sum_k A B = 2^(eA+eB-14) * sum_d 2^(-8 d) G_d,   G_d = sum_{s+t=d} sum_k a_s b_t
// and the triangular truncation keeps d < S (S(S+1)/2 slice pairs).  The
// tensor cores accumulate G_d in FP32 over chunks of at most 1024 products,
// which keeps every partial sum an integer of at most 2^24 and therefore
// exact; the epilogue converts each chunk to an integer and accumulates
//     R = sum_d 2^(8 (S-1-d)) G_d
// exactly in int64 in tensor memory.  The only roundings of the whole
// product are the digit truncation and the final int64 -> FP64 conversion.
// This is the scheme of Ozaki, Ogita, Oishi and Rump (Numer. Algorithms 59,
// 2012) as mapped to integer-exact tensor-core products by Ootomo, Ozaki and
// Yokota (IJHPCA 2024), with BF16 digits and FP32 accumulation.
#pragma once

#include <climits>

#include <cuda.h>

#include "common.cuh"

namespace eg::split {

constexpr int kBits = 8;        // digit width
constexpr int kTopBits = 7;     // magnitude bits of the leading digit
constexpr int kMaxSlices = 6;   // keeps the scaled digits and the int64 accumulator in range
constexpr int kBM = 128, kBN = 128, kBK = 64;
constexpr int kChunkKB = 16;    // 16 x 64 = 1024 products per exact FP32 chunk
constexpr int kKStep = 2 * kBK;  // K is padded to whole groups of two K blocks

struct TcGemmParams {
    int S;
    int nkb;  // K blocks in this pass
    int kb0;  // first K block of this pass
    int mtiles, ntiles, nbatch;
    int64_t M, N;
    int Mp, Np;
    ModeGroup bg, mg, ng; // output offsets in C (component 2)
    double *C;
    double cp, ab;
    int ab_pow2; // ab = +-2^k: folded into the exponent (ab_neg gives the sign)
    int ab_neg;
    int zero;
    const int *eA; // [nbatch][Mp] row exponents; INT_MIN marks a non-finite row
    const int *eB; // [nbatch][Np]
    int shift_const; // -14 - 8 (S-1), plus k when ab = +-2^k
    int *status;
    unsigned long long timeout_ns;
    // Optional per-CTA cycle counters (null in normal runs): see kProf* in tc_gemm.cu.
    unsigned long long *prof;
    // Per-CTA scratch of gridDim.x * 128 * 128 int64: a finished tile's sums
    // wait here until the epilogue converts them during the next tile.
    long long *rbuf;
    // K slices run in parallel when there are few output tiles: entry t of the
    // schedule is K slice t % ksplit (kslice K blocks, even; the last slice takes
    // the rest) of tile t / ksplit.  The slices' exact int64 sums are added into
    // racc ([tile][128 columns][128 rows]) and the last slice to arrive at a
    // region of an epilogue warp (counted in rcnt, [tile][8]) finishes it.  Both
    // are zeroed by the host before the launch; unused when ksplit == 1.
    int ksplit, kslice;
    long long *racc;
    int *rcnt;
    // Launch as CTA pairs (cta_group::2, 256x128 tiles; B's tensor map has
    // 64-row boxes): single contractions only.
    int pair;
    // Slice groups d0 <= d < d1 (anti-diagonals s + t = d of the digit pairs)
    // summed by this launch: all of them (0, S) unless a long K is split into
    // group ranges whose exact sums each fit int64 (finished into C one by one).
    int d0, d1;
    // Grouped launches: two tensor maps per item (A, B) over the item's own digit
    // planes with its own row and K extents, so that TMA fills the tile's rows
    // past M (N) and K blocks past K with zeros instead of reading the padding.
    const CUtensorMap *item_maps;
};

// One item of a grouped launch: an independent contraction whose digit planes
// start at plane zA / zB of the shared plane arrays and whose exponents start
// at eAoff / eBoff.  Work entries (int4) are {item, batch index, mt, nt}.
struct TcItem {
    double *C;
    int64_t M, N;
    int nkb;
    int zA, zB;
    int eAoff, eBoff;
    int Mp, Np;
    ModeGroup bg, mg, ng;
};

// IEEE bit pattern of |x|: for non-negative doubles (and NaN above Inf) the
// unsigned order of the patterns is the numeric order.  Integer ops only: an
// FP64 abs would run on this GPU's slow FP64 pipe, once per element.
__device__ __forceinline__ unsigned long long abs_bits(double x) {
    return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}

// round(x * 2^sh) to nearest, ties to even, for |x| 2^sh < 2^52, built from the
// IEEE fields with integer operations (the FP64 pipe of this GPU runs about two
// operations per clock per SM; this is the splitting kernels' inner loop).
__device__ __forceinline__ long long scaled_round(double x, int sh) {
    const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((bits >> 52) & 0x7ff);
    const unsigned long long mant = (bits & 0xFFFFFFFFFFFFFull) | ((unsigned long long)(ex != 0) << 52);
    const int r = 1075 - (ex != 0 ? ex : 1) - sh; // |x| 2^sh = mant 2^-r
    unsigned long long q;
    if (r <= 0) {
        q = mant << (-r < 11 ? -r : 11); // not reached while |x| 2^sh < 2^52
    } else if (r > 62) {
        q = 0; // below 1/2
    } else {
        // round half to even in one add: the carry out of the r low bits happens
        // exactly when they exceed half, or equal half with an odd quotient
        q = (mant + ((1ull << (r - 1)) - 1ull) + ((mant >> r) & 1ull)) >> r;
    }
    return (bits >> 63) ? -(long long)q : (long long)q;
}

__device__ __forceinline__ double scale_pow2(double v, int e) {
    if (v == 0.0) return v;
    const long long bits = __double_as_longlong(v);
    const int ex = (int)((bits >> 52) & 0x7ff);
    const int ne = ex + e;
    if (ex != 0 && ne > 0 && ne < 2047) return __longlong_as_double(bits + ((long long)e << 52));
    return scalbn(v, e);
}

// R * 2^e rounded to nearest (ties to even), built with integer operations so
// the FP64 pipe -- about 1.75 operations per clock per SM on this GPU -- is
// left for the one fused multiply-add with C.  Falls back to the FP64 path
// when the result would not be a normal number.
__device__ __forceinline__ double int_times_pow2_rn(long long R, int e) {
    if (R == 0) return 0.0;
    const unsigned long long sign = R < 0 ? 0x8000000000000000ull : 0ull;
    const unsigned long long a = R < 0 ? (unsigned long long)(-R) : (unsigned long long)R;
    const int lz = __clzll((long long)a);
    const unsigned long long x = a << lz;      // leading one at bit 63
    unsigned long long mant = x >> 11;         // 53 bits, leading one at bit 52
    const unsigned long long rem = x & 0x7FFull;
    if (rem > 0x400ull || (rem == 0x400ull && (mant & 1ull))) mant++;
    int exp = 63 - lz + e;
    if (mant >> 53) {
        mant >>= 1;
        exp++;
    }
    const int biased = exp + 1023;
    if (biased <= 0 || biased >= 2047) return scale_pow2(__ll2double_rn(R), e);
    return __longlong_as_double((long long)(sign | ((unsigned long long)biased << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// Balanced base-256 digits of x * 2^(7 + 8(S-1) - e) rounded to an integer,
// most significant first: dig[0] in [-128, 128], the others in [-127, 128].
__device__ __forceinline__ void to_digits(double x, int e, int S, int *dig) {
    long long F = scaled_round(x, kTopBits + kBits * (S - 1) - e);
#pragma unroll
    for (int s = S - 1; s >= 1; s--) {
        int d = (int)(F & 255);
        if (d > 128) d -= 256;
        dig[s] = d;
        F = (F - d) >> 8; // exact: F - d is a multiple of 256
    }
    dig[0] = (int)F;
}

// The digits of two values as BF16 pairs: out[s] holds digit s of x0 in its low
// half and digit s of x1 in its high half — the same digits as to_digits.  With
// B = 127 (256^(S-2) + ... + 256 + 1), G = F + B has the ordinary base-256
// digits d_s + 127 in [0, 255] for s >= 1 and G >> 8(S-1) = d_0, so one 64-bit
// add replaces the subtract-and-shift chain.  A byte u becomes the float u - 127
// exactly as (2^23 + u) - (2^23 + 127) (bit OR, then an FP32 add), and d_0 as
// (1.5 * 2^23 + d_0) - 1.5 * 2^23; every digit has at most 8 significant bits,
// so its BF16 is the float's upper half, and one byte permute packs the pair.
template <int S>
__device__ __forceinline__ void digits_bf16x2(double x0, double x1, int e, uint32_t *out) {
    constexpr long long bias = [] {
        long long b = 0;
        for (int s = 1; s < S; s++) b = b * 256 + 127;
        return b;
    }();
    const int sh = kTopBits + kBits * (S - 1) - e;
    const long long G0 = scaled_round(x0, sh) + bias, G1 = scaled_round(x1, sh) + bias;
    const uint32_t g0[2] = {(uint32_t)G0, (uint32_t)((unsigned long long)G0 >> 32)};
    const uint32_t g1[2] = {(uint32_t)G1, (uint32_t)((unsigned long long)G1 >> 32)};
#pragma unroll
    for (int s = 1; s < S; s++) {
        // byte S-1-s of G next to the bytes 00 00 4B: the float 2^23 + u in one permute
        const int byte = S - 1 - s, w = byte >> 2;
        const uint32_t sel = 0x7440u | (uint32_t)(byte & 3);
        const float f0 = __uint_as_float(__byte_perm(g0[w], 0x4B000000u, sel)) - 8388735.0f;
        const float f1 = __uint_as_float(__byte_perm(g1[w], 0x4B000000u, sel)) - 8388735.0f;
        out[s] = __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632);
    }
    const int t0 = (int)(G0 >> (8 * (S - 1))), t1 = (int)(G1 >> (8 * (S - 1)));
    const float f0 = __int_as_float(0x4B400000 + t0) - 12582912.0f;
    const float f1 = __int_as_float(0x4B400000 + t1) - 12582912.0f;
    out[0] = __byte_perm(__float_as_uint(f0), __float_as_uint(f1), 0x7632);
}

// Sets the kernels' shared-memory attribute once (call outside stream capture).
eg_status ensure_tc_attributes();
// Clusters of two k_tc_split_gemm CTAs that fit on the GPU at once, when CTA
// pairs are requested with EINSUMS_GB300_TC_PAIRS=1 (else 0: single-CTA tiles).
int tc_pair_clusters();
eg_status launch_tc_gemm(const CUtensorMap &tmA, const CUtensorMap &tmB, const TcGemmParams &p, cudaStream_t s);
// Grouped form: `ntiles_total` work entries, per-tile parameters from `items`.
eg_status launch_tc_gemm_grouped(const CUtensorMap &tmA, const CUtensorMap &tmB, const TcGemmParams &p,
                                 const TcItem *items, const int4 *work, int ntiles_total, cudaStream_t s);

// Bytes of the per-CTA sum scratch a tensor launch needs (TcGemmParams::rbuf).
inline size_t rbuf_bytes() { return (size_t)num_sms() * kBM * kBN * sizeof(long long); }

// Largest K (a multiple of kKStep) one pass may sum without the int64
// accumulator overflowing 2^62 for S slices.
// Largest K (a multiple of kKStep) for which the exact sum over slice groups
// d0 <= d < d1, R = sum_d 2^(8 (d1-1-d)) G_d, stays below 2^62 in magnitude:
// |G_d| <= (d+1) K 2^14.
inline int64_t max_k_per_pass_groups(int d0, int d1) {
    double w = 0.0;
    for (int d = d0; d < d1; d++) w += (d + 1) * std::ldexp(1.0, 8 * (d1 - 1 - d));
    double kmax = std::ldexp(1.0, 62) / (std::ldexp(1.0, 14) * w);
    int64_t k = kmax > 9.0e18 ? INT64_MAX : (int64_t)kmax;
    return (k / kKStep) * kKStep;
}

inline int64_t max_k_per_pass(int S) { return max_k_per_pass_groups(0, S); }

// A-priori bound on the relative error of one product, relative to
// sum_k |A_row| |B_col| scaled to the row maxima: the dropped digit tail of
// both operands plus the dropped cross terms with s + t >= S.
inline double error_bound(int S) {
    const double u = std::ldexp(1.0, -(kTopBits + kBits * (S - 1))); // one unit of the last digit, relative
    return (S + 2) * u;
}

} // namespace eg::split
