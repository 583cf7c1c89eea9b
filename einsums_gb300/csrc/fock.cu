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
// Six multiply-adds per canonical element, 0.75 n^4 in all, against 2 n^4 for
// the two general contractions.  On this GPU the FP64 pipe retires about one
// warp-wide FMA per 64 cycles per SM sub-partition, a sixty-fourth of the FP32
// rate, so those multiply-adds bound the FP64 form.  The split form moves four
// of the six terms (T1, T2, T4, T5) to the FP32 pipe: g and D are cut into S
// balanced 8-bit digits at a power-of-two scale per summed line -- the digits
// of the split-BF16 contraction (split.cuh) -- whose products, integers below
// 2^14, add up exactly in FP32 over at most 64 elements and then exactly in
// integers (Horner over the digit groups d = s + t < S), converted to FP64
// once per line.  T3 and T6 stay FP64 and run on the FP64 pipe beside them.
//
// Every pass is a set of sums along lines of g read by 32 lanes at 32
// consecutive addresses: the symmetries of g give each sum a layout whose
// fastest index is the lanes' own.  Each lane keeps its sums in registers; no
// shared-memory tiles, no atomics.  Every partial has one home and the last
// passes add them in a fixed order, so the result is deterministic.
//   k_fock_digits_d   (split form) the digits of every row of D.
//   k_fock_rows<S>    unit r, a lane per pair (p, q): T1 and T4, sums over s
//                     of g[r,s,p,q] (= g[p,q,r,s]), consecutive lanes along q.
//   k_fock_cols<S>    unit p, a lane per pair (r, s): T2, T5 and T3, sums over
//                     q of g[p,q,r,s], consecutive lanes along s.
//   k_fock_exchange   warp (q, p, 32 s): T6, sums over r of g[q,p,r,s]
//                     (= g[p,q,r,s]) D[p,r], lanes along s.
//   k_fock_reduce     CTA (i, 32 j): YJ and XK from the partials.
//   k_fock_combine    J = 2 (YJ + YJ^T), K = XK + XK^T and the prefactors.
#include <algorithm>
#include <climits>
#include <cmath>

#include "split.cuh"

namespace eg {
void set_split_report(const eg_split_report &r);

namespace {

using split::int_times_pow2_rn;
using split::scaled_round;

constexpr int kWarps = 4;      // warps per CTA of the line passes (consecutive r)
constexpr int kRedWarps = 8;   // warps of a reduction CTA
constexpr int kFockMaxN = 384; // g is 174 GB at n = 384
constexpr int kFlush = 64;     // elements per exact FP32 digit-group sum (a multiple of kBatch)
constexpr int kBatch = 8;      // independent loads in flight per lane in the line passes

// x / 2 rounded to nearest even, on the IEEE fields with integer operations
// only: an exponent decrement for normal numbers, a mantissa shift for the rest
// (an FP64 multiply here would be if-converted into every element's path and
// cost the FP64 pipe more than the element's own multiply-adds).  Inf and NaN
// keep their exponent field and stay what they are.
__device__ __forceinline__ double half_exact(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned long long ex = (b >> 52) & 0x7ff;
    if (ex > 1 && ex < 0x7ff) return __longlong_as_double((long long)(b - (1ull << 52)));
    if (ex == 0x7ff) return x;
    const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (ex << 52); // ex = 1: the implicit one
    const unsigned long long h = (m >> 1) + (m & (m >> 1) & 1ull);     // halve, ties to even
    return __longlong_as_double((long long)((b & 0x8000000000000000ull) | h));
}

// Scale exponent of a set whose largest |x| has IEEE bits mx: |x| < 2^e
// (0 for an all-zero set, INT_MIN when it holds an Inf or NaN).
__device__ __forceinline__ int set_exponent(unsigned long long mx) {
    const int ex = (int)(mx >> 52);
    if (ex == 0x7ff) return INT_MIN;
    if (mx == 0) return 0;
    if (ex != 0) return ex - 1022;
    int e = 0;
    frexp(__longlong_as_double((long long)mx), &e); // subnormal maximum
    return e;
}

// The S balanced digits of round(x 2^sh) as floats, most significant first:
// with the bias B = 127 (256^(S-2) + ... + 1) the lower digits are plain bytes
// of F + B, each made a float exactly as (2^23 + u) - (2^23 + 127), and the top
// digit is (F + B) >> 8 (S - 1) -- the digits of split.cuh's digits_bf16x2.
template <int S>
__device__ __forceinline__ void digits_f32(double x, int sh, float (&f)[S]) {
    constexpr long long bias = [] {
        long long b = 0;
        for (int s = 1; s < S; s++) b = b * 256 + 127;
        return b;
    }();
    const long long G = scaled_round(x, sh) + bias;
    const uint32_t w[2] = {(uint32_t)G, (uint32_t)((unsigned long long)G >> 32)};
#pragma unroll
    for (int s = 1; s < S; s++) {
        const int byte = S - 1 - s;
        const uint32_t u = (w[byte >> 2] >> (8 * (byte & 3))) & 255u;
        f[s] = __uint_as_float(0x4B000000u | u) - 8388735.0f;
    }
    const int t0 = (int)(G >> (8 * (S - 1)));
    f[0] = __int_as_float(0x4B400000 + t0) - 12582912.0f;
}

// acc[d] += sum_{s + t = d} a[s] b[t] for d < S: the triangular digit product.
template <int S>
__device__ __forceinline__ void digit_fma(const float (&a)[S], const float (&b)[S], float (&acc)[S]) {
#pragma unroll
    for (int d = 0; d < S; d++)
#pragma unroll
        for (int s = 0; s <= d; s++) acc[d] = fmaf(a[s], b[d - s], acc[d]);
}

// The FP32 group sums (integers below 2^24) folded into int32 running sums.
template <int S>
__device__ __forceinline__ void digit_flush(float (&acc)[S], int (&run)[S]) {
#pragma unroll
    for (int d = 0; d < S; d++) {
        run[d] += __float2int_rn(acc[d]);
        acc[d] = 0.0f;
    }
}

// The FP64 value of sum_d run[d] 256^(S-1-d) 2^e (INT_MIN: NaN).
template <int S>
__device__ __forceinline__ double digit_value(const int (&run)[S], int e) {
    if (e == INT_MIN) return __longlong_as_double(0x7ff8000000000000ll);
    long long R = 0;
#pragma unroll
    for (int d = 0; d < S; d++) R = R * 256 + run[d];
    return int_times_pow2_rn(R, e);
}

template <int S>
__device__ __forceinline__ void load_digits(const float *p, float (&b)[S]) {
#pragma unroll
    for (int t = 0; t < S; t++) b[t] = __ldg(p + t);
}

struct FockScratch {
    double *S1;      // [p][r][q]   T1: sum over s
    double *S4;      // [q][p][r]   T4: sum over s
    double *S2;      // [r][p][s]   T2: sum over q
    double *S5;      // [p][r][s]   T5: sum over q
    double *X3;      // [p][r][s]   T3: sum over q
    double *X6;      // [q][p][s]   T6: sum over r
    double *YJ;      // [i][j], i >= j
    double *XK;      // [i][j]
    const float *Dd; // split form: [row][k][S] digits of D
    const int *De;   //             [row] scale exponents of D's rows
    int nsc;         // chunks of 32 s
};

// Digits of every row of D at the row's own scale: De[row] with |D[row][k]| < 2^e.
template <int S>
__global__ void __launch_bounds__(128) k_fock_digits_d(const double *__restrict__ D, int n, float *Dd, int *De) {
    const int row = blockIdx.x;
    __shared__ unsigned long long red[4];
    unsigned long long mx = 0;
    for (int k = threadIdx.x; k < n; k += 128) mx = max(mx, split::abs_bits(D[(size_t)row * n + k]));
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
    __syncthreads();
    mx = max(max(red[0], red[1]), max(red[2], red[3]));
    const int e = set_exponent(mx);
    if (threadIdx.x == 0) De[row] = e;
    const int sh = split::kTopBits + split::kBits * (S - 1) - (e == INT_MIN ? 0 : e);
    for (int k = threadIdx.x; k < n; k += 128) {
        float f[S];
        digits_f32<S>(e == INT_MIN ? 0.0 : D[(size_t)row * n + k], sh, f);
#pragma unroll
        for (int t = 0; t < S; t++) Dd[((size_t)row * n + k) * S + t] = f[t];
    }
}

constexpr int kShift(int S) { return -2 * split::kTopBits - split::kBits * (S - 1); }

// Flattened lanes.  For the rows pass, one r and the pairs (p, q) with p >= r,
// q <= p, numbered p-major from 0: pair f has p with start(p) <= f < start(p + 1),
// start(p) = (p (p + 1) - r (r + 1)) / 2.  For the columns pass, one p and the
// pairs (r, s) with s <= r <= p: start(r) = r (r + 1) / 2.  Consecutive lanes take
// consecutive pairs, so warps stay full however small p or r is.
__device__ __forceinline__ int tri_row(long long K) { // largest x with x (x + 1) <= K
    int x = (int)((sqrtf(4.0f * (float)K + 1.0f) - 1.0f) * 0.5f);
    while ((long long)(x + 1) * (x + 2) <= K) x++;
    while (x > 0 && (long long)x * (x + 1) > K) x--;
    return x;
}

// CTA x of a pass whose units u = 0 .. n-1 have count(u) pairs: the unit and the
// first pair of the CTA (kWarps * 32 pairs per CTA; the units with more pairs first).
template <typename Count>
__device__ __forceinline__ void unit_of_cta(int x, int n, Count count, int &u, int &first) {
    for (int k = 0; k < n; k++) {
        const int uu = n - 1 - k;
        const int ctas = (count(uu) + kWarps * 32 - 1) / (kWarps * 32);
        if (x < ctas) {
            u = uu;
            first = x * kWarps * 32;
            return;
        }
        x -= ctas;
    }
    u = -1;
    first = 0;
}

__device__ __forceinline__ int rows_pairs(int n, int r) { return (n * (n + 1) - r * (r + 1)) / 2; }
__device__ __forceinline__ int cols_pairs(int p) { return (p + 1) * (p + 2) / 2; }

// T1 and T4.  Unit r, lane (p, q): sums over s <= r (s <= q when p == r) of
// f g[p,q,r,s] {D[r,s], D[p,s]}, reading g[r,s,p,q] -- consecutive lanes read
// consecutive q.  The loop runs over the warp's common range in batches of
// kBatch independent loads (a lane outside its own range adds nothing).
template <int S>
__global__ void __launch_bounds__(kWarps * 32) k_fock_rows(const double *__restrict__ g,
                                                           const double *__restrict__ D, int n, FockScratch sc) {
    int r, first;
    unit_of_cta(blockIdx.x, n, [&](int u) { return rows_pairs(n, u); }, r, first);
    if (r < 0) return;
    const int f = first + threadIdx.x;
    const bool on = f < rows_pairs(n, r);
    int p = tri_row(2ll * (on ? f : 0) + (long long)r * (r + 1));
    if (p < r) p = r;
    if (p >= n) p = n - 1;
    const int q = on ? f - (p * (p + 1) - r * (r + 1)) / 2 : 0;
    const bool diag = p == r;
    const int smax = diag ? q : r; // this lane's last s
    const size_t step = (size_t)n * n; // s -> s + 1 in g[r][s][p][q]
    const double *gl = g + (((size_t)r * n) * n + p) * n + q;
    const double *Dr = D + (size_t)r * n, *Dp = D + (size_t)p * n;
    auto scale = [&](double v, int s) {
        if (q == p) v = half_exact(v);
        if (s == r) v = half_exact(v);
        if (diag && s == q) v = half_exact(v);
        return v;
    };
    double v1 = 0.0, v4 = 0.0;
    if constexpr (S == 0) {
        double a1 = 0.0, a4 = 0.0;
        for (int s0 = 0; s0 <= r; s0 += kBatch) {
            double v[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; u++) v[u] = s0 + u <= r ? __ldcs(gl + (s0 + u) * step) : 0.0;
#pragma unroll
            for (int u = 0; u < kBatch; u++) {
                const int s = s0 + u;
                if (s <= smax && on) {
                    const double w = scale(v[u], s);
                    a1 = fma(w, __ldg(Dr + s), a1);
                    a4 = fma(w, __ldg(Dp + s), a4);
                }
            }
        }
        v1 = a1;
        v4 = a4;
    } else {
        unsigned long long mx = 0;
        for (int s0 = 0; s0 <= r; s0 += kBatch) {
            unsigned long long b[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; u++) b[u] = s0 + u <= r ? split::abs_bits(__ldg(gl + (s0 + u) * step)) : 0ull;
#pragma unroll
            for (int u = 0; u < kBatch; u++)
                if (s0 + u <= smax) mx = max(mx, b[u]);
        }
        const int e = set_exponent(mx);
        const int sh = split::kTopBits + split::kBits * (S - 1) - (e == INT_MIN ? 0 : e);
        float acc1[S] = {}, acc4[S] = {};
        int run1[S] = {}, run4[S] = {};
        const float *Drd = sc.Dd + (size_t)r * n * S, *Dpd = sc.Dd + (size_t)p * n * S;
        for (int s0 = 0; s0 <= r; s0 += kBatch) {
            double v[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; u++) v[u] = s0 + u <= r ? __ldcs(gl + (s0 + u) * step) : 0.0;
#pragma unroll
            for (int u = 0; u < kBatch; u++) {
                const int s = s0 + u;
                if (s <= smax && on) {
                    float a[S], w[S];
                    digits_f32<S>(e == INT_MIN ? 0.0 : scale(v[u], s), sh, a);
                    load_digits<S>(Drd + s * S, w);
                    digit_fma<S>(a, w, acc1);
                    load_digits<S>(Dpd + s * S, w);
                    digit_fma<S>(a, w, acc4);
                }
            }
            if (((s0 + kBatch) % kFlush) == 0) { // every kFlush elements: exact FP32 group sums
                digit_flush<S>(acc1, run1);
                digit_flush<S>(acc4, run4);
            }
        }
        digit_flush<S>(acc1, run1);
        digit_flush<S>(acc4, run4);
        const int eDr = __ldg(sc.De + r), eDp = __ldg(sc.De + p);
        v1 = digit_value<S>(run1, (e == INT_MIN || eDr == INT_MIN) ? INT_MIN : e + eDr + kShift(S));
        v4 = digit_value<S>(run4, (e == INT_MIN || eDp == INT_MIN) ? INT_MIN : e + eDp + kShift(S));
    }
    if (on) {
        sc.S1[((size_t)p * n + r) * n + q] = v1;
        sc.S4[((size_t)q * n + p) * n + r] = v4;
    }
}

// T2, T5 and T3.  Unit p, lane (r, s): sums over q <= p (q >= s when p == r) of
// f g[p,q,r,s] {D[p,q], D[q,r], D[q,s]} -- consecutive lanes read consecutive s;
// batches of kBatch loads as in the rows pass.  Each lane's T3 sum over q is
// added over s by the reduction.
template <int S>
__global__ void __launch_bounds__(kWarps * 32) k_fock_cols(const double *__restrict__ g,
                                                           const double *__restrict__ D, int n, FockScratch sc) {
    int p, first;
    unit_of_cta(blockIdx.x, n, [&](int u) { return cols_pairs(u); }, p, first);
    if (p < 0) return;
    const int f = first + threadIdx.x;
    const bool on = f < cols_pairs(p);
    int r = tri_row(2ll * (on ? f : 0));
    if (r > p) r = p;
    const int s = on ? f - r * (r + 1) / 2 : 0;
    const bool diag = p == r;
    const int qmin = diag ? s : 0; // this lane's first q
    const size_t step = (size_t)n * n; // q -> q + 1 in g[p][q][r][s]
    const double *gl = g + (((size_t)p * n) * n + r) * n + s;
    const double *Dp = D + (size_t)p * n;
    auto scale = [&](double v, int q) {
        if (q == p) v = half_exact(v);
        if (s == r) v = half_exact(v);
        if (diag && s == q) v = half_exact(v);
        return v;
    };
    double a3 = 0.0, v2 = 0.0, v5 = 0.0;
    if constexpr (S == 0) {
        double a2 = 0.0, a5 = 0.0;
        for (int q0 = 0; q0 <= p; q0 += kBatch) {
            double v[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; u++) v[u] = q0 + u <= p ? __ldcs(gl + (q0 + u) * step) : 0.0;
#pragma unroll
            for (int u = 0; u < kBatch; u++) {
                const int q = q0 + u;
                if (q <= p && q >= qmin && on) {
                    const double w = scale(v[u], q);
                    a2 = fma(w, __ldg(Dp + q), a2);
                    a5 = fma(w, __ldg(D + (size_t)q * n + r), a5);
                    a3 = fma(w, __ldg(D + (size_t)q * n + s), a3);
                }
            }
        }
        v2 = a2;
        v5 = a5;
    } else {
        unsigned long long mx = 0;
        for (int q0 = 0; q0 <= p; q0 += kBatch) {
            unsigned long long b[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; u++) b[u] = q0 + u <= p ? split::abs_bits(__ldg(gl + (q0 + u) * step)) : 0ull;
#pragma unroll
            for (int u = 0; u < kBatch; u++)
                if (q0 + u >= qmin) mx = max(mx, b[u]);
        }
        const int e = set_exponent(mx);
        const int sh = split::kTopBits + split::kBits * (S - 1) - (e == INT_MIN ? 0 : e);
        float acc2[S] = {}, acc5[S] = {};
        int run2[S] = {}, run5[S] = {};
        const float *Dpd = sc.Dd + (size_t)p * n * S, *Drd = sc.Dd + (size_t)r * n * S;
        for (int q0 = 0; q0 <= p; q0 += kBatch) {
            double v[kBatch];
#pragma unroll
            for (int u = 0; u < kBatch; u++) v[u] = q0 + u <= p ? __ldcs(gl + (q0 + u) * step) : 0.0;
#pragma unroll
            for (int u = 0; u < kBatch; u++) {
                const int q = q0 + u;
                if (q <= p && q >= qmin && on) {
                    const double w = scale(v[u], q);
                    float a[S], b[S];
                    digits_f32<S>(e == INT_MIN ? 0.0 : w, sh, a);
                    load_digits<S>(Dpd + q * S, b);
                    digit_fma<S>(a, b, acc2);
                    load_digits<S>(Drd + q * S, b);
                    digit_fma<S>(a, b, acc5);
                    a3 = fma(w, __ldg(D + (size_t)q * n + s), a3);
                }
            }
            if (((q0 + kBatch) % kFlush) == 0) {
                digit_flush<S>(acc2, run2);
                digit_flush<S>(acc5, run5);
            }
        }
        digit_flush<S>(acc2, run2);
        digit_flush<S>(acc5, run5);
        const int eDp = __ldg(sc.De + p), eDr = __ldg(sc.De + r);
        v2 = digit_value<S>(run2, (e == INT_MIN || eDp == INT_MIN) ? INT_MIN : e + eDp + kShift(S));
        v5 = digit_value<S>(run5, (e == INT_MIN || eDr == INT_MIN) ? INT_MIN : e + eDr + kShift(S));
    }
    if (on) {
        sc.S2[((size_t)r * n + p) * n + s] = v2;
        sc.S5[((size_t)p * n + r) * n + s] = v5;
        sc.X3[((size_t)p * n + r) * n + s] = a3;
    }
}

// T6: XK[q,s] = sum over canonical (p, r) -- p >= q, s <= r <= p, without r = p
// when q < s -- of f g[q,p,r,s] D[p,r].  Warp (q, 32 s, p), lane = s: the sum
// over r for one p, so that every warp has at most n terms (the sums over p
// would leave a few long warps running alone); the reduction adds over p.
__global__ void __launch_bounds__(kWarps * 32) k_fock_exchange(const double *__restrict__ g,
                                                               const double *__restrict__ D, int n, int nsc,
                                                               double *__restrict__ X6) {
    const int q = blockIdx.x / nsc, s0 = (blockIdx.x - q * nsc) * 32;
    const int p = blockIdx.y * kWarps + (threadIdx.x >> 5);
    const int s = s0 + (threadIdx.x & 31);
    if (p >= n || p < q || p < s0) return; // whole warps leave together
    const int sl = s < n ? s : n - 1;
    const int rend = s >= n ? -1 : (q < s ? p - 1 : p); // this lane's canonical r in [s, rend]
    const double *gl = g + (((size_t)q * n + p) * n) * n + sl;
    const double *Dp = D + (size_t)p * n;
    double acc = 0.0;
    // the warp walks r over [s0, p] in batches of kBatch loads
    for (int r0 = s0; r0 <= p; r0 += kBatch) {
        double v[kBatch];
#pragma unroll
        for (int u = 0; u < kBatch; u++) v[u] = r0 + u <= p ? __ldcs(gl + (size_t)(r0 + u) * n) : 0.0;
#pragma unroll
        for (int u = 0; u < kBatch; u++) {
            const int r = r0 + u;
            if (r >= s && r <= rend) {
                double w = v[u];
                if (p == q) w = half_exact(w);
                if (r == s) w = half_exact(w);
                if (p == r && q == s) w = half_exact(w);
                acc = fma(w, __ldg(Dp + r), acc);
            }
        }
    }
    if (s < n) X6[((size_t)q * n + p) * n + s] = acc;
}

// Row i, columns j of one chunk of 32, of YJ (j <= i) and XK from the partials.
// Lanes run over j (every read is contiguous); warp w takes the terms t = w,
// w + 8, ... of each sum over p or r, and the eight warps' sums are added in
// warp order.
__global__ void __launch_bounds__(kRedWarps * 32) k_fock_reduce(int n, FockScratch sc) {
    __shared__ double sr[2][kRedWarps][32];
    const int i = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j = blockIdx.y * 32 + lane;
    if (j < n) {
        double xk = 0.0, yj = 0.0;
        if (warp == 0) {

        }
        for (int t = warp; t < n; t += kRedWarps) {
            if (t >= max(i, j)) xk += sc.S4[((size_t)i * n + t) * n + j]; // T4 of (p = t, r = j), q = i
            if (t >= max(i, j & ~31)) xk += sc.X6[((size_t)i * n + t) * n + j]; // T6 of (q = i, p = t), s = j
            if (i >= j && t <= j) xk += sc.X3[((size_t)i * n + j) * n + t];      // T3 of (p = i, r = j), s = t
            if (i >= j) {
                if (t >= j && t <= i) xk += sc.S5[((size_t)i * n + t) * n + j]; // T5 of (p = i, r = t), s = j
                if (t <= i) yj += sc.S1[((size_t)i * n + t) * n + j];           // T1 of (p = i, r = t), q = j
                if (t >= i) yj += sc.S2[((size_t)i * n + t) * n + j];           // T2 of (p = t, r = i), s = j
            }
        }
        sr[0][warp][lane] = xk;
        sr[1][warp][lane] = yj;
    }
    __syncthreads();
    if (warp == 0 && j < n) {
        double xk = 0.0, yj = 0.0;
        for (int w = 0; w < kRedWarps; w++) {
            xk += sr[0][w][lane];
            yj += sr[1][w][lane];
        }
        sc.XK[(size_t)i * n + j] = xk;
        if (i >= j) sc.YJ[(size_t)i * n + j] = yj;
    }
}

// F = fp F + jp J + kp K with J = 2 (YJ + YJ^T) and K = XK + XK^T.
__global__ void __launch_bounds__(128) k_fock_combine(double *F, int n, FockScratch sc, double fp, double jp,
                                                      double kp, int zero_f) {
    const int i = blockIdx.x;
    for (int j = threadIdx.x; j < n; j += 128) {
        const double yj = sc.YJ[(size_t)max(i, j) * n + min(i, j)];
        const double J = (i == j ? 4.0 : 2.0) * yj;
        const double K = sc.XK[(size_t)i * n + j] + sc.XK[(size_t)j * n + i];
        double *f = F + (size_t)i * n + j;
        const double add = jp * J + kp * K;
        *f = zero_f ? add : fma(fp, *f, add);
    }
}

template <int S>
eg_status launch_lines(const double *g, const double *D, int n, const FockScratch &sc, cudaStream_t s) {
    unsigned rows_ctas = 0, cols_ctas = 0;
    for (int u = 0; u < n; u++) {
        rows_ctas += (unsigned)(((n * (n + 1) - u * (u + 1)) / 2 + kWarps * 32 - 1) / (kWarps * 32));
        cols_ctas += (unsigned)(((u + 1) * (u + 2) / 2 + kWarps * 32 - 1) / (kWarps * 32));
    }
    if constexpr (S > 0) {
        {
            LaunchScope ls_("k_fock_digits_d", s);
            k_fock_digits_d<S><<<n, 128, 0, s>>>(D, n, (float *)sc.Dd, (int *)sc.De);
        }
        EG_CHECK_LAUNCH("k_fock_digits_d");
    }
    {
        LaunchScope ls_("k_fock_rows", s);
        k_fock_rows<S><<<rows_ctas, kWarps * 32, 0, s>>>(g, D, n, sc);
    }
    EG_CHECK_LAUNCH("k_fock_rows");
    {
        LaunchScope ls_("k_fock_cols", s);
        k_fock_cols<S><<<cols_ctas, kWarps * 32, 0, s>>>(g, D, n, sc);
    }
    EG_CHECK_LAUNCH("k_fock_cols");
    return EG_SUCCESS;
}

} // namespace

} // namespace eg

extern "C" eg_status eg_fock_jk_symmetric(double F_prefactor, double *F, double J_prefactor, double K_prefactor,
                                          const double *g, const double *D, int64_t n, const eg_options *opt,
                                          void *stream) {
    using namespace eg;
    set_error("");
    eg_options o;
    eg_options_default(&o);
    if (opt) o = *opt;
    if (o.precision != EG_PRECISION_FP64 && o.precision != EG_PRECISION_SPLIT_BF16)
        return fail(EG_ERROR_INVALID_ARGUMENT, "eg_fock_jk_symmetric: unknown precision");
    const int S = o.precision == EG_PRECISION_SPLIT_BF16 ? (o.slices ? o.slices : 5) : 0;
    if (S != 0 && (S < 3 || S > 6))
        return fail(EG_ERROR_INVALID_ARGUMENT, "eg_fock_jk_symmetric: slices must be in 3..6");
    if (n < 0) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_fock_jk_symmetric: negative n");
    if (n == 0) return EG_SUCCESS;
    if (!F || !g || !D) return fail(EG_ERROR_INVALID_ARGUMENT, "eg_fock_jk_symmetric: NULL pointer");
    if (n > kFockMaxN)
        return fail(EG_ERROR_NOT_SUPPORTED, "eg_fock_jk_symmetric: n = " + std::to_string(n) +
                                                " exceeds the largest supported (" + std::to_string(kFockMaxN) + ")");
    const int nn = (int)n;
    const int nsc = (nn + 31) / 32;
    const size_t n3 = (size_t)nn * nn * nn, n2 = (size_t)nn * nn;
    const size_t elems = 6 * n3 + 2 * n2;
    const size_t dd_bytes = S ? (n2 * S * sizeof(float) + (size_t)nn * sizeof(int) + 256) : 0;
    cudaStream_t s = (cudaStream_t)stream;
    void *ws = nullptr;
    eg_status st = workspace(s, elems * sizeof(double) + dd_bytes, &ws);
    if (st != EG_SUCCESS) return st;
    FockScratch sc;
    sc.S1 = (double *)ws;
    sc.S4 = sc.S1 + n3;
    sc.S2 = sc.S4 + n3;
    sc.S5 = sc.S2 + n3;
    sc.X3 = sc.S5 + n3;
    sc.X6 = sc.X3 + n3;
    sc.YJ = sc.X6 + n3;
    sc.XK = sc.YJ + n2;
    sc.Dd = S ? (const float *)(sc.XK + n2) : nullptr;
    sc.De = S ? (const int *)(sc.Dd + n2 * S) : nullptr;
    sc.nsc = nsc;
    switch (S) {
    case 0: st = launch_lines<0>(g, D, nn, sc, s); break;
    case 3: st = launch_lines<3>(g, D, nn, sc, s); break;
    case 4: st = launch_lines<4>(g, D, nn, sc, s); break;
    case 5: st = launch_lines<5>(g, D, nn, sc, s); break;
    default: st = launch_lines<6>(g, D, nn, sc, s); break;
    }
    if (st != EG_SUCCESS) return st;
    {
        LaunchScope ls_("k_fock_exchange", s);
        k_fock_exchange<<<dim3((unsigned)(nn * nsc), (unsigned)((nn + kWarps - 1) / kWarps)), kWarps * 32, 0, s>>>(
            g, D, nn, nsc, sc.X6);
    }
    EG_CHECK_LAUNCH("k_fock_exchange");
    {
        LaunchScope ls_("k_fock_reduce", s);
        k_fock_reduce<<<dim3((unsigned)nn, (unsigned)nsc), kRedWarps * 32, 0, s>>>(nn, sc);
    }
    EG_CHECK_LAUNCH("k_fock_reduce");
    {
        LaunchScope ls_("k_fock_combine", s);
        k_fock_combine<<<(unsigned)nn, 128, 0, s>>>(F, nn, sc, F_prefactor, J_prefactor, K_prefactor,
                                                   F_prefactor == 0.0 ? 1 : 0);
    }
    EG_CHECK_LAUNCH("k_fock_combine");
    if (S) set_split_report(eg_split_report{S, S * (S + 1) / 2, split::kBits, split::error_bound(S)});
    return EG_SUCCESS;
}
