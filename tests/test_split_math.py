"""CPU check of the split-BF16 arithmetic used by the GPU kernels: row
exponents, balanced base-256 digits (each exact in BF16), triangular
truncation of the digit products, and exact integer accumulation.  A numpy
restatement of einsums_gb300/csrc/split.cuh:to_digits and the epilogue's
R = sum_d 2^(8(S-1-d)) G_d; checks the reconstruction and the stated error
bound, and the FP32-exactness limits the kernel relies on.  A bit-level
restatement of the device's scaled_round / digits_bf16x2 (one add-and-shift
rounding, bias, byte permute, FP32 add) is checked against the definition."""
import math

import numpy as np
import pytest

BITS, TOP = 8, 7


def exponents(X):
    mx = np.max(np.abs(X), axis=1)
    e = np.zeros(len(mx), dtype=np.int64)
    nz = mx > 0
    _, e[nz] = np.frexp(mx[nz])
    return e


def digits(X, e, S):
    """Balanced base-256 digits, leading digit first, like to_digits()."""
    y = np.ldexp(X, (TOP + BITS * (S - 1) - e)[:, None])
    F = np.rint(y).astype(np.int64)
    out = np.zeros((S,) + X.shape, dtype=np.int64)
    for s in range(S - 1, 0, -1):
        d = F & 255
        d = np.where(d > 128, d - 256, d)
        out[s] = d
        F = (F - d) // 256
    out[0] = F
    return out


def split_product(A, B, S):
    """A (M x K) times B^T (N x K) by the split scheme, with exact integers."""
    eA, eB = exponents(A), exponents(B)
    a, b = digits(A, eA, S), digits(B, eB, S)
    R = np.zeros((A.shape[0], B.shape[0]), dtype=object)
    for d in range(S):
        G = sum(a[s].astype(object) @ b[d - s].T.astype(object) for s in range(d + 1))
        R = R * 256 + G
    shift = eA[:, None] + eB[None, :] - 2 * TOP - BITS * (S - 1)
    out = np.empty(R.shape)
    for i in range(R.shape[0]):
        for j in range(R.shape[1]):
            out[i, j] = math.ldexp(float(R[i, j]), int(shift[i, j]))
    return out


def split_product_fast(A, B, S):
    """split_product with the digit products summed in FP64 (exact while
    K * 2^14 < 2^53) and the Horner combination in int64 (|R| < 2^62 for one
    exact pass of K)."""
    assert A.shape[1] * 2 ** 14 < 2 ** 53
    eA, eB = exponents(A), exponents(B)
    a, b = digits(A, eA, S), digits(B, eB, S)
    R = np.zeros((A.shape[0], B.shape[0]), dtype=np.int64)
    for d in range(S):
        G = sum(a[s].astype(np.float64) @ b[d - s].T.astype(np.float64) for s in range(d + 1))
        R = R * 256 + G.astype(np.int64)
    shift = eA[:, None] + eB[None, :] - 2 * TOP - BITS * (S - 1)
    return np.ldexp(R.astype(np.float64), shift.astype(np.int64))


def max_k_per_pass_groups(d0, d1, kstep=128):
    """Restates split.cuh max_k_per_pass_groups: the largest K (a multiple of 128)
    for which sum_{d0 <= d < d1} 2^(8 (d1-1-d)) G_d stays below 2^62, |G_d| <= (d+1) K 2^14."""
    w = sum((d + 1) * 2.0 ** (8 * (d1 - 1 - d)) for d in range(d0, d1))
    k = int(2.0 ** 62 / (2.0 ** 14 * w))
    return k // kstep * kstep


def slice_group_ranges(S, Kp):
    """Restates the launch plan of split.cu: greedy ranges of slice groups whose exact
    sums fit int64 over the whole (padded) K."""
    ranges, d0 = [], 0
    while d0 < S:
        d1 = d0 + 1
        while d1 < S and max_k_per_pass_groups(d0, d1 + 1) >= Kp:
            d1 += 1
        ranges.append((d0, d1))
        d0 = d1
    return ranges


def split_product_ranges(A, B, S):
    """The split product as the GPU forms it when K needs several slice-group
    ranges: each range's exact int64 sum rounded to FP64 on its own, the ranges
    added in FP64 in order (the first stores, the others add)."""
    K = A.shape[1]
    assert K * 2 ** 14 < 2 ** 53
    Kp = -(-K // 128) * 128
    eA, eB = exponents(A), exponents(B)
    a, b = digits(A, eA, S), digits(B, eB, S)
    shift = (eA[:, None] + eB[None, :] - 2 * TOP - BITS * (S - 1)).astype(np.int64)
    out = None
    for d0, d1 in slice_group_ranges(S, Kp):
        assert max_k_per_pass_groups(d0, d1) >= Kp
        R = np.zeros((A.shape[0], B.shape[0]), dtype=np.int64)
        for d in range(d0, d1):
            G = sum(a[s].astype(np.float64) @ b[d - s].T.astype(np.float64) for s in range(d + 1))
            R = R * 256 + G.astype(np.int64)
        v = np.ldexp(R.astype(np.float64), shift + BITS * (S - d1))
        out = v if out is None else out + v
    return out


def test_slice_group_ranges():
    assert max_k_per_pass_groups(0, 5) == 65024
    assert slice_group_ranges(5, 1024) == [(0, 5)]
    assert slice_group_ranges(5, 65024) == [(0, 5)]
    assert slice_group_ranges(5, 65152) == [(0, 4), (4, 5)]
    assert max_k_per_pass_groups(0, 6) == 128
    assert slice_group_ranges(6, 128) == [(0, 6)]
    assert slice_group_ranges(6, 16384) == [(0, 5), (5, 6)]
    assert slice_group_ranges(3, 1 << 20) == [(0, 3)]
    rng = np.random.default_rng(8)
    A, B = rng.standard_normal((7, 300)), rng.standard_normal((5, 300))
    # one range: the same numbers as the single exact sum
    assert np.array_equal(split_product_ranges(A, B, 5).view(np.uint64), split_product_fast(A, B, 5).view(np.uint64))
    # two ranges for S = 6 and K = 300: within one FP64 rounding of the exact sum
    two = split_product_ranges(A, B, 6)
    assert slice_group_ranges(6, 384) == [(0, 5), (5, 6)]
    assert np.allclose(two, split_product_fast(A, B, 6), rtol=4e-16, atol=0)


def test_fast_split_product_matches_exact_integers():
    rng = np.random.default_rng(4)
    A = rng.standard_normal((9, 150)) * np.exp2(rng.integers(-30, 30, size=(9, 1)))
    B = rng.standard_normal((7, 150))
    A[2] = 0.0
    for S in (3, 5, 6):
        assert np.array_equal(split_product(A, B, S).view(np.uint64), split_product_fast(A, B, S).view(np.uint64))


@pytest.mark.parametrize("S", [2, 3, 4, 5, 6])
def test_digits_are_bf16_exact_and_reconstruct(S):
    rng = np.random.default_rng(S)
    X = rng.standard_normal((16, 40)) * np.exp(rng.uniform(-20, 20, size=(16, 1)))
    X[3] = 0.0
    e = exponents(X)
    D = digits(X, e, S)
    assert np.all(np.abs(D) <= 128)  # integers of magnitude <= 2^7: exact in BF16 (8 significant bits)
    rec = sum(np.ldexp(D[s].astype(float), (e - TOP - BITS * s)[:, None]) for s in range(S))
    # residual below half a unit of the last digit, relative to the row's 2^e
    err = np.abs(rec - X) / np.ldexp(1.0, e)[:, None]
    assert np.all(err <= 0.5 * 2.0 ** -(TOP + BITS * (S - 1)) + 1e-300)


@pytest.mark.parametrize("S", [3, 4, 5, 6])
def test_split_product_error_bound(S):
    rng = np.random.default_rng(10 + S)
    A = rng.standard_normal((12, 200))
    B = rng.standard_normal((9, 200))
    ref = A @ B.T
    got = split_product(A, B, S)
    scale = np.ldexp(1.0, exponents(A))[:, None] * np.ldexp(1.0, exponents(B))[None, :] * A.shape[1]
    bound = (S + 2) * 2.0 ** -(TOP + BITS * (S - 1))
    assert np.all(np.abs(got - ref) <= bound * scale)
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    if S >= 5:
        assert rel < 1e-10


def test_chunk_sums_stay_fp32_exact():
    """1024 products of digits bounded by 128 stay within 2^24: the FP32
    accumulators of one chunk hold exact integers."""
    assert 1024 * 128 * 128 <= 2 ** 24


def test_int64_accumulator_limit():
    """R = sum_d 2^(8(S-1-d)) G_d stays below 2^62 for the per-pass K limit."""
    for S in range(2, 7):
        w = sum((d + 1) * 2.0 ** (8 * (S - 1 - d)) for d in range(S))
        kmax = int(2 ** 62 / (2 ** 14 * w)) // 64 * 64
        assert kmax * 2 ** 14 * w <= 2 ** 62
        assert kmax >= 64


# ---- bit-level restatement of the device digit arithmetic (split.cuh) ------
def _scaled_round_dev(x, sh):
    """scaled_round: round(x 2^sh) half to even in one add-and-shift on the IEEE fields."""
    import struct
    bits = struct.unpack("<Q", struct.pack("<d", x))[0]
    ex = (bits >> 52) & 0x7FF
    mant = (bits & 0xFFFFFFFFFFFFF) | ((1 if ex else 0) << 52)
    r = 1075 - (ex if ex else 1) - sh
    if r <= 0:
        q = (mant << min(-r, 11)) & (2 ** 64 - 1)
    elif r > 62:
        q = 0
    else:
        q = ((mant + ((1 << (r - 1)) - 1) + ((mant >> r) & 1)) & (2 ** 64 - 1)) >> r
    return -q if bits >> 63 else q


def _byte_perm(x, y, s):
    b = [(x >> (8 * i)) & 255 for i in range(4)] + [(y >> (8 * i)) & 255 for i in range(4)]
    return sum(b[(s >> (4 * i)) & 7] << (8 * i) for i in range(4))


def _f32(u):
    import struct
    return np.float32(struct.unpack("<f", struct.pack("<I", u & 0xFFFFFFFF))[0])


def _digits_dev(x, e, S):
    """digits_bf16x2 for one value: bias, byte permute to 2^23 + u, one FP32 add per digit."""
    bias = 0
    for _ in range(1, S):
        bias = bias * 256 + 127
    G = _scaled_round_dev(x, TOP + BITS * (S - 1) - e) + bias
    Gu = G & (2 ** 64 - 1)
    words = [Gu & 0xFFFFFFFF, Gu >> 32]
    out = [0] * S
    for s in range(1, S):
        byte = S - 1 - s
        f = _f32(_byte_perm(words[byte >> 2], 0x4B000000, 0x7440 | (byte & 3))) - np.float32(8388735.0)
        assert float(f).is_integer()
        out[s] = int(f)
    f0 = _f32(0x4B400000 + (G >> (8 * (S - 1)))) - np.float32(12582912.0)
    out[0] = int(f0)
    return out


@pytest.mark.parametrize("S", [2, 3, 4, 5, 6])
def test_device_digit_arithmetic_matches_the_definition(S):
    rng = np.random.default_rng(40 + S)
    X = rng.standard_normal((12, 24)) * np.exp2(rng.integers(-30, 30, size=(12, 1)))
    X[0, :5] = [0.0, -0.0, 5e-324, -1e-310, 1.0]
    X[1, :] = np.ldexp(np.round(rng.standard_normal(24) * 2 ** 20) + 0.5, -20)  # exact ties
    e = exponents(X)
    D = digits(X, e, S)
    for i in range(X.shape[0]):
        sh = TOP + BITS * (S - 1) - int(e[i])
        for j in range(X.shape[1]):
            assert _scaled_round_dev(float(X[i, j]), sh) == int(np.rint(np.ldexp(X[i, j], sh)))
            assert _digits_dev(float(X[i, j]), int(e[i]), S) == [int(D[s, i, j]) for s in range(S)]


def _int_times_pow2_rn_dev(R, e):
    """int_times_pow2_rn of split.cuh (the tensor kernel's epilogue): R * 2^e rounded to nearest
    even, built on the IEEE fields (leading-zero count, 53-bit mantissa with
    half-even rounding of the 11 dropped bits); None where the kernel leaves the
    result to its FP64 fallback (exponent out of the normal range)."""
    if R == 0:
        return 0.0
    a = -R if R < 0 else R
    lz = 64 - a.bit_length()
    x = (a << lz) & (2 ** 64 - 1)
    mant, rem = x >> 11, x & 0x7FF
    if rem > 0x400 or (rem == 0x400 and (mant & 1)):
        mant += 1
    exp = 63 - lz + e
    if mant >> 53:
        mant >>= 1
        exp += 1
    biased = exp + 1023
    if biased <= 0 or biased >= 2047:
        return None
    import struct
    bits = ((1 << 63) if R < 0 else 0) | (biased << 52) | (mant & 0xFFFFFFFFFFFFF)
    return struct.unpack("<d", struct.pack("<Q", bits))[0]


def test_epilogue_int64_to_double_rounds_half_even():
    rng = np.random.default_rng(77)
    cases = [1, -1, 2 ** 53 - 1, 2 ** 53, 2 ** 53 + 1, 2 ** 53 + 3, -(2 ** 54 + 2), 2 ** 62 + 2 ** 9,
             2 ** 62 + 2 ** 10, 2 ** 62 + 3 * 2 ** 9, 2 ** 63 - 1, -(2 ** 63 - 1), (2 ** 53 - 1) << 10]
    cases += [int(v) for v in rng.integers(-2 ** 62, 2 ** 62, size=400)]
    cases += [int(v) << int(s) for v, s in zip(rng.integers(-2 ** 20, 2 ** 20, size=100), rng.integers(0, 40, size=100))]
    for R in cases:
        for e in (-1074 + 64, -200, -46, 0, 17, 900):
            got = _int_times_pow2_rn_dev(R, e)
            if got is None:
                continue  # out of the normal range: the kernel's FP64 fallback handles it
            assert got == math.ldexp(float(R), e), (R, e)  # float(int) rounds half to even
