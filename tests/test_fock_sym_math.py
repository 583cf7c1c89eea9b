"""CPU restatement of the symmetric Fock build's decomposition (the device
kernels of einsums_gb300/csrc/fock.cu), checked without a GPU against the two
general contractions it replaces:

    J[p,q] = sum_rs g[p,q,r,s] D[r,s]        (einsum pq <- pqrs, rs)
    K[p,q] = sum_rs g[p,r,q,s] D[r,s]        (einsum pq <- prqs, rs)

for g with 8-fold permutational symmetry and symmetric D.  Only the canonical
quartets (p >= q, r >= s, pair(p,q) >= pair(r,s)) are read.  Each canonical
element g, scaled by its degeneracy f = 1/2 for each of p == q, r == s and
pair(p,q) == pair(r,s), makes six contributions to two non-symmetric
accumulators YJ and XK (J = 2 (YJ + YJ^T), K = XK + XK^T):

    T1  YJ[p,q] += f g D[r,s]        rows pass: per (p, r, q), sum over s
    T2  YJ[r,s] += f g D[p,q]        columns pass: per (p, r, s), sum over q
    T3  XK[p,r] += f g D[q,s]        columns pass: per (p, r), sum over (q, s)
    T4  XK[q,r] += f g D[p,s]        rows pass
    T5  XK[p,s] += f g D[q,r]        columns pass
    T6  XK[q,s] += f g D[p,r]        exchange pass: per (q, s), sum over (p, r)

The rows pass reads g[r,s,p,q] (= g[p,q,r,s]) and the exchange pass g[q,p,r,s]
(= g[p,q,r,s]), so that each line's lanes read consecutive addresses; the
per-line results go to scratch and a reduction adds them in a fixed order.
"""
import numpy as np
import pytest


def sym_inputs(n, seed):
    r = np.random.default_rng(seed)
    g = r.uniform(-1.0, 1.0, size=(n, n, n, n))
    g = g + g.transpose(1, 0, 2, 3)
    g = g + g.transpose(0, 1, 3, 2)
    g = g + g.transpose(2, 3, 0, 1)
    C = r.standard_normal((n, 3))
    return g, C @ C.T


def fock_jk_restated(g, D):
    n = g.shape[0]
    S1 = np.zeros((n, n, n))  # [p][r][q]
    S4 = np.zeros((n, n, n))  # [q][p][r]
    S2 = np.zeros((n, n, n))  # [r][p][s]
    S5 = np.zeros((n, n, n))  # [p][r][s]
    X3 = np.zeros((n, n))     # [p][r]
    X6 = np.zeros((n, n))     # [q][s]

    def f(p, q, r, s):
        return (0.5 if p == q else 1.0) * (0.5 if r == s else 1.0) * (0.5 if (p == r and q == s) else 1.0)

    for p in range(n):
        for r in range(p + 1):
            for q in range(p + 1):  # rows pass: line (p, r, q) over s, read as g[r,s,p,q]
                for s in range(r + 1 if p > r else q + 1):
                    v = f(p, q, r, s) * g[r, s, p, q]
                    S1[p, r, q] += v * D[r, s]
                    S4[q, p, r] += v * D[p, s]
            for s in range(r + 1):  # columns pass: line (p, r, s) over q
                for q in range(s if p == r else 0, p + 1):
                    v = f(p, q, r, s) * g[p, q, r, s]
                    S2[r, p, s] += v * D[p, q]
                    S5[p, r, s] += v * D[q, r]
                    X3[p, r] += v * D[q, s]
    for q in range(n):  # exchange pass: (q, s) over p >= q, s <= r <= p (r < p when q < s), read as g[q,p,r,s]
        for s in range(n):
            for p in range(max(q, s), n):
                for r in range(s, (p - 1 if q < s else p) + 1):
                    X6[q, s] += f(p, q, r, s) * g[q, p, r, s] * D[p, r]
    YJ = np.zeros((n, n))
    XK = X6.copy()
    for i in range(n):
        for j in range(n):
            XK[i, j] += sum(S4[i, p, j] for p in range(max(i, j), n))
            if i >= j:
                XK[i, j] += X3[i, j] + sum(S5[i, r, j] for r in range(j, i + 1))
                YJ[i, j] = sum(S1[i, r, j] for r in range(i + 1)) + sum(S2[i, p, j] for p in range(i, n))
    return 2.0 * (YJ + YJ.T), XK + XK.T


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (5, 2), (9, 3)])
def test_restated_symmetric_fock_matches_the_two_contractions(n, seed):
    g, D = sym_inputs(n, seed)
    J, K = fock_jk_restated(g, D)
    J_ref = np.einsum("pqrs,rs->pq", g, D)
    K_ref = np.einsum("prqs,rs->pq", g, D)
    assert np.allclose(J, J_ref, rtol=1e-13, atol=1e-13 * np.abs(J_ref).max())
    assert np.allclose(K, K_ref, rtol=1e-13, atol=1e-13 * np.abs(K_ref).max())


def _half_exact(x):
    """half_exact of fock.cu: x / 2 with integer operations on the IEEE fields."""
    import struct
    b = struct.unpack("<Q", struct.pack("<d", x))[0]
    ex = (b >> 52) & 0x7FF
    if 1 < ex < 0x7FF:
        b -= 1 << 52
    elif ex != 0x7FF:
        m = (b & 0xFFFFFFFFFFFFF) | (ex << 52)
        h = (m >> 1) + (m & (m >> 1) & 1)
        b = (b & 0x8000000000000000) | h
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def test_half_exact_matches_the_rounded_half():
    import struct
    rng = np.random.default_rng(7)
    bits = rng.integers(0, 2 ** 63, size=20000, dtype=np.uint64) * 2 + rng.integers(0, 2, size=20000, dtype=np.uint64)
    bits[::3] &= np.uint64(0x801FFFFFFFFFFFFF)  # exponents near zero: subnormal results and their edge
    xs = [struct.unpack("<d", struct.pack("<Q", int(b)))[0] for b in bits]
    xs += [0.0, -0.0, 5e-324, -5e-324, 2.2250738585072014e-308, 2.225073858507201e-308, 1.0, float("inf")]
    for x in xs:
        if np.isnan(x):
            continue
        assert struct.pack("<d", _half_exact(x)) == struct.pack("<d", x * 0.5), x


def _tri_row(K):
    x = int((np.sqrt(np.float32(4.0 * K + 1.0)) - 1.0) * 0.5)
    while (x + 1) * (x + 2) <= K:
        x += 1
    while x > 0 and x * (x + 1) > K:
        x -= 1
    return x


@pytest.mark.parametrize("n", [1, 2, 5, 33, 70])
def test_flattened_lanes_cover_every_pair_once(n):
    """The lane mapping of fock.cu's rows and columns passes: CTAs of 128 pairs,
    units with more pairs first; every (p, q) of a rows unit r and every (r, s) of a
    columns unit p is taken by exactly one lane."""
    per_cta = 128
    rows_pairs = lambda r: (n * (n + 1) - r * (r + 1)) // 2
    cols_pairs = lambda p: (p + 1) * (p + 2) // 2
    for count, kind in ((rows_pairs, "rows"), (cols_pairs, "cols")):
        seen = set()
        ctas = sum((count(u) + per_cta - 1) // per_cta for u in range(n))
        for x in range(ctas):
            k, xx = 0, x
            for k in range(n):
                u = n - 1 - k
                c = (count(u) + per_cta - 1) // per_cta
                if xx < c:
                    break
                xx -= c
            first = xx * per_cta
            for t in range(per_cta):
                f = first + t
                if f >= count(u):
                    continue
                if kind == "rows":
                    r = u
                    p = min(max(_tri_row(2 * f + r * (r + 1)), r), n - 1)
                    q = f - (p * (p + 1) - r * (r + 1)) // 2
                    assert r <= p < n and 0 <= q <= p
                    seen.add((r, p, q))
                else:
                    p = u
                    r = min(_tri_row(2 * f), p)
                    s = f - r * (r + 1) // 2
                    assert 0 <= s <= r <= p
                    seen.add((p, r, s))
        want = (sum(rows_pairs(r) for r in range(n)) if kind == "rows" else sum(cols_pairs(p) for p in range(n)))
        assert len(seen) == want
