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

    T1  YJ[p,q] += f g D[r,s]        row sums of a (p, r) block over s
    T2  YJ[r,s] += f g D[p,q]        column sums over q
    T3  XK[p,r] += f g D[q,s]        the block's weighted total
    T4  XK[q,r] += f g D[p,s]        row sums over s
    T5  XK[p,s] += f g D[q,r]        column sums over q
    T6  XK[q,s] += f g D[p,r]        the weighted total of a (q, s) block

T1-T5 come from "pair blocks" B[q, s] = g[p, q, r, s] (p >= r; q <= p; s <= r,
and s <= q when p == r); T6 from "exchange blocks" over (p, r) for fixed
(q, s), read through g[p,q,r,s] = g[q,p,s,r].  The per-block vectors go to
scratch and are summed in a fixed order by a final pass.
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
    S1 = np.zeros((n, n, n))  # [p][r][q]  T1
    S2 = np.zeros((n, n, n))  # [r][p][s]  T2
    S4 = np.zeros((n, n, n))  # [r][p][q]  T4
    S5 = np.zeros((n, n, n))  # [p][r][s]  T5
    X3 = np.zeros((n, n))     # [p][r]     T3 (p >= r)
    X6 = np.zeros((n, n))     # [q][s]     T6
    for p in range(n):
        for r in range(p + 1):
            B = np.zeros((p + 1, r + 1))
            for q in range(p + 1):
                smax = r if p > r else q
                B[q, :smax + 1] = g[p, q, r, :smax + 1]
            B = B.copy()
            B[p, :] *= 0.5                 # p == q
            B[:, r] *= 0.5                 # r == s
            if p == r:
                B[np.arange(p + 1), np.arange(p + 1)] *= 0.5   # pair(p,q) == pair(r,s)
            S1[p, r, :p + 1] = B @ D[r, :r + 1]
            S4[r, p, :p + 1] = B @ D[p, :r + 1]
            S2[r, p, :r + 1] = D[p, :p + 1] @ B
            S5[p, r, :r + 1] = D[:p + 1, r] @ B
            X3[p, r] = np.sum(B * D[:p + 1, :r + 1])
    for q in range(n):
        for s in range(n):
            acc = 0.0
            for p in range(q, n):
                for rr in range(s, n):
                    if not (p > rr or (p == rr and q >= s)):
                        continue
                    f = (0.5 if p == q else 1.0) * (0.5 if rr == s else 1.0) * (0.5 if (p == rr and q == s) else 1.0)
                    acc += f * g[q, p, s, rr] * D[p, rr]
            X6[q, s] = acc
    YJ = np.zeros((n, n))
    XK = X6.copy()
    for i in range(n):
        for j in range(n):
            if i >= j:
                YJ[i, j] = sum(S1[i, r, j] for r in range(i + 1)) + sum(S2[i, p, j] for p in range(i, n))
                XK[i, j] += X3[i, j] + sum(S5[i, r, j] for r in range(j, i + 1))
            XK[i, j] += sum(S4[j, p, i] for p in range(max(i, j), n))
    return 2.0 * (YJ + YJ.T), XK + XK.T


@pytest.mark.parametrize("n,seed", [(1, 0), (2, 1), (5, 2), (9, 3)])
def test_restated_symmetric_fock_matches_the_two_contractions(n, seed):
    g, D = sym_inputs(n, seed)
    J, K = fock_jk_restated(g, D)
    J_ref = np.einsum("pqrs,rs->pq", g, D)
    K_ref = np.einsum("prqs,rs->pq", g, D)
    assert np.allclose(J, J_ref, rtol=1e-13, atol=1e-13 * np.abs(J_ref).max())
    assert np.allclose(K, K_ref, rtol=1e-13, atol=1e-13 * np.abs(K_ref).max())
