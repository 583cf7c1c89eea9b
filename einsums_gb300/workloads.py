"""Seeded synthetic inputs for the benchmark configurations.

Every generator takes a seed and a backend: ``"numpy"`` (PCG64,
``np.random.default_rng(seed)``) or ``"cuda"`` (a seeded ``torch.Generator``
on the current CUDA device, for full-size inputs that would take too long to
build on the host).  The two backends give different numbers for the same
seed; each test or benchmark uses one backend for both the checked and the
checking side.

Configurations (sizes are the benchmark defaults):
  * Fock two-electron build, n orbitals: g[p,q,r,s] ~ U(-1,1), symmetrised to
    8-fold permutational symmetry and scaled by exp(-0.1(|p-q|+|r-s|));
    D = Cocc Cocc^T with Cocc the first min(20, n) columns of a random
    orthogonal matrix (QR of N(0,1)).
  * CCD W intermediates, o occupied / v virtual: t_ijab ~ N(0, 0.01^2),
    antisymmetrised in (i,j) and (a,b); g_oooo, g_oovv, g_vvvv, g_ovvo ~
    U(-1,1), antisymmetrised in the bra pair and the ket pair (g_ovvo mixes
    the two spaces in each pair, so its antisymmetry relates it to other
    blocks and it stays plain uniform).
  * Sweep: N(0,1) operands for C[i,k,j,l] = sum_mn A[i,m,j,n] B[m,k,n,l].
  * Batched: 2048 contractions C_k[a,b] = sum_ij A_k[i,j,a] B_k[i,j,b] with
    extents log-uniform, i,j in [4,32] and a,b in [20,120].
"""
from __future__ import annotations

import math

import numpy as np


def _rng(seed):
    return np.random.default_rng(seed)


def _torch_gen(seed):
    import torch
    g = torch.Generator(device="cuda")
    g.manual_seed(int(seed))
    return g


# ------------------------------------------------------------------ Fock --
def fock_inputs(n: int, seed: int = 0, backend: str = "numpy", nocc: int = 20):
    nocc = min(nocc, n)
    if backend == "numpy":
        r = _rng(seed)
        g = r.uniform(-1.0, 1.0, size=(n, n, n, n))
        g = g + g.transpose(1, 0, 2, 3)
        g = g + g.transpose(0, 1, 3, 2)
        g = g + g.transpose(2, 3, 0, 1)
        g *= 0.125
        idx = np.arange(n)
        d = np.abs(idx[:, None] - idx[None, :])
        g *= np.exp(-0.1 * (d[:, :, None, None] + d[None, None, :, :]))
        Q, _ = np.linalg.qr(r.standard_normal((n, n)))
        Cocc = Q[:, :nocc]
        return g, Cocc @ Cocc.T
    import torch
    gen = _torch_gen(seed)
    g = torch.rand((n, n, n, n), generator=gen, dtype=torch.float64, device="cuda") * 2.0 - 1.0
    g = g + g.permute(1, 0, 2, 3)
    g = g + g.permute(0, 1, 3, 2)
    g = g + g.permute(2, 3, 0, 1)
    g *= 0.125
    idx = torch.arange(n, device="cuda", dtype=torch.float64)
    d = (idx[:, None] - idx[None, :]).abs()
    g *= torch.exp(-0.1 * (d[:, :, None, None] + d[None, None, :, :]))
    Q, _ = torch.linalg.qr(torch.randn((n, n), generator=gen, dtype=torch.float64, device="cuda"))
    Cocc = Q[:, :nocc]
    return g.contiguous(), (Cocc @ Cocc.T).contiguous()


# ------------------------------------------------------------------- CCD --
def _antisym_np(x):
    x = 0.5 * (x - x.transpose(1, 0, 2, 3))
    return 0.5 * (x - x.transpose(0, 1, 3, 2))


def _antisym_t(x):
    x = 0.5 * (x - x.permute(1, 0, 2, 3))
    return (0.5 * (x - x.permute(0, 1, 3, 2))).contiguous()


def ccd_inputs(o: int, v: int, seed: int = 0, backend: str = "numpy", with_vvvv: bool = True):
    """Returns dict with t (oovv), g_oooo, g_oovv, g_vvvv (or None), g_ovvo."""
    if backend == "numpy":
        r = _rng(seed)
        t = _antisym_np(r.normal(0.0, 0.01, size=(o, o, v, v)))
        out = {"t": t,
               "g_oooo": _antisym_np(r.uniform(-1, 1, size=(o, o, o, o))),
               "g_oovv": _antisym_np(r.uniform(-1, 1, size=(o, o, v, v))),
               "g_vvvv": _antisym_np(r.uniform(-1, 1, size=(v, v, v, v))) if with_vvvv else None,
               "g_ovvo": r.uniform(-1, 1, size=(o, v, v, o))}
        return out
    import torch
    gen = _torch_gen(seed)
    u = lambda *s: torch.rand(s, generator=gen, dtype=torch.float64, device="cuda") * 2.0 - 1.0
    t = _antisym_t(torch.randn((o, o, v, v), generator=gen, dtype=torch.float64, device="cuda") * 0.01)
    out = {"t": t, "g_oooo": _antisym_t(u(o, o, o, o)), "g_oovv": _antisym_t(u(o, o, v, v)),
           "g_vvvv": None, "g_ovvo": u(o, v, v, o)}
    if with_vvvv:
        # built in place to keep the peak at one v^4 buffer plus one v^4 temporary
        g = u(v, v, v, v)
        g.sub_(g.permute(1, 0, 2, 3).contiguous()).mul_(0.5)
        g.sub_(g.permute(0, 1, 3, 2).contiguous()).mul_(0.5)
        out["g_vvvv"] = g
    return out


# ----------------------------------------------------------------- sweep --
def sweep_contraction_inputs(n: int, seed: int = 0, backend: str = "numpy"):
    if backend == "numpy":
        r = _rng(seed)
        return r.standard_normal((n, n, n, n)), r.standard_normal((n, n, n, n))
    import torch
    gen = _torch_gen(seed)
    mk = lambda: torch.randn((n, n, n, n), generator=gen, dtype=torch.float64, device="cuda")
    return mk(), mk()


# --------------------------------------------------------------- batched --
def batched_shapes(count: int = 2048, seed: int = 0, ij=(4, 32), ab=(20, 120)):
    r = _rng(seed)
    lu = lambda lo, hi, k: np.exp(r.uniform(math.log(lo), math.log(hi + 1), size=k)).astype(int).clip(lo, hi)
    i, j = lu(*ij, count), lu(*ij, count)
    a, b = lu(*ab, count), lu(*ab, count)
    return [(int(i[k]), int(j[k]), int(a[k]), int(b[k])) for k in range(count)]


def batched_inputs(shapes, seed: int = 0, backend: str = "numpy"):
    if backend == "numpy":
        r = _rng(seed)
        As = [r.standard_normal((i, j, a)) for (i, j, a, b) in shapes]
        Bs = [r.standard_normal((i, j, b)) for (i, j, a, b) in shapes]
        return As, Bs
    import torch
    gen = _torch_gen(seed)
    As = [torch.randn((i, j, a), generator=gen, dtype=torch.float64, device="cuda") for (i, j, a, b) in shapes]
    Bs = [torch.randn((i, j, b), generator=gen, dtype=torch.float64, device="cuda") for (i, j, a, b) in shapes]
    return As, Bs
