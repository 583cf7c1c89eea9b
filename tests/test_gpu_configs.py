"""The benchmark configurations at their full sizes on the GPU, each checked
against the CPU oracle:

* Fock two-electron build, n = 100: F = 2 J - K with J = einsum(pq <- pqrs, rs)
  (GEMV) and K = einsum(pq <- prqs, rs) (GENERIC), as in the reference's
  QChemTests.cpp:300-303;
* CCD W intermediates, o = 32, v = 160: Wmnij, Wabef (GEMM), Wmbej (GENERIC)
  and E (DOT) in FP64 against oracle slabs, and the split-BF16 form against
  FP64 within 1e-10;
* all 24 rank-4 permutations at n = 64, bit-exact (Permute.hpp:338-407);
* the generic contraction ikjl <- imjn * mknl at n = 64, FP64 against an
  oracle slab and split-BF16 with 3..6 slices against FP64;
* 2048 uneven contractions ab <- ija * ijb in one grouped plan, every item
  against the oracle (Dispatch.hpp:1264-1286);
* the autograd binding at o = 24, v = 96: FP64 central differences on 64
  seeded entries of each input and the oracle's adjoint einsums.
"""
import itertools

import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12        # FP64 contractions against the oracle (relative Frobenius)
SPLIT_TOL = 1e-10  # split-BF16 (5 slices) against FP64


@pytest.fixture(scope="module")
def eg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import einsums_gb300
    from einsums_gb300 import build
    build.build()
    return einsums_gb300


def cu(x):
    return torch.from_numpy(np.array(x, dtype=np.float64, order="C", copy=True)).cuda()


def test_fock_n100(eg):
    from einsums_gb300 import workloads
    n = 100
    g, D = workloads.fock_inputs(n, seed=0)
    F_ref = np.zeros((n, n))
    assert oracle.einsum("pq", F_ref, 0.0, 2.0, "pqrs", g, "rs", D).name == "GEMV"
    assert oracle.einsum("pq", F_ref, 1.0, -1.0, "prqs", g, "rs", D).name == "GENERIC"
    tF = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    tg, tD = cu(g), cu(D)
    assert eg.einsum(0.0, "pq", tF, 2.0, "pqrs", tg, "rs", tD) == "GEMV"
    assert eg.einsum(1.0, "pq", tF, -1.0, "prqs", tg, "rs", tD) == "GENERIC"
    assert oracle.rel_fro(tF.cpu().numpy(), F_ref) < TOL


def test_ccd_o32_v160(eg):
    from einsums_gb300 import workloads
    o, v, rows = 32, 160, 2
    T = workloads.ccd_inputs(o, v, seed=0, backend="cuda")
    t, g = T["t"], T["g_oovv"]
    W = {}
    for prec in ("fp64", "split_bf16"):
        Wmnij, Wabef, Wmbej = T["g_oooo"].clone(), T["g_vvvv"].clone(), T["g_ovvo"].clone()
        E = torch.zeros((), dtype=torch.float64, device="cuda")
        assert eg.einsum(1.0, "mnij", Wmnij, 0.25, "ijef", t, "mnef", g, precision=prec) == "GEMM"
        assert eg.einsum(1.0, "abef", Wabef, 0.25, "mnef", g, "mnab", t, precision=prec) == "GEMM"
        assert eg.einsum(1.0, "mbej", Wmbej, -0.5, "jnfb", t, "mnef", g, precision=prec) == "GENERIC"
        assert eg.einsum(0.0, "", E, 0.25, "ijab", t, "ijab", g) == "DOT"
        W[prec] = (Wmnij, Wabef, Wmbej, E)
    # FP64 against oracle slabs (rows of the leading output index)
    t_np, g_np = t.cpu().numpy(), g.cpu().numpy()
    Wmnij, Wabef, Wmbej, E = W["fp64"]
    ref = T["g_oooo"][:rows].cpu().numpy().copy()
    oracle.einsum("mnij", ref, 1.0, 0.25, "ijef", t_np, "mnef", np.ascontiguousarray(g_np[:rows]))
    assert oracle.rel_fro(Wmnij[:rows].cpu().numpy(), ref) < TOL
    ref = T["g_vvvv"][:rows].cpu().numpy().copy()
    oracle.einsum("abef", ref, 1.0, 0.25, "mnef", g_np, "mnab", np.ascontiguousarray(t_np[:, :, :rows]))
    assert oracle.rel_fro(Wabef[:rows].cpu().numpy(), ref) < TOL
    ref = T["g_ovvo"][:rows].cpu().numpy().copy()
    oracle.einsum("mbej", ref, 1.0, -0.5, "jnfb", t_np, "mnef", np.ascontiguousarray(g_np[:rows]))
    assert oracle.rel_fro(Wmbej[:rows].cpu().numpy(), ref) < TOL
    e = np.zeros(())
    oracle.einsum("", e, 0.0, 0.25, "ijab", t_np, "ijab", g_np)
    assert abs(float(E.item()) - float(e)) <= TOL * abs(float(e))
    # split-BF16 against FP64, on the contraction part of each W
    for name, init, a, b in zip(("Wmnij", "Wabef", "Wmbej"), ("g_oooo", "g_vvvv", "g_ovvo"), W["split_bf16"][:3],
                                W["fp64"][:3]):
        d_s, d_f = a - T[init], b - T[init]
        err = float(torch.linalg.vector_norm(d_s - d_f) / torch.linalg.vector_norm(d_f))
        assert err < SPLIT_TOL, (name, err)


@pytest.mark.parametrize("perm", list(itertools.permutations(range(4))))
def test_permute_n64(eg, perm):
    n = 64
    gen = torch.Generator(device="cuda")
    gen.manual_seed(64)
    A = torch.randn((n, n, n, n), generator=gen, dtype=torch.float64, device="cuda")
    Cl = "".join("abcd"[p] for p in perm)
    C = torch.empty_like(A)
    eg.permute(0.0, Cl, C, 1.0, "abcd", A)
    ref = np.empty([n] * 4)
    oracle.permute(Cl, ref, 0.0, 1.0, "abcd", A.cpu().numpy())
    assert np.array_equal(C.cpu().numpy().view(np.uint64), ref.view(np.uint64))


def test_contraction_sweep_n64(eg):
    from einsums_gb300 import workloads
    n = 64
    A, B = workloads.sweep_contraction_inputs(n, seed=n, backend="cuda")
    C64 = torch.zeros((n, n, n, n), dtype=torch.float64, device="cuda")
    eg.einsum(0.0, "ikjl", C64, 1.0, "imjn", A, "mknl", B)
    ri = 8
    ref = np.zeros((ri, n, n, n))
    oracle.einsum("ikjl", ref, 0.0, 1.0, "imjn", np.ascontiguousarray(A[:ri].cpu().numpy()), "mknl", B.cpu().numpy())
    assert oracle.rel_fro(C64[:ri].cpu().numpy(), ref) < TOL
    # error against FP64 falls with the slice count; 5 slices meet 1e-10
    bounds = {3: 1e-5, 4: 1e-7, 5: SPLIT_TOL, 6: 1e-12}
    C = torch.zeros_like(C64)
    for S, bound in bounds.items():
        eg.einsum(0.0, "ikjl", C, 1.0, "imjn", A, "mknl", B, precision="split_bf16", slices=S)
        assert eg.last_split_report()["slices"] == S
        err = float(torch.linalg.vector_norm(C - C64) / torch.linalg.vector_norm(C64))
        assert err < bound, (S, err)


@pytest.mark.parametrize("precision,tol", [("fp64", TOL), ("split_bf16", SPLIT_TOL)])
def test_batched_2048_every_item(eg, precision, tol):
    from einsums_gb300 import workloads
    shapes = workloads.batched_shapes(2048, seed=0)
    As, Bs = workloads.batched_inputs(shapes, seed=1)
    tA, tB = [cu(x) for x in As], [cu(x) for x in Bs]
    tC = [torch.zeros((a, b), dtype=torch.float64, device="cuda") for (i, j, a, b) in shapes]
    plan = eg.GroupedPlan(0.0, "ab", tC, 1.0, "ija", tA, "ijb", tB, precision=precision)
    plan.execute()
    torch.cuda.synchronize()
    worst = 0.0
    for k in range(len(shapes)):
        ref = np.zeros(tC[k].shape)
        oracle.einsum("ab", ref, 0.0, 1.0, "ija", As[k], "ijb", Bs[k])
        worst = max(worst, oracle.rel_fro(tC[k].cpu().numpy(), ref))
    plan.close()
    assert worst < tol, worst


def test_autograd_o24_v96(eg):
    from einsums_gb300 import autograd, workloads
    o, v = 24, 96
    T = workloads.ccd_inputs(o, v, seed=0, backend="numpy", with_vvvv=False)
    t_np, g_np = T["t"], T["g_oovv"]
    R_np = np.random.default_rng(9).standard_normal((o, v, v, o))
    R = cu(R_np)
    grads = {}
    for prec in ("fp64", "split_bf16"):
        t = cu(t_np).requires_grad_(True)
        g = cu(g_np).requires_grad_(True)
        C = autograd.einsum_ag("mbej", "jnfb", "mnef", t, g, precision=prec)
        ((C - R) ** 2).sum().backward()
        grads[prec] = (t.grad.detach(), g.grad.detach())
    # the oracle's forward and adjoint einsums (every index is in C or in both
    # operands, so the C++ generic loop and the Python plan semantics agree)
    Cn = np.zeros((o, v, v, o))
    oracle.einsum("mbej", Cn, 0.0, 1.0, "jnfb", t_np, "mnef", g_np)
    dC = 2.0 * (Cn - R_np)
    dt_ref = np.zeros_like(t_np)
    oracle.einsum("jnfb", dt_ref, 0.0, 1.0, "mbej", dC, "mnef", g_np)
    dg_ref = np.zeros_like(g_np)
    oracle.einsum("mnef", dg_ref, 0.0, 1.0, "mbej", dC, "jnfb", t_np)
    assert oracle.rel_fro(grads["fp64"][0].cpu().numpy(), dt_ref) < TOL
    assert oracle.rel_fro(grads["fp64"][1].cpu().numpy(), dg_ref) < TOL
    assert oracle.rel_fro(grads["split_bf16"][0].cpu().numpy(), dt_ref) < SPLIT_TOL
    assert oracle.rel_fro(grads["split_bf16"][1].cpu().numpy(), dg_ref) < SPLIT_TOL
    # FP64 central differences, h = 1e-6, on 64 seeded entries of each input;
    # the change in L is summed as (C+ - C-)(C+ + C- - 2R) to avoid cancellation
    rng = np.random.default_rng(4)
    h = 1e-6
    tt, gg = cu(t_np), cu(g_np)
    for which, X in ((0, tt), (1, gg)):
        grad = grads["fp64"][which]
        gmax = float(grad.abs().max())
        for f in rng.choice(X.numel(), size=64, replace=False):
            idx = np.unravel_index(int(f), tuple(X.shape))
            Xp, Xm = X.clone(), X.clone()
            Xp[idx] += h
            Xm[idx] -= h
            Cp = autograd.einsum_ag("mbej", "jnfb", "mnef", *((Xp, gg) if which == 0 else (tt, Xp))).detach()
            Cm = autograd.einsum_ag("mbej", "jnfb", "mnef", *((Xm, gg) if which == 0 else (tt, Xm))).detach()
            fd = float(((Cp - Cm) * (Cp + Cm - 2.0 * R)).sum()) / (2 * h)
            an = float(grad[idx])
            assert abs(fd - an) <= 1e-7 * max(abs(an), 1e-3 * gmax), (which, idx, fd, an)
