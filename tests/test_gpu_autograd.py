"""Autograd binding on the GPU: hand-written adjoint contractions against FP64
central finite differences (h = 1e-6, 64 seeded entries per input, relative
agreement 1e-7), against the CPU oracle's einsum of the adjoint patterns, and
against torch.einsum's own gradients on other patterns.  The split-BF16
forward/backward errors are stated against FP64."""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ag():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from einsums_gb300 import autograd, build
    build.build()
    return autograd


def ccd_inputs(o, v, seed):
    from einsums_gb300 import workloads
    T = workloads.ccd_inputs(o, v, seed=seed, backend="numpy", with_vvvv=False)
    R = np.random.default_rng(seed + 7).standard_normal((o, v, v, o))
    return T["t"], T["g_oovv"], R


def test_wmbej_gradients_fd_and_oracle(ag):
    o, v = 8, 24
    t_np, g_np, R_np = ccd_inputs(o, v, seed=1)
    t = torch.tensor(t_np, device="cuda", requires_grad=True)
    g = torch.tensor(g_np, device="cuda", requires_grad=True)
    R = torch.tensor(R_np, device="cuda")
    C = ag.einsum_ag("mbej", "jnfb", "mnef", t, g)
    L = ((C - R) ** 2).sum()
    L.backward()
    dt, dg = t.grad.detach(), g.grad.detach()

    # oracle: the adjoint einsums on the CPU (Python plan semantics)
    Cn = np.zeros((o, v, v, o))
    oracle.einsum("mbej", Cn, 0.0, 1.0, "jnfb", t_np, "mnef", g_np, semantics="py")
    dC = 2.0 * (Cn - R_np)
    dt_ref = np.zeros_like(t_np)
    oracle.einsum("jnfb", dt_ref, 0.0, 1.0, "mbej", dC, "mnef", g_np, semantics="py")
    dg_ref = np.zeros_like(g_np)
    oracle.einsum("mnef", dg_ref, 0.0, 1.0, "mbej", dC, "jnfb", t_np, semantics="py")
    assert oracle.rel_fro(dt.cpu().numpy(), dt_ref) < 1e-12
    assert oracle.rel_fro(dg.cpu().numpy(), dg_ref) < 1e-12

    # central differences on 64 seeded entries of each input; the change in L is
    # summed elementwise as (C+ - C-)(C+ + C- - 2R) to avoid cancellation
    rng = np.random.default_rng(3)
    h = 1e-6

    def fwd(tt, gg):
        return ag.einsum_ag("mbej", "jnfb", "mnef", tt, gg).detach()

    for X, grad, which in ((t, dt, 0), (g, dg, 1)):
        flat = rng.choice(X.numel(), size=64, replace=False)
        for f in flat:
            idx = np.unravel_index(int(f), tuple(X.shape))
            Xp = X.detach().clone()
            Xm = X.detach().clone()
            Xp[idx] += h
            Xm[idx] -= h
            Cp = fwd(Xp, g.detach()) if which == 0 else fwd(t.detach(), Xp)
            Cm = fwd(Xm, g.detach()) if which == 0 else fwd(t.detach(), Xm)
            dL = float(((Cp - Cm) * (Cp + Cm - 2.0 * R)).sum())
            fd = dL / (2.0 * h)
            an = float(grad[idx])
            assert abs(fd - an) <= 1e-7 * max(abs(an), 1e-3 * float(grad.abs().max())), (which, idx, fd, an)


def test_split_forward_backward_error(ag):
    o, v = 8, 24
    t_np, g_np, R_np = ccd_inputs(o, v, seed=2)
    R = torch.tensor(R_np, device="cuda")
    out = {}
    for prec in ("fp64", "split_bf16"):
        t = torch.tensor(t_np, device="cuda", requires_grad=True)
        g = torch.tensor(g_np, device="cuda", requires_grad=True)
        C = ag.einsum_ag("mbej", "jnfb", "mnef", t, g, precision=prec)
        ((C - R) ** 2).sum().backward()
        out[prec] = (C.detach(), t.grad.detach(), g.grad.detach())
    for a, b in zip(out["split_bf16"], out["fp64"]):
        err = float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))
        assert err < 1e-10, err


@pytest.mark.parametrize("pattern", [("ij", "ik", "kj"), ("", "ij", "ij"), ("ikjl", "imjn", "mknl"),
                                     ("i", "ij", "j"), ("ij", "i", "j"), ("bij", "bik", "bkj"), ("ia", "iab", "b")])
def test_gradients_match_torch_einsum(ag, pattern):
    Cl, Al, Bl = pattern
    dims = {l: 3 + (ord(l) % 5) for l in set(Cl + Al + Bl)}
    gen = torch.Generator(device="cuda")
    gen.manual_seed(5)
    A = torch.randn([dims[l] for l in Al], generator=gen, dtype=torch.float64, device="cuda", requires_grad=True)
    B = torch.randn([dims[l] for l in Bl], generator=gen, dtype=torch.float64, device="cuda", requires_grad=True)
    W = torch.randn([dims[l] for l in Cl], generator=gen, dtype=torch.float64, device="cuda")
    (ag.einsum_ag(Cl, Al, Bl, A, B) * W).sum().backward()
    gA, gB = A.grad.clone(), B.grad.clone()
    A.grad = None
    B.grad = None
    (torch.einsum(f"{Al},{Bl}->{Cl}", A, B) * W).sum().backward()
    assert torch.allclose(gA, A.grad, rtol=1e-12, atol=1e-12)
    assert torch.allclose(gB, B.grad, rtol=1e-12, atol=1e-12)
