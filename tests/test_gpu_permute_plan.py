"""Compiled permute plans on the GPU (eg_permute_plan_*): one plan, built from
the shapes, strides, permutation and prefactors, runs on several tensor pairs
and matches the oracle's permute bit for bit, as the reference's
compile_permute + permute(&C, A, plan) reuse one HPTT plan
(Permute.hpp:37-171, :292-297)."""
import itertools

import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("perm", [(0, 1, 2, 3), (3, 2, 1, 0), (1, 0, 3, 2), (2, 0, 3, 1)])
def test_plan_reused_on_several_tensors(eg, perm):
    rng = np.random.default_rng(sum(perm) + 7 * perm[0])
    shape = (9, 33, 17, 40)
    Al = "abcd"
    Cl = "".join(Al[p] for p in perm)
    cshape = [shape[p] for p in perm]
    tA0, tC0 = cu(rng.standard_normal(shape)), torch.zeros(cshape, dtype=torch.float64, device="cuda")
    plan = eg.compile_permute(0.0, Cl, tC0, 1.0, Al, tA0)
    for _ in range(3):
        A = rng.standard_normal(shape)
        ref = np.zeros(cshape)
        oracle.permute(Cl, ref, 0.0, 1.0, Al, A)
        tC = torch.full(cshape, 5.0, dtype=torch.float64, device="cuda")
        plan.execute(tC, cu(A))
        assert np.array_equal(tC.cpu().numpy().view(np.uint64), ref.view(np.uint64))
    plan.close()


def test_plan_with_prefactors_and_views(eg):
    rng = np.random.default_rng(3)
    big = rng.standard_normal((12, 20, 30))
    A = big[2:10, ::2, 5:25]
    plan = None
    for k in range(2):
        C0 = rng.standard_normal((20, 8, 10))
        ref = C0.copy()
        oracle.permute("kij", ref, 0.75, -1.5, "ijk", A * (k + 1))
        tbig = cu(big * (k + 1))
        tA = tbig[2:10, ::2, 5:25]
        tC = cu(C0)
        if plan is None:
            plan = eg.compile_permute(0.75, "kij", tC, -1.5, "ijk", tA)
        plan.execute(tC, tA)
        got = tC.cpu().numpy()
        assert np.array_equal(got.view(np.uint64), ref.view(np.uint64))
    from einsums_gb300._lib import DimensionError
    with pytest.raises(DimensionError):
        plan.execute(torch.zeros((20, 8, 11), dtype=torch.float64, device="cuda"), tA)


def _launched(eg, name):
    from einsums_gb300 import _lib
    import ctypes
    buf = ctypes.create_string_buffer(1 << 16)
    _lib.check(_lib.load().eg_profile_summary(buf, len(buf)))
    return name in buf.value.decode()


@pytest.mark.parametrize("shape,perm,ap,expect_tma", [
    ((100, 70), (1, 0), 1.0, True),                  # rank 2, partial boxes on both edges
    ((33, 40, 34), (2, 0, 1), 1.0, True),            # rank 3, partial boxes
    ((64, 64, 64, 64), (3, 1, 0, 2), 2.5, True),     # rank 4, scaled copy
    ((6, 34, 4, 2, 40), (4, 3, 0, 2, 1), 1.0, True),  # rank 5, nothing folds
    ((33, 35), (1, 0), 1.0, False),                  # odd row stride (not a 16-byte multiple): tile kernel
    ((20, 8, 100), (2, 1, 0), 1.0, False),           # C's fastest extent below one box: tile kernel
    ((40, 36, 8), (1, 0, 2), -0.75, False),          # fastest modes shared: row copies
])
def test_permute_tma_and_fallbacks_bit_exact(eg, shape, perm, ap, expect_tma):
    """The transposing case runs through TMA boxes (k_permute_tma) when its
    strides allow; edge boxes, ranks 2..5 and the scaled copy match NumPy bit for
    bit, as do the shapes that take the other kernels."""
    from einsums_gb300 import _lib
    rng = np.random.default_rng(sum(shape))
    A = rng.standard_normal(shape)
    ref = np.ascontiguousarray(np.transpose(A, perm)) * ap if ap != 1.0 else np.ascontiguousarray(np.transpose(A, perm))
    Al = "abcde"[:len(shape)]
    Cl = "".join(Al[p] for p in perm)
    C = torch.full(ref.shape, np.nan, dtype=torch.float64, device="cuda")
    lib = _lib.load()
    lib.eg_profile_enable(1)
    lib.eg_profile_reset()
    eg.permute(0.0, Cl, C, ap, Al, cu(A))
    torch.cuda.synchronize()
    tma = _launched(eg, "k_permute_tma")
    lib.eg_profile_enable(0)
    assert np.array_equal(C.cpu().numpy().view(np.uint64), ref.view(np.uint64))
    assert tma == expect_tma, (shape, perm)
    # the same through a compiled plan on a second pair of tensors
    A2 = rng.standard_normal(shape)
    C2 = torch.zeros(ref.shape, dtype=torch.float64, device="cuda")
    plan = eg.compile_permute(0.0, Cl, C2, ap, Al, cu(A2))
    plan.execute(C2, cu(A2))
    ref2 = np.ascontiguousarray(np.transpose(A2, perm))
    ref2 = ref2 * ap if ap != 1.0 else ref2
    assert np.array_equal(C2.cpu().numpy().view(np.uint64), ref2.view(np.uint64))
    plan.close()
