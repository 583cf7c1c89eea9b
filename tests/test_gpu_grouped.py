"""Grouped (batched) execution on the GPU: persistent grouped launches over a
device work list, captured as CUDA graphs, against the oracle per item."""
import os

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


def make_batch(count, seed):
    from einsums_gb300 import workloads
    shapes = workloads.batched_shapes(count, seed=seed)
    As, Bs = workloads.batched_inputs(shapes, seed=seed + 1)
    Cs = [np.random.default_rng(seed + 2 + k).standard_normal((a, b)) for k, (i, j, a, b) in enumerate(shapes)]
    return shapes, As, Bs, Cs


def check_batch(Cs_gpu, As, Bs, Cs0, cp, ab, tol):
    for k in range(len(As)):
        ref = Cs0[k].copy()
        oracle.einsum("ab", ref, cp, ab, "ija", As[k], "ijb", Bs[k])
        err = oracle.rel_fro(Cs_gpu[k].cpu().numpy(), ref)
        assert err < tol, (k, err)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("split_bf16", 1e-10)])
def test_grouped_plan_matches_oracle(eg, precision, tol):
    shapes, As, Bs, Cs0 = make_batch(96, seed=3)
    tA, tB, tC = [cu(x) for x in As], [cu(x) for x in Bs], [cu(x) for x in Cs0]
    plan = eg.GroupedPlan(0.5, "ab", tC, -1.25, "ija", tA, "ijb", tB, precision=precision)
    assert plan.algorithm == "GEMM"
    plan.execute()
    torch.cuda.synchronize()
    check_batch(tC, As, Bs, Cs0, 0.5, -1.25, tol)
    # the graph reads the tensors' current contents: new inputs, replay, new result
    for k in range(len(As)):
        As[k] = As[k] * 2.0
        tA[k].copy_(cu(As[k]))
        tC[k].copy_(cu(Cs0[k]))
    plan.execute()
    torch.cuda.synchronize()
    check_batch(tC, As, Bs, Cs0, 0.5, -1.25, tol)
    plan.close()


def test_batched_einsum_uses_cached_plan(eg):
    shapes, As, Bs, Cs0 = make_batch(64, seed=5)
    tA, tB = [cu(x) for x in As], [cu(x) for x in Bs]
    for _ in range(2):
        tC = [cu(x) for x in Cs0]
        alg = eg.einsum(1.0, "ab", tC, 0.25, "ija", tA, "ijb", tB)
        torch.cuda.synchronize()
        assert alg == "GEMM"
        check_batch(tC, As, Bs, Cs0, 1.0, 0.25, 1e-12)
    # the Python list form of Plan.execute goes the same way
    tC = [cu(x) for x in Cs0]
    eg.compile_plan("ab", "ija", "ijb").execute(0.0, tC, 1.0, tA, tB, precision="split_bf16")
    torch.cuda.synchronize()
    check_batch(tC, As, Bs, [np.zeros_like(c) for c in Cs0], 0.0, 1.0, 1e-10)


def test_non_groupable_list_runs_item_by_item(eg):
    rng = np.random.default_rng(9)
    As = [rng.standard_normal(50 + 7 * k) for k in range(5)]
    Bs = [rng.standard_normal(50 + 7 * k) for k in range(5)]
    tC = [torch.zeros((), dtype=torch.float64, device="cuda") for _ in range(5)]
    alg = eg.einsum(0.0, "", tC, 1.0, "i", [cu(a) for a in As], "i", [cu(b) for b in Bs])
    assert alg == "DOT"
    for k in range(5):
        assert abs(tC[k].item() - float(np.dot(As[k], Bs[k]))) < 1e-12 * max(1.0, abs(np.dot(As[k], Bs[k])))
    from einsums_gb300._lib import NotSupportedError
    with pytest.raises(NotSupportedError):
        eg.GroupedPlan(0.0, "", tC, 1.0, "i", [cu(a) for a in As], "i", [cu(b) for b in Bs])


def test_autotuner_cache_written(eg):
    shapes, As, Bs, Cs0 = make_batch(40, seed=13)
    tA, tB, tC = [cu(x) for x in As], [cu(x) for x in Bs], [cu(x) for x in Cs0]
    eg.GroupedPlan(0.0, "ab", tC, 1.0, "ija", tA, "ijb", tB).close()
    path = os.environ["EINSUMS_GB300_AUTOTUNE_CACHE"]
    assert os.path.exists(path)
    lines = open(path).read().strip().split("\n")
    assert any("|f64|" in l and l.rsplit("=", 1)[1] in ("32", "64") for l in lines)


@pytest.mark.parametrize("pattern", [("ab", "ai", "ib"), ("zab", "zai", "zbi"), ("ab", "ia", "bi")])
def test_grouped_split_operand_layouts(eg, pattern):
    """Operands contiguous along K, along their rows, and with a batch index;
    odd K, rows spanning several 32-row splitting units and two row tiles."""
    Cl, Al, Bl = pattern
    rng = np.random.default_rng(17)
    dims_list = [dict(z=2, a=7, b=33, i=5), dict(z=1, a=150, b=64, i=129), dict(z=3, a=40, b=200, i=300),
                 dict(z=2, a=3, b=5, i=2), dict(z=1, a=65, b=97, i=64)]
    As, Bs, Cs0 = [], [], []
    for d in dims_list:
        As.append(rng.standard_normal([d[c] for c in Al]) * 10.0 ** rng.integers(-3, 3))
        Bs.append(rng.standard_normal([d[c] for c in Bl]))
        Cs0.append(rng.standard_normal([d[c] for c in Cl]))
    tA, tB, tC = [cu(x) for x in As], [cu(x) for x in Bs], [cu(x) for x in Cs0]
    plan = eg.GroupedPlan(0.5, Cl, tC, 2.0, Al, tA, Bl, tB, precision="split_bf16")
    for _ in range(2):  # a replay rewrites the digit planes from the current inputs
        for k in range(len(tC)):
            tC[k].copy_(cu(Cs0[k]))
        plan.execute()
        torch.cuda.synchronize()
        for k in range(len(As)):
            ref = Cs0[k].copy()
            oracle.einsum(Cl, ref, 0.5, 2.0, Al, As[k], Bl, Bs[k])
            assert oracle.rel_fro(tC[k].cpu().numpy(), ref) < 1e-10, k
    plan.close()


@pytest.mark.parametrize("precision", ["fp64", "split_bf16"])
def test_list_einsum_with_empty_items(eg, precision):
    """A list with empty items (an output extent 0): a grouped plan refuses it, and
    the list form of execute runs the items one by one with the other items'
    results correct."""
    rng = np.random.default_rng(17)
    shapes = [(3, 4, 20, 30), (3, 4, 0, 10), (2, 5, 12, 0), (6, 7, 33, 41)]
    As = [rng.standard_normal((i, j, a)) for i, j, a, b in shapes]
    Bs = [rng.standard_normal((i, j, b)) for i, j, a, b in shapes]
    Cs = [rng.standard_normal((a, b)) for i, j, a, b in shapes]
    from einsums_gb300 import _lib
    with pytest.raises(_lib.NotSupportedError):
        eg.GroupedPlan(0.5, "ab", [cu(c) for c in Cs], -1.25, "ija", [cu(a) for a in As], "ijb",
                       [cu(b) for b in Bs], precision=precision)
    tC = [cu(c) for c in Cs]
    eg.compile_plan("ab", "ija", "ijb").execute(0.5, tC, -1.25, [cu(a) for a in As], [cu(b) for b in Bs],
                                                 precision=precision)
    torch.cuda.synchronize()
    tol = 1e-12 if precision == "fp64" else 1e-10
    for a, b, c0, c in zip(As, Bs, Cs, tC):
        ref = c0.copy()
        oracle.einsum("ab", ref, 0.5, -1.25, "ija", a, "ijb", b)
        if ref.size:
            assert oracle.rel_fro(c.cpu().numpy(), ref) < tol
