"""Parity of the split-BF16 tensor-core path with the CPU oracle (GPU).

Tolerance: relative Frobenius error <= 1e-10 at the default 5 slices, and the
error reported for every slice count (3..6) must fall with the count and stay
under the a-priori bound the library reports."""
import os

import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL_SPLIT = 1e-10


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


def status_ok(eg):
    import ctypes

    from einsums_gb300 import _lib
    code = ctypes.c_int32(0)
    st = _lib.load().eg_stream_status(ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), ctypes.byref(code))
    return st == 0 and code.value == 0


def run_case(eg, Cl, Al, Bl, dims, cp=0.0, ab=1.0, slices=5, seed=0, scale_rows=False):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal([dims[l] for l in Al])
    B = rng.standard_normal([dims[l] for l in Bl])
    if scale_rows:
        A *= np.exp(rng.uniform(-30, 30, size=A.shape[:1]))[(...,) + (None,) * (A.ndim - 1)]
    C = rng.standard_normal([dims[l] for l in Cl])
    ref = C.copy()
    oracle.einsum(Cl, ref, cp, ab, Al, A, Bl, B)
    tC = cu(C)
    eg.einsum(cp, Cl, tC, ab, Al, cu(A), Bl, cu(B), precision="split_bf16", slices=slices)
    got = tC.cpu().numpy()
    assert status_ok(eg)
    return oracle.rel_fro(got, ref), eg.last_split_report()


def test_single_tile_gemm(eg):
    err, rep = run_case(eg, "ij", "ik", "kj", {"i": 128, "j": 128, "k": 64})
    assert rep["slices"] == 5 and rep["slice_pairs"] == 15
    assert err < TOL_SPLIT, err


@pytest.mark.parametrize("dims", [{"i": 200, "j": 300, "k": 1000}, {"i": 37, "j": 129, "k": 70},
                                  {"i": 1, "j": 250, "k": 3000}, {"i": 640, "j": 384, "k": 2500}])
def test_gemm_shapes(eg, dims):
    err, _ = run_case(eg, "ij", "ik", "kj", dims, cp=0.5, ab=-1.25)
    assert err < TOL_SPLIT, err


@pytest.mark.parametrize("S", [3, 4, 5, 6])
def test_error_per_slice_count(eg, S):
    err, rep = run_case(eg, "ikjl", "imjn", "mknl", {"i": 12, "k": 12, "j": 12, "l": 12, "m": 20, "n": 20}, slices=S,
                        seed=S)
    assert rep["slices"] == S and rep["slice_pairs"] == S * (S + 1) // 2
    assert err <= 50 * rep["error_bound"], (S, err, rep)
    if S >= 5:
        assert err < TOL_SPLIT


def test_generic_wmbej_pattern(eg):
    err, _ = run_case(eg, "mbej", "jnfb", "mnef", {"m": 8, "b": 24, "e": 24, "j": 8, "n": 8, "f": 24}, cp=1.0,
                      ab=-0.5)
    assert err < TOL_SPLIT, err


def test_wabef_pattern(eg):
    err, _ = run_case(eg, "abef", "mnef", "mnab", {"a": 20, "b": 20, "e": 20, "f": 20, "m": 8, "n": 8}, cp=1.0,
                      ab=0.25)
    assert err < TOL_SPLIT, err


def test_batched_pattern_and_gemv_shape(eg):
    err, _ = run_case(eg, "bij", "bik", "bkj", {"b": 3, "i": 70, "j": 90, "k": 150})
    assert err < TOL_SPLIT, err
    err, _ = run_case(eg, "pq", "prqs", "rs", {"p": 12, "q": 12, "r": 12, "s": 12}, cp=1.0, ab=-1.0)
    assert err < TOL_SPLIT, err


def test_gemv_shapes_run_fp64(eg):
    # M or N at most 4: the FP64 kernels run (report: 0 slices), bitwise equal to precision="fp64"
    rng = np.random.default_rng(9)
    for dims in ({"i": 3, "j": 500, "k": 700}, {"i": 400, "j": 4, "k": 300}):
        A = cu(rng.standard_normal((dims["i"], dims["k"])))
        B = cu(rng.standard_normal((dims["k"], dims["j"])))
        outs = []
        for prec in ("split_bf16", "fp64"):
            C = torch.zeros((dims["i"], dims["j"]), dtype=torch.float64, device="cuda")
            eg.einsum(0.0, "ij", C, 1.0, "ik", A, "kj", B, precision=prec)
            outs.append(C.cpu().numpy())
            if prec == "split_bf16":
                assert eg.last_split_report()["slices"] == 0
        assert np.array_equal(outs[0], outs[1])
    # one above the limit takes the split form
    err, rep = run_case(eg, "ij", "ik", "kj", {"i": 5, "j": 300, "k": 400})
    assert rep["slices"] == 5 and err < TOL_SPLIT, err


def test_k_slices_in_parallel(eg):
    # few output tiles and a long K: the K range runs in slices on different CTAs whose
    # exact int64 sums are added atomically; the result is exact-order independent
    err, rep = run_case(eg, "ij", "ik", "kj", {"i": 130, "j": 120, "k": 8192}, cp=0.7, ab=-0.3)
    assert rep["slices"] == 5 and err < TOL_SPLIT, err
    rng = np.random.default_rng(21)
    A, B = cu(rng.standard_normal((200, 6000))), cu(rng.standard_normal((6000, 140)))
    C0 = cu(rng.standard_normal((200, 140)))
    outs = []
    for _ in range(3):
        C = C0.clone()
        eg.einsum(0.5, "ij", C, 1.5, "ik", A, "kj", B, precision="split_bf16")
        outs.append(C.cpu().numpy())
    assert np.array_equal(outs[0], outs[1]) and np.array_equal(outs[0], outs[2])
    ref = 0.5 * C0.cpu().numpy() + 1.5 * (A.cpu().numpy() @ B.cpu().numpy())
    assert oracle.rel_fro(outs[0], ref) < TOL_SPLIT


def test_rows_with_wide_dynamic_range(eg):
    err, _ = run_case(eg, "ij", "ik", "kj", {"i": 150, "j": 140, "k": 300}, scale_rows=True)
    assert err < TOL_SPLIT, err


def test_multi_pass_k_for_six_slices(eg):
    # six slices' exact sum fits int64 only up to K = 128; K = 700 runs slice
    # groups 0-4 and 5 as two launches, each over the whole K
    err, _ = run_case(eg, "ij", "ik", "kj", {"i": 100, "j": 100, "k": 700}, cp=0.3, ab=2.0, slices=6)
    assert err < 1e-12, err


@pytest.mark.parametrize("S,K", [(6, 1000), (6, 129), (5, 70000)])
def test_slice_group_ranges_match_cpu_restatement(eg, S, K):
    """When all slice groups' exact sum cannot take the whole K in int64, the groups
    run as ranges (S = 6: 0-4 and 5), each range's exact sum rounded to FP64 and the
    ranges added in order: bit for bit the CPU restatement of that plan."""
    from test_split_math import split_product_ranges
    rng = np.random.default_rng(S * K)
    M, N = (37, 130) if K < 10000 else (9, 12)
    A = rng.standard_normal((M, K)) * np.exp2(rng.integers(-8, 8, size=(M, 1)))
    B = rng.standard_normal((N, K))
    ref = split_product_ranges(A, B, S)
    C = torch.full((M, N), np.nan, dtype=torch.float64, device="cuda")
    eg.einsum(0.0, "ij", C, 1.0, "ik", cu(A), "jk", cu(B), precision="split_bf16", slices=S)
    assert np.array_equal(C.cpu().numpy().view(np.uint64), ref.view(np.uint64))


def test_nonfinite_row_gives_nan_row_only(eg):
    rng = np.random.default_rng(5)
    A = rng.standard_normal((64, 80))
    B = rng.standard_normal((80, 48))
    A[7, 3] = np.inf
    tC = torch.zeros((64, 48), dtype=torch.float64, device="cuda")
    eg.einsum(0.0, "ij", tC, 1.0, "ik", cu(A), "kj", cu(B), precision="split_bf16")
    got = tC.cpu().numpy()
    assert np.all(np.isnan(got[7]))
    mask = np.ones(64, bool)
    mask[7] = False
    assert oracle.rel_fro(got[mask], (A @ B)[mask]) < TOL_SPLIT


def test_deterministic(eg):
    rng = np.random.default_rng(8)
    A, B = cu(rng.standard_normal((300, 500))), cu(rng.standard_normal((500, 260)))
    outs = []
    for _ in range(2):
        C = torch.zeros((300, 260), dtype=torch.float64, device="cuda")
        eg.einsum(0.0, "ij", C, 1.0, "ik", A, "kj", B, precision="split_bf16")
        outs.append(C.cpu().numpy())
    assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))


def test_e2e_slab_pipeline_matches_whole_step(eg):
    """The host-buffer pipeline moves Wabef in row slabs through a ring of device
    buffers on three streams; every result must equal the whole-step contraction
    bit for bit (each element's row, column and K sum are unchanged by slabbing)."""
    import os
    import sys
    import types
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    from einsums_gb300 import workloads
    o, v = 6, 20
    T = workloads.ccd_inputs(o, v, seed=5, backend="torch")
    args = types.SimpleNamespace(steps=4, warmup=1, slices=5)
    _, out = bench.run_e2e(eg, T, "split_bf16", args, o, v, 1.0, chunks=3, return_outputs=True)
    W = bench.fresh_W(T)
    bench.ccd_step(eg, T, W, "split_bf16", 5)
    torch.cuda.synchronize()
    for k in ("Wmnij", "Wmbej", "Wabef"):
        assert torch.equal(out[k], W[k].cpu()), k
    assert abs(float(out["E"]) - float(W["E"])) <= 1e-14 * max(1.0, abs(float(W["E"])))


PAIR_CASES = [(300, 200, 256, 0.0), (260, 100, 2048, 0.0), (1000, 520, 384, 1.0), (128, 640, 512, 0.0)]


def pair_cases():
    """Runs PAIR_CASES in this process and returns the number of pair clusters
    the tensor kernel used; raises on the first result that is not bit-exact."""
    import ctypes
    import einsums_gb300 as eg
    from einsums_gb300 import _lib
    from test_split_math import split_product_fast
    for M, N, K, cp in PAIR_CASES:
        rng = np.random.default_rng(M + K)
        A = rng.standard_normal((M, K)) * np.exp2(rng.integers(-10, 10, size=(M, 1)))
        B = rng.standard_normal((N, K))
        ref = split_product_fast(A, B, 5)
        C0 = rng.standard_normal((M, N))
        C = cu(C0)
        eg.einsum(cp, "ij", C, 1.0, "ik", cu(A), "jk", cu(B), precision="split_bf16", slices=5)
        want = ref if cp == 0.0 else C0 + ref
        assert np.array_equal(C.cpu().numpy().view(np.uint64), want.view(np.uint64)), (M, N, K, cp)
        # C contiguous along the rows (the epilogue path that runs one thread per row)
        Ct = torch.zeros((N, M), dtype=torch.float64, device="cuda")
        eg.einsum(0.0, "ji", Ct, 1.0, "ik", cu(A), "jk", cu(B), precision="split_bf16", slices=5)
        assert np.array_equal(Ct.cpu().numpy().T.copy().view(np.uint64), ref.view(np.uint64)), (M, N, K, "rows")
    # a batch index: each batch's tiles are scheduled as their own pairs
    rng = np.random.default_rng(5)
    A = rng.standard_normal((2, 300, 192))
    B = rng.standard_normal((2, 140, 192))
    C = torch.zeros((2, 300, 140), dtype=torch.float64, device="cuda")
    eg.einsum(0.0, "bij", C, 1.0, "bik", cu(A), "bjk", cu(B), precision="split_bf16", slices=5)
    got = C.cpu().numpy()
    for b in range(2):
        want = split_product_fast(A[b], B[b], 5)
        assert np.array_equal(got[b].view(np.uint64), want.view(np.uint64)), ("batch", b)
    n = ctypes.c_int32(-1)
    _lib.check(_lib.load().eg_tc_pair_clusters(ctypes.byref(n)))
    return n.value


def test_single_cta_tiles_are_the_exact_split_product(eg):
    """Outputs of several 128-row tiles, odd tile counts and a K cut into slices
    (260 x 100, K = 2048): bit for bit the CPU restatement of the scheme."""
    clusters = pair_cases()
    if os.environ.get("EINSUMS_GB300_TC_PAIRS") != "1":
        assert clusters == 0  # this process runs single-CTA tiles


def test_pair_tiles_are_the_exact_split_product(eg):
    """The same cases on CTA pairs (256x128 tiles, cta_group::2), in a process
    started with EINSUMS_GB300_TC_PAIRS=1: an odd row-tile count leaves the
    second CTA of the last pair past the rows (300 and 1000 rows)."""
    import subprocess
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    path = os.pathsep.join([root, os.path.join(root, "oracle"), here, os.environ.get("PYTHONPATH", "")])
    env = dict(os.environ, EINSUMS_GB300_TC_PAIRS="1", PYTHONPATH=path)
    code = "import test_gpu_split as t; print('pairs', t.pair_cases())"
    r = subprocess.run([sys.executable, "-c", code], cwd=here, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    clusters = int(r.stdout.split("pairs")[-1])
    assert clusters > 0, r.stdout


@pytest.mark.parametrize("S,K", [(3, 300), (4, 257), (5, 1000), (5, 70), (6, 128)])
def test_split_result_is_the_exact_split_product(eg, S, K):
    """Digits, exact integer accumulation and the final int64 -> FP64 rounding
    together: C = A B^T through the split path equals, bit for bit, the CPU
    restatement of the scheme with Python integers (one exact pass of K)."""
    from test_split_math import split_product
    rng = np.random.default_rng(100 + S)
    M, N = 37, 130
    A = rng.standard_normal((M, K)) * np.exp2(rng.integers(-20, 20, size=(M, 1)))
    B = rng.standard_normal((N, K))
    A[3, :] = 0.0  # a zero row
    ref = split_product(A, B, S)
    C = torch.zeros((M, N), dtype=torch.float64, device="cuda")
    eg.einsum(0.0, "ij", C, 1.0, "ik", cu(A), "jk", cu(B), precision="split_bf16", slices=S)
    assert eg.last_split_report()["slices"] == S
    assert np.array_equal(C.cpu().numpy().view(np.uint64), ref.view(np.uint64))
    # the grouped launch computes every item the same way
    As = [A, A[:20, :]]
    Bs = [B, B[:9, :]]
    Cs = [torch.zeros((a.shape[0], b.shape[0]), dtype=torch.float64, device="cuda") for a, b in zip(As, Bs)]
    plan = eg.GroupedPlan(0.0, "ij", Cs, 1.0, "ik", [cu(a) for a in As], "jk", [cu(b) for b in Bs],
                          precision="split_bf16", slices=S)
    plan.execute()
    torch.cuda.synchronize()
    for a, b, c in zip(As, Bs, Cs):
        assert np.array_equal(c.cpu().numpy().view(np.uint64), split_product(a, b, S).view(np.uint64))
    plan.close()


@pytest.mark.parametrize("layout", ["rows_contiguous", "k_contiguous"])
def test_split_product_exact_for_both_operand_layouts(eg, layout):
    """Row maxima and digits read operands stored either way round: rows
    contiguous (A given as "bki", so the splitting kernels walk rows with k
    strided) or k contiguous ("bik").  Row counts that are not a multiple of
    the 256-row units, K not a multiple of the 8-load batches, two batches,
    and rows spread over 2^-40 .. 2^40: bit for bit the CPU restatement."""
    from test_split_math import split_product_fast
    S, nb, M, N, K = 5, 2, 300, 37, 1003
    rng = np.random.default_rng(7)
    A = rng.standard_normal((nb, M, K)) * np.exp2(rng.integers(-40, 40, size=(nb, M, 1)))
    B = rng.standard_normal((nb, N, K)) * np.exp2(rng.integers(-40, 40, size=(nb, N, 1)))
    A[1, 299, :] = 0.0  # a zero row in the last, partial unit
    if layout == "rows_contiguous":
        Al, Bl = "bki", "bkj"
        tA, tB = cu(A.transpose(0, 2, 1)), cu(B.transpose(0, 2, 1))
    else:
        Al, Bl = "bik", "bjk"
        tA, tB = cu(A), cu(B)
    C = torch.zeros((nb, M, N), dtype=torch.float64, device="cuda")
    eg.einsum(0.0, "bij", C, 1.0, Al, tA, Bl, tB, precision="split_bf16", slices=S)
    assert eg.last_split_report()["slices"] == S
    got = C.cpu().numpy()
    for b in range(nb):
        ref = split_product_fast(A[b], B[b], S)
        assert np.array_equal(got[b].view(np.uint64), ref.view(np.uint64)), b
