"""Parity of the plain FP64 CUDA path with the CPU oracle (GPU)."""
import itertools
import json
import os

import numpy as np
import pytest

import classify
import oracle
import qchem_driver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))
TOL = 1e-12  # relative Frobenius error bound for contractions (permute is bit-exact)


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


def cu_view(base_np, slicer):
    return cu(base_np)[slicer]


def test_known_answers(eg):
    A2 = np.arange(1, 10, dtype=float).reshape(3, 3)
    A3 = np.arange(1, 28, dtype=float).reshape(3, 3, 3)
    cases = {"ik=ij,jk": ("ij", "ik", A2, "kj", A2), "il=ijk,jkl": ("il", "ijk", A3, "jkl", A3)}
    for sec in GOLDEN["known_answers"]:
        Cl, Al, A, Bl, B = cases[sec["section"]]
        Cs = [torch.zeros(3, 3, dtype=torch.float64, device="cuda") for _ in range(10)]
        alg = eg.einsum(0.0, Cl, Cs, 1.0, Al, [cu(A)] * 10, Bl, [cu(B)] * 10)  # Batched.cpp
        assert alg == "GEMM"
        for C in Cs:
            Cn = C.cpu().numpy()
            for i, j, v in sec["values"]:
                assert Cn[i, j] == v


def _case_tensors(case, rng):
    labels = sorted(set(case["C"]) | set(case["A"]) | set(case["B"]))
    dims = {l: 3 + (i % 3) for i, l in enumerate(labels)}
    make = lambda labs: rng.standard_normal([dims[l] for l in labs]) if labs else np.zeros(())
    C, A, B = make(case["C"]), make(case["A"]), make(case["B"])
    tC, tA, tB = cu(C), cu(A), cu(B)
    w = case["where"]
    if w.endswith("Einsum7.cpp:209"):
        Q, i, a = A.shape
        big = rng.standard_normal((Q, i + a, i + a))
        A = big[:, 0:i, i:i + a]
        tA = cu(big)[:, 0:i, i:i + a]
    if w.endswith("Dot.cpp:112"):
        big = rng.standard_normal((A.shape[0] + 8, A.shape[1]))
        A = big[0:A.shape[0], :]
        tA = cu(big)[0:A.shape[0], :]
    if w.endswith("Einsum1.cpp:127"):
        bigC = np.zeros((10, 10))
        C = bigC[5:5 + C.shape[0], 5:5 + C.shape[1]]
        tC = cu(bigC)[5:5 + C.shape[0], 5:5 + C.shape[1]]
        bigB = rng.standard_normal((B.shape[0], B.shape[1] + 2))
        B = bigB[:, 2:]
        tB = cu(bigB)[:, 2:]
    return (C, A, B), (tC, tA, tB)


@pytest.mark.parametrize("case", GOLDEN["cpp_choices"], ids=lambda c: c["where"].split("/")[-1])
def test_cpp_choices_and_values(eg, case):
    rng = np.random.default_rng(7)
    (C, A, B), (tC, tA, tB) = _case_tensors(case, rng)
    ref = np.array(C, copy=True)
    want = oracle.einsum(case["C"], ref, 0.0, 1.0, case["A"], A, case["B"], B)
    alg = eg.einsum(0.0, case["C"], tC, 1.0, case["A"], tA, case["B"], tB)
    assert alg == case["expected"] == want.name
    assert oracle.rel_fro(tC.cpu().numpy(), ref) < TOL


PATTERNS = [
    ("ij", "ik", "kj"), ("ij", "ki", "jk"), ("ikjl", "imjn", "mknl"), ("mbej", "jnfb", "mnef"),
    ("pq", "prqs", "rs"), ("pq", "pqrs", "rs"), ("", "ijab", "ijab"), ("ijk", "ijk", "ijk"),
    ("ij", "i", "j"), ("iajb", "iajb", "iajb"), ("i", "ij", "ji"), ("ijkl", "ijpl", "pk"),
    ("ab", "ija", "ijb"), ("", "iajb", "ibja"), ("ij", "ii", "ij"), ("i", "ij", "j"), ("i", "j", "ij"),
    ("ijab", "ijef", "efab"), ("ijab", "ijab", ""), ("bia", "ij", "bja"), ("ii", "i", "i"),
    ("ijk", "ikl", "lkj"), ("ij", "ikq", "kjq"),
]


@pytest.mark.parametrize("pattern", PATTERNS, ids=lambda p: f"{p[0]}<-{p[1]}*{p[2]}")
@pytest.mark.parametrize("semantics", ["cpp", "py"])
@pytest.mark.parametrize("prefactors", [(0.0, 1.0), (0.5, -1.25), (1.0, 2.0)])
def test_patterns_vs_oracle(eg, pattern, semantics, prefactors):
    Cl, Al, Bl = pattern
    cpf, abf = prefactors
    rng = np.random.default_rng(abs(hash((pattern, semantics, prefactors))) % 2**32)
    labels = sorted(set(Cl + Al + Bl))
    dims = {l: [7, 5, 9, 6, 4, 11][i % 6] for i, l in enumerate(labels)}
    A = rng.standard_normal([dims[l] for l in Al])
    B = rng.standard_normal([dims[l] for l in Bl])
    C = rng.standard_normal([dims[l] for l in Cl]) if Cl else np.array(rng.standard_normal())
    ref = C.copy()
    want = oracle.einsum(Cl, ref, cpf, abf, Al, A, Bl, B, semantics=semantics)
    tC = cu(C)
    if semantics == "cpp":
        alg = eg.einsum(cpf, Cl, tC, abf, Al, cu(A), Bl, cu(B))
        assert alg == want.name
    else:
        plan = eg.compile_plan(Cl, Al, Bl)
        assert type(plan).__name__ == classify.PLAN_NAMES[want]
        plan.execute(cpf, tC, abf, cu(A), cu(B))
    assert oracle.rel_fro(tC.cpu().numpy(), ref) < TOL


@pytest.mark.parametrize("pattern", [("ij", "ik", "kj"), ("", "i", "i"), ("ij", "i", "j"), ("ij", "ij", "ij"),
                                     ("i", "ij", "j"), ("ij", "ji", "ij")])
def test_zero_prefactor_overwrites_nan(eg, pattern):
    """C_prefactor == 0 zeroes C (no NaN propagation) except where the reference
    multiplies (C++ DOT and GER keep NaN)."""
    Cl, Al, Bl = pattern
    dims = {"i": 5, "j": 6, "k": 7}
    rng = np.random.default_rng(2)
    A = rng.standard_normal([dims[l] for l in Al])
    B = rng.standard_normal([dims[l] for l in Bl])
    shape = [dims[l] for l in Cl]
    for semantics in ("cpp", "py"):
        tC = torch.full(shape, float("nan"), dtype=torch.float64, device="cuda")
        ref = np.full(shape, np.nan)
        want = oracle.einsum(Cl, ref, 0.0, 1.0, Al, A, Bl, B, semantics=semantics)
        if semantics == "cpp":
            eg.einsum(0.0, Cl, tC, 1.0, Al, cu(A), Bl, cu(B))
        else:
            eg.compile_plan(Cl, Al, Bl).execute(0.0, tC, 1.0, cu(A), cu(B))
        got = tC.cpu().numpy()
        assert np.array_equal(np.isnan(got), np.isnan(ref)), (semantics, want)
        mask = ~np.isnan(ref)
        if mask.any():
            assert oracle.rel_fro(got[mask], ref[mask]) < TOL


def test_dot_is_deterministic(eg):
    rng = np.random.default_rng(9)
    A = cu(rng.standard_normal((64, 64, 48, 33)))
    B = cu(rng.standard_normal((64, 64, 48, 33)))
    outs = []
    for _ in range(3):
        C = torch.zeros((), dtype=torch.float64, device="cuda")
        eg.einsum(0.0, "", C, 1.0, "ijab", A, "ijab", B)
        outs.append(C.item())
    assert outs[0] == outs[1] == outs[2]
    ref = np.dot(A.cpu().numpy().ravel(), B.cpu().numpy().ravel())
    assert abs(outs[0] - ref) <= 1e-12 * abs(ref) + 1e-9


@pytest.mark.parametrize("perm", list(itertools.permutations(range(4))))
def test_permute_bit_exact(eg, perm):
    rng = np.random.default_rng(3)
    A = rng.standard_normal((12, 17, 32, 9))
    A[0, 0, 0, :3] = [-0.0, np.inf, np.nan]
    Al = "abcd"
    Cl = "".join(Al[p] for p in perm)
    shape = [A.shape[p] for p in perm]
    ref = np.zeros(shape)
    oracle.permute(Cl, ref, 0.0, 1.0, Al, A)
    tC = torch.full(shape, 7.0, dtype=torch.float64, device="cuda")
    eg.permute(0.0, Cl, tC, 1.0, Al, cu(A))
    assert np.array_equal(tC.cpu().numpy().view(np.uint64), ref.view(np.uint64))
    # prefactors: alpha*A + beta*C, compared bit for bit with the oracle
    C0 = rng.standard_normal(shape)
    ref2 = C0.copy()
    oracle.permute(Cl, ref2, 0.75, -1.5, Al, A)
    tC2 = cu(C0)
    eg.permute(0.75, Cl, tC2, -1.5, Al, cu(A))
    got2 = tC2.cpu().numpy()
    nan = np.isnan(ref2)
    assert np.array_equal(np.isnan(got2), nan)  # NaN payloads are not compared
    assert np.array_equal(got2[~nan].view(np.uint64), ref2[~nan].view(np.uint64))


def test_permute_strided_views_and_errors(eg):
    rng = np.random.default_rng(4)
    big = rng.standard_normal((10, 20, 30))
    tA = cu(big)[2:8, ::2, 5:25]
    A = big[2:8, ::2, 5:25]
    ref = np.zeros((20, 6, 10))
    oracle.permute("kij", ref, 0.0, 3.0, "ijk", A)
    tC = torch.zeros((20, 6, 10), dtype=torch.float64, device="cuda")
    eg.permute(0.0, "kij", tC, 3.0, "ijk", tA)
    assert np.array_equal(tC.cpu().numpy(), ref)
    from einsums_gb300._lib import DimensionError
    with pytest.raises(DimensionError):
        eg.permute(0.0, "ji", torch.zeros((3, 3), dtype=torch.float64, device="cuda"), 1.0, "ij",
                   torch.zeros((3, 4), dtype=torch.float64, device="cuda"))


class _TorchOps:
    def __init__(self, eg, semantics):
        self.eg, self.semantics = eg, semantics

    def einsum(self, Cl, C, c, ab, Al, A, Bl, B):
        if self.semantics == "cpp":
            return self.eg.einsum(c, Cl, C, ab, Al, A, Bl, B)
        return self.eg.compile_plan(Cl, Al, Bl).execute(c, C, ab, A, B)

    array = staticmethod(lambda x: torch.tensor(np.asarray(x, dtype=np.float64), device="cuda"))
    numpy = staticmethod(lambda x: x.cpu().numpy())
    zeros = staticmethod(lambda s: torch.zeros(s, dtype=torch.float64, device="cuda"))
    scalar = staticmethod(lambda x: float(x.item()))

    @staticmethod
    def copy_into(dst, src):
        dst.copy_(torch.as_tensor(np.asarray(src, dtype=np.float64)))


@pytest.mark.parametrize("semantics", ["cpp", "py"])
def test_water_rhf_mp2_on_gpu(eg, semantics):
    q = GOLDEN["qchem"]
    res = qchem_driver.rhf_mp2(_TorchOps(eg, semantics), q["enuc"])
    assert abs(res["e_scf"] - q["e_scf"]) < q["tol"]
    assert abs(res["e_mp2"] - q["e_mp2"]) < q["tol"]
    assert abs(res["e_tot"] - q["e_tot"]) < q["tol"]


def test_fock_build_small(eg):
    """Config-1 shape at n=24: F = 2 J - K with J via GEMV and K via GENERIC."""
    from einsums_gb300 import workloads
    g, D = workloads.fock_inputs(24, seed=1)
    F_ref = np.zeros((24, 24))
    assert oracle.einsum("pq", F_ref, 0.0, 2.0, "pqrs", g, "rs", D).name == "GEMV"
    assert oracle.einsum("pq", F_ref, 1.0, -1.0, "prqs", g, "rs", D).name == "GENERIC"
    tF = torch.zeros((24, 24), dtype=torch.float64, device="cuda")
    tg, tD = cu(g), cu(D)
    assert eg.einsum(0.0, "pq", tF, 2.0, "pqrs", tg, "rs", tD) == "GEMV"
    assert eg.einsum(1.0, "pq", tF, -1.0, "prqs", tg, "rs", tD) == "GENERIC"
    assert oracle.rel_fro(tF.cpu().numpy(), F_ref) < TOL


def test_empty_and_degenerate(eg):
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device="cuda")
    C = z(0, 3)
    eg.einsum(0.0, "ij", C, 1.0, "ik", z(0, 4), "kj", z(4, 3))
    C = z(3, 3).fill_(2.0)
    eg.einsum(0.5, "ij", C, 1.0, "ik", z(3, 0), "kj", z(0, 3))
    assert torch.all(C == 1.0)


@pytest.mark.parametrize("case", ["rows_contig_odd", "rows_misaligned", "vector_times_matrix", "strided_k",
                                  "strided_k_rows_over_B", "tail_rows"])
def test_long_k_gemv_variants(eg, case):
    # long k (>= 2048) GEMV shapes: the multi-row kernel, contiguous (16-byte pairs or not),
    # strided through offset tables, and with the operands swapped when the rows run over B
    rng = np.random.default_rng(sum(map(ord, case)))
    if case == "rows_contig_odd":
        Cl, Al, Bl, A, B = "p", "pk", "k", rng.standard_normal((103, 3001)), rng.standard_normal(3001)
    elif case == "rows_misaligned":
        A_np, B_np = rng.standard_normal((40, 2501)), rng.standard_normal(2501)
        tA, tB = cu(A_np)[:, 1:], cu(B_np)[1:]  # 8-byte offsets: no 16-byte pairs
        ref = A_np[:, 1:] @ B_np[1:]
        C = torch.zeros(40, dtype=torch.float64, device="cuda")
        eg.einsum(0.0, "p", C, 1.0, "pk", tA, "k", tB)
        assert oracle.rel_fro(C.cpu().numpy(), ref) < TOL
        return
    elif case == "vector_times_matrix":
        Cl, Al, Bl, A, B = "q", "k", "kq", rng.standard_normal(2600), rng.standard_normal((2600, 77))
    elif case == "strided_k":
        Cl, Al, Bl, A, B = "pq", "prqs", "rs", rng.standard_normal((9, 60, 9, 50)), rng.standard_normal((60, 50))
    elif case == "strided_k_rows_over_B":
        Cl, Al, Bl, A, B = "pq", "rs", "prqs", rng.standard_normal((60, 50)), rng.standard_normal((9, 60, 9, 50))
    else:  # rows not a multiple of the rows per block
        Cl, Al, Bl, A, B = "p", "pk", "k", rng.standard_normal((7, 4096)), rng.standard_normal(4096)
    dims = {}
    for l, e in list(zip(Al, A.shape)) + list(zip(Bl, B.shape)):
        dims[l] = e
    C0 = rng.standard_normal([dims[l] for l in Cl])
    ref = C0.copy()
    oracle.einsum(Cl, ref, 0.5, -1.5, Al, A, Bl, B)
    tC = cu(C0)
    eg.einsum(0.5, Cl, tC, -1.5, Al, cu(A), Bl, cu(B))
    assert oracle.rel_fro(tC.cpu().numpy(), ref) < TOL


def test_fp64_probe_rates_and_clock(eg):
    """The FP64 probes report positive rates and the SM clock the DFMA loop ran
    at, from each block's cycles over its own duration: a plausible GB300 clock,
    not the lower figure a block's cycles over the whole launch would give."""
    import ctypes

    from einsums_gb300 import _lib
    lib = _lib.load()
    dfma, dmma, mhz = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    _lib.check(lib.eg_measure_fp64_peak_clock(ctypes.byref(dfma), ctypes.byref(dmma), ctypes.byref(mhz)))
    assert 0.1 < dfma.value < 5.0 and 0.1 < dmma.value < 5.0
    assert 300.0 < mhz.value < 2300.0
    # the DFMA loop cannot beat the FP64 pipe's rate, 4 flop per clock per SM
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    assert dfma.value <= 1.02 * 4.0 * sms * mhz.value * 1e6 / 1e12
