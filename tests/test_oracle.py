"""Pins the CPU oracle against the reference's own golden data (CPU only).

* every active ``REQUIRE(alg_choice == ...)`` of the reference's C++ unit
  tests (tests/golden/golden.json ``cpp_choices``), with the same tensor
  shapes and views where the choice depends on strides;
* every ``assert type(plan) is ...`` of the reference's pytest suite;
* the exact integer answers of ``Einsum1.cpp`` / ``Batched.cpp``;
* the water/STO-3G RHF and MP2 energies of ``QChemTests.cpp`` to 1e-6;
* the generic loops against an independent dense evaluation;
* permute against HPTT itself when ``oracle/_ref`` was built here.
"""
import itertools
import json
import os

import numpy as np
import pytest

import classify
import oracle
import qchem_driver

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "golden.json")))


def _case_arrays(case, rng):
    labels = sorted(set(case["C"]) | set(case["A"]) | set(case["B"]))
    dims = {l: 3 + (i % 3) for i, l in enumerate(labels)}
    make = lambda labs: rng.standard_normal([dims[l] for l in labs]) if labs else np.zeros(())
    C, A, B = make(case["C"]), make(case["A"]), make(case["B"])
    where = case["where"]
    if where.endswith("Einsum7.cpp:209"):
        # SECTION("11"): Qov = B_Qmo(All, Range{0, nocc}, Range{nocc, nocc+nvirt})
        Q, i, a = A.shape
        big = rng.standard_normal((Q, i + a, i + a))
        A = big[:, 0:i, i:i + a]
    if where.endswith("Dot.cpp:112"):
        # A_view = A(Range{0, l}, All) of a taller matrix
        big = rng.standard_normal((A.shape[0] + 8, A.shape[1]))
        A = big[0:A.shape[0], :]
    if where.endswith("Einsum1.cpp:127"):
        bigC = np.zeros((10, 10))
        C = bigC[5:5 + C.shape[0], 5:5 + C.shape[1]]
        bigB = rng.standard_normal((B.shape[0], B.shape[1] + 2))
        B = bigB[:, 2:]
    return C, A, B


@pytest.mark.parametrize("case", GOLDEN["cpp_choices"], ids=lambda c: c["where"].split("/")[-1])
def test_cpp_algorithm_choice(case):
    rng = np.random.default_rng(7)
    C, A, B = _case_arrays(case, rng)
    want = classify.Algorithm[case["expected"]]
    got = oracle.einsum(case["C"], C, 0.0, 1.0, case["A"], A, case["B"], B)
    assert got == want


@pytest.mark.parametrize("case", GOLDEN["py_plans"], ids=lambda c: c["where"])
def test_py_plan_type(case):
    got = classify.classify_py(case["C"], case["A"], case["B"])
    assert classify.PLAN_NAMES[got] == case["expected"]


@pytest.mark.parametrize("semantics", ["cpp", "py"])
def test_known_answers(semantics):
    A2 = np.arange(1, 10, dtype=float).reshape(3, 3)
    A3 = np.arange(1, 28, dtype=float).reshape(3, 3, 3)
    cases = {"ik=ij,jk": ("ij", "ik", A2, "kj", A2), "il=ijk,jkl": ("il", "ijk", A3, "jkl", A3)}
    for sec in GOLDEN["known_answers"]:
        Cl, Al, A, Bl, B = cases[sec["section"]]
        for _ in range(10):  # Batched.cpp repeats the same product over 10 tensors
            C = np.zeros((3, 3))
            alg = oracle.einsum(Cl, C, 0.0, 1.0, Al, A, Bl, B, semantics=semantics)
            assert alg == classify.Algorithm.GEMM
            for i, j, v in sec["values"]:
                assert C[i, j] == v


class _NumpyOps:
    def __init__(self, semantics):
        self.semantics = semantics

    def einsum(self, Cl, C, c, ab, Al, A, Bl, B):
        return oracle.einsum(Cl, C, c, ab, Al, A, Bl, B, semantics=self.semantics)

    array = staticmethod(lambda x: np.array(x, dtype=np.float64))
    numpy = staticmethod(lambda x: np.array(x))
    zeros = staticmethod(lambda s: np.zeros(s))
    scalar = staticmethod(lambda x: float(x))

    @staticmethod
    def copy_into(dst, src):
        dst[...] = src


@pytest.mark.parametrize("semantics", ["cpp", "py"])
def test_water_rhf_mp2(semantics):
    q = GOLDEN["qchem"]
    res = qchem_driver.rhf_mp2(_NumpyOps(semantics), q["enuc"])
    assert res["cycles"] < 50
    assert abs(res["e_scf"] - q["e_scf"]) < q["tol"]
    assert abs(res["e_mp2"] - q["e_mp2"]) < q["tol"]
    assert abs(res["e_tot"] - q["e_tot"]) < q["tol"]


PATTERNS = [
    ("ij", "ik", "kj"), ("ij", "ki", "jk"), ("ikjl", "imjn", "mknl"), ("mbej", "jnfb", "mnef"),
    ("pq", "prqs", "rs"), ("pq", "pqrs", "rs"), ("", "ijab", "ijab"), ("ijk", "ijk", "ijk"),
    ("ij", "i", "j"), ("iajb", "iajb", "iajb"), ("i", "ij", "ji"), ("ijkl", "ijpl", "pk"),
    ("ab", "ija", "ijb"), ("", "iajb", "ibja"), ("ij", "ii", "ij"),
]


@pytest.mark.parametrize("pattern", PATTERNS, ids=lambda p: f"{p[0]}<-{p[1]}*{p[2]}")
@pytest.mark.parametrize("generic", [False, True])
def test_oracle_matches_dense_sum(pattern, generic):
    """The oracle's loops and lowerings equal a dense einsum over the same
    index space (for patterns without operand-only free indices)."""
    Cl, Al, Bl = pattern
    rng = np.random.default_rng(11)
    labels = sorted(set(Cl + Al + Bl))
    dims = {l: [4, 5, 3, 6, 2, 7][i % 6] for i, l in enumerate(labels)}
    A = rng.standard_normal([dims[l] for l in Al])
    B = rng.standard_normal([dims[l] for l in Bl])
    C = rng.standard_normal([dims[l] for l in Cl]) if Cl else np.array(rng.standard_normal())
    want = 0.5 * C + (-1.25) * np.einsum(f"{Al},{Bl}->{Cl}", A, B)
    if len(set(Cl)) != len(Cl):
        pytest.skip("numpy einsum cannot write a repeated output index")
    got = C.copy()
    oracle.einsum(Cl, got, 0.5, -1.25, Al, A, Bl, B, only_generic=generic)
    assert oracle.rel_fro(got, want) < 1e-13


@pytest.mark.parametrize("perm", list(itertools.permutations(range(4))))
def test_permute_rank4(perm):
    rng = np.random.default_rng(3)
    A = rng.standard_normal((4, 5, 6, 7))
    Al = "abcd"
    Cl = "".join(Al[p] for p in perm)
    C = np.full([A.shape[p] for p in perm], np.nan)
    oracle.permute(Cl, C, 0.0, 1.0, Al, A)
    want = np.transpose(A, perm)
    assert np.array_equal(C.view(np.uint64), np.ascontiguousarray(want).view(np.uint64))


def test_permute_prefactors_and_errors():
    rng = np.random.default_rng(4)
    A = rng.standard_normal((3, 4))
    C0 = rng.standard_normal((4, 3))
    C = C0.copy()
    oracle.permute("ji", C, 0.5, 2.0, "ij", A)
    assert np.array_equal(C, 0.5 * C0 + 2.0 * A.T)
    with pytest.raises(ValueError):
        oracle.permute("ji", np.zeros((3, 3)), 0.0, 1.0, "ij", A)


def test_permute_matches_hptt_reference():
    ref = pytest.importorskip("hptt_ref")
    if not ref.available():
        pytest.skip("oracle/_ref not built (HPTT sources absent)")
    rng = np.random.default_rng(5)
    A = rng.standard_normal((6, 7, 8, 9))
    for perm in itertools.permutations(range(4)):
        Cl = "".join("abcd"[p] for p in perm)
        C = np.zeros([A.shape[p] for p in perm])
        oracle.permute(Cl, C, 0.0, 1.0, "abcd", A)
        H = ref.permute(A, perm, alpha=1.0)
        assert np.array_equal(C.view(np.uint64), H.view(np.uint64))
        C2 = rng.standard_normal(C.shape)
        C3 = C2.copy()
        oracle.permute(Cl, C2, 0.75, -1.5, "abcd", A)
        H2 = ref.permute(A, perm, alpha=-1.5, beta=0.75, out=C3)
        np.testing.assert_allclose(C2, H2, rtol=0, atol=1e-15)
