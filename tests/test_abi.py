"""C-ABI checks that need no GPU: the library loads, exports every symbol the
header declares, reports the reference's algorithm choices and plan types, and
rejects bad arguments with status codes (no device work is issued)."""
import ctypes
import json
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "einsums_gb300.h")
GOLDEN = json.load(open(os.path.join(ROOT, "tests", "golden", "golden.json")))


@pytest.fixture(scope="module")
def lib():
    from einsums_gb300 import _lib
    from einsums_gb300 import build
    build.build()
    return _lib.load()


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(eg_[a-z_0-9]+)\s*\(", text)))


def test_header_symbols_exported(lib):
    from einsums_gb300 import _lib
    syms = declared_symbols()
    assert len(syms) >= 15
    for s in syms:
        assert hasattr(lib, s), f"{s} declared in include/einsums_gb300.h but not exported"
        assert s in _lib.PROTOTYPES, f"{s} has no ctypes prototype"


def test_version_and_status_strings(lib):
    assert b"sm_103a" in lib.eg_version()
    assert lib.eg_status_string(3) == b"dimension error"


@pytest.mark.parametrize("case", GOLDEN["cpp_choices"], ids=lambda c: c["where"].split("/")[-1])
def test_cpp_choice_through_abi(lib, case):
    """Compile-time choice (before stride vetoes) equals the reference's, except
    where the reference test relies on a runtime veto of a strided view."""
    from einsums_gb300 import core
    from einsums_gb300._lib import SEMANTICS_CPP
    alg = core.ALGORITHMS[core.classify(case["C"], case["A"], case["B"], SEMANTICS_CPP)]
    if case["where"].endswith("Einsum7.cpp:209"):
        assert alg == "GEMM"  # the strided view vetoes it to GENERIC at run time (GPU test)
    else:
        assert alg == case["expected"]


@pytest.mark.parametrize("case", GOLDEN["py_plans"], ids=lambda c: c["where"])
def test_compile_plan_types(lib, case):
    import einsums_gb300 as eg
    plan = eg.compile_plan(case["C"], case["A"], case["B"])
    assert type(plan).__name__ == case["expected"]


def test_classifier_agrees_with_oracle_on_random_patterns(lib):
    import random

    import classify
    from einsums_gb300 import core
    from einsums_gb300._lib import SEMANTICS_CPP, SEMANTICS_PYTHON
    rng = random.Random(1)
    letters = "ijklmn"
    for _ in range(3000):
        mk = lambda: "".join(rng.choice(letters) for _ in range(rng.randint(0, 4)))
        C, A, B = mk(), mk(), mk()
        assert core.classify(C, A, B, SEMANTICS_CPP) == int(classify.classify_cpp(C, A, B)), (C, A, B)
        assert core.classify(C, A, B, SEMANTICS_PYTHON) == int(classify.classify_py(C, A, B)), (C, A, B)


def test_bad_arguments_return_status(lib):
    from einsums_gb300 import _lib
    T = _lib.EgTensor
    C, A, B = T(), T(), T()
    C.rank, A.rank, B.rank = 9, 1, 1
    lab = _lib.labels("ijklmnopq")
    st = lib.eg_einsum(0.0, lab, ctypes.byref(C), 1.0, lab, ctypes.byref(A), lab, ctypes.byref(B), None, None, None)
    assert st == 2  # rank error
    st = lib.eg_einsum(0.0, lab, None, 1.0, lab, ctypes.byref(A), lab, ctypes.byref(B), None, None, None)
    assert st == 1
    assert b"C is NULL" in lib.eg_last_error()
    # inconsistent extents: C(i) with i=3 against A(i) with i=4 (zero-size data, so no device access)
    C.rank, A.rank, B.rank = 1, 1, 1
    C.extent[0], A.extent[0], B.extent[0] = 3, 4, 0
    C.stride[0] = A.stride[0] = B.stride[0] = 1
    C.data = A.data = B.data = 16
    st = lib.eg_einsum(0.0, _lib.labels("i"), ctypes.byref(C), 1.0, _lib.labels("i"), ctypes.byref(A),
                       _lib.labels("j"), ctypes.byref(B), None, None, None)
    assert st == 3
    # permute with a too-small output
    st = lib.eg_permute(0.0, _lib.labels("i"), ctypes.byref(C), 1.0, _lib.labels("i"), ctypes.byref(A), None)
    assert st == 3
    # the wait self-test refuses limits outside (0, 2 s] before touching the device
    assert lib.eg_selftest_wait_timeout(0, None) == 1
    assert lib.eg_selftest_wait_timeout(3_000_000_000, None) == 1


def test_memory_budget_refuses(lib):
    assert lib.eg_set_memory_budget(1024) == 0
    p = ctypes.c_void_p()
    assert lib.eg_device_alloc(1 << 20, ctypes.byref(p)) == 6
    assert b"budget" in lib.eg_last_error()
    assert lib.eg_set_memory_budget(0) == 0
