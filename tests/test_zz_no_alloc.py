"""GPU test of eg_dot_noalloc, the entry point for callers that cannot let the
library allocate device memory (their memory belongs to another allocator, or
they run latency-critical loops).  It must match the regular dot entry point
(eg_einsum with a rank-0 output) within the contraction tolerance of the test
suite, on two calls in a row with different inputs, and reject lengths beyond
its fixed scratch.  Kept in a file collected last so a failing run has already
run every other test; it also passes alone in a fresh process."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative error bound used for contractions throughout the suite


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from einsums_gb300 import _lib, build
    build.build()
    return _lib.load()


def _regular_dot(lib, A, B, cp, ab, c0, semantics=0):
    from einsums_gb300 import _lib
    opt = _lib.EgOptions()
    lib.eg_options_default(ctypes.byref(opt))
    opt.semantics = semantics
    C = torch.full((), c0, dtype=torch.float64, device="cuda")
    tC, tA, tB = _lib.EgTensor(), _lib.EgTensor(), _lib.EgTensor()
    tC.data, tC.rank = C.data_ptr(), 0
    for t, x in ((tA, A), (tB, B)):
        t.data, t.rank = x.data_ptr(), 1
        t.extent[0], t.stride[0] = x.numel(), 1
    lab = _lib.labels("i")
    st = lib.eg_einsum(cp, lab, ctypes.byref(tC), ab, lab, ctypes.byref(tA), lab, ctypes.byref(tB), ctypes.byref(opt),
                       ctypes.c_void_p(torch.cuda.current_stream().cuda_stream), None)
    assert st == 0, lib.eg_last_error()
    return float(C.item())


def _noalloc_dot(lib, A, B, cp, ab, c0):
    C = torch.full((), c0, dtype=torch.float64, device="cuda")
    st = lib.eg_dot_noalloc(cp, ctypes.c_void_p(C.data_ptr()), ab, ctypes.c_void_p(A.data_ptr()),
                            ctypes.c_void_p(B.data_ptr()), A.numel(),
                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.eg_last_error()
    return float(C.item())


def test_noalloc_dot_matches_regular_entry_point_twice(lib):
    gen = torch.Generator(device="cuda")
    gen.manual_seed(11)
    for n, cp, ab, c0 in ((3_000_001, 0.5, 0.25, 2.0), (777_777, 1.0, -1.5, -3.0)):
        A = torch.randn(n, generator=gen, dtype=torch.float64, device="cuda")
        B = torch.randn(n, generator=gen, dtype=torch.float64, device="cuda")
        want = _regular_dot(lib, A, B, cp, ab, c0)
        got = _noalloc_dot(lib, A, B, cp, ab, c0)
        assert abs(got - want) <= TOL * max(abs(want), 1.0), (n, got, want)
        ref = cp * c0 + ab * float(np.dot(A.cpu().numpy(), B.cpu().numpy()))
        assert abs(got - ref) <= TOL * max(abs(ref), 1.0)


@pytest.mark.parametrize("n", [1, 255, 257, 65536, 65537, 2 * 65536 + 1])
def test_noalloc_dot_block_edges(lib, n):
    """Lengths below one block of threads, at and just past one 65536-element
    chunk, and with a final chunk of a single element."""
    gen = torch.Generator(device="cuda")
    gen.manual_seed(n)
    A = torch.randn(n, generator=gen, dtype=torch.float64, device="cuda")
    B = torch.randn(n, generator=gen, dtype=torch.float64, device="cuda")
    want = _regular_dot(lib, A, B, 0.75, 1.25, 0.5)
    ref = 0.75 * 0.5 + 1.25 * float(np.dot(A.cpu().numpy(), B.cpu().numpy()))
    for _ in range(2):
        got = _noalloc_dot(lib, A, B, 0.75, 1.25, 0.5)
        assert abs(got - want) <= TOL * max(abs(want), 1.0), (n, got, want)
        assert abs(got - ref) <= TOL * max(abs(ref), 1.0), (n, got, ref)


def test_noalloc_dot_zero_prefactor_keeps_cpp_dot_semantics(lib):
    """C is scaled by C_prefactor even when it is 0, as eg_einsum's C++ DOT
    choice does: a NaN in C survives.  With finite C the two entry points agree."""
    gen = torch.Generator(device="cuda")
    gen.manual_seed(5)
    A = torch.randn(1000, generator=gen, dtype=torch.float64, device="cuda")
    B = torch.randn(1000, generator=gen, dtype=torch.float64, device="cuda")
    assert np.isnan(_noalloc_dot(lib, A, B, 0.0, 1.0, float("nan")))
    assert np.isnan(_regular_dot(lib, A, B, 0.0, 1.0, float("nan")))
    got = _noalloc_dot(lib, A, B, 0.0, 1.0, 7.0)
    want = _regular_dot(lib, A, B, 0.0, 1.0, 7.0)
    assert abs(got - want) <= TOL * max(abs(want), 1.0)


def test_noalloc_dot_limits(lib):
    C = torch.full((), 4.0, dtype=torch.float64, device="cuda")
    # empty input: only the prefactor applies
    st = lib.eg_dot_noalloc(0.5, ctypes.c_void_p(C.data_ptr()), 1.0, None, None, 0,
                            ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0 and float(C.item()) == 2.0
    # beyond the fixed scratch: rejected before any device work
    st = lib.eg_dot_noalloc(0.0, ctypes.c_void_p(C.data_ptr()), 1.0, ctypes.c_void_p(16), ctypes.c_void_p(16),
                            (1 << 28) + 1, None)
    assert st == 4
    assert b"exceeds the maximum" in lib.eg_last_error()
