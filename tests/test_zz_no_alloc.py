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


def _regular_dot(lib, A, B, cp, ab, c0):
    from einsums_gb300 import _lib
    C = torch.full((), c0, dtype=torch.float64, device="cuda")
    tC, tA, tB = _lib.EgTensor(), _lib.EgTensor(), _lib.EgTensor()
    tC.data, tC.rank = C.data_ptr(), 0
    for t, x in ((tA, A), (tB, B)):
        t.data, t.rank = x.data_ptr(), 1
        t.extent[0], t.stride[0] = x.numel(), 1
    lab = _lib.labels("i")
    st = lib.eg_einsum(cp, lab, ctypes.byref(tC), ab, lab, ctypes.byref(tA), lab, ctypes.byref(tB), None,
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
