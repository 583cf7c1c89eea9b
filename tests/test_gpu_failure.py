"""Failure detection on the GPU without a fault: a bounded device wait that
nothing satisfies gives up after its limit, the kernel frees its tensor memory
and returns, the host reads EG_ERROR_TIMEOUT from the stream's status record,
and the context stays usable (a split-BF16 contraction on the same stream
afterwards runs and agrees with FP64)."""
import ctypes

import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

EG_ERROR_TIMEOUT = 7
SELFTEST_CODE = 6


@pytest.fixture(scope="module")
def lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from einsums_gb300 import _lib, build
    build.build()
    return _lib.load()


def _status(lib, stream):
    code = ctypes.c_int32(-1)
    st = lib.eg_stream_status(ctypes.c_void_p(stream), ctypes.byref(code))
    return st, code.value


def test_wait_timeout_is_reported_and_the_context_survives(lib):
    import einsums_gb300 as eg
    stream = torch.cuda.current_stream().cuda_stream
    assert _status(lib, stream) == (0, 0)
    assert lib.eg_selftest_wait_timeout(20_000_000, ctypes.c_void_p(stream)) == 0  # 20 ms
    st, code = _status(lib, stream)
    assert st == EG_ERROR_TIMEOUT and code == SELFTEST_CODE
    assert b"gave up" in lib.eg_last_error()
    assert _status(lib, stream) == (0, 0)  # reading the record clears it

    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    A = torch.randn((300, 200), generator=g, dtype=torch.float64, device="cuda")
    B = torch.randn((200, 250), generator=g, dtype=torch.float64, device="cuda")
    C = torch.zeros((300, 250), dtype=torch.float64, device="cuda")
    eg.einsum(0.0, "ij", C, 1.0, "ik", A, "kj", B, precision="split_bf16")
    ref = A @ B
    assert float(torch.linalg.vector_norm(C - ref) / torch.linalg.vector_norm(ref)) < 1e-10
    assert _status(lib, stream) == (0, 0)


def test_timeouts_on_two_streams_are_kept_apart(lib):
    s1 = torch.cuda.Stream()
    s2 = torch.cuda.Stream()
    assert lib.eg_selftest_wait_timeout(5_000_000, ctypes.c_void_p(s1.cuda_stream)) == 0
    s2.synchronize()
    assert _status(lib, s2.cuda_stream) == (0, 0)
    assert _status(lib, s1.cuda_stream) == (EG_ERROR_TIMEOUT, SELFTEST_CODE)
