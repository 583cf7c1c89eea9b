"""EinsumsPy plans on host NumPy buffers: Plan.execute copies the operands to
the device, contracts there and copies the result back into C in place, as
the reference's execute accepts buffers (EinsumsPy/TensorAlgebra/src/Export.cpp:17-32).
Checked against the oracle with the Python plan semantics."""
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


@pytest.mark.parametrize("pattern", [("ij", "ik", "kj"), ("", "ij", "ij"), ("i", "ij", "j"), ("ikjl", "imjn", "mknl")])
def test_plan_execute_on_numpy(eg, pattern):
    Cl, Al, Bl = pattern
    rng = np.random.default_rng(7)
    dims = {l: 5 + (ord(l) % 4) for l in set(Cl + Al + Bl)}
    A = rng.standard_normal([dims[l] for l in Al])
    B = rng.standard_normal([dims[l] for l in Bl])
    C = rng.standard_normal([dims[l] for l in Cl]) if Cl else np.array(1.5)
    ref = C.copy()
    oracle.einsum(Cl, ref, 0.5, 2.0, Al, A, Bl, B, semantics="py")
    plan = eg.compile_plan(Cl, Al, Bl)
    plan.execute(0.5, C, 2.0, A, B)
    assert oracle.rel_fro(C, ref) < 1e-12


def test_plan_execute_on_numpy_lists_and_mixed(eg):
    rng = np.random.default_rng(8)
    As = [rng.standard_normal((6, 4 + k)) for k in range(3)]
    Bs = [rng.standard_normal((4 + k, 9)) for k in range(3)]
    Cs = [np.zeros((6, 9)) for _ in range(3)]
    plan = eg.compile_plan("ij", "ik", "kj")
    plan.execute(0.0, Cs, 1.0, As, Bs)
    for a, b, c in zip(As, Bs, Cs):
        assert np.allclose(c, a @ b, rtol=1e-12, atol=1e-12)
    # a device C with host operands, and a strided (non-contiguous) host C
    Cd = torch.zeros((6, 9), dtype=torch.float64, device="cuda")
    plan.execute(0.0, Cd, 1.0, As[0], Bs[0])
    assert np.allclose(Cd.cpu().numpy(), As[0] @ Bs[0], rtol=1e-12, atol=1e-12)
    big = np.ones((12, 18))
    view = big[::2, ::2]
    plan.execute(1.0, view, 1.0, As[1], Bs[1])
    assert np.allclose(view, 1.0 + As[1] @ Bs[1], rtol=1e-12, atol=1e-12)
    assert np.all(big[1::2] == 1.0)
    with pytest.raises(TypeError):
        plan.execute(0.0, np.zeros((6, 9), dtype=np.float32), 1.0, As[0], Bs[0])
