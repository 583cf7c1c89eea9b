"""Complex128 einsum with conjugation on the GPU (eg_einsum_complex): the
reference's einsum<ConjA, ConjB> on std::complex<double> tensors
(Dispatch.hpp:48,136; BaseAlgebra.hpp:33-38), checked against NumPy's complex
einsum of the same operands (conjugated where asked) to 1e-12 relative
Frobenius error in FP64 and 1e-10 in the split form, for every algorithm
choice and for complex prefactors."""
import numpy as np
import pytest

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


def crand(rng, shape):
    return rng.standard_normal(shape) + 1j * rng.standard_normal(shape)


def rel(a, b):
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


PATTERNS = [("ij", "ik", "kj", "GEMM"), ("i", "ij", "j", "GEMV"), ("", "ij", "ij", "DOT"),
            ("ikjl", "imjn", "mknl", "GENERIC"), ("ij", "i", "j", "GER"), ("ijk", "ijk", "ijk", "DIRECT")]


@pytest.mark.parametrize("conj", [(False, False), (True, False), (False, True), (True, True)])
@pytest.mark.parametrize("pattern", PATTERNS, ids=[p[3] for p in PATTERNS])
def test_complex_einsum_matches_numpy(eg, pattern, conj):
    Cl, Al, Bl, alg = pattern
    rng = np.random.default_rng(len(Al) * 7 + conj[0] + 2 * conj[1])
    dims = {l: 5 + (ord(l) % 4) for l in set(Cl + Al + Bl)}
    A = crand(rng, [dims[l] for l in Al])
    B = crand(rng, [dims[l] for l in Bl])
    C0 = crand(rng, [dims[l] for l in Cl]) if Cl else np.array(0.5 - 0.25j)
    cp, ab = 0.5 - 0.75j, 1.25 + 0.5j
    Aop = A.conj() if conj[0] else A
    Bop = B.conj() if conj[1] else B
    want = cp * C0 + ab * np.einsum(f"{Al},{Bl}->{Cl}", Aop, Bop)
    tC = torch.tensor(C0, dtype=torch.complex128, device="cuda")
    got_alg = eg.einsum(cp, Cl, tC, ab, Al, torch.tensor(A, device="cuda"), Bl, torch.tensor(B, device="cuda"),
                        conj_A=conj[0], conj_B=conj[1])
    assert got_alg == alg
    assert rel(tC.cpu().numpy(), want) < 1e-12


def test_complex_real_prefactors_split_and_plans(eg):
    rng = np.random.default_rng(5)
    A, B = crand(rng, (60, 70)), crand(rng, (70, 50))
    C0 = crand(rng, (60, 50))
    want = 0.0 * C0 + 2.0 * (A.conj() @ B)
    tC = torch.tensor(C0, device="cuda")
    eg.einsum(0.0, "ij", tC, 2.0, "ik", torch.tensor(A, device="cuda"), "kj", torch.tensor(B, device="cuda"),
              conj_A=True, precision="split_bf16")
    assert rel(tC.cpu().numpy(), want) < 1e-10
    # EinsumsPy plans take complex tensors too (Python semantics)
    tC = torch.zeros((60, 50), dtype=torch.complex128, device="cuda")
    eg.compile_plan("ij", "ik", "kj").execute(0.0, tC, 1.0, torch.tensor(A, device="cuda"),
                                              torch.tensor(B, device="cuda"))
    assert rel(tC.cpu().numpy(), A @ B) < 1e-12
    with pytest.raises(TypeError):
        eg.einsum(0.0, "ij", tC, 1.0, "ik", torch.zeros((60, 70), dtype=torch.float64, device="cuda"), "kj",
                  torch.tensor(B, device="cuda"))
