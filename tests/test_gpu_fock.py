"""eg_fock_jk_symmetric on the GPU: F = fp F + jp J + kp K for 8-fold
symmetric g and symmetric D, reading only the canonical eighth of g, against
the oracle's two general contractions (the reference's RHF Fock update
F += 2 einsum(pq <- pqrs, rs), F -= einsum(pq <- prqs, rs);
QChemTests.cpp:300-303): 1e-12 relative Frobenius error in FP64, 1e-10 in
the split form (5 slices), with the error falling as slices are added."""
import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12
SPLIT_TOL = 1e-10


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


def oracle_fock(F0, g, D, fp, jp, kp):
    F = F0.copy()
    oracle.einsum("pq", F, fp, jp, "pqrs", g, "rs", D)
    oracle.einsum("pq", F, 1.0, kp, "prqs", g, "rs", D)
    return F


# n = 33, 65, 70 and 100 cross the 32-lane chunks of q and s and the groups of
# four r of the line passes
@pytest.mark.parametrize("precision,tol", [("fp64", TOL), ("split_bf16", SPLIT_TOL)])
@pytest.mark.parametrize("n", [1, 2, 7, 24, 33, 65, 70, 100])
def test_fock_symmetric_matches_two_contractions(eg, n, precision, tol):
    from einsums_gb300 import workloads
    g, D = workloads.fock_inputs(n, seed=n)
    F0 = np.random.default_rng(n).standard_normal((n, n))
    want = oracle_fock(F0, g, D, 1.0, 2.0, -1.0)
    tF = cu(F0)
    eg.fock_jk_symmetric(tF, cu(g), cu(D), precision=precision)
    assert oracle.rel_fro(tF.cpu().numpy(), want) < tol


def test_fock_symmetric_split_error_falls_with_slices(eg):
    from einsums_gb300 import workloads
    n = 40
    g, D = workloads.fock_inputs(n, seed=4)
    want = oracle_fock(np.zeros((n, n)), g, D, 0.0, 2.0, -1.0)
    tg, tD = cu(g), cu(D)
    errs = {}
    for S in (3, 4, 5, 6):
        tF = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        eg.fock_jk_symmetric(tF, tg, tD, F_prefactor=0.0, precision="split_bf16", slices=S)
        rep = eg.last_split_report()
        assert rep["slices"] == S
        errs[S] = oracle.rel_fro(tF.cpu().numpy(), want)
        assert errs[S] < 100 * rep["error_bound"], (S, errs[S], rep["error_bound"])
    assert errs[3] > errs[4] > errs[5] > errs[6]


def test_fock_symmetric_prefactors_and_zero_f(eg):
    from einsums_gb300 import workloads
    n = 30
    g, D = workloads.fock_inputs(n, seed=3)
    F0 = np.random.default_rng(1).standard_normal((n, n))
    want = oracle_fock(F0, g, D, 0.5, 0.75, 1.25)
    tF = cu(F0)
    eg.fock_jk_symmetric(tF, cu(g), cu(D), F_prefactor=0.5, J_prefactor=0.75, K_prefactor=1.25)
    assert oracle.rel_fro(tF.cpu().numpy(), want) < TOL
    # F_prefactor == 0: F is not read (a NaN there does not survive)
    tF = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
    eg.fock_jk_symmetric(tF, cu(g), cu(D), F_prefactor=0.0)
    want = oracle_fock(np.zeros((n, n)), g, D, 0.0, 2.0, -1.0)
    assert oracle.rel_fro(tF.cpu().numpy(), want) < TOL


def test_fock_symmetric_is_deterministic_and_matches_gpu_einsum(eg):
    from einsums_gb300 import workloads
    n = 48
    g, D = workloads.fock_inputs(n, seed=5)
    tg, tD = cu(g), cu(D)
    outs = []
    for prec in ("fp64", "fp64", "split_bf16", "split_bf16"):
        tF = torch.zeros((n, n), dtype=torch.float64, device="cuda")
        eg.fock_jk_symmetric(tF, tg, tD, F_prefactor=0.0, precision=prec)
        outs.append(tF.cpu().numpy())
    assert np.array_equal(outs[0].view(np.uint64), outs[1].view(np.uint64))
    assert np.array_equal(outs[2].view(np.uint64), outs[3].view(np.uint64))
    ref = torch.zeros((n, n), dtype=torch.float64, device="cuda")
    eg.einsum(0.0, "pq", ref, 2.0, "pqrs", tg, "rs", tD)
    eg.einsum(1.0, "pq", ref, -1.0, "prqs", tg, "rs", tD)
    assert oracle.rel_fro(outs[0], ref.cpu().numpy()) < TOL


@pytest.mark.parametrize("precision", ["fp64", "split_bf16"])
def test_fock_symmetric_water_energy(eg, precision):
    """The RHF energy of the reference's water/STO-3G fixture with the Fock
    matrix built by the symmetric entry point (E_SCF to 1e-6)."""
    import json
    import os
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, here)
    import qchem_driver
    with open(os.path.join(here, "golden", "golden.json")) as f:
        q = json.load(f)["qchem"]

    class Ops:
        def einsum(self, Cl, C, c, ab, Al, A, Bl, B):
            return eg.einsum(c, Cl, C, ab, Al, A, Bl, B)

        def __init__(self, precision):
            self.precision = precision

        def fock(self, F, g, D):
            eg.fock_jk_symmetric(F, g, D, precision=self.precision)
        array = staticmethod(lambda x: torch.tensor(np.asarray(x, dtype=np.float64), device="cuda"))
        numpy = staticmethod(lambda x: x.cpu().numpy())
        zeros = staticmethod(lambda s: torch.zeros(s, dtype=torch.float64, device="cuda"))
        scalar = staticmethod(lambda x: float(x.item()))

        @staticmethod
        def copy_into(dst, src):
            dst.copy_(torch.as_tensor(np.asarray(src, dtype=np.float64)))

    res = qchem_driver.rhf_mp2(Ops(precision), q["enuc"])
    assert abs(res["e_scf"] - q["e_scf"]) < q["tol"]


def test_fock_symmetric_rejects_bad_arguments(eg):
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device="cuda")
    from einsums_gb300._lib import DimensionError
    with pytest.raises(DimensionError):
        eg.fock_jk_symmetric(z(3, 3), z(3, 3, 3, 4), z(3, 3))
    with pytest.raises(DimensionError):
        eg.fock_jk_symmetric(z(3, 3), z(3, 3, 3, 3), z(4, 4))
    from einsums_gb300._lib import EinsumsError
    with pytest.raises(EinsumsError):
        eg.fock_jk_symmetric(z(3, 3), z(3, 3, 3, 3), z(3, 3), precision="split_bf16", slices=2)
