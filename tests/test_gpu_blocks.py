"""Block-diagonal and tiled tensors on the GPU (eg_einsum_blocks through
einsums_gb300.BlockTensor / TiledTensor), against the oracle on the dense
tensors they stand for, and the reference's TEST_CASE("RHF symmetry")
(QChemTests.cpp:417): the water/STO-3G SCF in the C2v symmetry-adapted basis,
with block-diagonal one-electron matrices and tiled two-electron integrals,
to the golden E_SCF within 1e-6."""
import itertools
import json
import os

import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def eg():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import einsums_gb300
    from einsums_gb300 import build
    build.build()
    return einsums_gb300


def rand_block(eg, dims, rng):
    b = eg.BlockTensor(2, dims)
    for i, d in enumerate(dims):
        b.blocks[i].copy_(torch.from_numpy(rng.standard_normal((d, d))))
    return b


def rand_sym_tiles(eg, dims, rng, density=0.8):
    t = eg.TiledTensor([dims] * 4)
    for idx in itertools.product(*[range(len(dims))] * 4):
        i, j, k, l = idx
        if ((i == j and k == l) or (i == k and j == l) or (i == l and j == k)) and rng.random() < density:
            t.tile(idx).copy_(torch.from_numpy(rng.standard_normal(t.tile_shape(idx))))
    return t


@pytest.mark.parametrize("precision,tol", [("fp64", TOL), ("split_bf16", 1e-10)])
def test_block_gemm_matches_dense_oracle(eg, precision, tol):
    rng = np.random.default_rng(1)
    dims = [40, 0, 7, 130, 3]
    C, A, B = rand_block(eg, dims, rng), rand_block(eg, dims, rng), rand_block(eg, dims, rng)
    Cd, Ad, Bd = (x.to_dense().cpu().numpy() for x in (C, A, B))
    assert eg.einsum(0.5, "ij", C, -1.5, "ik", A, "kj", B, precision=precision) == "GEMM"
    oracle.einsum("ij", Cd, 0.5, -1.5, "ik", Ad, "kj", Bd)
    got = C.to_dense().cpu().numpy()
    assert oracle.rel_fro(got, Cd) < tol


@pytest.mark.parametrize("pattern", ["ijkl", "ikjl"])
def test_tiled_fock_build_matches_dense_oracle(eg, pattern):
    rng = np.random.default_rng(2)
    dims = [6, 0, 3, 5]
    F, D = rand_block(eg, dims, rng), rand_block(eg, dims, rng)
    g = rand_sym_tiles(eg, dims, rng)
    Fd, Dd, gd = F.to_dense().cpu().numpy(), D.to_dense().cpu().numpy(), g.to_dense().cpu().numpy()
    eg.einsum(1.0, "ij", F, 2.0, pattern, g, "kl", D)
    oracle.einsum("ij", Fd, 1.0, 2.0, pattern, gd, "kl", Dd)
    mask = eg.BlockTensor.from_dense(torch.ones(Fd.shape, dtype=torch.float64, device="cuda"), dims).to_dense()
    mask = mask.cpu().numpy() > 0
    got = F.to_dense().cpu().numpy()
    assert np.allclose(got[mask], Fd[mask], rtol=TOL, atol=TOL * np.abs(Fd).max())


def test_tiled_gemm_and_scalar(eg):
    rng = np.random.default_rng(3)
    dims = [17, 0, 33, 9]
    A, B, C = (eg.TiledTensor([dims, dims]) for _ in range(3))
    for t, dens in ((A, 0.6), (B, 0.6), (C, 0.3)):
        for idx in itertools.product(range(4), range(4)):
            if rng.random() < dens:
                t.tile(idx).copy_(torch.from_numpy(rng.standard_normal(t.tile_shape(idx))))
    Cd, Ad, Bd = (x.to_dense().cpu().numpy() for x in (C, A, B))
    eg.einsum(0.25, "ij", C, 1.0, "ik", A, "kj", B)
    oracle.einsum("ij", Cd, 0.25, 1.0, "ik", Ad, "kj", Bd)
    assert oracle.rel_fro(C.to_dense().cpu().numpy(), Cd) < TOL
    # scalar output: the sum over every pair of tiles
    E = torch.tensor(3.0, dtype=torch.float64, device="cuda")
    eg.einsum(0.5, "", E, 2.0, "ij", A, "ij", B)
    e = np.array(3.0)
    oracle.einsum("", e, 0.5, 2.0, "ij", Ad, "ij", Bd)
    assert abs(float(E.item()) - float(e)) <= TOL * max(1.0, abs(float(e)))


def _golden():
    with open(os.path.join(HERE, "golden", "golden.json")) as f:
        g = json.load(f)
    return g["qchem"], g["qchem_symmetry"]


def test_rhf_symmetry_water(eg):
    """The reference's symmetry-blocked RHF (QChemTests.cpp:417): symmetrise S, H, X and the
    TEI with the C2v adaptation matrix, cut them into irrep blocks and tiles, and run the SCF
    with every contraction on block-diagonal / tiled operands."""
    import sys
    sys.path.insert(0, HERE)
    import qchem_driver
    q, qs = _golden()
    w = qchem_driver.load_water()
    sizes = qs["irrep_sizes"]
    n = sum(sizes)
    cu = lambda x: torch.tensor(np.asarray(x, dtype=np.float64), device="cuda")
    Symm = cu(np.array(qs["symm"]).reshape(n, n))
    S, H = cu(w["S"]), cu(w["T"] + w["V"])
    ew, U = np.linalg.eigh(w["S"])
    X = cu((U * ew ** -0.5) @ U.T)
    TEI = cu(w["TEI"])
    z = lambda *s: torch.zeros(s, dtype=torch.float64, device="cuda")

    def sym2(M):
        t1, t2 = z(n, n), z(n, n)
        eg.einsum(0.0, "ij", t1, 1.0, "ik", M, "kj", Symm)
        eg.einsum(0.0, "ij", t2, 1.0, "ki", Symm, "kj", t1)
        return t2

    S_sym = eg.BlockTensor.from_dense(sym2(S), sizes)
    H_sym = eg.BlockTensor.from_dense(sym2(H), sizes)
    X_sym = eg.BlockTensor.from_dense(sym2(X), sizes)
    t1, t2 = z(n, n, n, n), z(n, n, n, n)
    eg.einsum(0.0, "ijkl", t1, 1.0, "mjkl", TEI, "mi", Symm)
    eg.einsum(0.0, "ijkl", t2, 1.0, "imkl", t1, "mj", Symm)
    eg.einsum(0.0, "ijkl", t1, 1.0, "ijml", t2, "mk", Symm)
    eg.einsum(0.0, "ijkl", t2, 1.0, "ijkm", t1, "ml", Symm)
    TEI_sym = eg.TiledTensor.from_dense(t2, [sizes] * 4, tiles=qs["tei_tiles"])
    # the tiles hold every non-zero element of the symmetrised integrals
    assert torch.allclose(TEI_sym.to_dense(), t2, atol=1e-12)
    del S_sym

    nb = len(sizes)
    temp1, Ft, C, Cocc, D = (eg.BlockTensor(2, sizes) for _ in range(5))
    Elec = torch.zeros((), dtype=torch.float64, device="cuda")

    def diag_and_density(F):
        eg.einsum(0.0, "ij", temp1, 1.0, "ik", F, "kj", X_sym)
        eg.einsum(0.0, "ij", Ft, 1.0, "kj", temp1, "ki", X_sym)
        evals = []
        Ct = eg.BlockTensor(2, sizes)
        for b in range(nb):
            if sizes[b] == 0:
                evals.append(np.zeros(0))
                continue
            e, v = np.linalg.eigh(Ft[b].cpu().numpy())
            evals.append(e)
            Ct[b] = v
        eg.einsum(0.0, "ij", C, 1.0, "kj", Ct, "ik", X_sym)
        # aufbau over the irreps (the reference's update_Cocc): 5 doubly occupied orbitals
        occ = [0] * nb
        for _ in range(5):
            best, pick = np.inf, -1
            for b in range(nb):
                if occ[b] < sizes[b] and evals[b][occ[b]] < best:
                    best, pick = evals[b][occ[b]], b
            occ[pick] += 1
        Cocc.zero()
        for b in range(nb):
            if occ[b]:
                Cocc.blocks[b][:, :occ[b]] = C.blocks[b][:, :occ[b]]
        eg.einsum(0.0, "ij", D, 1.0, "im", Cocc, "jm", Cocc)

    def energy(F):
        eg.einsum(0.0, "", Elec, 1.0, "ij", F, "ij", D)
        eg.einsum(1.0, "", Elec, 1.0, "ij", H_sym, "ij", D)
        return float(Elec.item()) + q["enuc"]

    F = H_sym.copy()
    diag_and_density(F)
    e0, e1, cycles = energy(F), 0.0, 0
    while abs(e0 - e1) > 1e-10 and cycles < 50:
        e1 = e0
        F = H_sym.copy()
        eg.einsum(1.0, "ij", F, 2.0, "ijkl", TEI_sym, "kl", D)
        eg.einsum(1.0, "ij", F, -1.0, "ikjl", TEI_sym, "kl", D)
        diag_and_density(F)
        e0 = energy(F)
        cycles += 1
    assert cycles < 50
    assert abs(e0 - q["e_scf"]) < q["tol"], (e0, q["e_scf"])
