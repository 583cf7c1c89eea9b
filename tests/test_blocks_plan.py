"""Host logic of the block-sparse einsum, without a GPU: the tile combinations
that einsums_gb300.blocks.block_items lists, run item by item with the
oracle under eg_einsum_blocks' rules (every distinct C block scaled by
C_prefactor once, zeroed when it is 0; later items add), must reproduce the
oracle's einsum of the dense tensors the blocked ones stand for (missing
tiles are zero).  The reference loops over the same combinations
(Backends/BlockAlgebra.hpp:21-50, Backends/TileAlgebra.hpp:21-97)."""
import itertools

import numpy as np
import pytest

import oracle

torch = pytest.importorskip("torch")


def run_items(cp, ab, Cl, Al, Bl, Cs, As, Bs):
    first = {}
    for c, a, b in zip(Cs, As, Bs):
        key = (c.data_ptr(), tuple(c.shape), tuple(c.stride()))
        cn = c.numpy()
        if key not in first:
            first[key] = True
            if cp == 0.0:
                cn[...] = 0.0
            else:
                cn *= cp
        oracle.einsum(Cl, cn, 1.0, ab, Al, np.ascontiguousarray(a.numpy()), Bl, np.ascontiguousarray(b.numpy()))


def random_tiled(sizes_per_index, density, rng):
    from einsums_gb300.blocks import TiledTensor
    t = TiledTensor(sizes_per_index, device="cpu")
    for idx in itertools.product(*[range(len(s)) for s in sizes_per_index]):
        if rng.random() < density:
            t.tile(idx).copy_(torch.from_numpy(rng.standard_normal(t.tile_shape(idx))))
    return t


def random_symmetric_tiled(dims, density, rng):
    """Rank-4 tiles whose irreps pair up ((I,I,K,K), (I,K,I,K), (I,K,K,I)), as the tiles of
    two-electron integrals over symmetry-adapted orbitals do."""
    from einsums_gb300.blocks import TiledTensor
    t = TiledTensor([dims] * 4, device="cpu")
    for idx in itertools.product(*[range(len(dims))] * 4):
        i, j, k, l = idx
        if not ((i == j and k == l) or (i == k and j == l) or (i == l and j == k)):
            continue
        if rng.random() < density:
            t.tile(idx).copy_(torch.from_numpy(rng.standard_normal(t.tile_shape(idx))))
    return t


def random_block(rank, dims, rng):
    from einsums_gb300.blocks import BlockTensor
    b = BlockTensor(rank, dims, device="cpu")
    for i, d in enumerate(dims):
        b.blocks[i].copy_(torch.from_numpy(rng.standard_normal((d,) * rank)))
    return b


@pytest.mark.parametrize("case", ["block_gemm", "tiled_gemm", "fock_j", "fock_k", "block_dot", "dense_times_block",
                                  "tiled_to_dense"])
def test_block_items_reproduce_dense_einsum(case):
    from einsums_gb300 import blocks
    rng = np.random.default_rng(sum(map(ord, case)))
    dims = [3, 0, 5, 2]
    cp, ab = 0.5, -1.25
    if case == "block_gemm":
        Cl, Al, Bl = "ij", "ik", "kj"
        C, A, B = random_block(2, dims, rng), random_block(2, dims, rng), random_block(2, dims, rng)
    elif case == "tiled_gemm":
        Cl, Al, Bl = "ij", "ik", "kj"
        C = random_tiled([dims, dims], 0.5, rng)
        A, B = random_tiled([dims, dims], 0.6, rng), random_tiled([dims, dims], 0.6, rng)
    elif case == "fock_j":
        Cl, Al, Bl = "ij", "ijkl", "kl"
        C, A, B = random_block(2, dims, rng), random_symmetric_tiled(dims, 0.7, rng), random_block(2, dims, rng)
    elif case == "fock_k":
        Cl, Al, Bl = "ij", "ikjl", "kl"
        C, A, B = random_block(2, dims, rng), random_symmetric_tiled(dims, 0.7, rng), random_block(2, dims, rng)
    elif case == "block_dot":
        Cl, Al, Bl = "", "ij", "ij"
        C, A, B = torch.tensor(2.0, dtype=torch.float64), random_block(2, dims, rng), random_block(2, dims, rng)
    elif case == "dense_times_block":
        Cl, Al, Bl = "ij", "ik", "kj"
        n = sum(dims)
        C = torch.from_numpy(rng.standard_normal((n, n)))
        A, B = torch.from_numpy(rng.standard_normal((n, n))), random_block(2, dims, rng)
    else:
        Cl, Al, Bl = "ij", "ik", "kj"
        n = sum(dims)
        C = torch.from_numpy(rng.standard_normal((n, n)))
        A, B = random_tiled([dims, dims], 0.7, rng), random_tiled([dims, dims], 0.7, rng)

    def dense(x):
        return x.to_dense().numpy().copy() if blocks.is_blocked(x) else x.numpy().copy()

    Ad, Bd = dense(A), dense(B)
    Cs, As, Bs, untouched = blocks.block_items(Cl, C, Al, A, Bl, B)
    assert len(Cs) == len(As) == len(Bs)
    # the expected result: dense einsum on the combinations' support
    want = dense(C)
    run_items(cp, ab, Cl, Al, Bl, Cs, As, Bs)
    for t in untouched:
        t.mul_(cp)
    got = dense(C)
    if case in ("block_gemm", "fock_j", "fock_k"):
        # a BlockTensor C holds only its diagonal blocks: compare those
        ref = want.copy()
        oracle.einsum(Cl, ref, cp, ab, Al, Ad, Bl, Bd)
        mask = dense(blocks.BlockTensor.from_dense(torch.ones(ref.shape, dtype=torch.float64), dims)) > 0
        assert np.allclose(got[mask], ref[mask], rtol=1e-12, atol=1e-12)
    elif case == "tiled_gemm":
        ref = want.copy()
        oracle.einsum(Cl, ref, cp, ab, Al, Ad, Bl, Bd)
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-12)
    elif case == "block_dot":
        ref = np.array(float(want))
        oracle.einsum("", ref, cp, ab, Al, Ad, Bl, Bd)
        assert abs(float(got) - float(ref)) < 1e-12 * max(1.0, abs(float(ref)))
    else:
        ref = want.copy()
        oracle.einsum(Cl, ref, 1.0, ab, Al, Ad, Bl, Bd)
        # a dense C is scaled only where a combination writes it (its tile views)
        written = np.zeros(ref.shape, dtype=bool)
        for c in Cs:
            off = (c.storage_offset() // c.stride(0), c.storage_offset() % c.stride(0))
            written[off[0]:off[0] + c.shape[0], off[1]:off[1] + c.shape[1]] = True
        base = np.where(written, cp * want, want)
        oracle.einsum(Cl, base, 1.0, ab, Al, Ad, Bl, Bd)
        assert np.allclose(got, base, rtol=1e-12, atol=1e-12)


def test_block_items_reject_an_off_diagonal_block_c():
    from einsums_gb300 import blocks
    from einsums_gb300._lib import NotSupportedError
    rng = np.random.default_rng(1)
    dims = [2, 3]
    with pytest.raises(NotSupportedError):
        blocks.block_items("ij", random_block(2, dims, rng), "ik", torch.from_numpy(rng.standard_normal((5, 5))),
                           "kj", random_block(2, dims, rng))


def test_block_items_reject_mismatched_tiling():
    from einsums_gb300 import blocks
    from einsums_gb300._lib import DimensionError
    rng = np.random.default_rng(0)
    with pytest.raises(DimensionError):
        blocks.block_items("ij", random_block(2, [2, 3], rng), "ik", random_block(2, [3, 2], rng), "kj",
                           random_block(2, [2, 3], rng))
