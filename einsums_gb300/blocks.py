"""Block-diagonal and tiled tensors on the GPU, contracted through the grouped launch.

``BlockTensor`` is the reference's block-diagonal tensor (Einsums/Tensor/BlockTensor.hpp):
block ``i`` is a dense tensor whose every index runs over ``block_range(i)``.
``TiledTensor`` is the reference's tiled tensor (Einsums/Tensor/TiledTensor.hpp): each
index is cut into tiles of given sizes and only the tiles that were created are stored.
Both hold their blocks as CUDA float64 tensors.

``einsum`` on these operands follows the reference's special dispatch
(Backends/BlockAlgebra.hpp:21-50, Backends/TileAlgebra.hpp:21-97): every combination of
tiles over the unique indices, in the order of the indices of C, then A, then B, is one
contraction of A's tile with B's tile into C's tile; missing and empty tiles are skipped,
C is scaled by C_prefactor once.  Dense operands (and a dense C) take the view of the tile
ranges.  The combinations go to ``eg_einsum_blocks`` as one list: items that write
different C tiles share one grouped launch, and contributions to one C tile add in order.
"""
from __future__ import annotations

import ctypes
import itertools
from typing import Dict, List, Sequence, Tuple

import torch

from . import _lib
from .core import ALGORITHMS, _check_device, _options, _stream, _tensor
from ._lib import SEMANTICS_CPP


def _ranges(sizes: Sequence[int]) -> List[Tuple[int, int]]:
    out, off = [], 0
    for s in sizes:
        out.append((off, int(s)))
        off += int(s)
    return out


class BlockTensor:
    """Block-diagonal tensor of ``rank`` indices with blocks of the given sizes."""

    def __init__(self, rank: int, block_dims: Sequence[int], device="cuda", dtype=torch.float64):
        self.rank = int(rank)
        self.block_dims = [int(d) for d in block_dims]
        self.blocks = [torch.zeros((d,) * self.rank, dtype=dtype, device=device) for d in self.block_dims]

    @property
    def num_blocks(self) -> int:
        return len(self.blocks)

    def block_range(self, i: int) -> Tuple[int, int]:
        off = sum(self.block_dims[:i])
        return off, off + self.block_dims[i]

    def block(self, i: int) -> torch.Tensor:
        return self.blocks[i]

    def __getitem__(self, i: int) -> torch.Tensor:
        return self.blocks[i]

    def __setitem__(self, i: int, value) -> None:
        self.blocks[i].copy_(torch.as_tensor(value, dtype=self.blocks[i].dtype))

    def dim(self) -> int:
        return sum(self.block_dims)

    def zero(self) -> None:
        for b in self.blocks:
            b.zero_()

    def copy(self) -> "BlockTensor":
        out = BlockTensor(self.rank, self.block_dims, device=self.blocks[0].device if self.blocks else "cuda")
        for d, s in zip(out.blocks, self.blocks):
            d.copy_(s)
        return out

    def to_dense(self) -> torch.Tensor:
        n = self.dim()
        dev = self.blocks[0].device if self.blocks else "cuda"
        out = torch.zeros((n,) * self.rank, dtype=torch.float64, device=dev)
        for i, b in enumerate(self.blocks):
            lo, hi = self.block_range(i)
            out[(slice(lo, hi),) * self.rank] = b
        return out

    @classmethod
    def from_dense(cls, dense: torch.Tensor, block_dims: Sequence[int]) -> "BlockTensor":
        t = cls(dense.dim(), block_dims, device=dense.device)
        for i in range(t.num_blocks):
            lo, hi = t.block_range(i)
            t.blocks[i].copy_(dense[(slice(lo, hi),) * dense.dim()])
        return t

    # the tiled view: index d is cut by the block sizes; only diagonal tiles exist
    def _tile_sizes(self, d: int) -> List[int]:
        return self.block_dims

    def _get_tile(self, idx: Tuple[int, ...]):
        if len(set(idx)) != 1:
            return None
        return self.blocks[idx[0]]


class TiledTensor:
    """Tensor whose index d is cut into tiles of ``tile_sizes[d]``; only created tiles are stored."""

    def __init__(self, tile_sizes: Sequence[Sequence[int]], device="cuda", dtype=torch.float64):
        self.tile_sizes = [[int(s) for s in ts] for ts in tile_sizes]
        self.rank = len(self.tile_sizes)
        self.device, self.dtype = device, dtype
        self.tiles: Dict[Tuple[int, ...], torch.Tensor] = {}

    def has_tile(self, idx: Sequence[int]) -> bool:
        return tuple(idx) in self.tiles

    def tile_shape(self, idx: Sequence[int]) -> Tuple[int, ...]:
        return tuple(self.tile_sizes[d][i] for d, i in enumerate(idx))

    def tile(self, idx: Sequence[int]) -> torch.Tensor:
        """The tile at ``idx``, created (zero) when missing, as the reference's tile() does."""
        idx = tuple(idx)
        if idx not in self.tiles:
            self.tiles[idx] = torch.zeros(self.tile_shape(idx), dtype=self.dtype, device=self.device)
        return self.tiles[idx]

    def dims(self) -> Tuple[int, ...]:
        return tuple(sum(ts) for ts in self.tile_sizes)

    def zero(self) -> None:
        for t in self.tiles.values():
            t.zero_()

    def to_dense(self) -> torch.Tensor:
        out = torch.zeros(self.dims(), dtype=torch.float64, device=self.device)
        rng = [_ranges(ts) for ts in self.tile_sizes]
        for idx, t in self.tiles.items():
            sl = tuple(slice(rng[d][i][0], rng[d][i][0] + rng[d][i][1]) for d, i in enumerate(idx))
            out[sl] = t
        return out

    @classmethod
    def from_dense(cls, dense: torch.Tensor, tile_sizes: Sequence[Sequence[int]],
                   tiles: Sequence[Sequence[int]] | None = None) -> "TiledTensor":
        t = cls(tile_sizes, device=dense.device)
        rng = [_ranges(ts) for ts in t.tile_sizes]
        keys = tiles if tiles is not None else itertools.product(*[range(len(ts)) for ts in t.tile_sizes])
        for idx in keys:
            idx = tuple(idx)
            sl = tuple(slice(rng[d][i][0], rng[d][i][0] + rng[d][i][1]) for d, i in enumerate(idx))
            t.tile(idx).copy_(dense[sl])
        return t

    def _tile_sizes(self, d: int) -> List[int]:
        return self.tile_sizes[d]

    def _get_tile(self, idx: Tuple[int, ...]):
        return self.tiles.get(tuple(idx))


def is_blocked(x) -> bool:
    return isinstance(x, (BlockTensor, TiledTensor))


def block_items(C_indices, C, A_indices, A, B_indices, B):
    """The tile combinations of a blocked einsum, in the reference's order: lists of the C, A
    and B pieces of every contributing combination, and the C tiles no combination writes."""
    C_indices, A_indices, B_indices = list(C_indices), list(A_indices), list(B_indices)
    ops = [("C", C_indices, C), ("A", A_indices, A), ("B", B_indices, B)]
    unique: List = []
    for _, labels, _x in ops:
        for l in labels:
            if l not in unique:
                unique.append(l)
    # tile sizes of every unique index, from the blocked operands (they must agree)
    sizes: Dict = {}
    extent: Dict = {}
    for name, labels, x in ops:
        if is_blocked(x):
            if x.rank != len(labels):
                raise _lib.RankError(2, f"{name} has rank {x.rank} but {len(labels)} indices")
            for d, l in enumerate(labels):
                ts = list(x._tile_sizes(d))
                if l in sizes and sizes[l] != ts:
                    raise _lib.DimensionError(3, f"index {l!r} is tiled differently in the operands")
                sizes[l] = ts
        elif isinstance(x, torch.Tensor):
            if x.dim() != len(labels):
                raise _lib.RankError(2, f"{name} has rank {x.dim()} but {len(labels)} indices")
            for d, l in enumerate(labels):
                extent[l] = int(x.shape[d])
    for l in unique:
        if l not in sizes:
            sizes[l] = [extent.get(l, 0)]
        elif l in extent and extent[l] != sum(sizes[l]):
            raise _lib.DimensionError(3, f"index {l!r}: dense extent {extent[l]} != tiled extent {sum(sizes[l])}")
    rng = {l: _ranges(sizes[l]) for l in unique}

    def piece(x, labels, combo):
        idx = tuple(combo[l] for l in labels)
        if is_blocked(x):
            t = x._get_tile(idx)
            return t
        if x.dim() == 0:
            return x
        sl = tuple(slice(rng[l][i][0], rng[l][i][0] + rng[l][i][1]) for l, i in zip(labels, idx))
        return x[sl]

    Cs, As, Bs = [], [], []
    for combo_t in itertools.product(*[range(len(sizes[l])) for l in unique]):
        combo = dict(zip(unique, combo_t))
        a, b = piece(A, A_indices, combo), piece(B, B_indices, combo)
        if a is None or b is None or a.numel() == 0 or b.numel() == 0:
            continue
        if isinstance(C, TiledTensor):
            cidx = tuple(combo[l] for l in C_indices)
            if any(C.tile_sizes[d][i] == 0 for d, i in enumerate(cidx)):
                continue
            c = C.tile(cidx)
        elif isinstance(C, BlockTensor):
            c = C._get_tile(tuple(combo[l] for l in C_indices))
            if c is None:
                raise _lib.NotSupportedError(4, "a block combination writes an off-diagonal block of a BlockTensor C")
        else:
            c = piece(C, C_indices, combo)
        if c.numel() == 0 and c.dim() > 0:
            continue
        Cs.append(c)
        As.append(a)
        Bs.append(b)
    touched = {id(c) for c in Cs}
    untouched = []
    if isinstance(C, TiledTensor):
        untouched = [t for t in C.tiles.values() if id(t) not in touched]
    elif isinstance(C, BlockTensor):
        untouched = [t for t in C.blocks if id(t) not in touched]
    return Cs, As, Bs, untouched


def einsum_blocked(C_prefactor, C_indices, C, AB_prefactor, A_indices, A, B_indices, B, *, precision="fp64",
                   slices=0, tolerance=1e-10, stream=None) -> str:
    """einsum with BlockTensor / TiledTensor operands (at least one), C++ semantics."""
    C_indices, A_indices, B_indices = list(C_indices), list(A_indices), list(B_indices)
    Cs, As, Bs, untouched = block_items(C_indices, C, A_indices, A, B_indices, B)
    # C tiles that no combination writes are still scaled by C_prefactor (the reference
    # scales the whole of C first)
    from . import core
    for t in untouched:
        if t.numel() == 0:
            continue
        if C_prefactor == 0.0:
            t.zero_()
        elif C_prefactor != 1.0:
            lab = [f"_u{d}" for d in range(t.dim())]
            core.permute(0.0, lab, t, C_prefactor, lab, t.clone(), stream=stream)
    if not Cs:
        if not is_blocked(C) and isinstance(C, torch.Tensor):
            # nothing contributes: C = C_prefactor * C
            if C_prefactor == 0.0:
                C.zero_()
            elif C_prefactor != 1.0:
                C.mul_(C_prefactor)
        return "INDETERMINATE"
    _check_device(*Cs, *As, *Bs)
    n = len(Cs)
    ec, ea, eb = (_lib.EgTensor * n)(), (_lib.EgTensor * n)(), (_lib.EgTensor * n)()
    for i in range(n):
        ec[i], ea[i], eb[i] = _tensor(Cs[i], "C"), _tensor(As[i], "A"), _tensor(Bs[i], "B")
    opt = _options(precision, slices, SEMANTICS_CPP, False, tolerance)
    alg = ctypes.c_int32(0)
    _lib.check(_lib.load().eg_einsum_blocks(float(C_prefactor), _lib.labels(C_indices), ec, float(AB_prefactor),
                                            _lib.labels(A_indices), ea, _lib.labels(B_indices), eb, n,
                                            ctypes.byref(opt), ctypes.c_void_p(_stream(stream)), ctypes.byref(alg)))
    return ALGORITHMS[alg.value]
