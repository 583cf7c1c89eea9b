"""Differentiable einsum: a ``torch.autograd.Function`` whose backward runs the
adjoint contractions through the same CUDA kernels.

For ``C[c] = sum A[a] B[b]`` (every index not in C summed, the EinsumsPy
plan semantics) the adjoints are again contractions of the same kind:

    dA[a] = sum_{indices not in a} dC[c] * B[b]      (pattern  a <- c * b)
    dB[b] = sum_{indices not in b} dC[c] * A[a]      (pattern  b <- c * a)

An index that occurs only in C broadcasts in the forward pass and is summed in
the adjoint; an index that occurs only in A is summed in the forward pass and
broadcasts in the adjoint.  Both follow from the unique-index-space semantics
the kernels implement.  Permuted operands are never materialised: the forward
and the adjoint kernels read A, B and dC in place through their index maps, so
the backward pass stores only the two inputs it needs.

    C = einsum_ag("mbej", "jnfb", "mnef", t, g)           # FP64
    C = einsum_ag("mbej", "jnfb", "mnef", t, g, precision="split_bf16")
"""
from __future__ import annotations

import torch

from . import core
from ._lib import SEMANTICS_PYTHON


def _run(C_idx, A_idx, B_idx, A, B, precision, slices, shape):
    C = torch.empty(shape, dtype=torch.float64, device=A.device)
    core._run_einsum(0.0, C_idx, C, 1.0, A_idx, A, B_idx, B, semantics=SEMANTICS_PYTHON, precision=precision,
                     slices=slices)
    return C


def _extents(idx_pairs):
    dims = {}
    for labels, t in idx_pairs:
        for l, d in zip(labels, t.shape):
            if l in dims and dims[l] != d:
                raise ValueError(f"index {l!r} has extents {dims[l]} and {d}")
            dims[l] = d
    return dims


class Einsum(torch.autograd.Function):
    """``C = einsum(C_indices <- A_indices * B_indices)(A, B)`` with adjoint
    contractions in backward.  Index strings are one character per mode."""

    @staticmethod
    def forward(ctx, C_indices: str, A_indices: str, B_indices: str, A: torch.Tensor, B: torch.Tensor,
                precision: str = "fp64", slices: int = 0):
        dims = _extents([(A_indices, A), (B_indices, B)])
        for l in C_indices:
            if l not in dims:
                raise ValueError(f"output index {l!r} occurs in neither operand; its extent is unknown")
        shape = [dims[l] for l in C_indices]
        ctx.idx = (C_indices, A_indices, B_indices)
        ctx.precision, ctx.slices = precision, slices
        ctx.save_for_backward(A, B)
        return _run(C_indices, A_indices, B_indices, A.detach(), B.detach(), precision, slices, shape)

    @staticmethod
    def backward(ctx, dC: torch.Tensor):
        C_idx, A_idx, B_idx = ctx.idx
        A, B = ctx.saved_tensors
        dC = dC if dC.dtype == torch.float64 else dC.to(torch.float64)
        dA = dB = None
        if ctx.needs_input_grad[3]:
            dA = _run(A_idx, C_idx, B_idx, dC, B.detach(), ctx.precision, ctx.slices, list(A.shape))
        if ctx.needs_input_grad[4]:
            dB = _run(B_idx, C_idx, A_idx, dC, A.detach(), ctx.precision, ctx.slices, list(B.shape))
        return None, None, None, dA, dB, None, None


def einsum_ag(C_indices: str, A_indices: str, B_indices: str, A: torch.Tensor, B: torch.Tensor, *,
              precision: str = "fp64", slices: int = 0) -> torch.Tensor:
    """Differentiable einsum over CUDA float64 tensors (see module docstring)."""
    return Einsum.apply(C_indices, A_indices, B_indices, A, B, precision, slices)


def central_difference(loss_fn, X: torch.Tensor, index, h: float = 1e-6) -> float:
    """FP64 central difference of ``loss_fn`` with respect to ``X[index]``."""
    X_plus = X.detach().clone()
    X_plus[index] += h
    X_minus = X.detach().clone()
    X_minus[index] -= h
    return (loss_fn(X_plus) - loss_fn(X_minus)) / (2.0 * h)
