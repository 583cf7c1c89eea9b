"""Python front end mirroring the reference's EinsumsPy ``core`` module.

``compile_plan(C, A, B)`` returns a plan object of the same class names as
``libs/EinsumsPy/TensorAlgebra/src/Export.cpp:12-140`` and
``plan.execute(C_prefactor, C, AB_prefactor, A, B)`` runs it, either on
single tensors or on equal-length lists of tensors (the list overload).
Operands are CUDA float64 ``torch.Tensor`` objects (any strides), or, for plans,
host NumPy buffers that are copied in and the result copied back; all work
goes through the C ABI of libeinsums_gb300.so on the current CUDA stream.

``einsum`` / ``permute`` mirror the C++ ``einsum(C_prefactor, Indices{...},
&C, AB_prefactor, Indices{...}, A, Indices{...}, B)`` and ``permute`` calls
(with C++ semantics) for callers that name indices as strings or sequences.
"""
from __future__ import annotations

import ctypes
from typing import Sequence

import numpy as np
import torch

from . import _lib
from ._lib import (PRECISION_FP64, PRECISION_SPLIT_BF16, SEMANTICS_CPP, SEMANTICS_PYTHON, EgOptions,
                   EgSplitReport, EgTensor)

ALGORITHMS = ["GENERIC", "DOT", "DIRECT", "GER", "GEMV", "GEMM", "INDETERMINATE"]


def _tensor(t: torch.Tensor, name: str, complex_ok: bool = False) -> EgTensor:
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if t.dtype != torch.float64 and not (complex_ok and t.dtype == torch.complex128):
        raise TypeError(f"{name} must be float64{' or complex128' if complex_ok else ''} (got {t.dtype})")
    if not t.is_cuda:
        raise TypeError(f"{name} must live on a CUDA device")
    if t.dim() > _lib.MAX_RANK:
        raise _lib.RankError(2, f"{name} has rank {t.dim()} (max {_lib.MAX_RANK})")
    e = EgTensor()
    e.data = t.data_ptr() if t.numel() else None
    e.rank = t.dim()
    for i, (n, s) in enumerate(zip(t.shape, t.stride())):
        e.extent[i] = n
        e.stride[i] = s
    return e


def _options(precision: str, slices: int, semantics: int, only_generic: bool, tolerance: float) -> EgOptions:
    o = EgOptions()
    _lib.load().eg_options_default(ctypes.byref(o))
    o.precision = {"fp64": PRECISION_FP64, "split_bf16": PRECISION_SPLIT_BF16}[precision]
    o.slices = int(slices)
    o.tolerance = float(tolerance)
    o.semantics = semantics
    o.only_generic = int(bool(only_generic))
    return o


def _stream(stream) -> int:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    return stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream)


def _check_device(*ts):
    dev = None
    for t in ts:
        if dev is None:
            dev = t.device
        elif t.device != dev:
            raise ValueError("all operands must be on the same device")
    if dev is not None and dev.index is not None and dev.index != torch.cuda.current_device():
        raise ValueError("operands must be on the current CUDA device")


def _run_einsum(C_prefactor, C_labels, C, AB_prefactor, A_labels, A, B_labels, B, *, semantics, precision="fp64",
                slices=0, tolerance=1e-10, only_generic=False, stream=None, conj_A=False, conj_B=False) -> int:
    lib = _lib.load()
    if C.dim() != len(C_labels) or A.dim() != len(A_labels) or B.dim() != len(B_labels):
        raise _lib.RankError(2, "tensor ranks do not match the indices")
    _check_device(C, A, B)
    if any(t.dtype == torch.complex128 for t in (C, A, B)):
        if not all(t.dtype == torch.complex128 for t in (C, A, B)):
            raise TypeError("complex einsum: C, A and B must all be complex128")
        ec, ea, eb = _tensor(C, "C", True), _tensor(A, "A", True), _tensor(B, "B", True)
        opt = _options(precision, slices, semantics, only_generic, tolerance)
        alg = ctypes.c_int32(-1)
        cpf, abf = complex(C_prefactor), complex(AB_prefactor)
        cpa, aba = (ctypes.c_double * 2)(cpf.real, cpf.imag), (ctypes.c_double * 2)(abf.real, abf.imag)
        _lib.check(lib.eg_einsum_complex(cpa, _lib.labels(C_labels), ctypes.byref(ec), aba, _lib.labels(A_labels),
                                         ctypes.byref(ea), _lib.labels(B_labels), ctypes.byref(eb), int(bool(conj_A)),
                                         int(bool(conj_B)), ctypes.byref(opt), ctypes.c_void_p(_stream(stream)),
                                         ctypes.byref(alg)))
        return alg.value
    if conj_A or conj_B:
        pass  # conjugating a real operand changes nothing (the reference's ConjA/ConjB on real data)
    ec, ea, eb = _tensor(C, "C"), _tensor(A, "A"), _tensor(B, "B")
    opt = _options(precision, slices, semantics, only_generic, tolerance)
    alg = ctypes.c_int32(-1)
    _lib.check(lib.eg_einsum(float(C_prefactor), _lib.labels(C_labels), ctypes.byref(ec), float(AB_prefactor),
                             _lib.labels(A_labels), ctypes.byref(ea), _lib.labels(B_labels), ctypes.byref(eb),
                             ctypes.byref(opt), ctypes.c_void_p(_stream(stream)), ctypes.byref(alg)))
    return alg.value


def _run_batched(C_prefactor, C_labels, Cs, AB_prefactor, A_labels, As, B_labels, Bs, *, semantics,
                 precision="fp64", slices=0, tolerance=1e-10, stream=None) -> int:
    lib = _lib.load()
    if not (len(Cs) == len(As) == len(Bs)):
        raise ValueError("The lengths of the collections need to be the same!")
    n = len(Cs)
    if n == 0:
        return -1
    arrC, arrA, arrB = (EgTensor * n)(), (EgTensor * n)(), (EgTensor * n)()
    for i in range(n):
        if Cs[i].dim() != len(C_labels) or As[i].dim() != len(A_labels) or Bs[i].dim() != len(B_labels):
            raise _lib.RankError(2, "tensor ranks do not match the indices")
        _check_device(Cs[i], As[i], Bs[i])
        arrC[i], arrA[i], arrB[i] = _tensor(Cs[i], "C"), _tensor(As[i], "A"), _tensor(Bs[i], "B")
    opt = _options(precision, slices, semantics, False, tolerance)
    alg = ctypes.c_int32(-1)
    _lib.check(lib.eg_einsum_batched(float(C_prefactor), _lib.labels(C_labels), arrC, float(AB_prefactor),
                                     _lib.labels(A_labels), arrA, _lib.labels(B_labels), arrB, n, ctypes.byref(opt),
                                     ctypes.c_void_p(_stream(stream)), ctypes.byref(alg)))
    return alg.value


class GroupedPlan:
    """A list einsum lowered once and captured as a CUDA graph
    (eg_grouped_plan_create); ``execute()`` replays it on the current stream.
    The tensors must stay alive (and keep their storage) while the plan is used."""

    def __init__(self, C_prefactor, C_indices, Cs, AB_prefactor, A_indices, As, B_indices, Bs, *,
                 precision="fp64", slices=0, tolerance=1e-10, semantics=SEMANTICS_CPP, stream=None):
        lib = _lib.load()
        n = len(Cs)
        if not (n == len(As) == len(Bs)) or n == 0:
            raise ValueError("lists must be non-empty and of equal length")
        self._keep = (list(Cs), list(As), list(Bs))
        arrC, arrA, arrB = (EgTensor * n)(), (EgTensor * n)(), (EgTensor * n)()
        for i in range(n):
            if Cs[i].dim() != len(C_indices) or As[i].dim() != len(A_indices) or Bs[i].dim() != len(B_indices):
                raise _lib.RankError(2, "tensor ranks do not match the indices")
            _check_device(Cs[i], As[i], Bs[i])
            arrC[i], arrA[i], arrB[i] = _tensor(Cs[i], "C"), _tensor(As[i], "A"), _tensor(Bs[i], "B")
        opt = _options(precision, slices, semantics, False, tolerance)
        handle = ctypes.c_void_p()
        alg = ctypes.c_int32(-1)
        _lib.check(lib.eg_grouped_plan_create(float(C_prefactor), _lib.labels(C_indices), arrC, float(AB_prefactor),
                                              _lib.labels(A_indices), arrA, _lib.labels(B_indices), arrB, n,
                                              ctypes.byref(opt), ctypes.c_void_p(_stream(stream)),
                                              ctypes.byref(handle), ctypes.byref(alg)))
        self._handle = handle
        self.algorithm = ALGORITHMS[alg.value]
        self.count = n

    def execute(self, stream=None):
        _lib.check(_lib.load().eg_grouped_plan_execute(self._handle, ctypes.c_void_p(_stream(stream))))

    def close(self):
        if getattr(self, "_handle", None):
            _lib.load().eg_grouped_plan_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def classify(C_labels, A_labels, B_labels, semantics: int = SEMANTICS_CPP) -> int:
    lib = _lib.load()
    alg = ctypes.c_int32(-1)
    _lib.check(lib.eg_classify(len(C_labels), _lib.labels(C_labels), len(A_labels), _lib.labels(A_labels),
                               len(B_labels), _lib.labels(B_labels), semantics, ctypes.byref(alg)))
    return alg.value


# --------------------------------------------------------------- plans ----
class EinsumGenericPlan:
    """A compiled index pattern (``compile_plan`` result)."""

    algorithm = "GENERIC"

    def __init__(self, C: str, A: str, B: str):
        self.C_indices, self.A_indices, self.B_indices = C, A, B

    def execute(self, C_prefactor, C, AB_prefactor, A, B, *, precision: str = "fp64", slices: int = 0,
                tolerance: float = 1e-10, stream=None):
        """C = C_prefactor*C + AB_prefactor * A*B contracted over the plan's pattern.
        ``C``, ``A``, ``B`` are CUDA tensors or equal-length lists of them, or host buffers
        (NumPy arrays; C writable), which are copied to the device, contracted there and
        copied back into C -- the reference's execute also takes buffers (Export.cpp:17-32)."""
        if _is_host(C) or _is_host(A) or _is_host(B):
            return _execute_host(self, C_prefactor, C, AB_prefactor, A, B, precision=precision, slices=slices,
                                 tolerance=tolerance, stream=stream)
        if isinstance(C, (list, tuple)):
            _run_batched(C_prefactor, self.C_indices, list(C), AB_prefactor, self.A_indices, list(A),
                         self.B_indices, list(B), semantics=SEMANTICS_PYTHON, precision=precision, slices=slices,
                         tolerance=tolerance, stream=stream)
            return
        _run_einsum(C_prefactor, self.C_indices, C, AB_prefactor, self.A_indices, A, self.B_indices, B,
                    semantics=SEMANTICS_PYTHON, precision=precision, slices=slices, tolerance=tolerance,
                    stream=stream)

    def __repr__(self):
        return f"{type(self).__name__}({self.C_indices!r} <- {self.A_indices!r} * {self.B_indices!r})"


def _is_host(x) -> bool:
    if isinstance(x, (list, tuple)):
        return any(_is_host(y) for y in x)
    return not isinstance(x, torch.Tensor)


def _to_device(x, s):
    """A float64 CUDA copy of a host buffer (or the tensor itself when already on the GPU),
    copied on stream ``s`` through the library's copy entry point."""
    if isinstance(x, torch.Tensor):
        return x
    arr = np.array(x, dtype=np.float64, order="C", copy=True)  # keeps a 0-d buffer 0-d
    dev = torch.empty(arr.shape, dtype=torch.float64, device="cuda")
    if arr.size:
        _lib.check(_lib.load().eg_copy_to_device(ctypes.c_void_p(dev.data_ptr()), ctypes.c_void_p(arr.ctypes.data),
                                                 arr.nbytes, ctypes.c_void_p(s)))
    return dev, arr


def _execute_host(plan, C_prefactor, C, AB_prefactor, A, B, **kw):
    lib = _lib.load()
    stream = kw.pop("stream", None)
    s = _stream(stream)
    lists = isinstance(C, (list, tuple))
    Cs, As, Bs = (list(C), list(A), list(B)) if lists else ([C], [A], [B])
    keep = []  # host arrays that must outlive the asynchronous copies
    dC, dA, dB = [], [], []
    for dst, src in ((dA, As), (dB, Bs)):
        for x in src:
            r = _to_device(x, s)
            if isinstance(r, tuple):
                keep.append(r[1])
                r = r[0]
            dst.append(r)
    hosts = []
    for x in Cs:
        if isinstance(x, torch.Tensor):
            dC.append(x)
            hosts.append(None)
            continue
        if not isinstance(x, np.ndarray) or x.dtype != np.float64 or not x.flags.writeable:
            raise TypeError("a host C must be a writable float64 NumPy array")
        r = _to_device(x, s)
        keep.append(r[1])
        dC.append(r[0])
        hosts.append(x)
    if lists:
        plan.execute(C_prefactor, dC, AB_prefactor, dA, dB, stream=stream, **kw)
    else:
        plan.execute(C_prefactor, dC[0], AB_prefactor, dA[0], dB[0], stream=stream, **kw)
    outs = []
    for d, h in zip(dC, hosts):
        if h is None:
            continue
        out = np.empty(h.shape, dtype=np.float64)
        if out.size:
            _lib.check(lib.eg_copy_to_host(ctypes.c_void_p(out.ctypes.data), ctypes.c_void_p(d.data_ptr()),
                                           out.nbytes, ctypes.c_void_p(s)))
        outs.append((h, out))
    _lib.check(lib.eg_stream_synchronize(ctypes.c_void_p(s)))
    for h, out in outs:
        h[...] = out


class EinsumDotPlan(EinsumGenericPlan):
    algorithm = "DOT"


class EinsumDirectProductPlan(EinsumGenericPlan):
    algorithm = "DIRECT"


class EinsumGerPlan(EinsumGenericPlan):
    algorithm = "GER"


class EinsumGemvPlan(EinsumGenericPlan):
    algorithm = "GEMV"


class EinsumGemmPlan(EinsumGenericPlan):
    algorithm = "GEMM"


_PLAN_CLASSES = {0: EinsumGenericPlan, 1: EinsumDotPlan, 2: EinsumDirectProductPlan, 3: EinsumGerPlan,
                 4: EinsumGemvPlan, 5: EinsumGemmPlan}


def compile_plan(C_indices: str, A_indices: str, B_indices: str) -> EinsumGenericPlan:
    """Pattern analysis of compile_plan (PyTensorAlgebra.cpp:168-554): returns the plan class
    the reference returns for the same strings."""
    alg = classify(C_indices, A_indices, B_indices, SEMANTICS_PYTHON)
    return _PLAN_CLASSES[alg](C_indices, A_indices, B_indices)


# ------------------------------------------------------ C++-style calls ----
def einsum(C_prefactor, C_indices: Sequence, C, AB_prefactor, A_indices: Sequence, A, B_indices: Sequence, B, *,
           precision: str = "fp64", slices: int = 0, tolerance: float = 1e-10, only_generic: bool = False,
           stream=None, conj_A: bool = False, conj_B: bool = False) -> str:
    """C++-semantics einsum; returns the reference's AlgorithmChoice name.  C, A, B may also
    be equal-length lists (the batched overload), or BlockTensor / TiledTensor operands
    (blocks.py: every tile combination through one block-sparse call)."""
    from . import blocks
    if any(blocks.is_blocked(x) for x in (C, A, B)):
        return blocks.einsum_blocked(C_prefactor, C_indices, C, AB_prefactor, A_indices, A, B_indices, B,
                                     precision=precision, slices=slices, tolerance=tolerance, stream=stream)
    if isinstance(C, (list, tuple)):
        alg = _run_batched(C_prefactor, list(C_indices), list(C), AB_prefactor, list(A_indices), list(A),
                           list(B_indices), list(B), semantics=SEMANTICS_CPP, precision=precision, slices=slices,
                           tolerance=tolerance, stream=stream)
        return ALGORITHMS[alg] if alg >= 0 else "INDETERMINATE"
    alg = _run_einsum(C_prefactor, list(C_indices), C, AB_prefactor, list(A_indices), A, list(B_indices), B,
                      semantics=SEMANTICS_CPP, precision=precision, slices=slices, tolerance=tolerance,
                      only_generic=only_generic, stream=stream, conj_A=conj_A, conj_B=conj_B)
    return ALGORITHMS[alg]


def permute(C_prefactor, C_indices: Sequence, C, A_prefactor, A_indices: Sequence, A, *, stream=None) -> None:
    """C = C_prefactor*C + A_prefactor*A[perm] (Permute.hpp:330-407)."""
    lib = _lib.load()
    C_indices, A_indices = list(C_indices), list(A_indices)
    if C.dim() != len(C_indices) or A.dim() != len(A_indices):
        raise _lib.RankError(2, "tensor ranks do not match the indices")
    _check_device(C, A)
    ec, ea = _tensor(C, "C"), _tensor(A, "A")
    _lib.check(lib.eg_permute(float(C_prefactor), _lib.labels(C_indices), ctypes.byref(ec), float(A_prefactor),
                              _lib.labels(A_indices), ctypes.byref(ea), ctypes.c_void_p(_stream(stream))))


def fock_jk_symmetric(F, g, D, *, F_prefactor=1.0, J_prefactor=2.0, K_prefactor=-1.0, precision="fp64",
                      slices=0, stream=None) -> None:
    """F = F_prefactor*F + J_prefactor*J + K_prefactor*K with J = einsum(pq <- pqrs, rs) and
    K = einsum(pq <- prqs, rs), for g with 8-fold permutational symmetry and symmetric D
    (not checked); reads only the canonical eighth of g.  The defaults give the reference's
    RHF update F += 2 J - K (QChemTests.cpp:300-303).  F, g, D: contiguous CUDA float64.
    precision="split_bf16" sums four of the six contributions per element as exact 8-bit
    digit products on the FP32 pipe (last_split_report() gives the bound)."""
    lib = _lib.load()
    if g.dim() != 4 or len(set(g.shape)) != 1:
        raise _lib.DimensionError(3, "g must be n x n x n x n")
    n = g.shape[0]
    if tuple(D.shape) != (n, n) or tuple(F.shape) != (n, n):
        raise _lib.DimensionError(3, "D and F must be n x n")
    for t, name in ((F, "F"), (g, "g"), (D, "D")):
        _tensor(t, name)
        if not t.is_contiguous():
            raise ValueError(f"{name} must be contiguous")
    _check_device(F, g, D)
    opt = _options(precision, slices, SEMANTICS_CPP, False, 1e-10)
    _lib.check(lib.eg_fock_jk_symmetric(float(F_prefactor), ctypes.c_void_p(F.data_ptr()), float(J_prefactor),
                                        float(K_prefactor), ctypes.c_void_p(g.data_ptr()),
                                        ctypes.c_void_p(D.data_ptr()), n, ctypes.byref(opt),
                                        ctypes.c_void_p(_stream(stream))))


class PermutePlan:
    """A compiled permute (compile_permute of Permute.hpp:37-171): fixed permutation, shapes,
    strides and prefactors; ``execute(C, A)`` runs it on any tensors with those shapes and
    strides (the reference's permute(&C, A, plan), Permute.hpp:292-297)."""

    def __init__(self, C_prefactor, C_indices: Sequence, C, A_prefactor, A_indices: Sequence, A):
        lib = _lib.load()
        C_indices, A_indices = list(C_indices), list(A_indices)
        if C.dim() != len(C_indices) or A.dim() != len(A_indices):
            raise _lib.RankError(2, "tensor ranks do not match the indices")
        self._shape = (tuple(C.shape), tuple(C.stride()), tuple(A.shape), tuple(A.stride()))
        ec, ea = _tensor(C, "C"), _tensor(A, "A")
        h = ctypes.c_void_p()
        _lib.check(lib.eg_permute_plan_create(float(C_prefactor), _lib.labels(C_indices), ctypes.byref(ec),
                                              float(A_prefactor), _lib.labels(A_indices), ctypes.byref(ea),
                                              ctypes.byref(h)))
        self._h = h

    def execute(self, C, A, *, stream=None) -> None:
        if (tuple(C.shape), tuple(C.stride()), tuple(A.shape), tuple(A.stride())) != self._shape:
            raise _lib.DimensionError(3, "C and A must have the plan's shapes and strides")
        _tensor(C, "C")
        _tensor(A, "A")
        _check_device(C, A)
        _lib.check(_lib.load().eg_permute_plan_execute(self._h, ctypes.c_void_p(C.data_ptr() if C.numel() else None),
                                                       ctypes.c_void_p(A.data_ptr() if A.numel() else None),
                                                       ctypes.c_void_p(_stream(stream))))

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.load().eg_permute_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001 -- interpreter shutdown
            pass


def compile_permute(C_prefactor, C_indices: Sequence, C, A_prefactor, A_indices: Sequence, A) -> PermutePlan:
    return PermutePlan(C_prefactor, C_indices, C, A_prefactor, A_indices, A)


def last_split_report() -> dict:
    r = EgSplitReport()
    _lib.check(_lib.load().eg_last_split_report(ctypes.byref(r)))
    return {"slices": r.slices, "slice_pairs": r.slice_pairs, "bits_per_slice": r.bits_per_slice,
            "error_bound": r.error_bound}
