"""CPU oracle for the einsum / permute hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` may import this module, and only to check
results (or, in ``bench.py --impl reference``, as the timed CPU reference).
The product path never routes through it.

What it restates (reference paths relative to the Einsums project root):

* ``einsum(..., semantics="cpp")`` -- the C++ ``einsum`` entry
  (``libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Backends/Dispatch.hpp:960-1262``)
  through ``detail::einsum`` (:859-957): the compile-time algorithm choice
  (``oracle/classify.py``), the runtime stride vetoes of
  ``einsum_do_outer_product`` (:267-401), ``einsum_do_matrix_vector``
  (:444-560) and ``einsum_do_matrix_product`` (:614-837), the BLAS lowering
  of each choice, and the generic loops (``oracle_ref.c``).
* ``einsum(..., semantics="py")`` -- ``compile_plan`` + ``execute`` of
  ``libs/EinsumsPy/TensorAlgebra`` (every CPU plan runs
  ``execute_generic``, ``PyTensorAlgebra.hpp:520-605``, so values follow the
  full unique-index sum and C is zeroed when ``C_prefactor == 0``).
* ``permute`` -- ``Permute.hpp:338-407``.

The arithmetic of the BLAS-lowered choices lives in a third-party library that
is not part of the reference tree: whatever BLAS the reference is linked with
(OpenBLAS 0.3.29 in its documentation).  Here it is numpy's bundled OpenBLAS
(``dgemm``/``dgemv``/``ddot`` through ``np.matmul``/``np.dot``).  Parity is
pinned on the reference's own known answers and golden physics (tests/golden).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, _HERE)
from classify import Algorithm, Analysis, classify_cpp, classify_py  # noqa: E402

_LIB = None
_LOCK = threading.Lock()
_BUILD_DIR = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD_DIR, "liboracle.so")


def build(force: bool = False) -> str:
    """Compile oracle_ref.c with gcc + OpenMP into oracle/_build/liboracle.so."""
    src = os.path.join(_HERE, "oracle_ref.c")
    if (not force and os.path.exists(_SO)
            and os.path.getmtime(_SO) >= os.path.getmtime(src)):
        return _SO
    os.makedirs(_BUILD_DIR, exist_ok=True)
    tmp = _SO + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O3", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _SO)
    return _SO


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            path = build()
            L = ctypes.CDLL(path)
            P = ctypes.POINTER
            i64p = P(ctypes.c_int64)
            dp = P(ctypes.c_double)
            L.oracle_generic_cpp.argtypes = [ctypes.c_int, i64p, i64p, i64p, i64p, ctypes.c_int,
                                             i64p, i64p, i64p, ctypes.c_double, dp, dp, dp,
                                             ctypes.c_int]
            L.oracle_generic_py.argtypes = [ctypes.c_int, i64p, i64p, i64p, i64p, ctypes.c_double,
                                            dp, dp, dp]
            L.oracle_permute.argtypes = [ctypes.c_int, i64p, i64p, i64p, ctypes.c_double, dp,
                                         ctypes.c_double, dp]
            L.oracle_permute_copy.argtypes = [ctypes.c_int, i64p, i64p, i64p, dp, dp]
            L.oracle_num_threads.restype = ctypes.c_int
            _LIB = L
    return _LIB


def _i64(seq):
    a = (ctypes.c_int64 * max(1, len(seq)))()
    for i, v in enumerate(seq):
        a[i] = int(v)
    return a


def _estrides(x: np.ndarray):
    return [s // x.itemsize for s in x.strides]


def _base_ptr(x: np.ndarray):
    return x.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _stride_for(labels, strides, want):
    """get_stride_for (Detail/Utilities.hpp:560-596): sum of the strides of
    every position where ``want`` occurs (0 if absent)."""
    return sum(s for l, s in zip(labels, strides) if l == want)


# --- runtime vetoes (Dispatch.hpp) --------------------------------------------

def _totally_vectorable(x: np.ndarray) -> bool:
    """TensorImpl::is_totally_vectorable (TensorImpl.hpp:756-777)."""
    if x.ndim == 0:
        return False
    if x.ndim == 1:
        return True
    s = _estrides(x)
    if s[0] < s[-1]:
        return x.shape[-1] * s[-1] == x.size * s[0]
    return x.shape[0] * s[0] == x.size * s[-1]


def _two_groups_ok(x: np.ndarray, s0: int, s1: int) -> bool:
    """Row-major stride check of Dispatch.hpp:481-504 (and its copies at
    :664-684, :717-737, :770-790): the tensor must be two contiguous blocks."""
    st = _estrides(x)
    if x.ndim == 2:
        return not (st[0] != 1 and st[1] != 1)
    cutoff = max(s0, s1)
    check = 1
    for i in range(x.ndim - 1, -1, -1):
        if st[i] == cutoff:
            check = cutoff
        if st[i] != check:
            return False
        check *= x.shape[i]
    return True


def _last_stride(pairs, x):
    """last_stride (Detail/Utilities.hpp:384-391), row-major: stride of the
    last listed position."""
    return _estrides(x)[pairs[-1][1]]


def _gemv_veto(an: Analysis, A, B, C) -> bool:
    """True when einsum_do_matrix_vector (Dispatch.hpp:444-560) returns false."""
    if not _totally_vectorable(B) or not _totally_vectorable(C):
        return True
    sA0 = _last_stride(an.target_pos_A, A)
    sA1 = _last_stride(an.link_pos_A, A)
    return not _two_groups_ok(A, sA0, sA1)


def _gemm_veto(an: Analysis, A, B, C) -> bool:
    """True when einsum_do_matrix_product (Dispatch.hpp:614-837) returns false."""
    if not _two_groups_ok(A, _last_stride(an.target_pos_A, A), _last_stride(an.link_pos_A, A)):
        return True
    if not _two_groups_ok(B, _last_stride(an.link_pos_B, B), _last_stride(an.target_pos_B, B)):
        return True
    if not _two_groups_ok(C, _last_stride(an.A_target_pos_C, C), _last_stride(an.B_target_pos_C, C)):
        return True
    return False


def _ger_veto(an: Analysis, A, B, C) -> bool:
    """True when einsum_do_outer_product (Dispatch.hpp:267-401) returns false."""
    if not _totally_vectorable(A) or not _totally_vectorable(B):
        return True
    return not _two_groups_ok(C, _last_stride(an.A_target_pos_C, C), _last_stride(an.B_target_pos_C, C))


# --- lowering -----------------------------------------------------------------

def _group(x: np.ndarray, labels, first, second):
    """View x as a matrix (prod(first) x prod(second)) after ordering its modes
    as first+second (a transpose of a row-major view; numpy hands BLAS the
    transposed operand without copying when possible)."""
    order = [labels.index(l) for l in first] + [labels.index(l) for l in second]
    y = np.transpose(x, order)
    m = int(np.prod([x.shape[labels.index(l)] for l in first])) if first else 1
    n = int(np.prod([x.shape[labels.index(l)] for l in second])) if second else 1
    return y.reshape(m, n)


def _generic_cpp(Cl, C, Al, A, Bl, B, ab):
    an = Analysis(Cl, Al, Bl)
    dims = {}
    for l, d in zip(Cl, C.shape):
        dims.setdefault(l, d)
    ldims = {}
    for l, d in zip(Al, A.shape):
        ldims.setdefault(l, d)
    sC, sA, sB = _estrides(C), _estrides(A), _estrides(B)
    targets = an.C_unique
    links = an.link_unique
    tdims = [dims[l] for l in targets]
    ldims_v = [ldims[l] for l in links]
    L = lib()
    L.oracle_generic_cpp(len(targets), _i64(tdims), _i64([_stride_for(Cl, sC, l) for l in targets]),
                         _i64([_stride_for(Al, sA, l) for l in targets]),
                         _i64([_stride_for(Bl, sB, l) for l in targets]), len(links), _i64(ldims_v),
                         _i64([_stride_for(Al, sA, l) for l in links]),
                         _i64([_stride_for(Bl, sB, l) for l in links]), float(ab), _base_ptr(C),
                         _base_ptr(A), _base_ptr(B), 0)


def _generic_py(Cl, C, Al, A, Bl, B, ab):
    uniq = []
    for l in list(Al) + list(Bl) + list(Cl):
        if l not in uniq:
            uniq.append(l)
    dims = {}
    for lab, arr in ((Cl, C), (Al, A), (Bl, B)):
        for l, d in zip(lab, arr.shape):
            dims.setdefault(l, d)
    sC, sA, sB = _estrides(C), _estrides(A), _estrides(B)
    # create_perm_table maps each mode to its unique index; the loop adds
    # stride(mode) * unique_index for every mode (PyTensorAlgebra.hpp:588-598).
    lib().oracle_generic_py(len(uniq), _i64([dims[u] for u in uniq]),
                            _i64([_stride_for(Cl, sC, u) for u in uniq]),
                            _i64([_stride_for(Al, sA, u) for u in uniq]),
                            _i64([_stride_for(Bl, sB, u) for u in uniq]), float(ab), _base_ptr(C),
                            _base_ptr(A), _base_ptr(B))


def _prefactor_c(C, c):
    """einsum_generic_algorithm's prologue (BaseAlgebra.hpp:129-133)."""
    if c == 0.0:
        C[...] = 0.0
    else:
        C *= c


def einsum(C_labels, C: np.ndarray, c_pref: float, ab_pref: float, A_labels, A: np.ndarray,
           B_labels, B: np.ndarray, semantics: str = "cpp", only_generic: bool = False) -> Algorithm:
    """C = c_pref * C + ab_pref * sum_links A * B, in place on C.  Returns the
    algorithm the reference reports for the call."""
    Cl, Al, Bl = list(C_labels), list(A_labels), list(B_labels)
    if C.ndim != len(Cl) or A.ndim != len(Al) or B.ndim != len(Bl):
        raise ValueError("rank of a tensor does not match its indices")
    for arr in (C, A, B):
        if arr.dtype != np.float64:
            raise TypeError("oracle handles float64 only")
    if semantics == "py":
        alg = classify_py(Cl, Al, Bl)
        # Every CPU plan type runs execute_generic (PyTensorAlgebra.hpp:520-605).
        _prefactor_c(C, c_pref)
        if alg == Algorithm.GENERIC or only_generic:
            _generic_py(Cl, C, Al, A, Bl, B, ab_pref)
        else:
            _lowered(alg, Cl, C, 1.0, ab_pref, Al, A, Bl, B, prescaled=True)
        return alg

    alg = Algorithm.GENERIC if only_generic else classify_cpp(Cl, Al, Bl)
    an = Analysis(Cl, Al, Bl)
    if alg == Algorithm.GER and _ger_veto(an, A, B, C):
        alg = Algorithm.GENERIC
    elif alg == Algorithm.GEMV:
        swap = not an.is_gemv(False)
        if (_gemv_veto(Analysis(Cl, Bl, Al), B, A, C) if swap else _gemv_veto(an, A, B, C)):
            alg = Algorithm.GENERIC
    elif alg == Algorithm.GEMM and _gemm_veto(an, A, B, C):
        alg = Algorithm.GENERIC
    if alg == Algorithm.GENERIC:
        _prefactor_c(C, c_pref)
        _generic_cpp(Cl, C, Al, A, Bl, B, ab_pref)
        return alg
    _lowered(alg, Cl, C, c_pref, ab_pref, Al, A, Bl, B, prescaled=False)
    return alg


def _drop_free(x: np.ndarray, labels, other, Cl, how):
    """Remove modes of one operand that occur neither in C nor in the other
    operand.  The C++ lowering builds its BLAS views from the target and link
    modes only, so such a mode stays at index 0 (Dispatch.hpp:467-546,
    :641-826); the Python CPU plans walk the full unique-index space and so
    sum over it (PyTensorAlgebra.hpp:585-601)."""
    labels = list(labels)
    keep = [i for i, l in enumerate(labels) if l in Cl or l in other]
    free = [i for i in range(len(labels)) if i not in keep]
    if not free:
        return x, labels
    if how == "sum":
        y = x.sum(axis=tuple(free))
    else:
        sl = tuple(0 if i in free else slice(None) for i in range(len(labels)))
        y = x[sl]
    return y, [labels[i] for i in keep]


def _lowered(alg, Cl, C, c_pref, ab_pref, Al, A, Bl, B, prescaled):
    """The BLAS lowering of each specialised choice (Dispatch.hpp:900-951)."""
    how = "sum" if prescaled else "first"
    if alg not in (Algorithm.DOT, Algorithm.DIRECT):
        A, Al2 = _drop_free(A, Al, Bl, Cl, how)
        B, Bl2 = _drop_free(B, Bl, Al, Cl, how)
        Al, Bl = Al2, Bl2
    an = Analysis(Cl, Al, Bl)
    if alg == Algorithm.DOT:
        # dot then C = C_prefactor * C + AB_prefactor * dot (Dispatch.hpp:903-909);
        # C is multiplied, not zeroed, when C_prefactor == 0.
        temp = float(np.dot(np.ascontiguousarray(A).ravel(), np.ascontiguousarray(B).ravel()))
        if not prescaled:
            C *= c_pref
        C += ab_pref * temp
        return
    if alg == Algorithm.DIRECT:
        # direct_product(AB, A, B, C_prefactor, C): C = C_prefactor*C + AB*A.*B
        if not prescaled:
            _prefactor_c(C, c_pref)
        C += ab_pref * (A * B)
        return
    if alg == Algorithm.GER:
        # scale when C_prefactor != 1 (Dispatch.hpp:343-346), then ger.
        if not prescaled and c_pref != 1.0:
            C *= c_pref
        a_t = [l for l in Cl if l in Al]
        b_t = [l for l in Cl if l in Bl]
        C2 = _group(C, Cl, a_t, b_t)
        C2 += ab_pref * np.outer(_group(A, Al, a_t, []).ravel(), _group(B, Bl, b_t, []).ravel())
        return
    if alg == Algorithm.GEMV:
        swap = not an.is_gemv(False)
        Ml, Mx, Vl, Vx = (Bl, B, Al, A) if swap else (Al, A, Bl, B)
        links = [l for l in Ml if l in Vl and l not in Cl]
        targets = [l for l in Cl]
        A2 = _group(Mx, Ml, targets, links)
        x = _group(Vx, Vl, links, []).ravel()
        C1 = _group(C, Cl, targets, []).reshape(-1)
        y = ab_pref * (A2 @ x)
        if prescaled or c_pref == 0.0:
            if prescaled:
                y = y + C1
            C1[...] = y
        else:
            C1[...] = y + c_pref * C1
        return
    if alg == Algorithm.GEMM:
        links = [l for l in Al if l in Bl and l not in Cl]
        a_t = [l for l in Cl if l in Al]
        b_t = [l for l in Cl if l in Bl]
        A2 = _group(A, Al, a_t, links)
        B2 = _group(B, Bl, links, b_t)
        C2 = _group(C, Cl, a_t, b_t)
        y = ab_pref * (A2 @ B2)
        if prescaled:
            C2 += y
        elif c_pref == 0.0:
            C2[...] = y
        else:
            C2[...] = y + c_pref * C2
        return
    raise AssertionError(alg)


def permute(C_labels, C: np.ndarray, beta: float, alpha: float, A_labels, A: np.ndarray) -> None:
    """permute(beta, Cidx, &C, alpha, Aidx, A) (Permute.hpp:338-407):
    C[idx] = beta * C[idx] + alpha * A[perm(idx)]; C is zeroed first when
    beta == 0.  Raises ValueError (the reference's dimension_error) when a
    dimension of C is smaller than the matching dimension of A."""
    Cl, Al = list(C_labels), list(A_labels)
    if len(Cl) != len(Al) or sorted(map(str, Cl)) != sorted(map(str, Al)):
        raise ValueError("permute needs the same index set on both sides")
    for d, l in enumerate(Cl):
        if C.shape[d] < A.shape[Al.index(l)]:
            raise ValueError(f"dimension {d} of the output is smaller than the input")
    if beta == 0.0:
        C[...] = 0.0
    sA = _estrides(A)
    sA_c = [sA[Al.index(l)] for l in Cl]
    cdims = [A.shape[Al.index(l)] for l in Cl]
    L = lib()
    if alpha == 1.0 and beta == 0.0:
        L.oracle_permute_copy(len(Cl), _i64(cdims), _i64(_estrides(C)), _i64(sA_c), _base_ptr(C),
                              _base_ptr(A))
    else:
        L.oracle_permute(len(Cl), _i64(cdims), _i64(_estrides(C)), _i64(sA_c), float(beta),
                         _base_ptr(C), float(alpha), _base_ptr(A))


def rel_fro(x: np.ndarray, ref: np.ndarray) -> float:
    """Relative Frobenius error ||x - ref|| / ||ref||, computed in long double
    where the platform has it."""
    xd = np.asarray(x, dtype=np.longdouble)
    rd = np.asarray(ref, dtype=np.longdouble)
    den = np.sqrt(np.sum(rd * rd))
    num = np.sqrt(np.sum((xd - rd) * (xd - rd)))
    if den == 0:
        return float(num)
    return float(num / den)
