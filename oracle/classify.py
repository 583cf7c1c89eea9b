"""Oracle restatement of the reference's einsum pattern analysis.

TEST INFRASTRUCTURE ONLY.  This module is part of the CPU oracle: only the
tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg may
import it, and only to check results.  The product path classifies patterns in
``include/einsums_gb300/classify.hpp`` (compiled into the CUDA library) and
never calls into ``oracle/``.

Two variants exist in the reference and both are restated here:

* ``classify_cpp`` follows the compile-time ``if constexpr`` chain of
  ``libs/Einsums/TensorAlgebra/include/Einsums/TensorAlgebra/Backends/Dispatch.hpp:859-957``
  with the predicates ``einsum_is_dot_product`` (:215-221),
  ``einsum_is_direct_product`` (:226-238), ``einsum_is_outer_product``
  (:243-266), ``einsum_is_matrix_vector`` (:407-439) and
  ``einsum_is_matrix_product`` (:565-609), built from the set algebra of
  ``Detail/Utilities.hpp`` (``IntersectT``/``DifferenceT``/``UniqueT``,
  ``find_type_with_position`` :133-136, ``contiguous_positions`` :320-327,
  ``is_same_ordering`` :336-345).
* ``classify_py`` follows the runtime string analysis of
  ``libs/EinsumsPy/TensorAlgebra/src/PyTensorAlgebra.cpp:168-554``.

Labels are any hashable items (characters for the Python form, index-tag
names for the C++ form).  ``Algorithm`` numbering is the reference's
``AlgorithmChoice`` enum (``Detail/Utilities.hpp:26-34``).
"""
from __future__ import annotations

import enum
from typing import Sequence


class Algorithm(enum.IntEnum):
    GENERIC = 0
    DOT = 1
    DIRECT = 2
    GER = 3
    GEMV = 4
    GEMM = 5
    INDETERMINATE = 6


PLAN_NAMES = {
    Algorithm.GENERIC: "EinsumGenericPlan",
    Algorithm.DOT: "EinsumDotPlan",
    Algorithm.DIRECT: "EinsumDirectProductPlan",
    Algorithm.GER: "EinsumGerPlan",
    Algorithm.GEMV: "EinsumGemvPlan",
    Algorithm.GEMM: "EinsumGemmPlan",
}


# --- set algebra (Detail/Utilities.hpp) -------------------------------------

def intersect(x: Sequence, y: Sequence) -> list:
    """Elements of x (in x's order, duplicates kept) that occur in y."""
    return [e for e in x if e in y]


def difference(x: Sequence, y: Sequence) -> list:
    """Elements of x (in x's order, duplicates kept) that do not occur in y."""
    return [e for e in x if e not in y]


def unique(x: Sequence) -> list:
    out = []
    for e in x:
        if e not in out:
            out.append(e)
    return out


def find_with_pos(x: Sequence, y: Sequence) -> list:
    """For each element of x in x's order, every position where it occurs in y."""
    return [(e, j) for e in x for j, f in enumerate(y) if f == e]


def contiguous(pairs: list) -> bool:
    return all(pairs[i][1] == pairs[i + 1][1] - 1 for i in range(len(pairs) - 1))


def same_ordering(x: list, y: list) -> bool:
    if len(x) == 0 or len(y) == 0 or len(x) != len(y):
        return False
    return all(a[0] == b[0] for a, b in zip(x, y))


class Analysis:
    """All the intermediate sets the reference computes for a pattern."""

    def __init__(self, C, A, B):
        self.C, self.A, self.B = list(C), list(A), list(B)
        C, A, B = self.C, self.A, self.B
        self.linksAB = intersect(A, B)
        self.links = difference(self.linksAB, C)
        self.C_unique = unique(C)
        self.link_unique = unique(self.links)
        self.link_pos_A = find_with_pos(self.link_unique, A)
        self.link_pos_B = find_with_pos(self.link_unique, B)
        self.target_pos_A = find_with_pos(self.C_unique, A)
        self.target_pos_B = find_with_pos(self.C_unique, B)
        self.target_pos_C = find_with_pos(self.C_unique, C)
        self.A_target_pos_C = find_with_pos(A, C)
        self.B_target_pos_C = find_with_pos(B, C)
        self.hadamard = (len(unique(A)) != len(A) or len(unique(B)) != len(B)
                         or len(unique(C)) != len(C))

    def is_dot(self):
        return len(self.C) == 0 and self.A == self.B

    def is_direct(self):
        return self.C == self.A and self.C == self.B

    def is_outer(self):
        return (len(self.linksAB) == 0 and contiguous(self.target_pos_A)
                and contiguous(self.target_pos_B))

    def is_gemv(self, swap=False):
        # einsum_is_matrix_vector(C, A, B); swap=True evaluates it for (C, B, A).
        lpA, lpB = (self.link_pos_B, self.link_pos_A) if swap else (self.link_pos_A, self.link_pos_B)
        tpA, tpB = (self.target_pos_B, self.target_pos_A) if swap else (self.target_pos_A, self.target_pos_B)
        AtC, BtC = (self.B_target_pos_C, self.A_target_pos_C) if swap else (self.A_target_pos_C, self.B_target_pos_C)
        return (contiguous(lpA) and contiguous(lpB) and contiguous(tpA)
                and same_ordering(lpA, lpB) and same_ordering(tpA, AtC)
                and not same_ordering(tpB, BtC) and len(BtC) == 0)

    def is_gemm(self):
        CminusA = difference(self.C, self.A)
        CminusB = difference(self.C, self.B)
        return (len(CminusA) > 0 and len(CminusB) > 0
                and contiguous(self.link_pos_A) and contiguous(self.link_pos_B)
                and contiguous(self.target_pos_A) and contiguous(self.target_pos_B)
                and contiguous(self.A_target_pos_C) and contiguous(self.B_target_pos_C)
                and same_ordering(self.link_pos_A, self.link_pos_B)
                and same_ordering(self.target_pos_A, self.A_target_pos_C)
                and same_ordering(self.target_pos_B, self.B_target_pos_C))


def classify_cpp(C, A, B) -> Algorithm:
    """Compile-time choice of Dispatch.hpp:893-951 for real, same-typed basic tensors.

    The runtime stride vetoes (``einsum_do_*`` returning false) are applied
    separately by ``oracle.einsum`` because they depend on strides.
    """
    an = Analysis(C, A, B)
    if an.hadamard:
        return Algorithm.GENERIC
    if an.is_dot():
        return Algorithm.DOT
    if an.is_direct():
        return Algorithm.DIRECT
    if an.is_outer():
        return Algorithm.GER
    if an.is_gemv(False) or an.is_gemv(True):
        return Algorithm.GEMV
    if len(an.C) >= 2 and len(an.A) >= 2 and len(an.B) >= 2 and an.is_gemm():
        return Algorithm.GEMM
    return Algorithm.GENERIC


def classify_py(C, A, B) -> Algorithm:
    """Plan type chosen by compile_plan (PyTensorAlgebra.cpp:168-554)."""
    an = Analysis(C, A, B)
    if an.hadamard:
        # Every specialised plan requires !hadamard in PyTensorAlgebra.cpp.
        return Algorithm.GENERIC
    if len(an.C) == 0 and an.A == an.B:
        return Algorithm.DOT
    if an.C == an.A and an.C == an.B:
        return Algorithm.DIRECT
    if an.is_outer():
        return Algorithm.GER
    if an.is_gemv(False) or an.is_gemv(True):
        return Algorithm.GEMV
    if an.is_gemm():
        return Algorithm.GEMM
    return Algorithm.GENERIC
