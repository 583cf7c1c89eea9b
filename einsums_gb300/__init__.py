"""einsums_gb300: GB300-native (sm_103a) tensor-contraction hot path of Einsums.

The product is the C-ABI library ``libeinsums_gb300.so`` (include/einsums_gb300.h);
this package is its Python front end (``core``) plus the autograd binding.
Importing it loads the CUDA library; there is no CPU fallback.
"""
from . import _lib
from .autograd import Einsum, einsum_ag
from .blocks import BlockTensor, TiledTensor
from .core import (ALGORITHMS, EinsumDirectProductPlan, EinsumDotPlan, EinsumGemmPlan, EinsumGemvPlan,
                   EinsumGenericPlan, EinsumGerPlan, GroupedPlan, PermutePlan, compile_permute, compile_plan, einsum,
                   fock_jk_symmetric, last_split_report,
                   permute)

__all__ = ["compile_plan", "einsum", "permute", "compile_permute", "PermutePlan", "fock_jk_symmetric", "BlockTensor", "TiledTensor", "GroupedPlan", "Einsum", "einsum_ag", "last_split_report", "ALGORITHMS", "EinsumGenericPlan",
           "EinsumDotPlan", "EinsumDirectProductPlan", "EinsumGerPlan", "EinsumGemvPlan", "EinsumGemmPlan"]
