"""ctypes binding of the C ABI in include/einsums_gb300.h.

Loads ``einsums_gb300/_build/libeinsums_gb300.so`` (built in-tree by
``einsums_gb300.build``).  There is no fallback: when the library is missing
every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_build", "libeinsums_gb300.so")
MAX_RANK = 8

EG_SUCCESS = 0
STATUS = {
    1: "invalid argument", 2: "rank error", 3: "dimension error", 4: "not supported", 5: "CUDA error",
    6: "out of memory", 7: "device wait timed out", 8: "precision target not reachable",
}

PRECISION_FP64, PRECISION_SPLIT_BF16 = 0, 1
SEMANTICS_CPP, SEMANTICS_PYTHON = 0, 1


class EinsumsError(RuntimeError):
    """Base class of errors reported by the library."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, 'error')}: {message}")
        self.status = status


class RankError(EinsumsError, ValueError):
    pass


class DimensionError(EinsumsError, ValueError):
    pass


class NotSupportedError(EinsumsError, NotImplementedError):
    pass


class DeviceTimeoutError(EinsumsError):
    pass


_ERRORS = {2: RankError, 3: DimensionError, 4: NotSupportedError, 7: DeviceTimeoutError}


class EgTensor(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("rank", ctypes.c_int32),
                ("extent", ctypes.c_int64 * MAX_RANK), ("stride", ctypes.c_int64 * MAX_RANK)]


class EgOptions(ctypes.Structure):
    _fields_ = [("precision", ctypes.c_int32), ("slices", ctypes.c_int32), ("tolerance", ctypes.c_double),
                ("semantics", ctypes.c_int32), ("only_generic", ctypes.c_int32)]


class EgSplitReport(ctypes.Structure):
    _fields_ = [("slices", ctypes.c_int32), ("slice_pairs", ctypes.c_int32), ("bits_per_slice", ctypes.c_int32),
                ("error_bound", ctypes.c_double)]


# Every symbol the header declares, with its ctypes prototype.
_P = ctypes.POINTER
_i32p = _P(ctypes.c_int32)
_T = _P(EgTensor)
PROTOTYPES = {
    "eg_options_default": (None, [_P(EgOptions)]),
    "eg_einsum": (ctypes.c_int, [ctypes.c_double, _i32p, _T, ctypes.c_double, _i32p, _T, _i32p, _T,
                                 _P(EgOptions), ctypes.c_void_p, _i32p]),
    "eg_classify": (ctypes.c_int, [ctypes.c_int32, _i32p, ctypes.c_int32, _i32p, ctypes.c_int32, _i32p,
                                   ctypes.c_int32, _i32p]),
    "eg_permute": (ctypes.c_int, [ctypes.c_double, _i32p, _T, ctypes.c_double, _i32p, _T, ctypes.c_void_p]),
    "eg_permute_plan_create": (ctypes.c_int, [ctypes.c_double, _i32p, _T, ctypes.c_double, _i32p, _T,
                                              _P(ctypes.c_void_p)]),
    "eg_permute_plan_execute": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "eg_permute_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "eg_einsum_batched": (ctypes.c_int, [ctypes.c_double, _i32p, _T, ctypes.c_double, _i32p, _T, _i32p, _T,
                                         ctypes.c_int64, _P(EgOptions), ctypes.c_void_p, _i32p]),
    "eg_einsum_complex": (ctypes.c_int, [_P(ctypes.c_double), _i32p, _T, _P(ctypes.c_double), _i32p, _T, _i32p,
                                         _T, ctypes.c_int32, ctypes.c_int32, _P(EgOptions), ctypes.c_void_p, _i32p]),
    "eg_einsum_blocks": (ctypes.c_int, [ctypes.c_double, _i32p, _T, ctypes.c_double, _i32p, _T, _i32p, _T,
                                        ctypes.c_int64, _P(EgOptions), ctypes.c_void_p, _i32p]),
    "eg_dot_noalloc": (ctypes.c_int, [ctypes.c_double, ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p]),
    "eg_fock_jk_symmetric": (ctypes.c_int, [ctypes.c_double, ctypes.c_void_p, ctypes.c_double, ctypes.c_double,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, _P(EgOptions),
                                            ctypes.c_void_p]),
    "eg_grouped_plan_create": (ctypes.c_int, [ctypes.c_double, _i32p, _T, ctypes.c_double, _i32p, _T, _i32p, _T,
                                              ctypes.c_int64, _P(EgOptions), ctypes.c_void_p,
                                              _P(ctypes.c_void_p), _i32p]),
    "eg_grouped_plan_execute": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "eg_grouped_plan_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "eg_last_split_report": (ctypes.c_int, [_P(EgSplitReport)]),
    "eg_device_alloc": (ctypes.c_int, [ctypes.c_size_t, _P(ctypes.c_void_p)]),
    "eg_device_free": (ctypes.c_int, [ctypes.c_void_p]),
    "eg_set_memory_budget": (ctypes.c_int, [ctypes.c_size_t]),
    "eg_memory_in_use": (ctypes.c_int, [_P(ctypes.c_size_t)]),
    "eg_copy_to_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "eg_copy_to_host": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "eg_stream_synchronize": (ctypes.c_int, [ctypes.c_void_p]),
    "eg_stream_status": (ctypes.c_int, [ctypes.c_void_p, _P(ctypes.c_int32)]),
    "eg_measure_fp64_peak": (ctypes.c_int, [_P(ctypes.c_double), _P(ctypes.c_double)]),
    "eg_measure_fp64_peak_clock": (ctypes.c_int, [_P(ctypes.c_double), _P(ctypes.c_double), _P(ctypes.c_double)]),
    "eg_tc_pair_clusters": (ctypes.c_int, [_P(ctypes.c_int32)]),
    "eg_kernel_launches": (ctypes.c_int, [_P(ctypes.c_uint64)]),
    "eg_selftest_wait_timeout": (ctypes.c_int, [ctypes.c_uint64, ctypes.c_void_p]),
    "eg_profile_enable": (ctypes.c_int, [ctypes.c_int32]),
    "eg_profile_reset": (ctypes.c_int, []),
    "eg_profile_summary": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t]),
    "eg_last_error": (ctypes.c_char_p, []),
    "eg_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "eg_version": (ctypes.c_char_p, []),
}

_LIB = None
_LOCK = threading.Lock()


def load(path: str | None = None):
    """Load the library (once) and attach prototypes.  Raises when absent."""
    global _LIB
    with _LOCK:
        if _LIB is None:
            p = path or LIB_PATH
            if not os.path.exists(p):
                raise RuntimeError(
                    f"einsums_gb300 CUDA library not found at {p}; run `python -m einsums_gb300.build` "
                    "(there is no CPU fallback)")
            lib = ctypes.CDLL(p)
            for name, (res, args) in PROTOTYPES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _LIB = lib
    return _LIB


def check(status: int) -> None:
    if status != EG_SUCCESS:
        msg = load().eg_last_error().decode(errors="replace")
        raise _ERRORS.get(status, EinsumsError)(status, msg)


def label_id(name) -> int:
    """Stable 31-bit label for an index name: FNV-1a of its UTF-8 bytes (the
    C++ front end hashes index-tag letters the same way)."""
    h = 0x811C9DC5
    for b in str(name).encode():
        h ^= b
        h = (h * 0x01000193) & 0xFFFFFFFF
    return h & 0x7FFFFFFF


def labels(names) -> ctypes.Array:
    ids = [label_id(n) for n in names]
    arr = (ctypes.c_int32 * max(1, len(ids)))()
    for i, v in enumerate(ids):
        arr[i] = v
    return arr
