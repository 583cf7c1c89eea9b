"""ctypes access to the reference's HPTT built by oracle/Makefile.

TEST INFRASTRUCTURE ONLY (pins oracle.permute bit for bit).  The library
exists only where the reference checkout was present at build time.
"""
import ctypes
import os

import numpy as np

_SO = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref", "libhptt_ref.so")
_LIB = None


def available() -> bool:
    return os.path.exists(_SO)


def _lib():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(_SO)
        _LIB.hptt_ref_permute.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                          ctypes.POINTER(ctypes.c_size_t), ctypes.c_double,
                                          ctypes.c_void_p, ctypes.c_double, ctypes.c_void_p,
                                          ctypes.c_int]
    return _LIB


def permute(A: np.ndarray, perm, alpha=1.0, beta=0.0, out=None, threads=1) -> np.ndarray:
    """B[perm-ordered] = alpha * A + beta * B, like np.transpose(A, perm)."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    shape = [A.shape[p] for p in perm]
    B = np.zeros(shape) if out is None else out
    r = len(perm)
    p = (ctypes.c_int * r)(*perm)
    s = (ctypes.c_size_t * r)(*A.shape)
    rc = _lib().hptt_ref_permute(r, p, s, float(alpha), A.ctypes.data, float(beta), B.ctypes.data, threads)
    if rc != 0:
        raise RuntimeError("hptt plan failed")
    return B
