"""ctypes access to the reference's own atrousc.cpp (oracle/_ref), used only
to pin the oracle's restatements.  Test infrastructure only."""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


def available():
    return os.path.exists(build_oracle.REF_SO)


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_oracle.REF_SO)
        _lib.ref_atrousc.restype = ctypes.c_int
        _lib.ref_atrousc_error.restype = ctypes.c_char_p
    return _lib


def atrousc(S, F, M):
    """Reference atrousc(S, F, M*eye(2)) on FP64 (row, col)-indexed arrays.

    MATLAB arrays are column-major; the glue receives Fortran-ordered copies
    so that (row, col) means the same thing on both sides."""
    lib = _load()
    S = np.asfortranarray(S, dtype=np.float64)
    F = np.asfortranarray(F, dtype=np.float64)
    Sm, Sn = S.shape
    Fm, Fn = F.shape
    out = np.zeros((Sm - M * Fm + 1, Sn - M * Fn + 1), dtype=np.float64, order='F')
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    rc = lib.ref_atrousc(p(S), Sm, Sn, p(F), Fm, Fn, ctypes.c_double(M), p(out))
    if rc != 0:
        raise RuntimeError(lib.ref_atrousc_error().decode())
    return np.ascontiguousarray(out)
