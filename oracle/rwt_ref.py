"""ctypes access to the reference's own Rice Wavelet Toolbox templates
(shearcuda/src/mrdwt_r.h, mirdwt_r.h, mdwt_r.h via oracle/_ref/librwt_ref.so),
used only to pin the oracle's restatements.  Test infrastructure only.

Arrays are passed as Fortran-ordered copies so that (row, col) means the same
on both sides; the reference's m x 3nL yh is split into (3L, m, n) planes."""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


def available():
    return os.path.exists(build_oracle.RWT_SO)


def _load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build_oracle.RWT_SO)
        for f in ('ref_mrdwt', 'ref_mirdwt', 'ref_mdwt'):
            getattr(_lib, f).restype = None
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def mrdwt(x, h, L):
    x = np.asfortranarray(x, dtype=np.float64)
    m, n = x.shape
    h = np.ascontiguousarray(h, dtype=np.float64)
    yl = np.zeros((m, n), order='F')
    yh = np.zeros((m, 3 * n * L), order='F')
    _load().ref_mrdwt(_p(x), m, n, _p(h), h.size, L, _p(yl), _p(yh))
    return np.ascontiguousarray(yl), np.stack([yh[:, p * n:(p + 1) * n] for p in range(3 * L)])


def mirdwt(yl, yh, h, L):
    yl = np.asfortranarray(yl, dtype=np.float64)
    m, n = yl.shape
    yhm = np.asfortranarray(np.concatenate(list(yh), axis=1), dtype=np.float64)
    h = np.ascontiguousarray(h, dtype=np.float64)
    x = np.zeros((m, n), order='F')
    _load().ref_mirdwt(_p(x), m, n, _p(h), h.size, L, _p(yl), _p(yhm))
    return np.ascontiguousarray(x)


def mdwt(x, h, L):
    x = np.asfortranarray(x, dtype=np.float64)
    m, n = x.shape
    h = np.ascontiguousarray(h, dtype=np.float64)
    y = np.zeros((m, n), order='F')
    _load().ref_mdwt(_p(x), m, n, _p(h), h.size, L, _p(y))
    return np.ascontiguousarray(y)
