"""ctypes access to the oracle's C restatement (oracle/atrous_port.c).
Test infrastructure only."""
import ctypes
import os

import numpy as np

from . import build_oracle

_lib = None


def _load():
    global _lib
    if _lib is None:
        if not os.path.exists(build_oracle.PORT_SO):
            build_oracle.build_port()
        _lib = ctypes.CDLL(build_oracle.PORT_SO)
        for name in ('symext_port', 'atrous_level'):
            getattr(_lib, name).restype = ctypes.c_int
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def atrousc(S, F, M):
    """atrousc.cpp:43-73 restated: 'valid' conv of S with F upsampled by M."""
    lib = _load()
    S = np.ascontiguousarray(S, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.float64)
    Sr, Sc = S.shape
    Fr, Fc = F.shape
    out = np.empty((Sr - M * Fr + 1, Sc - M * Fc + 1))
    lib.atrousc_port(_p(S), Sr, Sc, _p(F), Fr, Fc, M, _p(out))
    return out


def symext(x, p, q, s1, s2):
    lib = _load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    m, n = x.shape
    out = np.empty((m + p - 1, n + q - 1))
    if lib.symext_port(_p(x), m, n, p, q, s1, s2, _p(out)) != 0:
        raise ValueError('symmetric extension exceeds one reflection')
    return out


def atrous_level(x, F, M, shift, nthreads=1):
    """atrousc(symext(x, upsample2df(F, log2 M), shift), F, M) in one call."""
    lib = _load()
    x = np.ascontiguousarray(x, dtype=np.float64)
    F = np.ascontiguousarray(F, dtype=np.float64)
    m, n = x.shape
    out = np.empty((m, n))
    rc = lib.atrous_level(_p(x), m, n, _p(F), F.shape[0], M, shift, _p(out), nthreads)
    if rc != 0:
        raise ValueError('atrous_level failed (%d)' % rc)
    return out
