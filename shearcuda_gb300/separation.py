"""Undecimated wavelets and the points / curves image separation, the Python
face of nsst_onfilter, nsst_mrdwt, nsst_mirdwt, nsst_tv_correction and
nsst_separate (include/nsst.h).

Names and argument meaning follow the reference's MATLAB API:
MakeONFilter(Type, Par), [yl, yh] = mrdwt_cuda(x, h, L),
x = mirdwt_cuda(yl, yh, h, L), TVCorrection_cuda(x, gamma) and
[C, P] = separate(img, level2, itermax, stop, gamma, coeff, display, shear)
(shearcuda/MakeONFilter.m, src_cuda/mrdwt_cuda.cpp, src_cuda/mirdwt_cuda.cpp,
shearcuda/separate.m).  Images are row-major (H, W) float32 CUDA tensors, or
batches (n, H, W); yh is (3L, H, W) per image, per level the planes LH, HL, HH.
"""
import ctypes

import numpy as np
import torch

from ._lib import NsstError, NsstSeparateInfo, check, lib
from .ops import _dev, _stream

__all__ = ['MakeONFilter', 'mrdwt_cuda', 'mirdwt_cuda', 'tv_correction_cuda', 'separate']

MAX_QMF = 64


def MakeONFilter(family, par=0):  # noqa: N802 (the reference's name)
    """Orthonormal QMF of MakeONFilter.m, f / norm(f), as float64 numpy."""
    out = (ctypes.c_double * MAX_QMF)()
    n = ctypes.c_int()
    check(lib().nsst_onfilter(family.encode(), int(par), out, ctypes.byref(n)))
    return np.array(out[:n.value], dtype=np.float64)


def _batch(x, name):
    if x.dim() == 2:
        return x.unsqueeze(0), True
    if x.dim() != 3:
        raise NsstError(1, '%s must be (H, W) or (n, H, W)' % name)
    return x, False


def _qmf(h):
    h = np.ascontiguousarray(np.asarray(h, dtype=np.float64).ravel())
    return h, h.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def mrdwt_cuda(x, h, L, yl=None, yh=None, stream=None):
    """Redundant DWT (mrdwt.m / mrdwt_cuda): returns (yl, yh) with yl like x
    and yh (3L, H, W), or (n, 3L, H, W) for a batch."""
    xb, single = _batch(x, 'x')
    n, H, W = xb.shape
    hv, hp = _qmf(h)
    if yl is None:
        yl = torch.empty_like(x)
    if yh is None:
        yh = torch.empty(((3 * L, H, W) if single else (n, 3 * L, H, W)), device=x.device, dtype=torch.float32)
    check(lib().nsst_mrdwt(_dev(xb, 'x'), n, H, W, hp, hv.size, int(L), _dev(yl, 'yl', tuple(x.shape)),
                           _dev(yh, 'yh', (3 * L, H, W) if single else (n, 3 * L, H, W)), _stream(stream)))
    return yl, yh


def mirdwt_cuda(yl, yh, h, L, x=None, stream=None):
    """Inverse redundant DWT (mirdwt.m / mirdwt_cuda); yl and yh are unchanged."""
    yb, single = _batch(yl, 'yl')
    n, H, W = yb.shape
    hv, hp = _qmf(h)
    if x is None:
        x = torch.empty_like(yl)
    check(lib().nsst_mirdwt(_dev(yb, 'yl'), _dev(yh, 'yh', (3 * L, H, W) if single else (n, 3 * L, H, W)), n, H, W,
                            hp, hv.size, int(L), _dev(x, 'x', tuple(yl.shape)), _stream(stream)))
    return x


def tv_correction_cuda(x, gamma, out=None, stream=None):
    """TVCorrection_cuda (separate.m:278-285): Haar mrdwt of one level, soft
    threshold gamma on its highpass planes, mirdwt."""
    xb, _ = _batch(x, 'x')
    n, H, W = xb.shape
    if out is None:
        out = torch.empty_like(x)
    check(lib().nsst_tv_correction(_dev(xb, 'x'), n, H, W, float(gamma), _dev(out, 'out', tuple(x.shape)),
                                   _stream(stream)))
    return out


def separate(img, level2, itermax, stop, gamma, coeff, shear, display=0, stream=None):
    """Points / curves separation (separate.m) with the shearlets of ``shear``
    (a ShearPlan; a batch (n, H, W) needs batch capacity n).  Returns
    (C, P, info): curves, points, and per image a dict of the setup values
    sigma, stop, buff_shear, buff_wavelet, deltamax, lam.  ``display`` is
    accepted for signature parity and ignored, as the reference ignores it on
    the GPU (separate.m:47-53)."""
    xb, single = _batch(img, 'img')
    n, H, W = xb.shape
    if (H, W) != (shear.H, shear.W):
        raise NsstError(1, 'img is %dx%d, the plan %dx%d' % (H, W, shear.H, shear.W))
    w = np.ascontiguousarray(np.asarray(coeff, dtype=np.float64).ravel())
    C = torch.empty_like(img)
    P = torch.empty_like(img)
    info = (NsstSeparateInfo * n)()
    check(lib().nsst_separate(shear.handle, _dev(xb, 'img'), n, int(level2), int(itermax), float(stop), float(gamma),
                              w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), int(w.size),
                              _dev(C, 'C'), _dev(P, 'P'), info, _stream(stream)))
    recs = [{k: getattr(info[i], k) for k, _ in NsstSeparateInfo._fields_} for i in range(n)]
    return C, P, (recs[0] if single else recs)
