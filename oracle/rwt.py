"""Undecimated and decimated 2-D wavelets, MakeONFilter, and the points /
curves separation loop, restated in FP64 numpy.

Test infrastructure only: this is the oracle the GPU path is checked against.
It is pinned against the reference's own Rice Wavelet Toolbox templates
(shearcuda/src/mrdwt_r.h, mirdwt_r.h, mdwt_r.h) compiled into
oracle/_ref/librwt_ref.so (tests/test_rwt_oracle.py), and against golden
vectors produced by those templates (tests/golden/rwt_golden.json).

Arrays are row-major (H, W); "rows" filtering runs along W, as the
reference's "go by rows" loop runs along a MATLAB row.  yh is (3L, H, W): per
level the planes LH, HL, HH (first letter: row filtering).
"""
import json
import os

import numpy as np

from . import nsst2d

_TABLES = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'onfilter_tables.json')))['tables']


def make_on_filter(family, par=0):
    """MakeONFilter.m:51-289: tabulated coefficients (oracle/onfilter_tables.json,
    generated from MakeONFilter.m), the Battle mirror (:283-286), f / norm(f)."""
    has_par = family in ('Coiflet', 'Daubechies', 'Symmlet', 'Battle')
    for t in _TABLES:
        if t['type'] == family and (not has_par or t['par'] == par):
            v = np.asarray(t['values'], dtype=np.float64)
            f = np.concatenate([v[1:][::-1], v]) if t['half'] else v
            return f / np.sqrt(np.sum(f * f))
    raise ValueError('no MakeONFilter table for %s %s' % (family, par))


def _analysis_pair(h):
    """mrdwt_r.h:118-125 (and mdwt_r.h:113-120): h0 = reverse(h); h1 = h with
    the even entries negated."""
    h = np.asarray(h, dtype=np.float64)
    h0 = h[::-1].copy()
    h1 = h.copy()
    h1[0::2] = -h1[0::2]
    return h0, h1


def _synthesis_pair(h):
    """mirdwt_r.h:125-130: g0 = h / 2; g1 = reverse(h) / 2 with the odd entries
    negated."""
    h = np.asarray(h, dtype=np.float64)
    g0 = h / 2
    g1 = h[::-1] / 2
    g1[1::2] = -g1[1::2]
    return g0, g1


def _fpconv(x, h0, h1, sf, axis):
    """fpconv (mrdwt_r.h:84-101) along every dilated chain of one axis:
    lo[c] = sum_j x[(c + j sf) mod n] h0[lh-1-j], hi likewise with h1 (j ascending)."""
    lh = len(h0)
    lo = np.zeros_like(x)
    hi = np.zeros_like(x)
    for j in range(lh):
        s = np.roll(x, -j * sf, axis=axis)
        lo = lo + s * h0[lh - 1 - j]
        hi = hi + s * h1[lh - 1 - j]
    return lo, hi


def _bpconv(xl, xh, g0, g1, sf, axis):
    """bpconv (mirdwt_r.h:95-112): x[c] = sum_j xl[c - t sf] g0[t] + xh[c - t sf] g1[t],
    t = lh-1-j, j ascending, periodic."""
    lh = len(g0)
    out = np.zeros_like(xl)
    for j in range(lh):
        t = lh - 1 - j
        out = out + np.roll(xl, t * sf, axis=axis) * g0[t] + np.roll(xh, t * sf, axis=axis) * g1[t]
    return out


def mrdwt(x, h, L):
    """mrdwt_r.h:104-209 (2-D): per level rows (:149-178), then columns (:180-206)."""
    h0, h1 = _analysis_pair(h)
    yl = np.array(x, dtype=np.float64)
    H, W = yl.shape
    if H % 2 ** L or W % 2 ** L:
        raise ValueError('H and W must be multiples of 2^L')
    yh = np.zeros((3 * L, H, W))
    for lv in range(L):
        sf = 2 ** lv
        lo, hr = _fpconv(yl, h0, h1, sf, axis=1)
        yl, yh[3 * lv] = _fpconv(lo, h0, h1, sf, axis=0)           # LL, LH
        yh[3 * lv + 1], yh[3 * lv + 2] = _fpconv(hr, h0, h1, sf, axis=0)  # HL, HH
    return yl, yh


def mirdwt(yl, yh, h, L):
    """mirdwt_r.h:115-219 (2-D): levels L..1, columns (:163-189), then rows (:192-213)."""
    g0, g1 = _synthesis_pair(h)
    x = np.array(yl, dtype=np.float64)
    for lv in range(L - 1, -1, -1):
        sf = 2 ** lv
        x1 = _bpconv(x, yh[3 * lv], g0, g1, sf, axis=0)
        xh = _bpconv(yh[3 * lv + 1], yh[3 * lv + 2], g0, g1, sf, axis=0)
        x = _bpconv(x1, xh, g0, g1, sf, axis=1)
    return x


def _fpsconv(x, h0, h1, axis):
    """fpsconv (mdwt_r.h:81-99): the even samples of the periodic filtering."""
    lo, hi = _fpconv(x, h0, h1, 1, axis)
    sl = [slice(None)] * x.ndim
    sl[axis] = slice(0, None, 2)
    return lo[tuple(sl)], hi[tuple(sl)]


def mdwt(x, h, L):
    """mdwt_r.h:102-176 (2-D): decimated DWT in place, rows then columns per level."""
    h0, h1 = _analysis_pair(h)
    y = np.array(x, dtype=np.float64)
    am, an = y.shape
    for _ in range(L):
        lo, hi = _fpsconv(y[:am, :an], h0, h1, axis=1)
        y[:am, :an // 2], y[:am, an // 2:an] = lo, hi
        lo, hi = _fpsconv(y[:am, :an], h0, h1, axis=0)
        y[:am // 2, :an], y[am // 2:am, :an] = lo, hi
        am //= 2
        an //= 2
    return y


def mad(x):
    """MAD.m: median(|x - median(x)|) / .6745 over the non-NaN values."""
    x = np.asarray(x, dtype=np.float64).ravel()
    x = x[~np.isnan(x)]
    return float(np.median(np.abs(x - np.median(x))) / .6745)


def soft_thresh(y, t):
    """SoftThresh.m: sign(y) (|y| - t)_+."""
    res = np.abs(y) - t
    res = (res + np.abs(res)) / 2
    return np.sign(y) * res


def tv_correction(x, gamma):
    """separate.m:268-276 (TVCorrection): one Haar level, soft threshold of yh."""
    qmf = make_on_filter('Haar')
    ll, wc = mrdwt(x, qmf, 1)
    return mirdwt(ll, soft_thresh(wc, gamma), qmf, 1)


def _planes(dst):
    out = [dst[0]]
    for b in dst[1:]:
        out.extend(list(b))
    return out


def _unplanes(planes, like):
    out = [planes[0]]
    at = 1
    for b in like[1:]:
        out.append(np.stack(planes[at:at + b.shape[0]]))
        at += b.shape[0]
    return out


def separate(img, dcomp, dsize, level2, itermax, stop, gamma, coeff, fname='maxflat', nthreads=1,
             residual='gpu'):
    """separate.m:41-289.  Returns (C, P, info) with info the setup values
    (sigma, stop, buff_shear, buff_wavelet, deltamax, lambda).
    residual='gpu' forms (img - p1) - p2 as the GPUminus calls do
    (separate.m:146-148); 'cpu' forms img - (p1 + p2) (:150)."""
    img = np.asarray(img, dtype=np.float64)
    H, W = img.shape
    qmf = make_on_filter('Symmlet', 4)
    d4 = make_on_filter('Daubechies', 4)
    shear_f = nsst2d.shear_spectra(H, W, dcomp, dsize)
    E = nsst2d.com_norm(H, W, dcomp, dsize, fname, shear_f=shear_f, nthreads=nthreads)
    x = nsst2d.re_weight_band(img, coeff, fname, nthreads=nthreads)
    # separate.m:82-102
    wc = mdwt(x, d4, 1)
    sigma = mad(wc[H // 2:, W // 2:])
    stop_s = stop * sigma
    # separate.m:104-126
    dst, _ = nsst2d.nsst_dec2(x, dcomp, dsize, fname, shear_f=shear_f, nthreads=nthreads)
    b1 = nsst2d.thresh_maxi(_planes(dst), E)
    _, yh = mrdwt(x, qmf, level2)
    b2 = float(np.max(np.abs(yh)))
    deltamax = min(b1, b2)
    lam = (deltamax / stop_s) ** (1.0 / (1 - itermax)) if itermax > 1 else float('inf')
    delta = deltamax
    p1 = np.zeros((H, W))
    p2 = np.zeros((H, W))
    for _ in range(itermax):
        r = (x - p1) - p2 if residual == 'gpu' else x - (p1 + p2)
        ra = p1 + r
        ra2 = p2 + r
        dst, _ = nsst2d.nsst_dec2(ra, dcomp, dsize, fname, shear_f=shear_f, nthreads=nthreads)
        planes = [c * (np.abs(c) > 1 * (1.4 * delta) * e) for c, e in zip(_planes(dst), E)]
        p1 = tv_correction(nsst2d.nsst_rec2(_unplanes(planes, dst), shear_f, fname, nthreads=nthreads), gamma)
        yl, yh = mrdwt(ra2, qmf, level2)
        yh = yh * (np.abs(yh) > 1.4 * delta)
        p2 = mirdwt(yl, yh, qmf, level2)
        delta = delta * lam
    info = dict(sigma=sigma, stop=stop_s, buff_shear=b1, buff_wavelet=b2, deltamax=deltamax, lam=lam)
    return p1, p2, info
