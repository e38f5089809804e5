"""FP64 CPU oracle for the 2-D NSST decompose -> threshold -> reconstruct path.

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this module, and only as the
checker (or as the timed CPU baseline), never as part of the product path.

Each function restates one reference function of ``shearlet_toolbox_1`` in
NumPy / SciPy FP64 and cites it.  Arrays are (row, col) indexed; MATLAB's
column-major storage does not change the arithmetic.  Images may be H x W
(the reference forces square L x L at nsst_dec2.m:37; its ``./L`` at :50 is
cancelled by the ``./d`` normalisation at :55-57, so H x W is well defined).

The à trous inner loop runs either through the C restatement
(``oracle/atrous_port.c``) or, when built here, through the reference's own
``atrousc.cpp`` (``oracle/_ref``); both are pinned against each other by the
golden fixtures in tests/golden.
"""
import json
import math
import os

import numpy as np
from scipy import fft as sfft

from . import clib

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), '..', 'tests', 'golden')
_FILTER_TABLES = None


def _tables():
    global _FILTER_TABLES
    if _FILTER_TABLES is None:
        with open(os.path.join(GOLDEN, 'pyramid_filter_tables.json')) as f:
            _FILTER_TABLES = json.load(f)
    return _FILTER_TABLES


def _mirror(q):
    """atrousfilters.m:167-175: [q fliplr(q(:,1:end-1))]; then flipud likewise."""
    q = np.asarray(q, dtype=np.float64)
    q = np.concatenate([q, np.fliplr(q[:, :-1])], axis=1)
    return np.concatenate([q, np.flipud(q[:-1, :])], axis=0)


def atrousfilters(fname='maxflat'):
    """atrousfilters.m:26-237 -> (h0, h1, g0, g1) as FP64 2-D arrays."""
    t = _tables()[fname]
    if fname == '9-7':
        h0, h1, g0, g1 = (np.asarray(t[k], dtype=np.float64) for k in ('h0', 'h1', 'g0', 'g1'))
        return h0, h1 / 2.0, g0 / 2.0, g1  # atrousfilters.m:100-104
    return tuple(_mirror(t[k]) for k in ('h0', 'h1', 'g0', 'g1'))


# ----------------------------------------------------------------------------
# à trous pyramid (atrousdec.m / atrousrec.m / symext.m / upsample2df.m)
# ----------------------------------------------------------------------------
def symext(x, p, q, s1, s2):
    """symext.m:18-31 (filter p x q, shift (s1, s2))."""
    m, n = x.shape
    ss = p // 2 - s1 + 1
    rr = q // 2 - s2 + 1
    cols = np.concatenate([np.arange(ss - 1, -1, -1), np.arange(n), np.arange(n - 1, n - p - s1 - 1, -1)])
    yT = x[:, cols]
    rows = np.concatenate([np.arange(rr - 1, -1, -1), np.arange(m), np.arange(m - 1, m - q - s2 - 1, -1)])
    yT = yT[rows, :]
    return yT[: m + p - 1, : n + q - 1]


def _filter_step(x, F, M, shift, conv, nthreads):
    """One atrousc(symext(x, upsample2df(F, log2 M), shift), F, M) call; for
    M == 1 this is conv2(symext(x, F, shift), F, 'valid') (atrousdec.m:34)."""
    if conv == 'port':
        return clib.atrous_level(x, F, M, shift, nthreads)
    p = M * F.shape[0]
    S = symext(x, p, p, shift, shift)
    if conv == 'ref':
        from . import atrous_ref
        return atrous_ref.atrousc(S, F, M)
    return clib.atrousc(S, F, M)


def atrousdec(x, fname='maxflat', nlevels=4, conv='port', nthreads=1):
    """atrousdec.m:19-51.  Returns [lowpass, bandpass coarse ... fine]."""
    h0, h1, _, _ = atrousfilters(fname)
    y = [None] * (nlevels + 1)
    y0 = _filter_step(x, h0, 1, 1, conv, nthreads)
    y1 = _filter_step(x, h1, 1, 1, conv, nthreads)
    y[nlevels] = y1
    x = y0
    for i in range(1, nlevels):
        shift = -(2 ** (i - 1)) + 2
        L = 2 ** i
        y0 = _filter_step(x, h0, L, shift, conv, nthreads)
        y1 = _filter_step(x, h1, L, shift, conv, nthreads)
        y[nlevels - i] = y1
        x = y0
    y[0] = x
    return y


def atrousrec(y, fname='maxflat', conv='port', nthreads=1):
    """atrousrec.m:18-41."""
    _, _, g0, g1 = atrousfilters(fname)
    n = len(y) - 1
    x = y[0]
    for i in range(n - 1, 0, -1):
        y1 = y[n - i]
        shift = -(2 ** (i - 1)) + 2
        L = 2 ** i
        x = _filter_step(x, g0, L, shift, conv, nthreads) + _filter_step(y1, g1, L, shift, conv, nthreads)
    return _filter_step(x, g0, 1, 1, conv, nthreads) + _filter_step(y[n], g1, 1, 1, conv, nthreads)


# ----------------------------------------------------------------------------
# Meyer shearing filters (shearing_filters_Myer.m and helpers)
# ----------------------------------------------------------------------------
def _mround(v):
    """MATLAB round: half away from zero (numpy rounds half to even)."""
    return math.floor(v + 0.5) if v >= 0 else -math.floor(-v + 0.5)


def gen_x_y_cordinates(n):
    """gen_x_y_cordinates.m:22-80 -> (x1n, y1n, x2n, y2n, D), 1-based indices."""
    n = n + 1
    x1 = np.zeros((n, n)); y1 = np.zeros((n, n)); x2 = np.zeros((n, n)); y2 = np.zeros((n, n))
    for i in range(1, n + 1):
        y0, x0, x_n, y_n = 1, i, n - i + 1, n
        flag = x_n == x0
        m1 = None if flag else (y_n - y0) / (x_n - x0)
        xt = x0 + np.arange(n) * ((x_n - x0) / (n - 1))  # linspace(x0, x_n, n)
        xt[0], xt[-1] = x0, x_n
        for j in range(1, n + 1):
            if not flag:
                yv = _mround(m1 * (xt[j - 1] - x0) + y0)
                xv = _mround(xt[j - 1])
                y1[i - 1, j - 1] = yv
                x1[i - 1, j - 1] = xv
                x2[i - 1, j - 1] = yv
                y2[i - 1, j - 1] = xv
            else:
                x1[i - 1, j - 1] = (n - 1) / 2 + 1
                y1[i - 1, j - 1] = j
                x2[i - 1, j - 1] = j
                y2[i - 1, j - 1] = (n - 1) / 2 + 1
    n = n - 1
    x1n = x1[:n, :n].copy(); y1n = y1[:n, :n].copy()
    x2n = x2[1:n + 1, :n].copy(); y2n = y2[1:n + 1, :n].copy()
    x1n = np.flipud(x1n)
    y2n[n - 1, 0] = n
    D = avg_pol(n, x1n, y1n, x2n, y2n)
    return (x1n.astype(int), y1n.astype(int), x2n.astype(int), y2n.astype(int), D)


def avg_pol(L, x1, y1, x2, y2):
    """gen_x_y_cordinates.m:85-110."""
    D = np.zeros((L, L))
    for i in range(L):
        for j in range(L):
            D[int(y1[i, j]) - 1, int(x1[i, j]) - 1] += 1
    for i in range(L):
        for j in range(L):
            D[int(y2[i, j]) - 1, int(x2[i, j]) - 1] += 1
    return D


def meyer_wind(x):
    """meyer_wind.m:11-19."""
    if -1 / 3 + 1 / 2 < x < 1 / 3 + 1 / 2:
        return 1.0
    if (1 / 3 + 1 / 2 <= x <= 2 / 3 + 1 / 2) or (-2 / 3 + 1 / 2 <= x <= 1 / 3 + 1 / 2):
        w = 3 * abs(x - 1 / 2) - 1
        z = w ** 4 * (35 - 84 * w + 70 * w ** 2 - 20 * w ** 3)
        return math.cos(math.pi / 2 * z) ** 2
    return 0.0


def windowing(x, L):
    """windowing.m:11-27."""
    N = len(x)
    y = np.zeros((N, L))
    T = N / L
    g = np.array([meyer_wind((-1 * T / 2 + j - 1) / T) for j in range(1, int(2 * T) + 1)])
    for j in range(1, L + 1):
        index = 0
        k = -1 * T / 2
        while k <= 1.5 * T - 1:
            in_sig = int(math.floor((k + (j - 1) * T) % N))  # MATLAB mod is floor-mod
            y[in_sig, j - 1] = g[index] * x[in_sig]
            index += 1
            k += 1
    return y


def rec_from_pol(l, n, x1, y1, x2, y2, D):
    """rec_from_pol.m:16-35 (option 0: accumulate, then average by D)."""
    C = np.zeros((n, n))
    for i in range(n):
        for j in range(n):
            C[y1[i, j] - 1, x1[i, j] - 1] += l[i, j]
            C[y2[i, j] - 1, x2[i, j] - 1] += l[i + n, j]
    return C / D


def shearing_filters_Myer(n1, level):
    """shearing_filters_Myer.m:18-26 -> w_s, shape (2**level, n1, n1)."""
    x11, y11, x12, y12, F1 = gen_x_y_cordinates(n1)
    wf = windowing(np.ones(2 * n1), 2 ** level)
    w_s = np.zeros((2 ** level, n1, n1))
    for k in range(2 ** level):
        temp = np.outer(wf[:, k], np.ones(n1))
        C = rec_from_pol(temp, n1, x11, y11, x12, y12, F1)
        w_s[k] = np.real(np.fft.fftshift(np.fft.ifft2(np.fft.fftshift(C)))) / math.sqrt(n1)
    return w_s


def shear_spectra(H, W, dcomp, dsize):
    """nsst_dec2.m:46-57: W_k = fft2(w_k, H, W) (top-left zero pad), then
    divided by d = sqrt(sum_k |W_k|^2).  Returns a list of (ndir, H, W) complex128."""
    out = []
    for lev in range(len(dcomp)):
        w_s = shearing_filters_Myer(dsize[lev], dcomp[lev])
        F = np.stack([np.fft.fft2(w, (H, W)) for w in w_s])
        d = np.sqrt(np.sum((F * np.conj(F)).real, axis=0))
        out.append(F / d)
    return out


def conv2p(Xspec, y, workers=1):
    """conv2p.m:12: real(ifft2(X .* fft2(y)))."""
    return np.real(sfft.ifft2(Xspec * sfft.fft2(y, workers=workers), workers=workers))


def nsst_dec2(x, dcomp, dsize, fname='maxflat', shear_f=None, conv='port', nthreads=1):
    """nsst_dec2.m:37-59 -> (dst, shear_f); dst[0] lowpass, dst[i] (ndir, H, W)."""
    H, W = x.shape
    y = atrousdec(x, fname, len(dcomp), conv=conv, nthreads=nthreads)
    if shear_f is None:
        shear_f = shear_spectra(H, W, dcomp, dsize)
    dst = [y[0]]
    for i in range(len(dcomp)):
        Y = sfft.fft2(y[i + 1], workers=nthreads)
        dst.append(np.real(sfft.ifft2(shear_f[i] * Y[None], axes=(-2, -1), workers=nthreads)))
    return dst, shear_f


def nsst_rec2(dst, shear_f, fname='maxflat', conv='port', nthreads=1):
    """nsst_rec2.m:25-35."""
    y = [dst[0]]
    for i in range(1, len(dst)):
        C = sfft.fft2(dst[i], axes=(-2, -1), workers=nthreads)
        y.append(np.real(sfft.ifft2(np.sum(np.conj(shear_f[i - 1]) * C, axis=0), workers=nthreads)))
    return np.real(atrousrec(y, fname, conv=conv, nthreads=nthreads))


def band_thresholds(sigma, K, scalars):
    """Per-band thresholds K[level] * sigma * scalar (nsst_HT.m:34-46 with
    Tscalars generalised to one multiplier per level; index 0 is lowpass)."""
    th = [K[0] * sigma * scalars[0]]
    for i in range(1, len(scalars)):
        th.append(np.asarray([K[i] * sigma * s for s in scalars[i]]))
    return th


def nsst_HT(dst, sigma, K, scalars):
    """nsst_HT.m:32-47: keep c where abs(c) > threshold (strict)."""
    th = band_thresholds(sigma, K, scalars)
    out = [dst[0] * (np.abs(dst[0]) > th[0])]
    for i in range(1, len(dst)):
        t = th[i][:, None, None]
        out.append(dst[i] * (np.abs(dst[i]) > t))
    return out


def nsst_ST(dst, sigma, K, scalars):
    """Soft threshold per band, SoftThresh.m:11-13: sign(c) max(abs(c)-t, 0)."""
    th = band_thresholds(sigma, K, scalars)
    soft = lambda c, t: np.sign(c) * np.maximum(np.abs(c) - t, 0.0)
    out = [soft(dst[0], th[0])]
    for i in range(1, len(dst)):
        out.append(soft(dst[i], th[i][:, None, None]))
    return out


def mad_sigma(d):
    """nsst_scalars.m:36,43: median(abs(d - median(d))) / .6745."""
    d = d.ravel()
    return float(np.median(np.abs(d - np.median(d))) / 0.6745)


def nsst_scalars(H, W, shear_f, seed, fname='maxflat', conv='port', nthreads=1):
    """nsst_scalars.m:28-45 with a seeded N(0,1) image instead of randn."""
    noise = np.random.default_rng(seed).standard_normal((H, W))
    y = atrousdec(noise, fname, len(shear_f), conv=conv, nthreads=nthreads)
    scal = [mad_sigma(y[0])]
    for i in range(len(shear_f)):
        Y = sfft.fft2(y[i + 1], workers=nthreads)
        s = []
        for k in range(shear_f[i].shape[0]):
            s.append(mad_sigma(np.real(sfft.ifft2(shear_f[i][k] * Y, workers=nthreads))))
        scal.append(np.asarray(s))
    return scal


def denoise(x, sigma, K, scalars, dcomp, dsize, mode='hard', shear_f=None, fname='maxflat',
            conv='port', nthreads=1):
    """nsst_dec2 -> nsst_HT (or soft) -> nsst_rec2, the reference demo's
    hot path (denoise_shearlet_example.m:56,94,103)."""
    dst, shear_f = nsst_dec2(x, dcomp, dsize, fname, shear_f, conv, nthreads)
    dst_t = nsst_HT(dst, sigma, K, scalars) if mode == 'hard' else nsst_ST(dst, sigma, K, scalars)
    return nsst_rec2(dst_t, shear_f, fname, conv, nthreads), dst


def psnr(ref, x, peak=255.0):
    mse = np.mean((np.asarray(ref, np.float64) - np.asarray(x, np.float64)) ** 2)
    return 10 * math.log10(peak * peak / mse)


# ----------------------------------------------------------------------------
# Adjoints and the gradient of the denoising loss (FP64).  The reference has no
# adjoint; these are the exact transposes of the operators above, used to
# check the GPU adjoint kernels.
# ----------------------------------------------------------------------------
def _reflect_index(t, n):
    """Single mirror reflection with the edge sample repeated (symext.m)."""
    t = np.where(t < 0, -1 - t, t)
    return np.where(t >= n, 2 * n - 1 - t, t)


def _filter_step_matrix_apply(x, F, M, transpose=False):
    """One centred dilated filtering step y[r,c] = sum_ab hf[a,b] xe[r-M c0+M a, c-M c0+M b]
    (the atrousc(symext(...)) call, see _filter_step) or its transpose."""
    n, m = x.shape
    Fs = F.shape[0]
    c0 = (Fs - 1) // 2
    hf = F[::-1, ::-1]
    out = np.zeros_like(x)
    rows = np.arange(n)
    cols = np.arange(m)
    for a in range(Fs):
        ri = _reflect_index(rows - M * c0 + M * a, n)
        for b in range(Fs):
            w = hf[a, b]
            if w == 0.0:
                continue
            ci = _reflect_index(cols - M * c0 + M * b, m)
            if not transpose:
                out += w * x[np.ix_(ri, ci)]
            else:
                np.add.at(out, np.ix_(ri, ci), w * x)
    return out


def atrousdec_adjoint(gy, fname='maxflat'):
    """Transpose of atrousdec: gradients of the (nlev+1) outputs -> gradient of x."""
    h0, h1, _, _ = atrousfilters(fname)
    n = len(gy) - 1
    g_lo = gy[0].copy()  # gradient of the last lowpass
    for i in range(n - 1, 0, -1):
        M = 2 ** i
        g_lo = _filter_step_matrix_apply(g_lo, h0, M, True) + _filter_step_matrix_apply(gy[n - i], h1, M, True)
    return _filter_step_matrix_apply(g_lo, h0, 1, True) + _filter_step_matrix_apply(gy[n], h1, 1, True)


def atrousrec_adjoint(gx, nlevels, fname='maxflat'):
    """Transpose of atrousrec: gradient of the output -> gradients of y[0..nlev]."""
    _, _, g0, g1 = atrousfilters(fname)
    gy = [None] * (nlevels + 1)
    gy[nlevels] = _filter_step_matrix_apply(gx, g1, 1, True)
    g = _filter_step_matrix_apply(gx, g0, 1, True)
    for i in range(1, nlevels):
        M = 2 ** i
        gy[nlevels - i] = _filter_step_matrix_apply(g, g1, M, True)
        g = _filter_step_matrix_apply(g, g0, M, True)
    gy[0] = g
    return gy


def soft(c, t):
    return np.sign(c) * np.maximum(np.abs(c) - t, 0.0)


def denoise_tau(x, tau, shear_f, fname='maxflat', mode='soft', nthreads=1):
    """Forward of the differentiable pipeline with explicit per-band thresholds
    tau = [t_lowpass, level0 (ndir0,), level1 (ndir1,), ...]."""
    dst, _ = _dec_with(x, shear_f, fname, nthreads)
    thr = lambda c, t: soft(c, t) if mode == 'soft' else c * (np.abs(c) > t)
    dt = [thr(dst[0], tau[0])] + [thr(dst[i], np.asarray(tau[i])[:, None, None]) for i in range(1, len(dst))]
    return nsst_rec2(dt, shear_f, fname, nthreads=max(nthreads, 1)), dst


def _dec_with(x, shear_f, fname, nthreads):
    y = atrousdec(x, fname, len(shear_f), nthreads=max(nthreads, 1))
    dst = [y[0]]
    for i in range(len(shear_f)):
        Y = sfft.fft2(y[i + 1], workers=max(nthreads, 1))
        dst.append(np.real(sfft.ifft2(shear_f[i] * Y[None], axes=(-2, -1), workers=max(nthreads, 1))))
    return dst, shear_f


def denoise_tau_grad(x, tau, clean, shear_f, fname='maxflat', mode='soft', nthreads=1):
    """loss = ||rec(T(dec(x), tau)) - clean||^2 and its gradients w.r.t. x and tau."""
    w = max(nthreads, 1)
    xr, dst = denoise_tau(x, tau, shear_f, fname, mode, nthreads)
    r = xr - clean
    loss = float(np.sum(r * r))
    gxr = 2.0 * r
    L = len(shear_f)
    gyp = atrousrec_adjoint(gxr, L, fname)         # d loss / d y' (synthesis inputs)
    gct = [gyp[0]]                                  # d loss / d thresholded coefficients
    for i in range(L):
        G = sfft.fft2(gyp[i + 1], workers=w)
        gct.append(np.real(sfft.ifft2(shear_f[i] * G[None], axes=(-2, -1), workers=w)))
    gc, gtau = [], []
    for i, (c, g) in enumerate(zip(dst, gct)):
        t = tau[0] if i == 0 else np.asarray(tau[i])[:, None, None]
        keep = np.abs(c) > t
        gc.append(g * keep)
        if mode == 'soft':
            gt = -np.sum(g * np.sign(c) * keep, axis=(-2, -1))
        else:
            gt = np.zeros_like(np.asarray(t, float).reshape(-1)) if i else 0.0
        gtau.append(float(gt) if i == 0 else np.asarray(gt).reshape(-1))
    gy = [gc[0]]
    for i in range(L):
        C = sfft.fft2(gc[i + 1], axes=(-2, -1), workers=w)
        gy.append(np.real(sfft.ifft2(np.sum(np.conj(shear_f[i]) * C, axis=0), workers=w)))
    gx = atrousdec_adjoint(gy, fname)
    return loss, gx, gtau


def com_norm(H, W, dcomp, dsize, fname='maxflat', shear_f=None, nthreads=1):
    """com_norm.m:25-55: l2 norm of every band's shearlet from the transform
    of X = fftshift(real(ifft2(ones))) * sqrt(H W), an impulse at (H/2, W/2);
    flat in coefficient plane order (lowpass first)."""
    X = np.fft.fftshift(np.real(np.fft.ifft2(np.ones((H, W))))) * math.sqrt(H * W)
    dst, _ = nsst_dec2(X, dcomp, dsize, fname, shear_f=shear_f, nthreads=nthreads)
    planes = [dst[0]] + [p for lev in dst[1:] for p in lev]
    return np.array([math.sqrt(float(np.sum(p * p)) / (H * W)) for p in planes])


def thresh_maxi(coeffs, scalars):
    """thresh.m:38-41 (opt == 1): max over bands of max|c_b / E_b| of the
    thresholded coefficients (flat planes, flat scalars)."""
    return max(float(np.max(np.abs(c))) / s for c, s in zip(coeffs, scalars) if s > 0)


def re_weight_band(P, coeff, fname='maxflat', conv='port', nthreads=1):
    """re_weight_band.m:23-29: atrousdec with len(coeff)-1 levels, band j
    scaled by coeff[j] (lowpass first), atrousrec."""
    y = atrousdec(P, fname, len(coeff) - 1, conv=conv, nthreads=nthreads)
    y = [c * b for c, b in zip(coeff, y)]
    return atrousrec(y, fname, conv=conv, nthreads=nthreads)
