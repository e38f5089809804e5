"""FP64 CPU oracle for the 3-D shearlet denoising path (band-pass pyramid +
CONVNFFT directional filtering).  TEST INFRASTRUCTURE ONLY (same rules as
oracle/nsst2d.py).

Each function restates one reference function of ``shearcuda3d`` and cites
it.  Arrays keep MATLAB's axis order (axis 0 = MATLAB dim 1, ...); the
half spectrum of the pyramid lies along the last axis as in ccsym.m.

Volume sizes: Pyr_mode 1.5 needs every dimension divisible by 12 for three
levels (PrySDdec_onestep.m:41-44).  The reference pads with MarshalData.m
(edge replication up to the next multiple of 12, always adding planes, so
128 -> 132 and 192 -> 204, lengths with prime factors 11 and 17); here each
dimension is padded by the same edge replication to the smallest of the grids
96, 144, 192 that holds it (pad_size), whose level sizes (d, 2d/3, d/3, d/6)
are all 2^a 3^b, and the result is cropped back.  This convention is shared by
the oracle and the GPU path.
"""
import math
import os

import numpy as np
from scipy import fft as sfft

# FFT worker threads: the transforms split over independent 1-D sequences,
# so the result does not depend on the count
WORKERS = os.cpu_count() or 1

PYR_MODES = {1: ([0.5, 0.25], [1 / 6, 1 / 12], [1.0, 2.0]),
             1.5: ([0.5, 3 / 8], [1 / 7, 1 / 9], [1.5, 2.0]),
             2: ([1 / 3, 1 / 3], [1 / 7, 1 / 7], [2.0, 2.0])}


def pyr_params(mode, L):
    """PyrNDDec_mm.m:58-74 (w, tbw, D arrays for L levels)."""
    w, t, d = PYR_MODES[mode]
    if mode == 2:
        return [w[0]] * L, [t[0]] * L, [d[0]] * L
    return [w[0]] + [w[1]] * (L - 1), [t[0]] + [t[1]] * (L - 1), [d[0]] + [d[1]] * (L - 1)


def rcos(x):
    """rcos.m:1-13."""
    x = np.asarray(x, dtype=np.float64)
    th = 0.5 * (1 - np.cos(np.pi * x))
    th = np.where(x <= 0, 0.0, th)
    return np.where(x >= 1, 1.0, th)


def ccsym(x, k, kind):
    """ccsym.m:20-52 (k is 0-based here)."""
    if kind == 'c':
        sl = [slice(None)] * x.ndim
        sl[k] = slice(0, x.shape[k] // 2 + 1)
        return x[tuple(sl)]
    sz = list(x.shape)
    sz[k] = (sz[k] - 1) * 2
    idx = [np.concatenate([[0], np.arange(sz[m] - 1, 0, -1)]) for m in range(x.ndim)]
    idx[k] = np.arange(sz[k] // 2 - 1, 0, -1)
    return np.concatenate([x, np.conj(x[np.ix_(*idx)])], axis=k)


def _windows(szX, w, tbw, smooth=rcos):
    """The separable low-pass window of PrySDdec_onestep.m:48-82: returns
    (pbd index arrays (0-based), 1-D window values per axis, szF)."""
    N = len(szX)
    szF = list(szX)
    szF[-1] = (szX[-1] - 1) * 2
    pbds, vals = [], []
    for n in range(N):
        nr = szF[n]
        K = math.ceil(nr / 2 * (w + tbw))
        pbd = np.arange(K + 1)
        val = np.sqrt(smooth((pbd[-1] - pbd) / (K - math.floor(nr / 2 * (w - tbw)))))
        if n != N - 1:
            pbd = np.concatenate([pbd, np.arange(nr - pbd[-1], nr)])
            val = np.concatenate([val, val[1:][::-1]])
        pbds.append(pbd)
        vals.append(val)
    return pbds, vals, szF


def _lf(vals):
    Lf = vals[0][:, None, None] * vals[1][None, :, None] * vals[2][None, None, :]
    return Lf


def _small_index(pbds, szLp, szX):
    """PrySDdec_onestep.m:92-98: the negative-frequency half of each pbd moves
    to the end of the smaller array."""
    out = []
    for n, pbd in enumerate(pbds):
        pbd = pbd.copy()
        if n != len(pbds) - 1:
            h = (len(pbd) + 3) // 2 - 1  # MATLAB (len+3)/2 (1-based) -> 0-based
            pbd[h:] = pbd[h:] + szLp[n] - szX[n]
        out.append(pbd)
    return out


def prysd_dec_onestep(X, w, tbw, D, smooth=rcos):
    """PrySDdec_onestep.m:20-125 on a half spectrum X."""
    N = X.ndim
    szX = list(X.shape)
    pbds, vals, szF = _windows(szX, w, tbw, smooth)
    Lf = _lf(vals)
    szLp = [f / D for f in szF]
    if any(abs(v - round(v)) > 1e-9 for v in szLp):
        raise ValueError('The downsampling factor must divide the size of the FFT matrix')
    szLp = [int(round(v)) for v in szLp]
    szLp[-1] = szLp[-1] // 2 + 1
    small = _small_index(pbds, szLp, szX)
    Lp = np.zeros(szLp, dtype=np.complex128)
    Lp[np.ix_(*small)] = (Lf / D ** (N / 2)) * X[np.ix_(*pbds)]
    Hp = X.copy()
    Hp[np.ix_(*pbds)] = np.sqrt(1 - Lf ** 2) * X[np.ix_(*pbds)]
    return Lp, Hp


def prysd_rec_onestep(Lp, Hp, w, tbw, D, smooth=rcos):
    """PrySDrec_onestep.m:20-119."""
    N = Hp.ndim
    szX = list(Hp.shape)
    pbds, vals, szF = _windows(szX, w, tbw, smooth)
    Lf = _lf(vals)
    rec = Hp.copy()
    rec[np.ix_(*pbds)] = np.sqrt(1 - Lf ** 2) * rec[np.ix_(*pbds)]
    szLp = [int(round(f / D)) for f in szF]
    szLp[-1] = szLp[-1] // 2 + 1
    small = _small_index(pbds, szLp, szX)
    rec[np.ix_(*pbds)] = rec[np.ix_(*pbds)] + Lp[np.ix_(*small)] * (Lf * D ** (N / 2))
    return rec


def pyr_dec(x, L=3, mode=1.5):
    """PyrNDDec_mm.m:20-109 with OutD = 'S' (DoPyrDec.m): [HP fine ... coarse, LP]."""
    w, t, d = pyr_params(mode, L)
    N = x.ndim
    X = ccsym(sfft.fftn(x, workers=WORKERS), N - 1, 'c')
    subs = []
    for n in range(L):
        Lp, Hp = prysd_dec_onestep(X, w[n], t[n], d[n])
        X = Lp
        subs.append(np.real(sfft.ifftn(ccsym(Hp, N - 1, 'e'), workers=WORKERS)))
    subs.append(np.real(sfft.ifftn(ccsym(X, N - 1, 'e'), workers=WORKERS)))
    return subs


def pyr_rec(subs, mode=1.5):
    """PyrNDRec_mm.m:20-95 with InD = 'S' (DoPyrRec.m)."""
    L = len(subs) - 1
    w, t, d = pyr_params(mode, L)
    N = subs[0].ndim
    Lp = ccsym(sfft.fftn(subs[-1], workers=WORKERS), N - 1, 'c')
    for n in range(L - 1, -1, -1):
        Hp = ccsym(sfft.fftn(subs[n], workers=WORKERS), N - 1, 'c')
        Lp = prysd_rec_onestep(Lp, Hp, w[n], t[n], d[n])
    return np.real(sfft.ifftn(ccsym(Lp, N - 1, 'e'), workers=WORKERS))


# ----------------------------------------------------------------------------
# 3-D Meyer-based shearing filters (GetMeyerBasedFilter.m and helpers)
# ----------------------------------------------------------------------------
def _u16(v):
    """MATLAB conversion of a non-negative double to uint16 (round half away)."""
    return np.uint16(min(max(math.floor(v + 0.5), 0), 65535))


def generate_xyz(n):
    """GenerateXYZ.m:12-54 -> X, Y, Z (1-based uint16 index volumes)."""
    X = np.zeros((n, n, n), dtype=np.int64)
    Y = np.zeros((n, n, n), dtype=np.int64)
    Z = np.zeros((n, n, n), dtype=np.int64)
    mid = math.ceil(n / 2)
    for j in range(1, mid + 1):
        for i in range(1, mid + 1):
            dL2 = (n - 1) ** 2 + (n - i + 1 - i) ** 2
            dL3 = (dL2 + (n - j + 1 - j) ** 2) ** 0.5
            dL2 = dL2 ** 0.5
            sinA = (n - j + 1 - j) / dL3
            cosA = dL2 / dL3
            sinB = (n - i + 1 - i) / dL2
            cosB = (n - 1) / dL2
            dl3 = dL3 / (n - 1)
            for k in range(1, n + 1):
                l = dl3 * (k - 1)
                temp = l * sinA
                I, K, J = i - 1, k - 1, j - 1
                Ii, Jj = n - i, n - j
                Z[I, K, J] = _u16(j + temp)
                Z[Ii, K, J] = Z[I, K, J]
                Z[I, K, Jj] = _u16(n - j + 1 - temp)
                Z[Ii, K, Jj] = _u16(n - j + 1 - temp)
                temp = l * cosA
                t1 = temp * sinB
                Y[I, K, J] = _u16(i + t1)
                Y[Ii, K, J] = _u16(n - i + 1 - t1)
                X[I, K, J] = _u16(1 + temp * cosB)
                X[Ii, K, J] = X[I, K, J]
                X[I, K, Jj] = X[I, K, J]
                X[Ii, K, Jj] = X[I, K, J]
                Y[I, K, Jj] = Y[I, K, J]
                Y[Ii, K, Jj] = Y[Ii, K, J]
    return X, Y, Z


def pyramid_sections(n):
    """GeneratePyramidSection.m:1-14: the three cones' coordinate maps."""
    X, Y, Z = generate_xyz(n)
    return [(X, Y, Z), (Y, X, Z), (Z, Y, X)]


def polar_to_rec(idx, radial, n, P):
    """PolarToRec.m:10-19 (assignment, later writes win; loop order j, i, k)."""
    X, Y, Z = P
    out = np.zeros((n, n, n))
    (i0, i1), (k0, k1), (j0, j1) = idx
    for j in range(j0, j1 + 1):
        for i in range(i0, i1 + 1):
            for k in range(k0, k1 + 1):
                out[X[i - 1, k - 1, j - 1] - 1, Y[i - 1, k - 1, j - 1] - 1, Z[i - 1, k - 1, j - 1] - 1] = \
                    radial[i - i0, k - k0, j - j0]
    return out


def _radial(a, n, b, corner):
    r = np.ones((a, n, b))
    r[[0, a - 1], :, :] = 0.5
    r[:, :, [0, b - 1]] = 0.5
    if corner is not None:
        r[corner[0], :, corner[1]] = 1 / 3
    return r


def meyer_filters_3d(num_dirs, cube=24):
    """GetMeyerBasedFilter.m:12-150 -> F[cone][level] = list of numDir x numDir
    spatial filters (cube^3), indexed [l2][l1]; the cone rows 1 and 2 are
    swapped at the end (:148-150).  num_dirs[l] = numDir of level l (fine first)."""
    P = pyramid_sections(cube)
    F = [[None] * len(num_dirs) for _ in range(3)]
    for l, nd in enumerate(num_dirs):
        shift = cube // nd
        blocks = [[[None] * nd for _ in range(nd)] for _ in range(3)]
        A = np.zeros((cube, cube, cube))
        s1 = shift + 1

        def put(c, l2, l1, rad, idx):
            nonlocal A
            blocks[c][l2 - 1][l1 - 1] = polar_to_rec(idx, rad, cube, P[c])
            A = A + blocks[c][l2 - 1][l1 - 1]

        for c in range(3):
            # corner (1,1)
            put(c, 1, 1, _radial(s1, cube, s1, (0, 0)), ((1, s1), (1, cube), (1, s1)))
            r = _radial(s1, cube, s1, None)
            for l2 in range(2, nd):
                for l1 in range(2, nd):
                    put(c, l2, l1, r, (((l1 - 1) * shift + 1, l1 * shift + 1), (1, cube),
                                       ((l2 - 1) * shift + 1, l2 * shift + 1)))
            # (1, numDir)
            put(c, 1, nd, _radial(shift, cube, s1, (shift - 1, 0)),
                (((nd - 1) * shift + 1, nd * shift), (1, cube), (1, s1)))
            r = _radial(shift, cube, s1, None)
            for l2 in range(2, nd):
                put(c, l2, nd, r, (((nd - 1) * shift + 1, nd * shift), (1, cube),
                                   ((l2 - 1) * shift + 1, l2 * shift + 1)))
            r = _radial(s1, cube, s1, None)
            for l2 in range(2, nd):
                put(c, l2, 1, r, ((1, s1), (1, cube), ((l2 - 1) * shift + 1, l2 * shift + 1)))
            # (numDir, 1)
            put(c, nd, 1, _radial(s1, cube, shift, (0, shift - 1)),
                ((1, s1), (1, cube), ((nd - 1) * shift + 1, nd * shift)))
            r = _radial(s1, cube, shift, None)
            for l1 in range(2, nd):
                put(c, nd, l1, r, (((l1 - 1) * shift + 1, l1 * shift + 1), (1, cube),
                                   ((nd - 1) * shift + 1, nd * shift)))
            r = _radial(s1, cube, s1, None)
            for l1 in range(2, nd):
                put(c, 1, l1, r, (((l1 - 1) * shift + 1, l1 * shift + 1), (1, cube), (1, s1)))
            # (numDir, numDir)
            put(c, nd, nd, _radial(shift, cube, shift, (shift - 1, shift - 1)),
                (((nd - 1) * shift + 1, nd * shift), (1, cube), ((nd - 1) * shift + 1, nd * shift)))
        for c in range(3):
            F[c][l] = [[np.real(np.fft.fftshift(np.fft.ifftn(np.fft.fftshift(blocks[c][l2][l1] / A))))
                        for l1 in range(nd)] for l2 in range(nd)]
    F[0], F[1] = F[1], F[0]
    return F


def convnfft_same(A, B):
    """convnfft.m:79-201 with shape 'same' and power-of-two FFT lengths."""
    out = A.astype(np.complex128)
    Bs = B.astype(np.complex128)
    subs = []
    for dim in range(A.ndim):
        m, n = A.shape[dim], B.shape[dim]
        lf = 2 ** math.ceil(math.log2(m + n - 1))
        out = sfft.fft(out, lf, axis=dim, workers=WORKERS)
        Bs = sfft.fft(Bs, lf, axis=dim, workers=WORKERS)
        s0 = math.ceil((n - 1) / 2)
        subs.append(slice(s0, s0 + m))
    out = np.real(sfft.ifftn(out * Bs, workers=WORKERS))
    return out[tuple(subs)]


def convnfft_same_level(BPl, filters):
    """convnfft 'same' (convnfft.m:79-201) of one level's volume with each of
    several filters, restated with real FFTs at the smallest fast length >=
    m + n - 1 per axis and the volume's transform shared by the filters.  Any
    length >= m + n - 1 gives the same linear convolution (convnfft.m's
    power-of-two length included), so this equals convnfft_same up to FP64
    rounding (test_oracle3d.py checks 1e-12); it is several times faster on
    the large volumes."""
    shp = [sfft.next_fast_len(m + n - 1, real=True) for m, n in zip(BPl.shape, filters[0].shape)]
    A = sfft.rfftn(BPl, shp, workers=WORKERS)
    out = []
    for f in filters:
        s0 = [math.ceil((n - 1) / 2) for n in f.shape]
        full = sfft.irfftn(A * sfft.rfftn(f, shp, workers=WORKERS), shp, workers=WORKERS)
        out.append(full[tuple(slice(a, a + m) for a, m in zip(s0, BPl.shape))])
    return out


def band_list(F):
    """Flatten F into (cone, level, l2, l1, filter) in the order the GPU path
    uses: level-major, then cone, then l2, then l1."""
    out = []
    for l in range(len(F[0])):
        for c in range(3):
            nd = len(F[c][l])
            for l2 in range(nd):
                for l1 in range(nd):
                    out.append((c, l, l2, l1, F[c][l][l2][l1]))
    return out


def sh_dec_level(BPl, F, l):
    """ShDec.m:18-34 for every cone at one level -> list of coefficient volumes."""
    return [convnfft_same(BPl, f) for (c, ll, l2, l1, f) in band_list(F) if ll == l]


def nsst_scalars3(shape, F, seed, L=3, mode=1.5):
    """NsstScalars.m:1-19 with a seeded N(0,1) volume -> (lowpass, bands in band_list order)."""
    noise = np.random.default_rng(seed).standard_normal(shape)
    bp = pyr_dec(noise, L, mode)
    mad = lambda d: float(np.median(np.abs(d - np.median(d))) / 0.6745)
    out = []
    for (c, l, l2, l1, f) in band_list(F):
        out.append(mad(convnfft_same(bp[l], f)))
    return mad(bp[L]), np.asarray(out)


def denoise3(x, F, sigma, T, band_scalars, L=3, mode=1.5, fast=False):
    """The 3-D denoise of DenoiseDemo/main.m:35-75: pyramid, per band
    convnfft 'same', hard threshold (ThresholdShCoeff.m: zero where
    |c| <= T(l) sigma bandEst), band + cone sums (ShRec.m, main.m:58-63),
    lowpass untouched (main.m:67), pyramid reconstruction.  fast: the
    convolutions through convnfft_same_level (same results to FP64 rounding)."""
    bp = pyr_dec(x, L, mode)
    rec = [np.zeros_like(b) for b in bp[:L]] + [bp[L]]
    bands = band_list(F)
    if fast:
        coefs = {}
        for l in range(L):
            idx = [b for b, bd in enumerate(bands) if bd[1] == l]
            for b, c in zip(idx, convnfft_same_level(bp[l], [bands[b][4] for b in idx])):
                c[np.abs(c) <= T[l] * sigma * band_scalars[b]] = 0.0
                rec[l] += c
        return pyr_rec(rec, mode)
    for b, (c, l, l2, l1, f) in enumerate(bands):
        coef = convnfft_same(bp[l], f)
        coef[np.abs(coef) <= T[l] * sigma * band_scalars[b]] = 0.0
        rec[l] += coef
    return pyr_rec(rec, mode)


FFT_LENS = (16, 24, 32, 48, 64, 72, 96, 128, 144, 192, 256)


def level_sizes(g, L=3, mode=1.5):
    """Level sizes g, g/D0, g/D0/D1, ... of a grid, or None when one of them
    is not a supported transform length (2^a 3^b, multiple of 8) or has no
    supported linear-convolution length (>= m + 23)."""
    D = pyr_params(mode, L)[2]
    conv = lambda m: next((v for v in FFT_LENS if v >= m + 23), None)
    out = [g]
    if g not in FFT_LENS or conv(g) is None:
        return None
    v = float(g)
    for l in range(L):
        v /= D[l]
        iv = int(round(v))
        if abs(v - iv) > 1e-9 or iv not in FFT_LENS or iv % 8:
            return None
        if l + 1 < L and conv(iv) is None:
            return None
        out.append(iv)
    return out


def pad_size(n, L=3, mode=1.5):
    """Smallest grid >= n (at most 192) whose level sizes all work; for the
    3-level Pyr_mode 1.5 pyramid these are 96, 144 and 192."""
    for g in FFT_LENS:
        if n <= g <= 192 and level_sizes(g, L, mode):
            return g
    raise ValueError('volume dimension %d larger than 192' % n)


def marshal_data(X, level=3):
    """MarshalData.m:1-22 as the reference ships it: every dimension x gains
    d - rem(x, d) planes, d = divFactor(level) = [3 6 12 24](level), by
    replicating its last plane (so a multiple of d gains d planes: 128 -> 132,
    192 -> 204, 96 -> 108 for three levels)."""
    d = [3, 6, 12, 24][level - 1]
    return np.pad(X, [(0, d - (s % d)) for s in X.shape], mode='edge')


def pad_volume(x):
    """Edge replication to pad_size in every dimension (MarshalData.m's edge
    replication, to the GPU path's 2^a 3^b grid instead of marshal_data's)."""
    pads = [(0, pad_size(s) - s) for s in x.shape]
    return np.pad(x, pads, mode='edge')


def psnr3(ref, x):
    """PSNR.m:1-5 (peak 256)."""
    err = np.asarray(ref, np.float64) - np.asarray(x, np.float64)
    return 20 * math.log10(256 / math.sqrt(np.mean(err ** 2)))


def pad_volume_to(x, grid):
    """Edge replication of x up to the given grid dims."""
    return np.pad(x, [(0, g - s) for s, g in zip(x.shape, grid)], mode='edge')


# ----------------------------------------------------------------------------
# Adjoint of the 3-D denoise (hard threshold: the subgradient keeps the mask of
# the forward pass fixed).  The band-pass pyramid is a Parseval frame, so
# pyr_rec is the exact adjoint of pyr_dec and vice versa (checked by
# test_oracle3d.py); the adjoint of convnfft 'same' is the correlation
# corr_same below; the adjoint of edge padding folds the padded planes back.
# ----------------------------------------------------------------------------
def corr_same(G, B):
    """Adjoint of convnfft_same(., B) for an output G of A's shape: place G at
    offset ceil((n-1)/2) of the linear-convolution domain, correlate with B and
    keep the first A.shape samples."""
    sl = []
    L = []
    for dim in range(G.ndim):
        m, n = G.shape[dim], B.shape[dim]
        L.append(2 ** math.ceil(math.log2(m + n - 1)))
        s0 = math.ceil((n - 1) / 2)
        sl.append(slice(s0, s0 + m))
    Z = np.zeros(L)
    Z[tuple(sl)] = G
    Bp = np.zeros(L)
    Bp[tuple(slice(0, n) for n in B.shape)] = B
    out = np.real(sfft.ifftn(sfft.fftn(Z, workers=WORKERS) * np.conj(sfft.fftn(Bp, workers=WORKERS)), workers=WORKERS))
    return out[tuple(slice(0, m) for m in G.shape)]


def fold_edge(g, shape):
    """Adjoint of pad_volume_to(x, g.shape): sums the replicated planes back."""
    out = g
    for ax, n in enumerate(shape):
        head = np.take(out, np.arange(n - 1), axis=ax)
        tail = np.take(out, np.arange(n - 1, out.shape[ax]), axis=ax).sum(axis=ax, keepdims=True)
        out = np.concatenate([head, tail], axis=ax)
    return out


def denoise3_masks(x, F, sigma, T, band_scalars, L=3, mode=1.5, grid=None):
    """Forward pass with the keep-masks of every band (|c| > t)."""
    grid = grid or tuple(pad_size(s, L, mode) for s in x.shape)
    bp = pyr_dec(pad_volume_to(x, grid), L, mode)
    masks = []
    for b, (c, l, l2, l1, f) in enumerate(band_list(F)):
        coef = convnfft_same(bp[l], f)
        masks.append(np.abs(coef) > T[l] * sigma * band_scalars[b])
    return masks, grid


def denoise3_jvp(dx, masks, F, grid, L=3, mode=1.5):
    """J dx of the denoise linearised at fixed masks (crop of the grid)."""
    bp = pyr_dec(pad_volume_to(dx, grid), L, mode)
    rec = [np.zeros_like(b) for b in bp[:L]] + [bp[L]]
    for b, (c, l, l2, l1, f) in enumerate(band_list(F)):
        rec[l] += np.where(masks[b], convnfft_same(bp[l], f), 0.0)
    n = dx.shape
    return pyr_rec(rec, mode)[:n[0], :n[1], :n[2]]


def denoise3_vjp(gy, masks, F, grid, L=3, mode=1.5):
    """J^T gy: zero-pad, pyr_dec (= pyr_rec^T), masked correlations,
    pyr_rec (= pyr_dec^T), fold of the edge padding."""
    n = gy.shape
    g = np.zeros(grid)
    g[:n[0], :n[1], :n[2]] = gy
    u = pyr_dec(g, L, mode)
    gb = [np.zeros_like(b) for b in u[:L]] + [u[L]]
    for b, (c, l, l2, l1, f) in enumerate(band_list(F)):
        gb[l] += corr_same(np.where(masks[b], u[l], 0.0), f)
    return fold_edge(pyr_rec(gb, mode), n)
