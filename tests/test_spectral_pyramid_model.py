"""The spectral pyramid's mathematics on the CPU (no GPU): the DCT-II-domain
restatement that csrc/k_dct.cu and csrc/host_dct.cpp implement, in FP64 NumPy,
against the oracle's direct atrousdec / atrousrec (oracle/nsst2d.py).

* each pyramid step (a filter symmetric in both axes, dilated by M, on the
  half-sample symmetric extension reflected once) is the pointwise product
  with G[k1][k2] = sum_{a,b} h[a][b] cos(pi k1 M (a-c0)/H) cos(pi k2 M (b-c0)/W)
  in the 2-D DCT-II domain;
* the DCTs run as one N-point FFT each (Makhoul), unnormalised, as the kernels
  do: DCT-III(DCT-II(x)) = N x per axis;
* the analysis tables R_l, the synthesis tables Q_l and the lowpass tables
  chain the level responses as host_dct.cpp does, with 1/(H W) folded in;
* every pyramid operator is symmetric as a matrix (the adjoint the backward
  uses is the same operator with the tables swapped).
Tolerance: 1e-12 relative (FP64 against FP64).
"""
import numpy as np
import pytest

from oracle import nsst2d


def dct2(x, axis):
    """Makhoul's DCT-II: v = (x[0::2], reversed x[1::2]), V = FFT(v),
    C[k] = (w^k V[k] + conj(w^k) V[N-k]) / 2, w = exp(-i pi / (2N))."""
    x = np.moveaxis(x, axis, -1)
    N = x.shape[-1]
    v = np.concatenate([x[..., 0::2], x[..., 1::2][..., ::-1]], axis=-1)
    V = np.fft.fft(v, axis=-1)
    w = np.exp(-1j * np.pi * np.arange(N) / (2 * N))
    Vm = np.roll(V[..., ::-1], 1, axis=-1)  # V[(N - k) % N]
    return np.moveaxis((w * V + np.conj(w) * Vm) / 2, -1, axis)


def dct3(C, axis):
    """Z[k] = conj(w^k) (C[k] - i C[N-k]) (C[N] = 0), v = unscaled IFFT(Z),
    x[2n] = v[n], x[2n+1] = v[N-1-n]: N times the inverse of dct2."""
    C = np.moveaxis(C, axis, -1)
    N = C.shape[-1]
    w = np.exp(-1j * np.pi * np.arange(N) / (2 * N))
    Cm = np.concatenate([np.zeros_like(C[..., :1]), C[..., :0:-1]], axis=-1)
    v = np.fft.ifft(np.conj(w) * (C - 1j * Cm), axis=-1) * N
    x = np.empty_like(v)
    x[..., 0::2] = v[..., :N // 2]
    x[..., 1::2] = v[..., N // 2:][..., ::-1]
    return np.moveaxis(x, -1, axis)


def D2(x):
    return dct2(dct2(x, 0), 1)


def D3(C):
    return dct3(dct3(C, 0), 1)


def response(h, M, H, W):
    F = h.shape[0]
    a = np.arange(F) - (F - 1) // 2
    ch = np.cos(np.pi * np.outer(np.arange(H), M * a) / H)
    cw = np.cos(np.pi * np.outer(np.arange(W), M * a) / W)
    return ch @ h @ cw.T


def tables(fname, L, H, W):
    """host_dct.cpp:dct_pyramid_tables: per directional level l (dilation
    2^(L-1-l)) R_l and Q_l, then the lowpass round trip, analysis, synthesis."""
    h0, h1, g0, g1 = nsst2d.atrousfilters(fname)
    s = 1.0 / (H * W)
    R, Q = [None] * L, [None] * L
    ch, cg = np.ones((H, W)), np.ones((H, W))
    for i in range(L):
        M = 1 << i
        R[L - 1 - i] = s * ch * response(h1, M, H, W)
        Q[L - 1 - i] = s * response(g1, M, H, W) * cg
        ch = ch * response(h0, M, H, W)
        cg = cg * response(g0, M, H, W)
    return R, Q, s * ch * cg, s * ch, s * cg


@pytest.mark.parametrize('fname', ['maxflat', '9-7', 'pyr', 'pyrexc'])
@pytest.mark.parametrize('HW,L', [((96, 128), 3), ((64, 64), 2), ((80, 48), 1)])
def test_spectral_pyramid_equals_direct(fname, HW, L):
    H, W = HW
    F = max(f.shape[0] for f in nsst2d.atrousfilters(fname))
    if (1 << (L - 1)) * F + 1 > min(H, W):  # the plan's one-reflection rule
        pytest.skip('image too small for this depth')
    rng = np.random.default_rng(H + W + L)
    x = rng.standard_normal((H, W)) * 30 + 100
    y = nsst2d.atrousdec(x, fname, L)
    R, Q, T, Rlow, Glow = tables(fname, L, H, W)
    X = D2(x)
    # analysis: directional level l is pyramid plane l + 1, the lowpass plane 0
    for l in range(L):
        band = D3(X * R[l]).real
        assert np.abs(band - y[l + 1]).max() <= 1e-12 * np.abs(x).max()
    assert np.abs(D3(X * Rlow).real - y[0]).max() <= 1e-12 * np.abs(x).max()
    # synthesis of arbitrary planes, and the untouched lowpass round trip
    z = [p * (0.5 + k) for k, p in enumerate(y)]
    rec = nsst2d.atrousrec(z, fname)
    acc = D2(z[0]) * Glow + sum(D2(z[l + 1]) * Q[l] for l in range(L))
    assert np.abs(D3(acc).real - rec).max() <= 1e-12 * np.abs(rec).max()
    acc_t = X * T + sum(D2(y[l + 1]) * Q[l] for l in range(L))
    assert np.abs(D3(acc_t).real - x).max() <= 1e-12 * np.abs(x).max()


def test_pyramid_operators_are_symmetric():
    # <A u, v> = <u, A v> for a band operator A = IDCT2 diag(R) DCT2: the
    # backward swaps only the tables
    H, W, L = 64, 96, 2
    R, Q, T, Rlow, Glow = tables('maxflat', L, H, W)
    rng = np.random.default_rng(3)
    u, v = rng.standard_normal((2, H, W))
    for r in (R[0], R[1], Q[0], Glow):
        au, av = D3(D2(u) * r).real, D3(D2(v) * r).real
        assert abs(np.sum(au * v) - np.sum(u * av)) <= 1e-12 * np.sqrt(np.sum(au ** 2) * np.sum(v ** 2))


def test_makhoul_dct_matches_definition():
    rng = np.random.default_rng(1)
    x = rng.standard_normal(24)
    n = np.arange(24)
    ref = np.array([np.sum(x * np.cos(np.pi * k * (2 * n + 1) / 48)) for k in range(24)])
    assert np.abs(dct2(x, 0) - ref).max() <= 1e-12
    assert np.abs(dct3(dct2(x, 0), 0).real - 24 * x).max() <= 1e-11
    z = rng.standard_normal(24) + 1j * rng.standard_normal(24)  # complex-linear: packed columns
    assert np.abs(dct2(z, 0) - (dct2(z.real, 0) + 1j * dct2(z.imag, 0))).max() <= 1e-12
