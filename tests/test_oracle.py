"""The oracle, pinned: C restatement vs the reference's own atrousc.cpp
(golden fixtures), filter-bank identities and FP64 transform invariants."""
import numpy as np
import pytest
from scipy.signal import convolve2d

from conftest import DCOMP, DSIZE
from oracle import clib, nsst2d

GOLD = np.load(__import__('os').path.join(nsst2d.GOLDEN, 'atrousc_ref_cases.npz'))


@pytest.mark.parametrize('i', range(int(GOLD['n'][0])))
def test_atrousc_port_matches_reference_fixture(i):
    out = clib.atrousc(GOLD['S_%d' % i], GOLD['F_%d' % i], int(GOLD['M_%d' % i][0]))
    ref = GOLD['out_%d' % i]
    assert out.shape == ref.shape
    np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * max(1.0, np.abs(ref).max()))


def test_atrousc_reference_live_when_built():
    from oracle import atrous_ref
    if not atrous_ref.available():
        pytest.skip('reference atrousc not built here')
    rng = np.random.default_rng(7)
    S, F = rng.standard_normal((70, 61)), rng.standard_normal((7, 7))
    np.testing.assert_allclose(clib.atrousc(S, F, 4), atrous_ref.atrousc(S, F, 4), atol=1e-12)


@pytest.mark.parametrize('fname', ['maxflat', '9-7', 'pyr', 'pyrexc'])
def test_pyramid_filters_perfect_reconstruction(fname):
    # atrousfilters.m:16-18: conv2(h0,g0) + conv2(h1,g1) = delta
    h0, h1, g0, g1 = nsst2d.atrousfilters(fname)
    pr = convolve2d(h0, g0) + convolve2d(h1, g1)
    c = np.array(pr.shape) // 2
    pr[c[0], c[1]] -= 1.0
    assert np.abs(pr).max() < 1e-12


def test_symext_numpy_matches_c():
    rng = np.random.default_rng(3)
    x = rng.standard_normal((40, 52))
    for (p, s) in [(13, 1), (26, 1), (52, 0), (104, -2), (19, 1), (152, -2)]:
        if p + s > 40:
            continue
        np.testing.assert_array_equal(nsst2d.symext(x, p, p, s, s), clib.symext(x, p, p, s, s))


@pytest.mark.parametrize('HW', [(256, 256), (256, 384)])
def test_oracle_perfect_reconstruction_and_tight_frame(HW):
    H, W = HW
    x = np.random.default_rng(1).standard_normal((H, W)) * 40 + 100
    dst, sf = nsst2d.nsst_dec2(x, DCOMP, DSIZE, nthreads=4)
    for s in sf:
        assert np.abs(np.sum(np.abs(s) ** 2, axis=0) - 1).max() < 1e-12
    xr = nsst2d.nsst_rec2(dst, sf, nthreads=4)
    assert np.linalg.norm(xr - x) / np.linalg.norm(x) < 1e-12


def test_oracle_adjoint_directional_dot_product():
    # conj-spectrum synthesis is the adjoint of the directional analysis
    H = W = 128
    sf = nsst2d.shear_spectra(H, W, [2], [16])[0]
    rng = np.random.default_rng(2)
    y = rng.standard_normal((H, W))
    c = rng.standard_normal((sf.shape[0], H, W))
    Ay = np.real(np.fft.ifft2(sf * np.fft.fft2(y)[None]))
    Atc = np.real(np.fft.ifft2(np.sum(np.conj(sf) * np.fft.fft2(c), axis=0)))
    assert abs(np.sum(Ay * c) - np.sum(y * Atc)) < 1e-10 * abs(np.sum(Ay * c))


def test_oracle_conv_paths_agree():
    x = np.random.default_rng(4).standard_normal((256, 256))
    a = nsst2d.atrousdec(x, conv='port', nthreads=4)
    b = nsst2d.atrousdec(x, conv='numpy')
    for u, v in zip(a, b):
        np.testing.assert_allclose(u, v, atol=1e-12)


def test_threshold_rules():
    d = [np.array([[0.0, -1.0], [2.0, 3.0]]), np.array([[[1.0, -2.5], [2.0, -4.0]]])]
    ht = nsst2d.nsst_HT(d, 1.0, [0, 2], [1.0, np.array([1.0])])
    np.testing.assert_array_equal(ht[1], [[[0.0, -2.5], [0.0, -4.0]]])  # strict >
    st = nsst2d.nsst_ST(d, 1.0, [0, 2], [1.0, np.array([1.0])])
    np.testing.assert_allclose(st[1], [[[0.0, -0.5], [0.0, -2.0]]])


def test_oracle_pyramid_adjoints_dot_product():
    rng = np.random.default_rng(11)
    H = W = 192
    x = rng.standard_normal((H, W))
    gy = [rng.standard_normal((H, W)) for _ in range(5)]
    y = nsst2d.atrousdec(x, nlevels=4, conv='numpy')
    lhs = sum(np.sum(a * b) for a, b in zip(y, gy))
    rhs = np.sum(x * nsst2d.atrousdec_adjoint(gy))
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)
    xr = nsst2d.atrousrec(gy, conv='numpy')
    g = rng.standard_normal((H, W))
    lhs = np.sum(xr * g)
    rhs = sum(np.sum(a * b) for a, b in zip(gy, nsst2d.atrousrec_adjoint(g, 4)))
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)


def test_oracle_loss_gradient_finite_differences():
    from shearcuda_gb300.synth import noisy_image
    H = W = 160
    sf = nsst2d.shear_spectra(H, W, [2, 3], [16, 16])
    clean, noisy = noisy_image(H, W, 20.0, 3)
    tau = [10.0, np.full(4, 20.0), np.full(8, 15.0)]
    loss, gx, gt = nsst2d.denoise_tau_grad(noisy, tau, clean, sf, nthreads=4)
    rng = np.random.default_rng(2)
    h = 1e-4
    for _ in range(4):
        i, j = int(rng.integers(0, H)), int(rng.integers(0, W))
        xp, xm = noisy.copy(), noisy.copy()
        xp[i, j] += h
        xm[i, j] -= h
        fd = (np.sum((nsst2d.denoise_tau(xp, tau, sf, nthreads=4)[0] - clean) ** 2) -
              np.sum((nsst2d.denoise_tau(xm, tau, sf, nthreads=4)[0] - clean) ** 2)) / (2 * h)
        assert abs(fd - gx[i, j]) <= 1e-3 * max(1.0, abs(fd))
    tp = [tau[0], tau[1].copy(), tau[2].copy()]
    tm = [tau[0], tau[1].copy(), tau[2].copy()]
    tp[2][3] += h
    tm[2][3] -= h
    fd = (np.sum((nsst2d.denoise_tau(noisy, tp, sf, nthreads=4)[0] - clean) ** 2) -
          np.sum((nsst2d.denoise_tau(noisy, tm, sf, nthreads=4)[0] - clean) ** 2)) / (2 * h)
    assert abs(fd - gt[2][3]) <= 1e-3 * max(1.0, abs(fd))


def test_com_norm_is_the_noise_std():
    # for white N(0,1) noise every band is Gaussian with std = its shearlet's
    # l2 norm: the exact norms (com_norm.m) and the Monte-Carlo scalars
    # (nsst_scalars.m) agree up to Monte-Carlo error
    H = W = 128
    sf = nsst2d.shear_spectra(H, W, [2, 3], [16, 16])
    E = nsst2d.com_norm(H, W, [2, 3], [16, 16], shear_f=sf)
    mc = nsst2d.nsst_scalars(H, W, sf, seed=3)
    flat = np.concatenate([[mc[0]]] + [np.asarray(s) for s in mc[1:]])
    assert E.shape == flat.shape
    assert np.abs(E / flat - 1).max() < 0.1
