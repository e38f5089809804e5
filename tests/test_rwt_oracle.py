"""The wavelet oracle (oracle/rwt.py), pinned: against the golden outputs of
the reference's Rice Wavelet Toolbox templates (tests/golden/rwt_ref_cases.npz,
made by tests/golden/make_golden.py), against those templates themselves when
oracle/_ref is built, against MakeONFilter.m when the reference tree is here,
plus the transform's own identities.  No GPU."""
import json
import os

import numpy as np
import pytest

from oracle import rwt

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden', 'rwt_ref_cases.npz'))
from oracle.build_oracle import default_reference  # noqa: E402

REFERENCE = default_reference()


@pytest.mark.parametrize('i', range(int(GOLD['n'][0])))
def test_oracle_matches_reference_golden(i):
    x, h, L = GOLD['x_%d' % i], GOLD['h_%d' % i], int(GOLD['L_%d' % i][0])
    yl, yh = rwt.mrdwt(x, h, L)
    # the same sums in the same order as the reference loops: equal to the last bit or nearly
    assert np.abs(yl - GOLD['yl_%d' % i]).max() <= 1e-14
    assert np.abs(yh - GOLD['yh_%d' % i]).max() <= 1e-14
    inv = rwt.mirdwt(GOLD['yl_%d' % i], GOLD['yh2_%d' % i], h, L)
    assert np.abs(inv - GOLD['inv_%d' % i]).max() <= 1e-14
    assert np.abs(rwt.mdwt(x, h, min(L, 2)) - GOLD['mdwt_%d' % i]).max() <= 1e-14


def test_oracle_matches_reference_library_random():
    from oracle import rwt_ref
    if not rwt_ref.available():
        pytest.skip('oracle/_ref/librwt_ref.so not built (reference tree absent)')
    rng = np.random.default_rng(77)
    for (H, W, fam, par, L) in [(32, 64, 'Symmlet', 4, 4), (64, 32, 'Daubechies', 6, 3), (16, 16, 'Symmlet', 8, 4),
                                (8, 32, 'Haar', 0, 3), (32, 32, 'Beylkin', 0, 2)]:
        h = rwt.make_on_filter(fam, par)
        x = rng.standard_normal((H, W))
        a, b = rwt.mrdwt(x, h, L)
        c, d = rwt_ref.mrdwt(x, h, L)
        assert np.abs(a - c).max() <= 1e-13 and np.abs(b - d).max() <= 1e-13
        yh2 = d + rng.standard_normal(d.shape)
        assert np.abs(rwt.mirdwt(c, yh2, h, L) - rwt_ref.mirdwt(c, yh2, h, L)).max() <= 1e-13
        assert np.abs(rwt.mdwt(x, h, 2) - rwt_ref.mdwt(x, h, 2)).max() <= 1e-13


@pytest.mark.parametrize('fam,par', [('Symmlet', 4), ('Haar', 0), ('Daubechies', 4), ('Daubechies', 20),
                                     ('Vaidyanathan', 0)])
def test_mirdwt_inverts_mrdwt(fam, par):
    h = rwt.make_on_filter(fam, par)
    x = np.random.default_rng(3).standard_normal((32, 64))
    yl, yh = rwt.mrdwt(x, h, 3)
    # the tables carry 12 digits, so the filters are orthonormal to about 1e-12
    assert np.abs(rwt.mirdwt(yl, yh, h, 3) - x).max() < 1e-9


def test_mrdwt_rejects_indivisible_size():
    with pytest.raises(ValueError):
        rwt.mrdwt(np.zeros((12, 16)), rwt.make_on_filter('Haar'), 3)


def test_onfilter_tables_match_makeonfilter_source():
    src = os.path.join(REFERENCE, 'shearcuda', 'MakeONFilter.m')
    if not os.path.exists(src):
        pytest.skip('reference tree absent')
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        'gen_wavelet_tables', os.path.join(os.path.dirname(__file__), '..', 'shearcuda_gb300', 'csrc',
                                           'gen_wavelet_tables.py'))
    gen = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(gen)
    parsed = gen.parse(open(src).read())
    committed = json.load(open(os.path.join(os.path.dirname(rwt.__file__), 'onfilter_tables.json')))['tables']
    assert [(t, p, h, v) for (t, p, h, v) in parsed] == [(c['type'], c['par'], c['half'], c['values'])
                                                          for c in committed]


def test_onfilter_families():
    # MakeONFilter.m: lengths and unit norm
    for fam, par, n in [('Haar', 0, 2), ('Daubechies', 4, 4), ('Daubechies', 20, 20), ('Symmlet', 4, 8),
                        ('Symmlet', 10, 20), ('Coiflet', 5, 30), ('Beylkin', 0, 18), ('Vaidyanathan', 0, 24),
                        ('Battle', 1, 23), ('Battle', 5, 59)]:
        f = rwt.make_on_filter(fam, par)
        assert f.size == n
        assert abs(np.sum(f * f) - 1) < 1e-15
    h = rwt.make_on_filter('Haar')
    assert np.allclose(h, [2 ** -0.5, 2 ** -0.5], rtol=0, atol=2.3e-16)
    b = rwt.make_on_filter('Battle', 3)
    assert np.array_equal(b, b[::-1])  # the mirror construction is symmetric
    with pytest.raises(ValueError):
        rwt.make_on_filter('Symmlet', 3)


def test_mad_follows_matlab_median():
    # even count: mean of the two middle values; NaNs dropped
    x = np.array([1.0, 2.0, 4.0, 7.0, np.nan])
    med = 3.0
    dev = np.sort(np.abs(np.array([1.0, 2.0, 4.0, 7.0]) - med))  # 1 1 2 4
    assert rwt.mad(x) == pytest.approx(((dev[1] + dev[2]) / 2) / .6745, rel=0, abs=1e-15)


def test_soft_thresh_and_tv_identities():
    rng = np.random.default_rng(5)
    y = rng.standard_normal(100)
    s = rwt.soft_thresh(y, 0.5)
    assert np.allclose(s, np.sign(y) * np.maximum(np.abs(y) - 0.5, 0))
    x = rng.standard_normal((16, 32))
    assert np.abs(rwt.tv_correction(x, 0.0) - x).max() < 1e-12   # no threshold: perfect reconstruction
    c = np.full((16, 32), 3.25)
    assert np.abs(rwt.tv_correction(c, 10.0) - c).max() < 1e-12  # constants have no highpass


def test_separate_oracle_small():
    # a tiny separation: the parts are finite, the curve part carries the
    # smooth structure, the setup values follow separate.m:82-131
    from shearcuda_gb300.synth import points_and_curves
    img, noisy = points_and_curves(64, npoints=20, sigma=10.0, seed=2)
    C, P, info = rwt.separate(noisy, [2, 2], [16, 16], level2=2, itermax=3, stop=3.0, gamma=3.0,
                              coeff=[0.1, 1.5, 1.5])
    assert np.isfinite(C).all() and np.isfinite(P).all()
    assert info['deltamax'] == min(info['buff_shear'], info['buff_wavelet'])
    assert info['lam'] == pytest.approx((info['deltamax'] / info['stop']) ** (1 / (1 - 3)), rel=1e-15)
    assert np.linalg.norm(C + P) > 0.5 * np.linalg.norm(img - img.mean())
