"""GPU parity of the 2-D NSST path against the FP64 oracle (through the C ABI).

Tolerances (FP32 device arithmetic vs FP64 oracle):
  * coefficients and pyramid outputs: relative L2 <= 1e-5
  * denoised output: |PSNR_gpu - PSNR_oracle| <= 0.01 dB
  * thresholding of identical FP32 inputs: bit-exact
"""
import numpy as np
import pytest
import torch

from conftest import DCOMP, DSIZE, K_DEMO, flat_coeffs, flat_scalars, rel_l2
from oracle import nsst2d

pytestmark = pytest.mark.gpu

SIZES = [(256, 256), (256, 384), (384, 512), (512, 512)]
_cache = {}


def _setup(H, W, sigma=20.0, seed=0):
    key = (H, W, sigma, seed)
    if key not in _cache:
        import shearcuda_gb300 as sc
        from shearcuda_gb300.synth import noisy_image
        clean, noisy = noisy_image(H, W, sigma, seed)
        noisy32 = noisy.astype(np.float32)
        shear = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W)
        sf = nsst2d.shear_spectra(H, W, DCOMP, DSIZE)
        scal = nsst2d.nsst_scalars(H, W, sf, seed=100, nthreads=8)
        _cache[key] = (clean, noisy32, shear, sf, scal)
    return _cache[key]


@pytest.mark.parametrize('HW', SIZES)
def test_atrous_pyramid_matches_oracle(built_lib, cuda, HW):
    import shearcuda_gb300 as sc
    clean, noisy32, shear, sf, scal = _setup(*HW)
    x = torch.tensor(noisy32, device=cuda)
    y = sc.atrousdec(x, shear).cpu().numpy()
    ref = nsst2d.atrousdec(noisy32.astype(np.float64), nthreads=8)
    for i in range(len(ref)):
        assert rel_l2(y[i], ref[i]) <= 1e-5, (i, rel_l2(y[i], ref[i]))
    # synthesis on FP32-rounded oracle inputs
    y32 = np.stack([r.astype(np.float32) for r in ref])
    xr = sc.atrousrec(torch.tensor(y32, device=cuda), shear).cpu().numpy()
    xr_ref = nsst2d.atrousrec([r.astype(np.float64) for r in y32], nthreads=8)
    assert rel_l2(xr, xr_ref) <= 1e-5


@pytest.mark.parametrize('HW', SIZES)
def test_shear_trans_matches_oracle(built_lib, cuda, HW):
    import shearcuda_gb300 as sc
    clean, noisy32, shear, sf, scal = _setup(*HW)
    x = torch.tensor(noisy32, device=cuda)
    c = sc.shear_trans_cuda(x, 'maxflat', shear).cpu().numpy()
    dst, _ = nsst2d.nsst_dec2(noisy32.astype(np.float64), DCOMP, DSIZE, shear_f=sf, nthreads=8)
    ref = flat_coeffs(dst)
    assert rel_l2(c, ref) <= 1e-5
    for b in range(ref.shape[0]):
        assert rel_l2(c[b], ref[b]) <= 1e-5, (b, rel_l2(c[b], ref[b]))


@pytest.mark.parametrize('HW', SIZES)
def test_inverse_shear_matches_oracle(built_lib, cuda, HW):
    import shearcuda_gb300 as sc
    clean, noisy32, shear, sf, scal = _setup(*HW)
    dst, _ = nsst2d.nsst_dec2(noisy32.astype(np.float64), DCOMP, DSIZE, shear_f=sf, nthreads=8)
    c32 = flat_coeffs(dst).astype(np.float32)
    xr = sc.inverse_shear_cuda(torch.tensor(c32, device=cuda), 'maxflat', shear).cpu().numpy()
    parts = [c32[0].astype(np.float64)]
    at = 1
    for d in DCOMP:
        parts.append(c32[at:at + (1 << d)].astype(np.float64))
        at += 1 << d
    ref = nsst2d.nsst_rec2(parts, sf, nthreads=8)
    assert rel_l2(xr, ref) <= 1e-5
    assert rel_l2(xr, noisy32) <= 1e-5  # perfect reconstruction


@pytest.mark.parametrize('mode', [0, 1])
def test_thresh_is_exact_on_identical_inputs(built_lib, cuda, mode):
    import shearcuda_gb300 as sc
    clean, noisy32, shear, sf, scal = _setup(256, 256)
    x = torch.tensor(noisy32, device=cuda)
    c = sc.shear_trans_cuda(x, 'maxflat', shear)
    host = c.cpu().numpy()
    flat = flat_scalars(scal)
    sc.thresh_cuda(c, 20.0, K_DEMO, flat, shear, mode=mode)
    got = c.cpu().numpy()
    t = np.array([np.float32(K_DEMO[lv] * 20.0 * flat[b]) for b, lv in enumerate(shear.band_levels)],
                 dtype=np.float32)[:, None, None]
    if mode == 0:
        exp = np.where(np.abs(host) > t, host, np.float32(0))
    else:
        a = np.abs(host) - t
        exp = np.where(a > 0, np.copysign(a, host), np.float32(0)).astype(np.float32)
    np.testing.assert_array_equal(got, exp)


@pytest.mark.parametrize('HW', SIZES)
@pytest.mark.parametrize('mode', ['hard', 'soft'])
def test_denoise_matches_oracle_psnr(built_lib, cuda, HW, mode):
    import shearcuda_gb300 as sc
    clean, noisy32, shear, sf, scal = _setup(*HW)
    x = torch.tensor(noisy32, device=cuda)
    out = sc.nsst_denoise(x, shear, 20.0, K_DEMO, flat_scalars(scal), mode=0 if mode == 'hard' else 1)
    out = out.cpu().numpy().astype(np.float64)
    ref, _ = nsst2d.denoise(noisy32.astype(np.float64), 20.0, K_DEMO, scal, DCOMP, DSIZE, mode=mode, shear_f=sf,
                            nthreads=8)
    p_gpu, p_ref = nsst2d.psnr(clean, out), nsst2d.psnr(clean, ref)
    assert abs(p_gpu - p_ref) <= 0.01, (p_gpu, p_ref)
    assert p_gpu > nsst2d.psnr(clean, noisy32) + 3.0  # it actually denoises
    assert rel_l2(out, ref) <= 1e-3


@pytest.mark.parametrize('mode', [0, 1])
@pytest.mark.parametrize('batch', [1, 4])
def test_all_bands_thresholded_away(built_lib, cuda, mode, batch):
    # thresholds above every coefficient: each row tile of every band
    # thresholds to zero, so the row pass writes zero tiles without the
    # forward transform; the result is the lowpass band's reconstruction,
    # as in the oracle with the same thresholds
    import shearcuda_gb300 as sc
    clean, noisy32, _, sf, scal = _setup(512, 512)
    shear = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, 512, 512, batch=batch)
    K = [0.0, 1e6, 1e6, 1e6, 1e6]
    x = torch.tensor(noisy32, device=cuda)
    outs = sc.nsst_denoise_batch([x] * batch, shear, [20.0] * batch, K, flat_scalars(scal), mode=mode)
    ref, _ = nsst2d.denoise(noisy32.astype(np.float64), 20.0, K, scal, DCOMP, DSIZE,
                            mode='hard' if mode == 0 else 'soft', shear_f=sf, nthreads=8)
    for o in outs:
        assert rel_l2(o.cpu().numpy().astype(np.float64), ref) <= 1e-5


def test_fused_denoise_equals_materialised_chain(built_lib, cuda):
    # with the direct pyramid the fused pass runs the chain's kernels
    # (test_gpu_dct_pyramid.py covers the spectral pyramid)
    import shearcuda_gb300 as sc
    clean, noisy32, _, sf, scal = _setup(512, 512)
    shear = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, 512, 512, pyramid=sc.PYRAMID_DIRECT)
    shear.set_directional('split')  # test_gpu_fused.py covers the cluster kernel
    x = torch.tensor(noisy32, device=cuda)
    flat = flat_scalars(scal)
    fused = sc.nsst_denoise(x, shear, 20.0, K_DEMO, flat)
    c = sc.shear_trans_cuda(x, 'maxflat', shear)
    sc.thresh_cuda(c, 20.0, K_DEMO, flat, shear)
    chain = sc.inverse_shear_cuda(c, 'maxflat', shear)
    np.testing.assert_array_equal(fused.cpu().numpy(), chain.cpu().numpy())


@pytest.mark.parametrize('HW', [(1024, 1024), (768, 1024), (2048, 2048)])
def test_full_size_round_trip_and_linearity(built_lib, cuda, HW):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    H, W = HW
    shear = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W)
    _, a = noisy_image(H, W, 20.0, 1)
    _, b = noisy_image(H, W, 20.0, 2)
    xa = torch.tensor(a.astype(np.float32), device=cuda)
    xb = torch.tensor(b.astype(np.float32), device=cuda)
    ca = sc.shear_trans_cuda(xa, 'maxflat', shear)
    xr = sc.inverse_shear_cuda(ca, 'maxflat', shear)
    assert rel_l2(xr.cpu().numpy(), xa.cpu().numpy()) <= 1e-5
    cb = sc.shear_trans_cuda(xb, 'maxflat', shear)
    cab = sc.shear_trans_cuda(2.0 * xa - 0.5 * xb, 'maxflat', shear)
    assert rel_l2(cab.cpu().numpy(), (2.0 * ca - 0.5 * cb).cpu().numpy()) <= 1e-5
    # zero thresholds: fused denoise is the identity (perfect reconstruction)
    out = sc.nsst_denoise(xa, shear, 0.0, [0] * 5, np.ones(shear.nbands))
    assert rel_l2(out.cpu().numpy(), xa.cpu().numpy()) <= 1e-5
    del shear
    torch.cuda.empty_cache()


def test_monte_carlo_scalars_plausible(built_lib, cuda):
    import shearcuda_gb300 as sc
    clean, noisy32, shear, sf, scal = _setup(256, 256)
    got = sc.nsst_scalars(shear, seed=5)
    ref = flat_scalars(scal)
    # two independent one-draw Monte-Carlo estimates (nsst_scalars.m:28): a
    # 256x256 draw spreads by a few percent per band, more for the lowpass
    dev = np.abs(got / ref - 1)
    assert dev.max() < 0.2 and dev.mean() < 0.04, (dev.max(), dev.mean())


def test_empty_and_bad_calls_report_errors(built_lib, cuda):
    import shearcuda_gb300 as sc
    from shearcuda_gb300._lib import NsstError
    clean, noisy32, shear, sf, scal = _setup(256, 256)
    x = torch.tensor(noisy32, device=cuda)
    with pytest.raises(NsstError):
        sc.nsst_denoise(x, shear, -1.0, K_DEMO, flat_scalars(scal))
    with pytest.raises(NsstError):
        sc.nsst_denoise(x, shear, 20.0, K_DEMO, flat_scalars(scal)[:-1])
    with pytest.raises(NsstError):
        sc.shear_trans_cuda(x[:128], 'maxflat', shear)
    with pytest.raises(NsstError):
        sc.shear_trans_cuda(x, '9-7', shear)


def test_allocation_failure_is_reported(built_lib, cuda):
    import shearcuda_gb300 as sc
    from shearcuda_gb300._lib import NsstError, lib
    lib().nsst_debug_fail_next_alloc(1)
    try:
        with pytest.raises(NsstError) as e:
            sc.ShearPlan(DCOMP, DSIZE, 256, 256)
        assert e.value.status == 3
    finally:
        lib().nsst_debug_fail_next_alloc(0)
    sc.ShearPlan(DCOMP, DSIZE, 256, 256)  # and the library still works


def test_band_norms_and_thresh_max_match_oracle(built_lib, cuda):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    H = W = 256
    shear = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W)
    E = sc.com_norm(shear)
    sf = nsst2d.shear_spectra(H, W, DCOMP, DSIZE)
    E_ref = nsst2d.com_norm(H, W, DCOMP, DSIZE, shear_f=sf)
    assert np.abs(E / E_ref - 1).max() < 1e-5
    # thresh_cuda(..., opt=1) with the exact norms as scalars
    _, noisy = noisy_image(H, W, 20.0, 31)
    x = torch.tensor(noisy.astype(np.float32), device=cuda)
    c = sc.shear_trans_cuda(x, 'maxflat', shear)
    maxi = sc.thresh_cuda(c, 20.0, [0, 3, 3, 3, 4], E, shear, opt=1)
    got = c.cpu().numpy().astype(np.float64)
    assert maxi == pytest.approx(nsst2d.thresh_maxi(got, E), rel=1e-12)
    # the thresholded planes are the plain threshold's
    c2 = sc.shear_trans_cuda(x, 'maxflat', shear)
    sc.thresh_cuda(c2, 20.0, [0, 3, 3, 3, 4], E, shear)
    assert torch.equal(c2.cpu(), torch.tensor(got, dtype=torch.float32))


def test_re_weight_band_matches_oracle(built_lib, cuda):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    H, W = 256, 384
    shear = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W)
    _, noisy = noisy_image(H, W, 20.0, 41)
    x = torch.tensor(noisy.astype(np.float32), device=cuda)
    w = [0.5, 1.0, 1.5, 2.0, 0.25]
    got = sc.re_weight_band(x, w, shear).cpu().numpy().astype(np.float64)
    ref = nsst2d.re_weight_band(noisy.astype(np.float32).astype(np.float64), w)
    assert rel_l2(got, ref) <= 1e-5
    ones = sc.re_weight_band(x, [1.0] * 5, shear).cpu().numpy()
    assert rel_l2(ones, noisy) <= 1e-5  # perfect reconstruction
    # fewer levels than the plan: the separation demo's four weights (three levels)
    w3 = [0.1, 0.1, 1.5, 1.5]
    got3 = sc.re_weight_band(x, w3, shear).cpu().numpy().astype(np.float64)
    assert rel_l2(got3, nsst2d.re_weight_band(noisy.astype(np.float32).astype(np.float64), w3)) <= 1e-5
    for bad in ([1.0], [1.0] * 6):
        with pytest.raises(sc.NsstError):
            sc.re_weight_band(x, bad, shear)
