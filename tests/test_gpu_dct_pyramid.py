"""The fused denoise pipeline with its pyramid in the DCT-II domain
(NSST_PYRAMID_SPECTRAL, the default where the filters allow it) against the
same pipeline with the direct dilated-convolution pyramid and against the
FP64 oracle.

Both compute atrousdec.m / atrousrec.m exactly in real arithmetic (each step
is a pointwise product in the DCT-II domain of the symmetric extension); in
FP32 they differ by rounding.  Tolerances:
  * zero thresholds (perfect reconstruction): relative L2 <= 1e-5 to the input
  * soft threshold (a 1-Lipschitz map): relative L2 <= 1e-5 between the paths
  * hard threshold: relative L2 <= 1e-3 (coefficients within rounding of their
    threshold flip), |PSNR difference| <= 0.01 dB to the oracle
  * one image alone and the same image in a batch: bit-identical
"""
import numpy as np
import pytest
import torch

from conftest import DCOMP, DSIZE, K_DEMO, flat_scalars, rel_l2
from oracle import nsst2d

pytestmark = pytest.mark.gpu

_plans = {}


def _plan(H, W, pyramid, lpfilt='maxflat', batch=1):
    import shearcuda_gb300 as sc
    key = (H, W, pyramid, lpfilt, batch)
    if key not in _plans:
        p = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, lpfilt=lpfilt, pyramid=pyramid, batch=batch)
        p.set_scalars(np.linspace(0.5, 1.5, p.nbands))
        _plans[key] = p
    return _plans[key]


def _img(H, W, seed, cuda):
    from shearcuda_gb300.synth import noisy_image
    _, noisy = noisy_image(H, W, 20.0, seed)
    return torch.tensor(noisy.astype(np.float32), device=cuda)


def _stages(plan, x, K, mode=0):
    import shearcuda_gb300 as sc
    plan.enable_timers(True)
    try:
        sc.nsst_denoise(x, plan, 20.0, K, None, mode=mode)
        return [n for n, _ in plan.read_timers(40)]
    finally:
        plan.enable_timers(False)


@pytest.mark.parametrize('HW', [(256, 256), (256, 384), (384, 512), (512, 512), (768, 1024)])
@pytest.mark.parametrize('lpfilt', ['maxflat', '9-7', 'pyr', 'pyrexc'])
def test_spectral_pyramid_reconstructs(built_lib, cuda, HW, lpfilt):
    import shearcuda_gb300 as sc
    H, W = HW
    if lpfilt != 'maxflat' and HW not in [(256, 384), (512, 512)]:
        pytest.skip('other filter sets on two sizes')
    p = _plan(H, W, sc.PYRAMID_SPECTRAL, lpfilt)
    x = _img(H, W, 3, cuda)
    assert 'dct_rows_levels' in _stages(p, x, [0] * 5)  # the spectral path ran
    out = sc.nsst_denoise(x, p, 0.0, [0] * 5, None)
    assert rel_l2(out.cpu().numpy(), x.cpu().numpy()) <= 1e-5


@pytest.mark.parametrize('HW', [(256, 256), (384, 512), (512, 512)])
@pytest.mark.parametrize('lpfilt', ['maxflat', '9-7'])
def test_spectral_equals_direct(built_lib, cuda, HW, lpfilt):
    import shearcuda_gb300 as sc
    H, W = HW
    ps, pd = _plan(H, W, sc.PYRAMID_SPECTRAL, lpfilt), _plan(H, W, sc.PYRAMID_DIRECT, lpfilt)
    x = _img(H, W, 4, cuda)
    assert 'dct_rows_levels' not in _stages(pd, x, K_DEMO)
    for mode, tol in [(sc.THRESH_SOFT, 1e-5), (sc.THRESH_HARD, 1e-3)]:
        a = sc.nsst_denoise(x, ps, 20.0, K_DEMO, None, mode=mode).cpu().numpy()
        b = sc.nsst_denoise(x, pd, 20.0, K_DEMO, None, mode=mode).cpu().numpy()
        assert rel_l2(a, b) <= tol, (mode, rel_l2(a, b))


def test_spectral_matches_oracle_psnr(built_lib, cuda):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    H, W = 256, 384
    clean, noisy = noisy_image(H, W, 20.0, 9)
    n32 = noisy.astype(np.float32)
    p = _plan(H, W, sc.PYRAMID_SPECTRAL)
    sf = nsst2d.shear_spectra(H, W, DCOMP, DSIZE)
    scal = nsst2d.nsst_scalars(H, W, sf, seed=100, nthreads=8)
    out = sc.nsst_denoise(torch.tensor(n32, device=cuda), p, 20.0, K_DEMO, flat_scalars(scal)).cpu().numpy()
    ref, _ = nsst2d.denoise(n32.astype(np.float64), 20.0, K_DEMO, scal, DCOMP, DSIZE, shear_f=sf, nthreads=8)
    assert abs(nsst2d.psnr(clean, out) - nsst2d.psnr(clean, ref)) <= 0.01
    assert rel_l2(out, ref) <= 1e-3


def test_spectral_batch_equals_single_and_graphs(built_lib, cuda):
    import shearcuda_gb300 as sc
    H, W = 256, 384
    single = _plan(H, W, sc.PYRAMID_SPECTRAL)
    batch = _plan(H, W, sc.PYRAMID_SPECTRAL, batch=3)
    xs = [_img(H, W, 20 + i, cuda) for i in range(3)]
    sig = [12.0, 20.0, 35.0]
    outs = sc.nsst_denoise_batch(xs, batch, sig, K_DEMO, None)
    for x, o, s in zip(xs, outs, sig):
        ref = sc.nsst_denoise(x, single, s, K_DEMO, None)
        np.testing.assert_array_equal(o.cpu().numpy(), ref.cpu().numpy())
    batch.use_graphs(True)
    try:
        outs2 = sc.nsst_denoise_batch(xs, batch, sig, K_DEMO, None)
        for o, o2 in zip(outs, outs2):
            np.testing.assert_array_equal(o.cpu().numpy(), o2.cpu().numpy())
    finally:
        batch.use_graphs(False)


@pytest.mark.parametrize('HW', [(256, 256), (256, 384)])
def test_spectral_thresholded_lowpass(built_lib, cuda, HW):
    # the lowpass band leaves the DCT domain once: IDCT2, threshold, DCT2
    import shearcuda_gb300 as sc
    H, W = HW
    ps, pd = _plan(H, W, sc.PYRAMID_SPECTRAL), _plan(H, W, sc.PYRAMID_DIRECT)
    x = _img(H, W, 7, cuda)
    K = [0.9] + list(K_DEMO[1:])  # lowpass threshold 0.9 * 20 * 0.5: a part of the lowpass is cut
    assert 'dct_lowpass_threshold' in _stages(ps, x, K)
    for mode, tol in [(sc.THRESH_SOFT, 1e-5), (sc.THRESH_HARD, 1e-3)]:
        a = sc.nsst_denoise(x, ps, 20.0, K, None, mode=mode).cpu().numpy()
        b = sc.nsst_denoise(x, pd, 20.0, K, None, mode=mode).cpu().numpy()
        assert rel_l2(a, b) <= tol, (mode, rel_l2(a, b))
    # a lowpass threshold above every lowpass value removes the lowpass on both paths
    K = [1e6] + list(K_DEMO[1:])
    a = sc.nsst_denoise(x, ps, 20.0, K, None, mode=sc.THRESH_SOFT).cpu().numpy()
    b = sc.nsst_denoise(x, pd, 20.0, K, None, mode=sc.THRESH_SOFT).cpu().numpy()
    assert rel_l2(a, b) <= 1e-4


def test_direct_fallbacks(built_lib, cuda):
    import shearcuda_gb300 as sc
    H, W = 256, 256
    pa = _plan(H, W, sc.PYRAMID_AUTO)
    x = _img(H, W, 5, cuda)
    # under NSST_PYRAMID_AUTO an image 4 bytes off a 16-byte boundary takes the direct pyramid
    buf = torch.zeros(H * W + 1, device=cuda)
    buf[1:] = x.reshape(-1)
    xm = buf[1:].view(H, W)
    a = sc.nsst_denoise(xm, pa, 20.0, K_DEMO, None, mode=sc.THRESH_SOFT).cpu().numpy()
    b = sc.nsst_denoise(x, pa, 20.0, K_DEMO, None, mode=sc.THRESH_SOFT).cpu().numpy()
    assert rel_l2(a, b) <= 1e-5
    # NSST_PYRAMID_SPECTRAL refuses it rather than switching silently
    ps = _plan(H, W, sc.PYRAMID_SPECTRAL)
    with pytest.raises(sc.NsstError):
        sc.nsst_denoise(xm, ps, 20.0, K_DEMO, None, mode=sc.THRESH_SOFT)
    with pytest.raises(sc.NsstError):
        sc.shear_trans_cuda(xm, 'maxflat', ps)


def test_pyramid_modes(built_lib, cuda):
    import shearcuda_gb300 as sc
    with pytest.raises(sc.NsstError):
        sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, 256, 256, pyramid=3)
    # the default (auto) plan takes the spectral path for atrousfilters.m's sets
    p = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, 256, 256)
    p.set_scalars(np.ones(p.nbands))
    assert 'dct_rows_levels' in _stages(p, _img(256, 256, 6, cuda), K_DEMO)


@pytest.mark.parametrize('HW', [(256, 384), (512, 512)])
def test_spectral_shear_trans_and_inverse(built_lib, cuda, HW):
    # nsst_shear_trans / nsst_inverse_shear (shear_trans_cuda / inverse_shear_cuda) on the
    # spectral pyramid: coefficients and reconstructions within FP32 rounding of the direct ones
    import shearcuda_gb300 as sc
    H, W = HW
    ps, pd = _plan(H, W, sc.PYRAMID_SPECTRAL), _plan(H, W, sc.PYRAMID_DIRECT)
    x = _img(H, W, 8, cuda)
    ps.enable_timers(True)
    try:
        cs = sc.shear_trans_cuda(x, 'maxflat', ps)
        assert 'dct_lowpass' in [n for n, _ in ps.read_timers(40)]
    finally:
        ps.enable_timers(False)
    cd = sc.shear_trans_cuda(x, 'maxflat', pd)
    assert rel_l2(cs.cpu().numpy(), cd.cpu().numpy()) <= 1e-5
    assert rel_l2(cs[0].cpu().numpy(), cd[0].cpu().numpy()) <= 1e-5  # the lowpass plane alone
    rs = sc.inverse_shear_cuda(cs, 'maxflat', ps)
    rd = sc.inverse_shear_cuda(cs, 'maxflat', pd)
    assert rel_l2(rs.cpu().numpy(), rd.cpu().numpy()) <= 1e-5
    assert rel_l2(rs.cpu().numpy(), x.cpu().numpy()) <= 1e-5
    # under NSST_PYRAMID_AUTO an output 4 bytes off a 16-byte boundary takes the
    # direct pyramid; NSST_PYRAMID_SPECTRAL refuses it
    from shearcuda_gb300 import _lib
    buf = torch.zeros(H * W + 1, device=cuda)
    assert _lib.lib().nsst_inverse_shear(ps.handle, cs.data_ptr(), buf.data_ptr() + 4, None) == 1
    pa = _plan(H, W, sc.PYRAMID_AUTO)
    pa.enable_timers(True)
    try:
        _lib.check(_lib.lib().nsst_inverse_shear(pa.handle, cs.data_ptr(), buf.data_ptr() + 4, None))
        assert 'dct_lowpass' not in [n for n, _ in pa.read_timers(40)]
    finally:
        pa.enable_timers(False)
    torch.cuda.synchronize()
    assert rel_l2(buf[1:].view(H, W).cpu().numpy(), rd.cpu().numpy()) <= 1e-5


@pytest.mark.parametrize('mode', [0, 1])
def test_spectral_gradients_match_direct(built_lib, cuda, mode):
    # the differentiable forward and its backward on the spectral pyramid
    # (the pyramid operators are symmetric, so the adjoint swaps the analysis
    # and synthesis tables) against the direct pyramid's
    import shearcuda_gb300 as sc
    H, W = 256, 256
    grads = []
    for pyr in (sc.PYRAMID_SPECTRAL, sc.PYRAMID_DIRECT):
        p = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, pyramid=pyr, batch=2)
        sc.autograd.enable_grad(p)
        x = torch.stack([_img(H, W, 30, cuda), _img(H, W, 31, cuda)]).requires_grad_(True)
        tau = torch.tensor(np.linspace(20.0, 60.0, p.nbands), dtype=torch.float32, device=cuda,
                           requires_grad=True)
        p.enable_timers(True)
        out = sc.nsst_denoise_diff(x, tau, p, mode)
        gy = torch.sin(torch.arange(out.numel(), device=cuda, dtype=torch.float32)).view_as(out)
        out.backward(gy)
        names = [n for n, _ in p.read_timers(40)]
        p.enable_timers(False)
        assert ('gradient_pyramid' in names) == (pyr == sc.PYRAMID_SPECTRAL)
        grads.append((out.detach().cpu().numpy(), x.grad.cpu().numpy(), tau.grad.cpu().numpy()))
    (o1, gx1, gt1), (o2, gx2, gt2) = grads
    assert rel_l2(o1, o2) <= 1e-3
    assert rel_l2(gx1, gx2) <= 1e-3, rel_l2(gx1, gx2)
    if mode == 1:
        assert rel_l2(gt1, gt2) <= 1e-3, rel_l2(gt1, gt2)


def test_spectral_atrousdec_atrousrec(built_lib, cuda):
    # nsst_atrousdec / nsst_atrousrec (the reference's atrousdec / atrousrec) on
    # the spectral pyramid: every plane within FP32 rounding of the direct one
    import shearcuda_gb300 as sc
    H, W = 384, 512
    ps, pd = _plan(H, W, sc.PYRAMID_SPECTRAL), _plan(H, W, sc.PYRAMID_DIRECT)
    x = _img(H, W, 12, cuda)
    ys, yd = sc.atrousdec(x, ps), sc.atrousdec(x, pd)
    for k in range(ys.shape[0]):
        assert rel_l2(ys[k].cpu().numpy(), yd[k].cpu().numpy()) <= 1e-5, k
    ys2 = ys.clone()
    ys2[1:] *= 0.5  # a synthesis input that is not an analysis output
    rs, rd = sc.atrousrec(ys2, ps), sc.atrousrec(ys2, pd)
    assert rel_l2(rs.cpu().numpy(), rd.cpu().numpy()) <= 1e-5
    assert rel_l2(sc.atrousrec(ys, ps).cpu().numpy(), x.cpu().numpy()) <= 1e-5

