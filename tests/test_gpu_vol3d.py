"""3-D path parity: libnsst.so's volume kernels (through the C ABI) against the
FP64 oracle (oracle/nsst3d.py) on seeded volumes.  Tolerances: relative L2
<= 1e-5 on sub-bands and directional coefficients (FP32 arithmetic), and
<= 0.01 dB PSNR difference on the denoised volume."""
import json
import math
import os

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope='module')
def s3(built_lib, cuda):
    import shearcuda_gb300 as s
    return s


def _t(a, dev='cuda'):
    import torch
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device=dev)


def _np(t):
    return t.detach().cpu().numpy().astype(np.float64)


def test_plan_geometry(s3):
    p = s3.VolumePlan(128, 128, 128, num_dirs=(2, 2, 4), batch=1)
    assert p.grid == (144, 144, 144)
    assert [d[0] for d in p.level_dims] == [144, 96, 48, 24]
    assert [c[0] for c in p.conv_dims] == [192, 128, 64, 0]  # N >= m + 12
    assert p.nbands == 72
    assert p.band_info[0] == (0, 0, 0, 0) and p.band_info[71] == (2, 2, 3, 3)
    q = s3.VolumePlan(80, 96, 100, num_dirs=(2, 2, 4))
    assert q.grid == (96, 96, 144)
    assert q.level_dims[3] == (16, 16, 24)


def test_plan_rejects_bad_arguments(s3):
    with pytest.raises(s3.NsstError):
        s3.VolumePlan(200, 96, 96)
    with pytest.raises(s3.NsstError):
        s3.VolumePlan(96, 96, 96, num_dirs=(5, 2, 2))
    with pytest.raises(s3.NsstError):
        s3.VolumePlan(96, 96, 96, pyr_mode=3)
    p = s3.VolumePlan(40, 40, 40, num_dirs=(2, 2, 4), batch=1)
    import torch
    with pytest.raises(s3.NsstError):
        s3.do_pyr_dec(torch.zeros((2, 40, 40, 40), device='cuda'), p)
    with pytest.raises(s3.NsstError):
        s3.do_pyr_dec(torch.zeros((1, 40, 40, 41), device='cuda'), p)
    with pytest.raises(s3.NsstError):
        s3.denoise3(torch.zeros((1, 40, 40, 40), device='cuda'), p, 30.0)  # no scalars stored


def test_pyr_dec_rec_match_oracle(s3):
    from oracle import nsst3d
    shape = (80, 96, 100)
    _, x = s3.synth.noisy_volume(shape, 30.0, 11)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4))
    flat, subs = s3.do_pyr_dec(_t(x), p)
    ref = nsst3d.pyr_dec(nsst3d.pad_volume(x), 3, 1.5)
    for l in range(4):
        assert subs[l].shape[1:] == ref[l].shape
        assert rel_l2(_np(subs[l][0]), ref[l]) < TOL, l
    rec = s3.do_pyr_rec(flat, p)
    assert rel_l2(_np(rec[0]), x) < TOL
    # reconstruction from the oracle's sub-bands
    rec2 = s3.do_pyr_rec(p.pack([_t(r[None]) for r in ref]), p)
    ref_rec = nsst3d.pyr_rec(ref, 1.5)[:shape[0], :shape[1], :shape[2]]
    assert rel_l2(_np(rec2[0]), ref_rec) < TOL


@pytest.mark.parametrize('mode,L,shape', [(1.5, 2, (48, 64, 72)), (1, 2, (96, 96, 96))])
def test_pyramid_other_modes(s3, mode, L, shape):
    from oracle import nsst3d
    x = np.random.default_rng(4).standard_normal(shape) * 50 + 80
    p = s3.VolumePlan(*shape, num_dirs=(2,) * L, pyr_mode=mode)
    flat, subs = s3.do_pyr_dec(_t(x), p)
    ref = nsst3d.pyr_dec(nsst3d.pad_volume_to(x, p.grid), L, mode)
    for l in range(L + 1):
        assert rel_l2(_np(subs[l][0]), ref[l]) < TOL, l
    assert rel_l2(_np(s3.do_pyr_rec(flat, p)[0]), x) < TOL


def test_sh_dec_matches_oracle(s3):
    from oracle import nsst3d
    shape = (96, 96, 96)
    _, x = s3.synth.noisy_volume(shape, 30.0, 12)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4))
    flat, subs = s3.do_pyr_dec(_t(x), p)
    F = nsst3d.meyer_filters_3d([2, 2, 4])
    bands = nsst3d.band_list(F)
    for l in range(3):
        got = _np(s3.sh_dec(flat, l, p)[0])
        bp = _np(subs[l][0])
        mine = [b for b in bands if b[1] == l]
        assert got.shape[0] == len(mine)
        for k, (c, ll, l2, l1, f) in enumerate(mine):
            assert rel_l2(got[k], nsst3d.convnfft_same(bp, f)) < TOL, (l, k)


def test_sh_dec_demo_config_band_order(s3):
    # DenoiseDemo/main.m's dBand (8, 4, 4): check a spread of level-0 bands
    from oracle import nsst3d
    shape = (96, 96, 96)
    _, x = s3.synth.noisy_volume(shape, 30.0, 13)
    p = s3.VolumePlan(*shape, num_dirs=(8, 4, 4))
    assert p.nbands == 288
    flat, subs = s3.do_pyr_dec(_t(x), p)
    F = nsst3d.meyer_filters_3d([8, 4, 4])
    got = s3.sh_dec(flat, 0, p)[0]
    bp = _np(subs[0][0])
    for k in (0, 9, 63, 64, 100, 191):
        c, l2, l1 = k // 64, (k % 64) // 8, k % 8
        assert p.band_info[k] == (0, c, l2, l1)
        assert rel_l2(_np(got[k]), nsst3d.convnfft_same(bp, F[c][0][l2][l1])) < TOL, k


def test_sh_dec_th_rec_without_threshold_is_identity(s3):
    shape = (96, 96, 96)
    _, x = s3.synth.noisy_volume(shape, 30.0, 14)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4))
    flat, subs = s3.do_pyr_dec(_t(x), p)
    rec = s3.sh_dec_th_rec_cuda(flat, p, 30.0, [0, 0, 0], scalars=np.ones(p.nbands))
    rs = p.split(rec)
    for l in range(3):
        assert rel_l2(_np(rs[l]), _np(subs[l])) < TOL
    assert np.array_equal(_np(rs[3]), _np(subs[3]))


def test_sh_dec_th_rec_matches_oracle(s3):
    from oracle import nsst3d
    shape = (96, 96, 96)
    sigma = 30.0
    _, x = s3.synth.noisy_volume(shape, sigma, 15)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4))
    scal = s3.nsst_scalars3(p, seed=3)
    flat, subs = s3.do_pyr_dec(_t(x), p)
    T = [3.3, 3.0, 3.0]
    rec = p.split(s3.sh_dec_th_rec_cuda(flat, p, sigma, T))
    F = nsst3d.meyer_filters_3d([2, 2, 4])
    for l in range(3):
        bp = _np(subs[l][0])
        acc = np.zeros_like(bp)
        for b, (c, ll, l2, l1, f) in enumerate(nsst3d.band_list(F)):
            if ll != l:
                continue
            coef = nsst3d.convnfft_same(bp, f)
            t = np.float32(T[l] * sigma * scal[b])  # the kernel compares against the FP32 threshold
            coef[np.abs(coef) <= t] = 0.0
            acc += coef
        assert rel_l2(_np(rec[l][0]), acc) < 2 * TOL, l


def test_denoise3_matches_oracle(s3):
    from oracle import nsst3d
    shape = (96, 96, 96)
    sigma = 30.0
    clean, x = s3.synth.noisy_volume(shape, sigma, 16)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4))
    scal = s3.nsst_scalars3(p, seed=5)
    T = list(s3.DEMO_T)
    out = _np(s3.denoise3(_t(x), p, sigma, T))
    F = nsst3d.meyer_filters_3d([2, 2, 4])
    ref = nsst3d.denoise3(x, F, sigma, T, scal)
    p_gpu, p_ref, p_in = nsst3d.psnr3(clean, out), nsst3d.psnr3(clean, ref), nsst3d.psnr3(clean, x)
    assert abs(p_gpu - p_ref) <= 0.01
    assert p_gpu > p_in + 5.0
    assert rel_l2(out, ref) < 1e-4


def test_denoise3_batch_equals_single(s3):
    import torch
    shape = (80, 96, 100)
    vols = [s3.synth.noisy_volume(shape, sg, 20 + i)[1] for i, sg in enumerate((20.0, 30.0, 40.0))]
    sig = [20.0, 30.0, 40.0]
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4), batch=3)
    s3.nsst_scalars3(p, seed=1)
    xb = torch.stack([_t(v) for v in vols])
    out = s3.denoise3(xb, p, sig)
    for i in range(3):
        one = s3.denoise3(_t(vols[i]), p, sig[i])
        assert torch.equal(one, out[i])


def test_compute_scalars_match_reference_table(s3):
    # GPU Monte-Carlo noise scalars vs the reference's nsstScalarsData22222.mat
    gold = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden',
                                       'nsst3_scalar_tables.json')))['22222']
    p = s3.VolumePlan(96, 96, 96, num_dirs=tuple(gold['num_dirs']))
    sc = s3.nsst_scalars3(p, seed=7)
    assert np.abs(sc / np.asarray(gold['bands']) - 1).max() < 0.03


def test_vol3d_launch_count_and_determinism(s3):
    import torch
    shape = (48, 48, 48)
    _, x = s3.synth.noisy_volume(shape, 30.0, 17)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4))
    s3.nsst_scalars3(p, seed=1)
    a = s3.denoise3(_t(x), p, 30.0)
    n0 = s3.launch_count()
    b = s3.denoise3(_t(x), p, 30.0)
    torch.cuda.synchronize()
    assert s3.launch_count() > n0
    assert torch.equal(a, b)
    assert math.isfinite(float(a.abs().max()))


def _dot(a, b):
    return float(np.vdot(np.asarray(a, np.float64).ravel(), np.asarray(b, np.float64).ravel()))


def test_denoise3_backward_dot_product(s3):
    # the hard-threshold denoise is linear at fixed masks and f(x0) = J(x0) x0,
    # so <gy, f(x0)> = <J^T gy, x0> with the masks of the same forward call
    import torch
    shape = (80, 96, 100)  # padded to (96, 96, 144): the fold of the edge padding is exercised
    _, x = s3.synth.noisy_volume(shape, 30.0, 31)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4), batch=2)
    s3.nsst_scalars3(p, seed=2)
    p.enable_grad()
    xb = torch.stack([_t(x), _t(x[::-1].copy())])
    out = s3.denoise3(xb, p, [30.0, 20.0])
    # a cotangent correlated with the output (no cancellation in <gy, out>)
    # and a white one, checked against the Cauchy-Schwarz scale
    for gy in (out + 10.0 * torch.randn_like(out), torch.randn_like(out)):
        gx = s3.denoise3_backward(gy, p)
        for i in range(2):
            lhs, rhs = _dot(_np(gy[i]), _np(out[i])), _dot(_np(gx[i]), _np(xb[i]))
            scale = np.linalg.norm(_np(gy[i])) * np.linalg.norm(_np(out[i]))
            assert abs(lhs - rhs) <= 1e-6 * scale, (i, lhs, rhs, scale)


def test_denoise3_backward_identity_without_threshold(s3):
    # T = 0 keeps every coefficient: the denoise is the identity, so is its adjoint
    import torch
    shape = (80, 96, 100)
    _, x = s3.synth.noisy_volume(shape, 30.0, 32)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4))
    p.set_scalars(np.ones(p.nbands))
    p.enable_grad()
    out = s3.denoise3(_t(x), p, 30.0, [0, 0, 0])
    assert rel_l2(_np(out), x) < TOL
    gy = torch.randn((1,) + shape, device='cuda')
    gx = s3.denoise3_backward(gy, p)
    # a white-noise gradient through two pyramids and 36 band-pair transforms in FP32
    assert rel_l2(_np(gx), _np(gy)) < 2 * TOL


def test_denoise3_backward_matches_oracle(s3):
    from oracle import nsst3d
    import torch
    shape = (40, 44, 36)
    sigma = 30.0
    _, x = s3.synth.noisy_volume(shape, sigma, 33)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2))
    assert p.grid == (48, 48, 48)
    scal = s3.nsst_scalars3(p, seed=4)
    p.enable_grad()
    T = [3.0, 3.0]
    s3.denoise3(_t(x), p, sigma, T)
    gy = np.random.default_rng(34).standard_normal(shape)
    gx = _np(s3.denoise3_backward(_t(gy), p))
    F = nsst3d.meyer_filters_3d([2, 2])
    th = [np.float32(T[l] * sigma * scal[b]) / (T[l] * sigma) for b, (c, l, l2, l1, f) in
          enumerate(nsst3d.band_list(F))]
    masks, grid = nsst3d.denoise3_masks(x.astype(np.float32).astype(np.float64), F, sigma, T, np.asarray(th), L=2)
    ref = nsst3d.denoise3_vjp(gy, masks, F, grid, L=2)
    # masks can differ only where a coefficient sits within FP32 rounding of its threshold
    assert rel_l2(gx, ref) < 1e-4


def test_denoise3_autograd_function(s3):
    import torch
    shape = (48, 48, 48)
    clean, x = s3.synth.noisy_volume(shape, 30.0, 35)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4), batch=1)
    s3.nsst_scalars3(p, seed=6)
    xt = _t(x).requires_grad_(True)
    out = s3.denoise3_diff(xt, p, 30.0)
    loss = ((out - _t(clean)) ** 2).sum()
    # another forward on the plan overwrites its masks; backward must redo its own
    s3.denoise3(_t(np.zeros(shape)), p, 30.0)
    loss.backward()
    s3.denoise3(xt.detach(), p, 30.0)
    ref = s3.denoise3_backward((2 * (out.detach() - _t(clean))), p)
    assert torch.equal(xt.grad, ref)
