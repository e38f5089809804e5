"""Parity at the image sizes the workloads use above 512^2, against the FP64
oracle (nsst_dec2 / nsst_rec2 with the reference's atrousc loop restated):

  * P1k / P2k and the batch sizes 768 x 1024 and 1024^2: per-band coefficient
    relative L2 <= 1e-5, denoised |dPSNR| <= 0.01 dB (hard threshold) and
    relative L2 <= 1e-5 (soft threshold);
  * the uneven batch with its two largest sizes through one multi-plan graph;
  * the differentiable configuration at its own size (512^2): gradients for
    the image and the 49 thresholds against the FP64 oracle gradient.

The reference's GPU operators stop at 1024 (shear_trans_cuda.cpp:114-117);
these sizes are the ones the GB300 path adds.
"""
import os

import numpy as np
import pytest
import torch

from conftest import DCOMP, DSIZE, K_DEMO, flat_coeffs, flat_scalars, rel_l2
from oracle import nsst2d

pytestmark = pytest.mark.gpu
NT = os.cpu_count() or 8


@pytest.mark.parametrize('HW,seed', [((768, 1024), 3), ((1024, 1024), 1), ((2048, 2048), 2)])
def test_large_sizes_match_oracle(built_lib, cuda, HW, seed):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    H, W = HW
    clean, noisy = noisy_image(H, W, 20.0, seed)
    noisy32 = noisy.astype(np.float32)
    x64 = noisy32.astype(np.float64)
    shear = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W)
    # both sides use the same FP64 band scalars (the GPU's Monte-Carlo estimate)
    flat = sc.nsst_scalars(shear, 100 + H // 256)
    scal = [flat[0]]
    at = 1
    for d in DCOMP:
        scal.append(np.asarray(flat[at:at + (1 << d)]))
        at += 1 << d
    sf = nsst2d.shear_spectra(H, W, DCOMP, DSIZE)
    x = torch.tensor(noisy32, device=cuda)
    c = sc.shear_trans_cuda(x, 'maxflat', shear).cpu().numpy()
    dst, _ = nsst2d.nsst_dec2(x64, DCOMP, DSIZE, shear_f=sf, nthreads=NT)
    ref = flat_coeffs(dst)
    del dst
    worst = max(rel_l2(c[b], ref[b]) for b in range(ref.shape[0]))
    assert worst <= 1e-5, worst
    del c, ref
    modes = ['hard'] if H >= 2048 else ['hard', 'soft']
    for mode in modes:
        out = sc.nsst_denoise(x, shear, 20.0, K_DEMO, flat, mode=0 if mode == 'hard' else 1)
        out = out.cpu().numpy().astype(np.float64)
        r, _ = nsst2d.denoise(x64, 20.0, K_DEMO, scal, DCOMP, DSIZE, mode=mode, shear_f=sf, nthreads=NT)
        d = abs(nsst2d.psnr(clean, out) - nsst2d.psnr(clean, r))
        assert d <= 0.01, (mode, d)
        if mode == 'soft':
            assert rel_l2(out, r) <= 1e-5, rel_l2(out, r)
    del shear
    torch.cuda.empty_cache()


def test_uneven_batch_large_sizes_match_oracle(built_lib, cuda):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    sizes = [(768, 1024), (1024, 1024), (512, 512)]
    plans, sf, scal, items = [], {}, {}, []
    for (H, W) in sizes:
        p = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, batch=2)
        flat = sc.nsst_scalars(p, 200 + H // 256)
        plans.append(p)
        scal[(H, W)] = flat
    rng = np.random.default_rng(3)
    for i, (H, W) in enumerate([sizes[0], sizes[1], sizes[0], sizes[2], sizes[1]]):
        sigma = float(rng.uniform(10, 40))
        clean, noisy = noisy_image(H, W, sigma, 300 + i)
        items.append((clean, noisy.astype(np.float32), sigma))
    m = sc.MultiBatch(plans)
    outs = m.denoise([torch.tensor(n, device=cuda) for _, n, _ in items], [s for _, _, s in items], K_DEMO)
    for (clean, noisy32, sigma), o in zip(items, outs):
        key = noisy32.shape
        if key not in sf:
            sf[key] = nsst2d.shear_spectra(key[0], key[1], DCOMP, DSIZE)
        flat = scal[key]
        parts = [flat[0]]
        at = 1
        for d in DCOMP:
            parts.append(np.asarray(flat[at:at + (1 << d)]))
            at += 1 << d
        ref, _ = nsst2d.denoise(noisy32.astype(np.float64), sigma, K_DEMO, parts, DCOMP, DSIZE, shear_f=sf[key],
                                nthreads=NT)
        g = o.cpu().numpy().astype(np.float64)
        assert abs(nsst2d.psnr(clean, g) - nsst2d.psnr(clean, ref)) <= 0.01


def test_d16_size_gradients_match_oracle(built_lib, cuda):
    # the differentiable configuration's image size (16 x 512^2 in the bench):
    # two 512^2 images, soft thresholds at 3 sigma band_scalar
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    H = W = 512
    plan = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, batch=2)
    sc.autograd.enable_grad(plan)
    sf = nsst2d.shear_spectra(H, W, DCOMP, DSIZE)
    flat = sc.nsst_scalars(plan, 104)
    tau_flat = (3.0 * 20.0 * np.asarray(flat)).astype(np.float32)
    imgs = [noisy_image(H, W, 20.0, 4 + i) for i in range(2)]
    x = torch.tensor(np.stack([n for _, n in imgs]).astype(np.float32), device=cuda, requires_grad=True)
    tau = torch.tensor(tau_flat, device=cuda, requires_grad=True)
    clean = np.stack([c for c, _ in imgs])
    out = sc.nsst_denoise_diff(x, tau, plan, mode=1)
    loss = torch.sum((out.double() - torch.tensor(clean, device=cuda)) ** 2)
    loss.backward()
    parts = [np.float64(tau_flat[0])]
    at = 1
    for d in DCOMP:
        parts.append(tau_flat[at:at + (1 << d)].astype(np.float64))
        at += 1 << d
    gt_ref = np.zeros_like(tau_flat, dtype=np.float64)
    l_ref = 0.0
    for i in range(2):
        li, gx_ref, gt_i = nsst2d.denoise_tau_grad(x.detach()[i].cpu().numpy().astype(np.float64), parts, clean[i],
                                                   sf, mode='soft', nthreads=NT)
        l_ref += li
        gx = x.grad[i].cpu().numpy().astype(np.float64)
        assert rel_l2(gx, gx_ref) <= 1e-4, rel_l2(gx, gx_ref)
        gt_ref += flat_scalars(gt_i)
    assert abs(float(loss.detach()) - l_ref) <= 1e-4 * l_ref
    assert rel_l2(tau.grad.cpu().numpy().astype(np.float64), gt_ref) <= 1e-4
