"""Batched and uneven-size paths: every image of a batch must come out
bit-identical to the same image denoised alone (same kernels, same
arithmetic), with and without CUDA-graph replay."""
import numpy as np
import pytest
import torch

from conftest import DCOMP, DSIZE, K_DEMO, rel_l2
from oracle import nsst2d

pytestmark = pytest.mark.gpu


def _imgs(shape, n, seed0, cuda):
    from shearcuda_gb300.synth import noisy_image
    out = []
    for i in range(n):
        _, noisy = noisy_image(shape[0], shape[1], 20.0, seed0 + i)
        out.append(torch.tensor(noisy.astype(np.float32), device=cuda))
    return out


def test_batch_equals_single(built_lib, cuda):
    import shearcuda_gb300 as sc
    single = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, 256, 256)
    batch = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, 256, 256, batch=4)
    scal = sc.nsst_scalars(single, 100)
    batch.set_scalars(scal)
    xs = _imgs((256, 256), 3, 10, cuda)
    sig = [12.0, 20.0, 35.0]
    outs = sc.nsst_denoise_batch(xs, batch, sig, K_DEMO, scal)
    for x, o, s in zip(xs, outs, sig):
        ref = sc.nsst_denoise(x, single, s, K_DEMO, scal)
        np.testing.assert_array_equal(o.cpu().numpy(), ref.cpu().numpy())
    # graph replay gives the same bits, twice in a row
    batch.use_graphs(True)
    for _ in range(2):
        outs2 = sc.nsst_denoise_batch(xs, batch, sig, K_DEMO, None)
        for o, o2 in zip(outs, outs2):
            np.testing.assert_array_equal(o.cpu().numpy(), o2.cpu().numpy())
    # a smaller second call on the same plan (n < capacity)
    o1 = sc.nsst_denoise_batch(xs[:1], batch, sig[:1], K_DEMO, None)[0]
    np.testing.assert_array_equal(o1.cpu().numpy(), outs[0].cpu().numpy())


@pytest.mark.parametrize('HW,B,n', [((512, 512), 8, 5), ((768, 1024), 4, 3), ((384, 512), 6, 4)])
def test_level_kernels_partial_batch_equal_single(built_lib, cuda, HW, B, n):
    # the TMA column kernels run, per level, chunks of column groups across
    # all B items of the plan (the inactive items' CTAs leave at once); with
    # the level analysis forced, every image of an n < B call equals itself
    # denoised alone through a one-image plan running the same kernels
    import shearcuda_gb300 as sc
    H, W = HW
    batch = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, batch=B)
    single = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W)
    scal = sc.nsst_scalars(single, 100)
    batch.set_scalars(scal)
    name = 'split/level-tma/rows8/synthesis-regs'
    for p, m in ((batch, n), (single, 1)):
        p.select_directional(m, p.directional_candidates().index(name))
    xs = _imgs(HW, n, 40, cuda)
    sig = [12.0, 20.0, 35.0, 25.0, 18.0][:n]
    outs = sc.nsst_denoise_batch(xs, batch, sig, K_DEMO, scal)
    for x, o, s in zip(xs, outs, sig):
        ref = sc.nsst_denoise(x, single, s, K_DEMO, scal)
        assert torch.equal(o, ref)
    batch.check_device()


def test_uneven_multi_batch(built_lib, cuda):
    import shearcuda_gb300 as sc
    shapes = [(256, 256), (384, 512), (256, 384)]
    plans, singles = [], []
    for (H, W) in shapes:
        p = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, batch=3)
        s1 = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W)
        scal = sc.nsst_scalars(s1, 100)
        p.set_scalars(scal)
        s1.set_scalars(scal)
        plans.append(p)
        singles.append(s1)
    m = sc.MultiBatch(plans)
    xs, sig, owner = [], [], []
    rng = np.random.default_rng(0)
    for i in range(7):
        k = int(rng.integers(0, 3))
        if sum(1 for o in owner if o == k) >= 3:
            k = (k + 1) % 3
        owner.append(k)
        xs += _imgs(shapes[k], 1, 50 + i, cuda)
        sig.append(float(rng.uniform(10, 40)))
    for rep in range(2):
        outs = m.denoise(xs, sig, K_DEMO)
        for x, o, s, k in zip(xs, outs, sig, owner):
            ref = sc.nsst_denoise(x, singles[k], s, K_DEMO, None)
            np.testing.assert_array_equal(o.cpu().numpy(), ref.cpu().numpy())


def test_uneven_batch_matches_oracle(built_lib, cuda):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import uneven_batch
    items = uneven_batch(4, seed=3, sizes=((256, 256), (384, 512)))
    plans = {}
    for clean, noisy, sigma in items:
        key = noisy.shape
        if key not in plans:
            plans[key] = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, key[0], key[1], batch=4)
    order = list(plans)
    sf, scal = {}, {}
    for key in order:
        sf[key] = nsst2d.shear_spectra(key[0], key[1], DCOMP, DSIZE)
        sc_ = nsst2d.nsst_scalars(key[0], key[1], sf[key], seed=100, nthreads=8)
        scal[key] = sc_
        plans[key].set_scalars(np.concatenate([[sc_[0]]] + [np.asarray(v) for v in sc_[1:]]))
    m = sc.MultiBatch([plans[k] for k in order])
    xs = [torch.tensor(n.astype(np.float32), device=cuda) for _, n, _ in items]
    outs = m.denoise(xs, [s for _, _, s in items], K_DEMO)
    for (clean, noisy, sigma), o in zip(items, outs):
        key = noisy.shape
        ref, _ = nsst2d.denoise(noisy.astype(np.float32).astype(np.float64), sigma, K_DEMO, scal[key], DCOMP, DSIZE,
                                shear_f=sf[key], nthreads=8)
        g = o.cpu().numpy().astype(np.float64)
        assert abs(nsst2d.psnr(clean, g) - nsst2d.psnr(clean, ref)) <= 0.01
