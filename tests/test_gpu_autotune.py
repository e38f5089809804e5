"""The autotuner on a GPU: every directional-stage candidate it can select
passes parity, and it keeps the fastest one it measured.

Tolerances as in test_gpu_fused.py: against the FP64 oracle |dPSNR| <= 0.01 dB
(hard) and relative L2 <= 1e-5 (soft); candidates against each other
relative L2 <= 1e-5 (soft) / 1e-4 (hard)."""
import numpy as np
import pytest
import torch

from conftest import DCOMP, DSIZE, K_DEMO, flat_scalars, rel_l2
from oracle import nsst2d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize('HW,n', [((256, 256), 4), ((512, 512), 2), ((384, 512), 2)])
def test_autotune_picks_fastest_and_every_candidate_is_exact(built_lib, cuda, HW, n):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    H, W = HW
    shear = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, batch=n)
    sf = nsst2d.shear_spectra(H, W, DCOMP, DSIZE)
    scal = nsst2d.nsst_scalars(H, W, sf, seed=100, nthreads=8)
    flat = flat_scalars(scal)
    shear.set_scalars(flat)
    res = shear.autotune(n)
    names = shear.directional_candidates()
    assert [c[0] for c in res['candidates']] == names
    assert len(names) >= 4
    ms = [c[1] for c in res['candidates']]
    assert all(m > 0 for m in ms)
    assert res['chosen'] == names[int(np.argmin(ms))]
    assert shear.directional(n) == ('fused' if res['chosen'].startswith('fused') else 'split')
    # direct convolution: proven windows, and the bound far above the FFT path
    assert all(s > 0 for s in res['direct_support'])
    assert max(res['direct_err']) <= 1e-5
    assert res['direct_bound_ms'] > min(ms) and not res['direct_wins']

    clean, noisy = noisy_image(H, W, 20.0, 0)
    xs = [torch.tensor(noisy.astype(np.float32), device=cuda)]
    for s in range(1, n):
        xs.append(torch.tensor(noisy_image(H, W, 20.0, s)[1].astype(np.float32), device=cuda))
    ref_soft, _ = nsst2d.denoise(noisy.astype(np.float32).astype(np.float64), 20.0, K_DEMO, scal, DCOMP, DSIZE,
                                 mode='soft', shear_f=sf, nthreads=8)
    ref_hard, _ = nsst2d.denoise(noisy.astype(np.float32).astype(np.float64), 20.0, K_DEMO, scal, DCOMP, DSIZE,
                                 mode='hard', shear_f=sf, nthreads=8)
    first = {}
    for i, name in enumerate(names):
        shear.select_directional(n, i)
        for mode, ref in ((1, ref_soft), (0, ref_hard)):
            outs = [o.cpu().numpy() for o in sc.nsst_denoise_batch(xs, shear, [20.0] * n, K_DEMO, flat, mode=mode)]
            out0 = outs[0].astype(np.float64)
            if mode == 1:
                assert rel_l2(out0, ref) <= 1e-5, (name, rel_l2(out0, ref))
            assert abs(nsst2d.psnr(clean, out0) - nsst2d.psnr(clean, ref)) <= 0.01, name
            if mode in first:
                for o, f in zip(outs, first[mode]):
                    assert rel_l2(o, f) <= (1e-5 if mode == 1 else 1e-4), (name, rel_l2(o, f))
            else:
                first[mode] = outs
    shear.check_device()
    shear.select_directional(n, -1)


@pytest.mark.parametrize('HW,n', [((512, 512), 3), ((768, 1024), 2), ((256, 384), 3)])
def test_tma_staging_is_bit_identical_to_cp_async(built_lib, cuda, HW, n):
    # the TMA-staged column kernels change how a column group reaches shared
    # memory, not the arithmetic: each "-tma" candidate equals its cp.async
    # twin bit for bit (hard and soft thresholds); so does the synthesis with
    # the band sum in registers ("-regs") against the one summing in shared
    # memory
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    H, W = HW
    shear = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W, batch=n)
    sc.nsst_scalars(shear, seed=100)
    names = shear.directional_candidates()
    pairs = [(names.index(t), names.index(t.replace('-tma', ''))) for t in names if t.endswith('-tma')]
    pairs += [(names.index(t), names.index(t.replace('synthesis-regs', 'synthesis-tma'))) for t in names
              if t.endswith('synthesis-regs')]
    assert len(pairs) >= 12
    xs = [torch.tensor(noisy_image(H, W, 20.0, s)[1].astype(np.float32), device=cuda) for s in range(n)]
    for it, ic in pairs:
        for mode in (0, 1):
            got = []
            for i in (it, ic):
                shear.select_directional(n, i)
                got.append([o.cpu() for o in sc.nsst_denoise_batch(xs, shear, [20.0] * n, K_DEMO, None, mode=mode)])
            for a, b in zip(*got):
                assert torch.equal(a, b), (names[it], names[ic], mode)
    shear.check_device()
    shear.select_directional(n, -1)
