"""3-D parity at the volume sizes of the V3 workload (128^3 and 192^3, three
levels, 72 directional bands), against the FP64 oracle (oracle/nsst3d.py):

  * on the GPU path's own grid (edge replication to 144^3 / 192^3): every
    directional band relative L2 <= 1e-5, the denoised volume |dPSNR| <= 0.01 dB;
  * with NSST3_GRID_MARSHAL, on the reference's own padding (MarshalData.m:
    128 -> 132, 192 -> 204, oracle.nsst3d.marshal_data): the same bounds,
    through the radix-11 and radix-17 volume transforms, and the adjoint;
  * the fast grid against the reference's padding: the pyramid is periodic,
    so the planes added at the far edges differ and the results near those
    edges differ with them; the bounds below are the measured differences.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

T3 = (3.3, 3.0, 3.0)
SIGMA = 30.0


def _t(a):
    import torch
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float32, device='cuda')


def _np(t):
    return t.detach().cpu().numpy().astype(np.float64)


@pytest.fixture(scope='module')
def filters3():
    from oracle import nsst3d
    return nsst3d.meyer_filters_3d([2, 2, 4])


@pytest.mark.parametrize('n,seed', [(128, 7), (192, 8)])
def test_v3_sizes_match_oracle(built_lib, cuda, filters3, n, seed):
    import torch
    import shearcuda_gb300 as s3
    from oracle import nsst3d
    shape = (n, n, n)
    clean, x = s3.synth.noisy_volume(shape, SIGMA, seed)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4))
    assert p.grid == (nsst3d.pad_size(n),) * 3
    scal = s3.nsst_scalars3(p, seed=9)
    xg = _t(x)
    flat, subs = s3.do_pyr_dec(xg, p)
    xp = nsst3d.pad_volume(x.astype(np.float32).astype(np.float64))
    bp = nsst3d.pyr_dec(xp, 3, 1.5)
    for l in range(4):
        assert rel_l2(_np(subs[l][0]), bp[l]) <= 1e-5, l
    bands = nsst3d.band_list(filters3)
    for l in range(3):
        got = s3.sh_dec(flat, l, p)[0]
        idx = [b for b, bd in enumerate(bands) if bd[1] == l]
        ref = nsst3d.convnfft_same_level(_np(subs[l][0]), [bands[b][4] for b in idx])
        for k, r in enumerate(ref):
            assert rel_l2(_np(got[k]), r) <= 1e-5, (l, k)
        del got
        torch.cuda.empty_cache()
    out = _np(s3.denoise3(xg, p, SIGMA, T3))
    ref = nsst3d.denoise3(xp, filters3, SIGMA, T3, scal, fast=True)[:n, :n, :n]
    d = abs(nsst3d.psnr3(clean, out) - nsst3d.psnr3(clean, ref))
    assert d <= 0.01, d
    assert nsst3d.psnr3(clean, out) > nsst3d.psnr3(clean, x) + 3.0
    del p
    torch.cuda.empty_cache()


# measured on a GB300: 128^3 -0.088 dB, rel-L2 1.85e-2 (the reference's grid
# 132^3 vs 144^3 here); 192^3 +0.361 dB, rel-L2 4.63e-2 (204^3 vs 192^3: the
# reference adds 12 replicated planes to a volume that needs none)
@pytest.mark.parametrize('n,seed,max_dpsnr,max_rel', [(128, 7, 0.15, 0.03), (192, 8, 0.5, 0.07)])
def test_v3_against_reference_padding(built_lib, cuda, filters3, n, seed, max_dpsnr, max_rel):
    import torch
    import shearcuda_gb300 as s3
    from oracle import nsst3d
    shape = (n, n, n)
    clean, x = s3.synth.noisy_volume(shape, SIGMA, seed)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4))
    scal = s3.nsst_scalars3(p, seed=9)
    out = _np(s3.denoise3(_t(x), p, SIGMA, T3))
    xm = nsst3d.marshal_data(x.astype(np.float32).astype(np.float64), 3)
    assert xm.shape == ((n + 12 - n % 12),) * 3  # 132 / 204
    ref = nsst3d.denoise3(xm, filters3, SIGMA, T3, scal, fast=True)[:n, :n, :n]
    p_gpu, p_ref = nsst3d.psnr3(clean, out), nsst3d.psnr3(clean, ref)
    rel = rel_l2(out, ref)
    print('V3 %d^3 vs MarshalData grid %d^3: PSNR %.4f / %.4f dB (diff %.4f), rel-L2 %.3e'
          % (n, xm.shape[0], p_gpu, p_ref, p_gpu - p_ref, rel))
    assert abs(p_gpu - p_ref) <= max_dpsnr
    assert rel <= max_rel
    del p
    torch.cuda.empty_cache()


@pytest.mark.parametrize('n,seed', [(128, 7), (192, 8)])
def test_v3_marshal_grid_matches_reference_padding(built_lib, cuda, filters3, n, seed):
    # NSST3_GRID_MARSHAL pads as MarshalData.m does (128 -> 132, 192 -> 204):
    # the reference's any-size demo, reproduced to FP32 rounding
    import torch
    import shearcuda_gb300 as s3
    from oracle import nsst3d
    shape = (n, n, n)
    clean, x = s3.synth.noisy_volume(shape, SIGMA, seed)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4), grid='marshal')
    xm = nsst3d.marshal_data(x.astype(np.float32).astype(np.float64), 3)
    assert p.grid == xm.shape
    scal = s3.nsst_scalars3(p, seed=9)
    xg = _t(x)
    flat, subs = s3.do_pyr_dec(xg, p)
    bp = nsst3d.pyr_dec(xm, 3, 1.5)
    for l in range(4):
        assert subs[l].shape[1:] == bp[l].shape
        assert rel_l2(_np(subs[l][0]), bp[l]) <= 1e-5, l
    bands = nsst3d.band_list(filters3)
    for l in range(3):
        got = s3.sh_dec(flat, l, p)[0]
        idx = [b for b, bd in enumerate(bands) if bd[1] == l]
        ref = nsst3d.convnfft_same_level(_np(subs[l][0]), [bands[b][4] for b in idx])
        for k, r in enumerate(ref):
            assert rel_l2(_np(got[k]), r) <= 1e-5, (l, k)
        del got
        torch.cuda.empty_cache()
    rec = _np(s3.do_pyr_rec(flat, p)[0])
    assert rel_l2(rec, x) <= 1e-5  # perfect reconstruction through the odd-length transforms
    out = _np(s3.denoise3(xg, p, SIGMA, T3))
    ref = nsst3d.denoise3(xm, filters3, SIGMA, T3, scal, fast=True)[:n, :n, :n]
    d = abs(nsst3d.psnr3(clean, out) - nsst3d.psnr3(clean, ref))
    assert d <= 0.01, d
    del p
    torch.cuda.empty_cache()


def test_v3_marshal_grid_adjoint_dot_product(built_lib, cuda):
    # 132^3: the level boxes 132 and 44 are not multiples of the 8-sequence
    # group, so the keep bits use a padded row pitch
    import torch
    import shearcuda_gb300 as s3
    shape = (128, 128, 128)
    _, x = s3.synth.noisy_volume(shape, SIGMA, 41)
    p = s3.VolumePlan(*shape, num_dirs=(2, 2, 4), grid='marshal')
    s3.nsst_scalars3(p, seed=2)
    p.enable_grad()
    xb = _t(x)[None]
    out = s3.denoise3(xb, p, [SIGMA])
    for gy in (out + 10.0 * torch.randn_like(out), torch.randn_like(out)):
        gx = s3.denoise3_backward(gy, p)
        lhs = float(np.vdot(_np(gy[0]).ravel(), _np(out[0]).ravel()))
        rhs = float(np.vdot(_np(gx[0]).ravel(), _np(xb[0]).ravel()))
        scale = np.linalg.norm(_np(gy[0])) * np.linalg.norm(_np(out[0]))
        assert abs(lhs - rhs) <= 1e-6 * scale, (lhs, rhs, scale)
    del p
    torch.cuda.empty_cache()
