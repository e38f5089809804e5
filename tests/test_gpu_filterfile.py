"""Plans built from the reference's filter-bank file (SHFM0002) on the GPU:
a double file of the library's own bank gives the constructed plan's
coefficients bit for bit; a single file stays within the parity tolerance of
the FP64 oracle."""
import numpy as np
import pytest
import torch

from conftest import DCOMP, DSIZE, flat_coeffs, rel_l2
from oracle import nsst2d

pytestmark = pytest.mark.gpu


def test_plan_from_file_matches_constructed_plan(built_lib, cuda, tmp_path):
    import shearcuda_gb300 as sc
    from shearcuda_gb300.synth import noisy_image
    H, W = 256, 384
    _, noisy = noisy_image(H, W, 20.0, 21)
    x = torch.tensor(noisy.astype(np.float32), device=cuda)
    ref_plan = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W)
    c_ref = sc.shear_trans_cuda(x, 'maxflat', ref_plan)
    path = sc.save_shearing_filters(DSIZE, DCOMP, 'double', path=str(tmp_path / 'bank_d.bin'))
    fp = sc.ShearPlan.from_file(path, H, W)
    assert fp.nbands == ref_plan.nbands and fp.dcomp == DCOMP and fp.dsize == DSIZE
    assert torch.equal(sc.shear_trans_cuda(x, 'maxflat', fp), c_ref)
    np.testing.assert_array_equal(fp.level_spectra(2), ref_plan.level_spectra(2))

    path32 = sc.save_shearing_filters(DSIZE, DCOMP, 'single', path=str(tmp_path / 'bank_s.bin'))
    fs = sc.ShearPlan.from_file(path32, H, W)
    c32 = sc.shear_trans_cuda(x, 'maxflat', fs).cpu().numpy().astype(np.float64)
    dst, _ = nsst2d.nsst_dec2(noisy.astype(np.float32).astype(np.float64), DCOMP, DSIZE,
                              shear_f=nsst2d.shear_spectra(H, W, DCOMP, DSIZE))
    assert rel_l2(c32, flat_coeffs(dst)) <= 1e-5
    # round trip through the file's plan
    rec = sc.inverse_shear_cuda(torch.tensor(c32, dtype=torch.float32, device=cuda), 'maxflat', fs)
    assert rel_l2(rec.cpu().numpy(), noisy) <= 1e-5


def test_unknown_pyramid_mode_is_rejected(built_lib, cuda):
    import shearcuda_gb300 as sc
    with pytest.raises(sc.NsstError):
        sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, 256, 256, pyramid=7)
