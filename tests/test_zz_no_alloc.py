"""The à trous entry point that allocates nothing (nsst_atrousdec_noalloc).

It serves callers that cannot call cudaMalloc (for example a MEX host whose
GPU array runtime owns the device memory, or a loop under a fixed memory
budget): its one scratch image lives in a static device array of the library.
The tests call it through the C ABI twice in a row, on two different images,
and check each result against the plan-based nsst_atrousdec with the pyramid
tolerance used everywhere else (relative L2 <= 1e-5 per plane), for every
filter set of atrousfilters.m and 1 to 4 levels (odd and even level counts
swap the order in which the lowpass chain alternates between the caller's
plane 0 and the static array), and at 6 levels.  This file is collected last
so that a run stopping at the first failure has already run every other test.
"""
import numpy as np
import pytest
import torch

from conftest import DCOMP, DSIZE, rel_l2

pytestmark = pytest.mark.gpu


def _check_twice(sc, cuda, plan, H, W, L, lpfilt, seeds):
    from shearcuda_gb300.synth import noisy_image
    y = torch.empty((L + 1, H, W), device=cuda, dtype=torch.float32)
    for seed in seeds:  # two calls in a row share the static scratch
        _, noisy = noisy_image(H, W, 20.0, seed)
        x = torch.tensor(noisy.astype(np.float32), device=cuda)
        ref = sc.atrousdec(x, plan).cpu().numpy()
        got = sc.atrousdec_noalloc(x, L, y, lpfilt=lpfilt).cpu().numpy()
        for k in range(L + 1):
            assert rel_l2(got[k], ref[k]) <= 1e-5, (lpfilt, L, seed, k, rel_l2(got[k], ref[k]))


def test_noalloc_atrousdec_matches_plan_path_twice(built_lib, cuda):
    import shearcuda_gb300 as sc
    H, W, L = 512, 384, len(DCOMP)
    plan = sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, H, W)
    _check_twice(sc, cuda, plan, H, W, L, 'maxflat', (11, 12))


@pytest.mark.parametrize('lpfilt', ['maxflat', '9-7', 'pyr', 'pyrexc'])
@pytest.mark.parametrize('L', [1, 2, 3, 4])
def test_noalloc_every_filter_set_and_depth(built_lib, cuda, lpfilt, L):
    import shearcuda_gb300 as sc
    H, W = 256, 384
    plan = sc.prepare_shearing_filters_cuda(DCOMP[:L], DSIZE[:L], H, W, lpfilt=lpfilt)
    _check_twice(sc, cuda, plan, H, W, L, lpfilt, (21, 22))


def test_noalloc_six_levels(built_lib, cuda):
    # 6 levels dilate the 19-tap filter by 32: one reflection needs 609 px
    import shearcuda_gb300 as sc
    H, W, L = 768, 1024, 6
    plan = sc.prepare_shearing_filters_cuda([3, 3, 4, 4, 4, 4], [32, 32, 16, 16, 16, 16], H, W)
    _check_twice(sc, cuda, plan, H, W, L, 'maxflat', (31, 32))


def test_noalloc_rejects_oversized_images(built_lib, cuda):
    import shearcuda_gb300 as sc
    from shearcuda_gb300._lib import NsstError
    x = torch.zeros((2048, 2056), device=cuda, dtype=torch.float32)
    y = torch.zeros((5, 2048, 2056), device=cuda, dtype=torch.float32)
    with pytest.raises(NsstError) as e:
        sc.atrousdec_noalloc(x, 4, y)
    assert e.value.status == 2 and 'scratch limit' in str(e.value)
