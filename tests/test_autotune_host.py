"""Host side of the autotuner: the evaluation of direct (spatial) directional
convolution, checked against an FP64 NumPy computation on the oracle's own
normalised spectra (nsst_dec2.m:47-57).  No GPU."""
import numpy as np
import pytest

from conftest import DCOMP, DSIZE
from oracle import nsst2d


def _numpy_margins(H, W, dcomp, dsize, tol):
    """Per level: the smallest margin m such that every band's effective filter
    ifft2(W_k / d) has relative L2 energy <= tol outside the square window
    [-m, dsize + m)^2 (circular); None if none below the image size."""
    sf = nsst2d.shear_spectra(H, W, dcomp, dsize)
    out = []
    for l, S in enumerate(sf):
        ds = dsize[l]
        mmax = (min(H, W) - ds) // 2 - 1
        need = 0
        for k in range(S.shape[0]):
            e = np.real(np.fft.ifft2(S[k]))
            E = e ** 2

            def dist(a, n):
                return np.where(a < ds, 0, np.minimum(a - ds + 1, n - a))
            D = np.maximum(dist(np.arange(H), H)[:, None], dist(np.arange(W), W)[None, :])
            ring = np.bincount(D.ravel(), weights=E.ravel(), minlength=max(H, W))
            rel = np.sqrt(np.maximum(E.sum() - np.cumsum(ring), 0) / E.sum())[:mmax + 1]
            ok = np.nonzero(rel <= tol)[0]
            if ok.size == 0:
                need = None
                break
            need = max(need, int(ok[0]))
        out.append(need)
    return out


@pytest.mark.parametrize('HW', [(256, 256), (256, 384)])
def test_direct_support_matches_numpy(built_lib, HW):
    import shearcuda_gb300 as sc
    H, W = HW
    sup, err = sc.direct_support(DCOMP, DSIZE, H, W, 1e-5)
    ref = _numpy_margins(H, W, DCOMP, DSIZE, 1e-5)
    for l in range(len(DCOMP)):
        if ref[l] is None:
            assert sup[l] == 0
        else:
            assert sup[l] == DSIZE[l] + 2 * ref[l], (l, sup[l], ref[l])
            assert err[l] <= 1e-5


def test_direct_support_rejects_when_no_window_fits(built_lib):
    import shearcuda_gb300 as sc
    # at 128 x 128 the 32-px filters' effective support (204 px at 1e-5)
    # exceeds the image: direct convolution cannot be proven
    sup, err = sc.direct_support([3, 3], [32, 32], 128, 128, 1e-5)
    assert sup == [0, 0]
    assert min(err) > 1e-5
    # a loose tolerance admits a window
    sup2, err2 = sc.direct_support([3, 3], [32, 32], 128, 128, 1e-2)
    assert all(0 < s < 128 for s in sup2) and max(err2) <= 1e-2


def test_direct_support_argument_checks(built_lib):
    import shearcuda_gb300 as sc
    with pytest.raises(sc.NsstError):
        sc.direct_support(DCOMP, DSIZE, 256, 256, 0.0)
    with pytest.raises(sc.NsstError):
        sc.direct_support(DCOMP, DSIZE, 100, 256, 1e-5)
