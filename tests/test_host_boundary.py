"""C-ABI boundary checks that need no GPU: the library loads, exports every
declared symbol, builds the FP64 filter bank exactly like the oracle, and
rejects bad arguments with the documented status codes."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import DCOMP, DSIZE, ROOT
from oracle import nsst2d


def _declared_symbols():
    text = open(os.path.join(ROOT, 'include', 'nsst.h')).read()
    text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
    return sorted(set(re.findall(r'\b(nsst_\w+)\s*\(', text)))


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    names = _declared_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header(built_lib):
    from shearcuda_gb300 import _lib
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(_declared_symbols()) <= bound


@pytest.mark.parametrize('fname', ['maxflat', '9-7', 'pyr', 'pyrexc'])
def test_pyramid_filters_match_oracle(built_lib, fname):
    import shearcuda_gb300 as sc
    for a, b in zip(sc.pyramid_filters(fname), nsst2d.atrousfilters(fname)):
        np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize('n1,level', [(32, 3), (16, 4), (8, 2), (32, 4)])
def test_meyer_filters_match_oracle(built_lib, n1, level):
    import shearcuda_gb300 as sc
    np.testing.assert_allclose(sc.shearing_filters(n1, level), nsst2d.shearing_filters_Myer(n1, level),
                               rtol=0, atol=1e-15)


@pytest.mark.parametrize('HW', [(256, 256), (256, 384), (384, 512)])
def test_level_spectra_match_oracle(built_lib, HW):
    import shearcuda_gb300 as sc
    H, W = HW
    for lev, (c, s) in enumerate(zip(DCOMP[:2] + DCOMP[3:], DSIZE[:2] + DSIZE[3:])):
        got = sc.level_spectra(s, c, H, W)
        ref = nsst2d.shear_spectra(H, W, [c], [s])[0][:, :, :W // 2 + 1]
        assert np.abs(got - ref).max() < 1e-13


# Sizes that are not powers of two put Meyer-grid coordinates on rounding
# boundaries: the host build must not fuse multiply-adds (aarch64 gcc does by
# default), or the filter bank differs between machines.
HOST_SPECTRA_CASES = [(48, 4), (80, 3), (80, 4), (40, 2)]


def _check_host_spectra(n1, level):
    import shearcuda_gb300 as sc
    np.testing.assert_allclose(sc.shearing_filters(n1, level), nsst2d.shearing_filters_Myer(n1, level),
                               rtol=0, atol=1e-15)
    got = sc.level_spectra(n1, level, 256, 256)
    ref = nsst2d.shear_spectra(256, 256, [level], [n1])[0][:, :, :129]
    assert np.abs(got - ref).max() < 1e-13


@pytest.mark.parametrize('n1,level', HOST_SPECTRA_CASES)
def test_host_filters_non_power_of_two_sizes(built_lib, n1, level):
    _check_host_spectra(n1, level)


@pytest.mark.gpu
@pytest.mark.parametrize('n1,level', HOST_SPECTRA_CASES)
def test_host_filters_non_power_of_two_sizes_on_gpu_machine(built_lib, n1, level):
    # the same host-only check, run with the GPU suite so that the GPU
    # machine's own build of the host code is compared with the oracle
    _check_host_spectra(n1, level)


def test_status_codes_without_gpu(built_lib):
    import shearcuda_gb300 as sc
    from shearcuda_gb300._lib import NsstError
    with pytest.raises(NsstError) as e:
        sc.ShearPlan([3, 3], [32, 32], 300, 300)  # not a supported FFT length
    assert e.value.status == 2
    with pytest.raises(NsstError) as e:
        sc.ShearPlan([9], [32], 256, 256)  # dcomp out of range
    assert e.value.status == 1
    with pytest.raises(NsstError) as e:
        sc.ShearPlan([3], [31], 256, 256)  # odd dsize
    assert e.value.status == 1
    with pytest.raises(NsstError) as e:
        sc.ShearPlan([3, 3], [32, 32], 256, 256, lpfilt='nope')
    assert e.value.status in (1, 4)  # invalid name (4 only if no device at all)
    with pytest.raises(NsstError):
        sc.level_spectra(31, 3, 256, 256)
    # pyramid modes: AUTO (0), DIRECT (1) and SPECTRAL (2) exist, others are
    # rejected by the configuration check before any device call
    with pytest.raises(NsstError) as e:
        sc.ShearPlan([3, 3], [32, 32], 256, 256, pyramid=3)
    assert e.value.status == 1 and 'pyramid mode' in str(e.value)
    assert (sc.PYRAMID_AUTO, sc.PYRAMID_DIRECT, sc.PYRAMID_SPECTRAL) == (0, 1, 2)


def test_noalloc_rejects_overlapping_buffers_before_any_device_call(built_lib):
    # host-side argument checks: no GPU is touched (fake device addresses)
    import ctypes
    from shearcuda_gb300._lib import lib
    H, W, L = 256, 256, 4
    plane = H * W * 4
    y = 1 << 32
    for x in (y, y + plane, y + L * plane, y - plane + 4):  # inside y or straddling its start
        st = lib().nsst_atrousdec_noalloc(ctypes.c_void_p(x), ctypes.c_void_p(y), H, W, L, b'maxflat', None)
        assert st == 1, x
        assert b'overlaps' in lib().nsst_last_error()


def test_missing_library_fails_loudly(built_lib, monkeypatch, tmp_path):
    # no fallback: without libnsst.so every entry point raises, the host-only
    # ones included (nothing routes to the oracle or to PyTorch instead)
    import shearcuda_gb300 as sc
    from shearcuda_gb300 import _lib
    monkeypatch.setattr(_lib, '_lib', None)
    monkeypatch.setattr(_lib, 'LIB_PATH', str(tmp_path / 'libnsst.so'))
    with pytest.raises(OSError, match='not built'):
        sc.MakeONFilter('Haar')
    with pytest.raises(OSError, match='not built'):
        sc.launch_count()
    with pytest.raises(OSError, match='not built'):
        sc.prepare_shearing_filters_cuda(DCOMP, DSIZE, 256, 256)
