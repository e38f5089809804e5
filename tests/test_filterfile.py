"""The reference's shearing-filter bank file (SHFM0002,
save_shearing_filters.m:46-84 / shearconfig.cpp:26-78): the library's writer
and reader against the oracle's restatement of both, byte for byte, on CPU."""
import ctypes
import os

import numpy as np
import pytest

from conftest import DCOMP, DSIZE
from oracle import nsst2d, shfm


@pytest.fixture
def sc(built_lib):
    import shearcuda_gb300
    return shearcuda_gb300


def _bank(dcomp=DCOMP, dsize=DSIZE, fname='maxflat'):
    shear = [np.stack(nsst2d.shearing_filters_Myer(n, c)) for c, n in zip(dcomp, dsize)]
    return shear, list(nsst2d.atrousfilters(fname))


@pytest.mark.parametrize('data_type', ['single', 'double'])
def test_written_file_matches_oracle(sc, tmp_path, data_type):
    # same layout and length as the oracle's writer; values equal up to the
    # last bit of the two FP64 filter constructions (different FFTs) and, for
    # single, one FP32 rounding
    mine = sc.save_shearing_filters(DSIZE, DCOMP, data_type, path=str(tmp_path / 'mine.bin'))
    ref = str(tmp_path / 'ref.bin')
    shear, atrous = _bank()
    shfm.shfm_write(ref, shear, atrous, data_type)
    assert os.path.getsize(mine) == os.path.getsize(ref)
    assert open(mine, 'rb').read()[:16] == open(ref, 'rb').read()[:16]
    dt_m, sh_m, at_m = shfm.shfm_read(mine)
    dt_r, sh_r, at_r = shfm.shfm_read(ref)
    assert dt_m == dt_r == data_type
    for a, b in zip(sh_m, sh_r):
        assert a.shape == b.shape
        tol = 1e-16 if data_type == 'double' else 2.0 ** -23 * np.abs(b).max()
        assert np.abs(a - b).max() <= tol
    for a, b in zip(at_m, at_r):
        assert np.array_equal(a, b)


def test_default_name_is_the_references(sc, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    p = sc.save_shearing_filters([32, 32, 16, 16], [3, 3, 4, 4], 'single')
    assert p == 'shearFilters_3_3_4_4_single.bin' and os.path.exists(p)


def test_reader_orientation_and_types(sc, tmp_path):
    # non-symmetric filters written the way MATLAB writes them (column-major)
    rng = np.random.default_rng(1)
    shear = [rng.standard_normal((2, 8, 8)), rng.standard_normal((4, 6, 6))]
    atrous = [rng.standard_normal((f, f)) for f in (5, 7, 7, 5)]
    for dt in ('single', 'double'):
        path = str(tmp_path / ('r_%s.bin' % dt))
        shfm.shfm_write(path, shear, atrous, dt)
        got = sc.load_shearing_filters(path)
        dtype_ref, shear_ref, atrous_ref = shfm.shfm_read(path)
        assert got['data_type'] == dt == dtype_ref
        for a, b, c in zip(got['shear'], shear_ref, shear):
            assert np.array_equal(a, b)
            tol = 0 if dt == 'double' else 1e-6 * np.abs(c).max()
            assert np.abs(a - c).max() <= tol
        for a, b in zip(got['atrous'], atrous_ref):
            assert np.array_equal(a, b)


def test_round_trip_of_library_bank(sc, tmp_path):
    p = sc.save_shearing_filters(DSIZE, DCOMP, 'double', path=str(tmp_path / 'd.bin'))
    got = sc.load_shearing_filters(p)
    for a, c, n in zip(got['shear'], DCOMP, DSIZE):
        assert np.array_equal(a, sc.shearing_filters(n, c))
    for a, b in zip(got['atrous'], sc.pyramid_filters('maxflat')):
        assert np.array_equal(a, b)


def test_malformed_files_are_rejected(sc, tmp_path):
    good = sc.save_shearing_filters(DSIZE, DCOMP, 'single', path=str(tmp_path / 'g.bin'))
    raw = open(good, 'rb').read()
    cases = {'magic.bin': b'SHFM0001' + raw[8:], 'trunc.bin': raw[:len(raw) // 2],
             'dtype.bin': raw[:10] + b'\x01\x00' + raw[12:], 'empty.bin': b''}
    for name, data in cases.items():
        p = tmp_path / name
        p.write_bytes(data)
        with pytest.raises(sc.NsstError):
            sc.load_shearing_filters(str(p))
    with pytest.raises(sc.NsstError):
        sc.load_shearing_filters(str(tmp_path / 'missing.bin'))
    with pytest.raises(sc.NsstError):
        sc.save_shearing_filters(DSIZE, DCOMP, 'half', path=str(tmp_path / 'x.bin'))
