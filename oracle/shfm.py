"""FP64 oracle of the reference's shearing-filter bank file (SHFM0002).
TEST INFRASTRUCTURE ONLY: imported by tests/, never by the library.

Writer: save_shearing_filters.m:46-84 (MATLAB fwrite of the magic, the
uint16 counts and each n x n filter w_s{j}(:,:,k) in column-major order,
then the four atrousfilters of :77-83).  Reader:
demo_denoise/demoImageDenoise/shearconfig.cpp:26-78 (ShearConfig::
readFromFile).  Both little-endian, as MATLAB and the x86 reader produce.
"""
import numpy as np

DTYPES = {'single': (0, '<f4'), 'double': (2, '<f8')}


def shfm_write(path, shear, atrous, data_type='single'):
    """shear: list of (ndir, n, n) arrays (row-major [k][r][c]); atrous: 4 square arrays."""
    code, fmt = DTYPES[data_type]
    with open(path, 'wb') as f:
        f.write(b'SHFM0002')                                   # :56
        f.write(np.array([len(shear), code], '<u2').tobytes())  # :58-64
        for w in shear:
            nd, n, _ = w.shape
            f.write(np.array([n, nd], '<u2').tobytes())         # :68-71
            for k in range(nd):
                f.write(np.asarray(w[k], np.float64).T.astype(fmt).tobytes())  # column-major, :73-74
        for h in atrous:
            f.write(np.array([h.shape[0]], '<u2').tobytes())    # :80
            f.write(np.asarray(h, np.float64).T.astype(fmt).tobytes())        # :82


def shfm_read(path):
    """-> (data_type, [ (ndir, n, n) ], [h0, h1, g0, g1]) as FP64, row-major."""
    raw = open(path, 'rb').read()
    if raw[:8] != b'SHFM0002':
        raise ValueError('bad magic')
    nscales, code = (int(v) for v in np.frombuffer(raw, '<u2', 2, 8))
    fmt, es = ('<f4', 4) if code == 0 else ('<f8', 8)
    at = 12
    shear = []
    for _ in range(nscales):
        n, nd = (int(v) for v in np.frombuffer(raw, '<u2', 2, at))
        at += 4
        v = np.frombuffer(raw, fmt, nd * n * n, at).astype(np.float64)
        at += nd * n * n * es
        shear.append(v.reshape(nd, n, n).transpose(0, 2, 1))  # column-major filters
    atrous = []
    for _ in range(4):
        F = int(np.frombuffer(raw, '<u2', 1, at)[0])
        at += 2
        atrous.append(np.frombuffer(raw, fmt, F * F, at).astype(np.float64).reshape(F, F).T)
        at += F * F * es
    if at != len(raw):
        raise ValueError('trailing bytes')
    return ('single' if code == 0 else 'double'), shear, atrous
