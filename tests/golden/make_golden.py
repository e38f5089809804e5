"""Generate the golden fixtures under tests/golden/ from the reference tree.

Run in the container that holds the read-only reference checkout:

    python tests/golden/make_golden.py [--reference DIR]
(default: $SHEARCUDA_REFERENCE, else ``reference`` beside the repository)

It writes two kinds of fixtures, both small enough to commit:

* ``pyramid_filter_tables.json``: the tabulated à trous filter matrices of
  ``shearlet_toolbox_1/atrousfilters.m`` (cases '9-7' lines 27-104,
  'maxflat' lines 106-175, 'pyr' lines 178-206, 'pyrexc' lines 208-236),
  parsed from the MATLAB source text (the numbers are data that defines the
  filters; they are read, never retyped).  The mirroring / scaling steps that
  follow each table stay in code (oracle and product restate them).
* ``atrousc_ref_cases.npz``: inputs and outputs of the reference's own
  ``atrousc.cpp`` (compiled unchanged through the project-written MEX shim in
  ``oracle/mex_shim``; see ``oracle/build_oracle.py``) on seeded random
  signals, for every (filter size, dilation) pair the 4-level pyramid uses,
  plus odd-sized ragged cases.  These pin the C and NumPy restatements.
* ``nsst3_scalar_tables.json``: the 3-D noise scalars the reference ships
  (``shearcuda3d/DenoiseDemo/nsstScalarsData*.mat``, written by
  NsstScalars.m:1-19 — Monte-Carlo MAD/0.6745 per band of N(0,1) noise for
  the demo's data size), flattened to the band order level, cone, l2, l1.
  They pin the 3-D pyramid windows, the Meyer filters and the band order to
  within the Monte-Carlo and data-size spread.
* ``rwt_ref_cases.npz``: inputs and outputs of the reference's Rice Wavelet
  Toolbox templates (``shearcuda/src/mrdwt_r.h``, ``mirdwt_r.h``,
  ``mdwt_r.h``, compiled unchanged behind ``oracle/rwt_ref_glue.cpp``) on
  seeded random images with the MakeONFilter filters the separation loop uses
  (Symmlet 4, Haar, Daubechies 4) and a long one (Coiflet 2), including a
  level whose dilated chain is shorter than the filter.
"""
import argparse
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def _strip_comments(line):
    out = []
    in_str = False
    for ch in line:
        if ch == "'":
            in_str = not in_str
        if ch == '%' and not in_str:
            break
        out.append(ch)
    return ''.join(out)


def parse_matlab_case(text, case_name):
    """Return {var: 2-D list} for every ``var = [ ... ];`` literal inside
    ``case '<case_name>'`` of a MATLAB switch statement."""
    lines = text.splitlines()
    start = None
    for i, ln in enumerate(lines):
        if re.match(r"\s*case\s+'%s'" % re.escape(case_name), ln):
            start = i + 1
            break
    if start is None:
        raise ValueError('case %r not found' % case_name)
    body = []
    for ln in lines[start:]:
        if re.match(r"\s*(case\s+'|end\s*$|otherwise)", ln):
            break
        body.append(_strip_comments(ln))
    # join continuation lines
    joined = ' '.join(l.replace('...', ' ') for l in body)
    mats = {}
    for m in re.finditer(r"(\w+)\s*=\s*\[([^\]]*)\]", joined):
        name, inner = m.group(1), m.group(2)
        if not re.search(r'\d', inner) or re.search(r'[A-Za-z_]\w*\s*\(', inner):
            continue  # mirroring statements such as [h0 fliplr(h0(:,1:end-1))]
        rows = [r for r in inner.split(';') if r.strip()]
        mat = [[float(tok) for tok in r.replace(',', ' ').split()] for r in rows]
        widths = {len(r) for r in mat}
        if len(widths) != 1:
            raise ValueError('ragged matrix %s in case %s: %s' % (name, case_name, widths))
        mats[name] = mat
    return mats


def filter_tables(reference):
    path = os.path.join(reference, 'shearlet_toolbox_1', 'atrousfilters.m')
    text = open(path).read()
    out = {'source': 'shearlet_toolbox_1/atrousfilters.m'}
    for case in ('9-7', 'maxflat', 'pyr', 'pyrexc'):
        mats = parse_matlab_case(text, case)
        for v in ('h0', 'h1', 'g0', 'g1'):
            if v not in mats:
                raise ValueError('missing %s in case %s' % (v, case))
        out[case] = {v: mats[v] for v in ('h0', 'h1', 'g0', 'g1')}
    return out


def atrousc_cases(seed=1234):
    sys.path.insert(0, ROOT)
    from oracle import atrous_ref  # noqa: E402  (reference atrousc via the MEX shim)
    if not atrous_ref.available():
        raise SystemExit('oracle/_ref not built: run python oracle/build_oracle.py first')
    rng = np.random.default_rng(seed)
    cases = {}
    # (signal rows, signal cols, filter size, dilation)
    shapes = []
    for F in (13, 19):
        for M in (1, 2, 4, 8):
            shapes.append((12 + M * F, 10 + M * F, F, M))
    shapes += [(37, 29, 7, 3), (20, 33, 5, 2), (9, 9, 9, 1)]
    for idx, (sr, sc, F, M) in enumerate(shapes):
        S = rng.standard_normal((sr, sc))
        Fm = rng.standard_normal((F, F))
        out = atrous_ref.atrousc(S, Fm, M)
        cases['S_%d' % idx] = S
        cases['F_%d' % idx] = Fm
        cases['M_%d' % idx] = np.array([M])
        cases['out_%d' % idx] = out
    cases['n'] = np.array([len(shapes)])
    return cases


def scalar_tables3(reference):
    """nsstScalarsData<level><dBand digits>.mat -> {name: {num_dirs, lowpass, bands}}."""
    import scipy.io as sio
    out = {}
    demo = os.path.join(reference, 'shearcuda3d', 'DenoiseDemo')
    for fn in sorted(os.listdir(demo)):
        m = re.match(r'nsstScalarsData(\d+)\.mat$', fn)
        if not m:
            continue
        digits = m.group(1)
        level = int(digits[0])
        if len(digits) != 1 + 2 * level:
            continue
        num_dirs = [int(digits[1 + 2 * l]) for l in range(level)]
        s = sio.loadmat(os.path.join(demo, fn), squeeze_me=True, struct_as_record=False)['nsstScalars']
        be = np.asarray(s.bandEst, dtype=object).reshape(3, level)
        bands = []
        for l in range(level):
            for c in range(3):
                tab = np.asarray(be[c, l], dtype=np.float64).reshape(num_dirs[l], num_dirs[l])
                bands.extend(float(v) for v in tab.ravel())  # (l2, l1) row-major
        out[digits] = {'num_dirs': num_dirs, 'lowpass': float(s.lowPassEst), 'bands': bands}
    return out


RWT_SHAPES = [(8, 16, 'Symmlet', 4, 3), (8, 8, 'Symmlet', 4, 3), (16, 8, 'Haar', 0, 2),
              (16, 16, 'Daubechies', 4, 2), (16, 16, 'Coiflet', 2, 2)]


def rwt_cases(seed=4321):
    sys.path.insert(0, ROOT)
    from oracle import rwt, rwt_ref  # noqa: E402
    if not rwt_ref.available():
        raise SystemExit('oracle/_ref not built: run python oracle/build_oracle.py first')
    rng = np.random.default_rng(seed)
    cases = {'n': np.array([len(RWT_SHAPES)])}
    for i, (H, W, fam, par, L) in enumerate(RWT_SHAPES):
        h = rwt.make_on_filter(fam, par)
        x = rng.standard_normal((H, W))
        yl, yh = rwt_ref.mrdwt(x, h, L)
        # the inverse of perturbed coefficients, so that mirdwt is pinned off the identity
        yh2 = yh + 0.1 * rng.standard_normal(yh.shape)
        cases.update({'x_%d' % i: x, 'h_%d' % i: h, 'L_%d' % i: np.array([L]), 'yl_%d' % i: yl, 'yh_%d' % i: yh,
                      'yh2_%d' % i: yh2, 'inv_%d' % i: rwt_ref.mirdwt(yl, yh2, h, L),
                      'mdwt_%d' % i: rwt_ref.mdwt(x, h, min(L, 2))})
    return cases


def main():
    ap = argparse.ArgumentParser()
    sys.path.insert(0, ROOT)
    from oracle.build_oracle import default_reference
    ap.add_argument('--reference', default=default_reference())
    args = ap.parse_args()
    tables = filter_tables(args.reference)
    with open(os.path.join(HERE, 'pyramid_filter_tables.json'), 'w') as f:
        json.dump(tables, f, indent=1)
    np.savez_compressed(os.path.join(HERE, 'atrousc_ref_cases.npz'), **atrousc_cases())
    with open(os.path.join(HERE, 'nsst3_scalar_tables.json'), 'w') as f:
        json.dump(scalar_tables3(args.reference), f, indent=1)
    np.savez_compressed(os.path.join(HERE, 'rwt_ref_cases.npz'), **rwt_cases())
    print('wrote', os.listdir(HERE))


if __name__ == '__main__':
    main()
