"""Build recipe for the oracle's native parts (test infrastructure only).

* ``oracle/libatrous_port.so``: the project's C restatement (atrous_port.c).
* ``oracle/_ref/libatrousc_ref.so``: the reference's own
  ``shearlet_toolbox_1/atrousc.cpp``, compiled unchanged where it lies in the
  reference checkout, against the project-written MEX shim in
  ``oracle/mex_shim`` plus ``atrous_ref_glue.cpp``.
* ``oracle/_ref/librwt_ref.so``: the reference's Rice Wavelet Toolbox
  templates ``shearcuda/src/{mrdwt,mirdwt,mdwt}_r.h``, included where they lie,
  behind ``rwt_ref_glue.cpp``.
Both reference builds happen only when the reference checkout is present (it
is not on machines that only run tests).

Usage: python oracle/build_oracle.py [--reference DIR]  (default: $SHEARCUDA_REFERENCE, else
``reference`` beside the repository)
"""
import argparse
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, 'libatrous_port.so')
REF_DIR = os.path.join(HERE, '_ref')
REF_SO = os.path.join(REF_DIR, 'libatrousc_ref.so')
RWT_SO = os.path.join(REF_DIR, 'librwt_ref.so')


def default_reference():
    """The reference checkout: $SHEARCUDA_REFERENCE, else a directory named
    `reference` beside this repository's directory."""
    env = os.environ.get('SHEARCUDA_REFERENCE')
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), 'reference')


DEFAULT_REFERENCE = default_reference()


def _newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_port(force=False):
    src = os.path.join(HERE, 'atrous_port.c')
    if force or _newer(PORT_SO, [src, os.path.abspath(__file__)]):
        subprocess.check_call(['gcc', '-O3', '-ffp-contract=off', '-fPIC', '-shared', '-pthread', '-o', PORT_SO, src])
    return PORT_SO


def build_ref(reference=DEFAULT_REFERENCE, force=False):
    src = os.path.join(reference, 'shearlet_toolbox_1', 'atrousc.cpp')
    if not os.path.exists(src):
        return None
    glue = os.path.join(HERE, 'atrous_ref_glue.cpp')
    shim = os.path.join(HERE, 'mex_shim')
    os.makedirs(REF_DIR, exist_ok=True)
    deps = [src, glue, os.path.join(shim, 'mex.h'), os.path.join(shim, 'matrix.h')]
    if force or _newer(REF_SO, deps):
        subprocess.check_call(['g++', '-O2', '-ffp-contract=off', '-fPIC', '-shared', '-I', shim, '-o', REF_SO, glue, src])
    return REF_SO


def build_rwt_ref(reference=DEFAULT_REFERENCE, force=False):
    srcdir = os.path.join(reference, 'shearcuda', 'src')
    heads = [os.path.join(srcdir, f) for f in ('mrdwt_r.h', 'mirdwt_r.h', 'mdwt_r.h')]
    if not all(os.path.exists(h) for h in heads):
        return None
    glue = os.path.join(HERE, 'rwt_ref_glue.cpp')
    shim = os.path.join(HERE, 'mex_shim')
    os.makedirs(REF_DIR, exist_ok=True)
    if force or _newer(RWT_SO, heads + [glue, os.path.join(shim, 'matrix.h')]):
        subprocess.check_call(['g++', '-O2', '-ffp-contract=off', '-fPIC', '-shared', '-I', shim, '-I', srcdir, '-o', RWT_SO, glue])
    return RWT_SO


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument('--reference', default=DEFAULT_REFERENCE)
    ap.add_argument('--force', action='store_true')
    a = ap.parse_args()
    print(build_port(a.force))
    print(build_ref(a.reference, a.force))
    print(build_rwt_ref(a.reference, a.force))


if __name__ == '__main__':
    main()
