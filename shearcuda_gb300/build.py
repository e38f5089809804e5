"""In-tree build of libnsst.so for sm_103a (nvcc, no cmake).

Each translation unit is compiled in parallel, then linked into
``shearcuda_gb300/libnsst.so``.  Object files go to ``shearcuda_gb300/_build``.
"""
import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libnsst.so')
NVCC = os.environ.get('NVCC', '/usr/local/cuda/bin/nvcc')
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
SOURCES = ['k_directional.cu', 'k_dir_fused.cu', 'k_cols_tma.cu', 'k_atrous.cu', 'k_adjoint.cu', 'k_reduce.cu', 'k_wavelet.cu', 'k_vol3d.cu', 'k_vol3d_pass.cu', 'k_vol3d_pass_odd.cu', 'k_dct.cu', 'noalloc.cu', 'host_filters.cpp', 'host_filterfile.cpp',
           'host_wavelets.cpp', 'host_dct.cpp', 'host_filters3d.cpp', 'plan.cpp', 'plan3d.cpp']
HEADERS = ['fft_core.cuh', 'tiles.cuh', 'tma.cuh', 'vol3d_pass.cuh', 'internal.h', 'pyramid_tables.h', 'wavelet_tables.h']


def _flags(src):
    # -ffp-contract=off: the host's FP64 filter construction (grid rounding in
    # the Meyer windows) must give the same bits on x86-64 and on aarch64, whose
    # gcc would otherwise fuse multiply-adds
    common = ['-O3', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-ffp-contract=off',
              '-I', os.path.join(ROOT, 'include')]
    if src.endswith('.cu'):
        return common + ARCH + ['-lineinfo', '--expt-relaxed-constexpr']
    return common + ['-x', 'c++']


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose=False):
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + '.o')
    deps = [os.path.join(CSRC, src)] + [os.path.join(CSRC, h) for h in HEADERS] + \
        [os.path.join(ROOT, 'include', 'nsst.h'), os.path.abspath(__file__)]
    if not _newer(obj, deps):
        return obj, ''
    cmd = [NVCC] + _flags(src) + ['-c', os.path.join(CSRC, src), '-o', obj]
    if verbose:
        cmd.insert(1, '-Xptxas=-v')
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError('compile failed: %s\n%s\n%s' % (' '.join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, log in results:
            if log:
                print(log)
    if _newer(LIB, objs):
        cmd = [NVCC] + ARCH + ['-shared', '-o', LIB] + objs + ['-lcudart']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('link failed: %s\n%s' % (r.stdout, r.stderr))
    return LIB


if __name__ == '__main__':
    print(build(verbose='-v' in sys.argv))
