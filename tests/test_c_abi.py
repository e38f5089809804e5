"""The C ABI from C: tests/c_abi/nsst_c_example.c includes only
include/nsst.h (and the CUDA runtime), compiles as C99 against it and links
libnsst.so; on a GPU its output equals the Python path's."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, 'tests', 'c_abi', 'nsst_c_example.c')
CUDA = os.environ.get('CUDA_HOME', '/usr/local/cuda')


def _build(tmp_path):
    exe = str(tmp_path / 'nsst_c_example')
    lib_dir = os.path.join(ROOT, 'shearcuda_gb300')
    cmd = ['gcc', '-std=c99', '-Wall', '-Wextra', '-pedantic', '-O2', '-I', os.path.join(ROOT, 'include'),
           '-isystem', os.path.join(CUDA, 'include'), SRC, '-o', exe, '-L', lib_dir, '-lnsst',
           '-L', os.path.join(CUDA, 'lib64'), '-lcudart', '-lm', '-Wl,-rpath,' + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert 'warning' not in r.stderr, r.stderr
    return exe


def test_c_example_compiles_and_links_as_c99(built_lib, tmp_path):
    assert os.path.exists(_build(tmp_path))


@pytest.mark.gpu
def test_c_example_matches_python_path(built_lib, cuda, tmp_path):
    import torch
    import shearcuda_gb300 as sc
    exe = _build(tmp_path)
    H, W = 256, 384
    r = subprocess.run([exe, str(H), str(W)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    fields = r.stdout.split()
    checksum, rdwt_err = float(fields[1]), float(fields[3])
    rr, cc = np.mgrid[0:H, 0:W]
    x = torch.tensor(((rr * 7 + cc * 13) % 101).astype(np.float32), device=cuda)
    plan = sc.prepare_shearing_filters_cuda([3, 3, 4, 4], [32, 32, 16, 16], H, W)
    sc.nsst_scalars(plan, seed=4321)
    y = sc.nsst_denoise(x, plan, 20.0, [0, 3, 3, 3, 4])
    assert checksum == pytest.approx(float(y.double().sum()), rel=1e-9)
    assert rdwt_err <= 1e-4 * 100
