import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

DCOMP = [3, 3, 4, 4]
DSIZE = [32, 32, 16, 16]
K_DEMO = [0, 3, 3, 3, 4]  # Tscalars [0 3 4] of denoise_shearlet_example.m:38 per level


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')


@pytest.fixture(scope='session')
def built_lib():
    from shearcuda_gb300 import build
    build.build()
    from oracle import build_oracle
    build_oracle.build_port()
    return build.LIB


@pytest.fixture(scope='session')
def cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    return torch.device('cuda:0')


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def flat_scalars(scal):
    return np.concatenate([[scal[0]]] + [np.asarray(s) for s in scal[1:]])


def flat_coeffs(dst):
    return np.concatenate([dst[0][None]] + list(dst[1:]))
