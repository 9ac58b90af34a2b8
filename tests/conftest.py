import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, 'tkf-mixdom_gb300')
for p in (ROOT, PKG_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built library')


def load_golden(name):
    g = np.load(os.path.join(GOLDEN, name + '.npz'))
    return {k: g[k] for k in g.files}


def golden_params(g):
    p = {k[2:]: g[k] for k in g if k.startswith('p_')}
    return {k: (float(v) if np.ndim(v) == 0 else v) for k, v in p.items()}


@pytest.fixture(scope='session')
def cuda_lib():
    """The built CUDA library (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip('no CUDA device')
    from pairhmm import _lib
    return _lib.load()
