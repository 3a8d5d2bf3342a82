import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')
REFERENCE = os.environ.get('TRANSIFLOW_REFERENCE', '/root/reference')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built libtfcuda.so')


def load_golden(name):
    return dict(np.load(os.path.join(GOLDEN, name + '.npz'), allow_pickle=False))


def golden_params(g):
    import ast
    return ast.literal_eval(str(g['params']))


def golden_csr(g, t):
    """(begA, jcoA, coA) of state t of a discretisation fixture."""
    off = int(np.sum(g['nnz'][:t]))
    k = int(g['nnz'][t])
    return g['begA'][t], g['jcoA'][off:off + k], g['coA'][off:off + k]


DISC_FIXTURES = ['ldc2d_16_re1000', 'ldc2d_16_re0', 'ldc2d_12x10_stretched', 'ldc3d_4_ramp',
                 'ldc3d_5x4x3_stretched', 'ldc_semi2d_4', 'dhc2d_8_stretched', 'dhc3d_4_ramp',
                 'rb3d_4_ramp', 'rb2d_6x5', 'rbp2d_6x5', 'qg2d_4_ramp', 'qg2d_8x6',
                 'amoc2d_4_ramp', 'amoc2d_8x4']


@pytest.fixture(scope='session')
def built_lib():
    """libtfcuda.so, built in-tree if it is missing (host-only calls need no GPU)."""
    from transiflow_gb300 import _lib
    if not os.path.exists(_lib.LIBPATH):
        _lib.build()
    return _lib.load()


def has_reference():
    return os.path.isdir(os.path.join(REFERENCE, 'transiflow'))
