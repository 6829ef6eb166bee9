import os
import sys

# a few BLAS threads: the oracle's small dense solves slow down badly when
# OpenBLAS oversubscribes a shared host
os.environ.setdefault('OPENBLAS_NUM_THREADS', '2')

import numpy as np  # noqa: E402
import pytest  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, 'tests', 'golden')


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300) and the built libttals.so')


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + '.npz'))

    def cores(prefix):
        return [z[f'{prefix}_{i}'] for i in range(int(z[prefix + '_n']))]

    return z, cores


@pytest.fixture
def golden():
    return load_golden
