"""Index arithmetic of every contraction descriptor, checked on the CPU: a host
program evaluates each descriptor with the kernels' own offset/sum code on
random data, compares with naive loop nests and bounds-checks every access."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_descriptors_on_host(tmp_path):
    nvcc = shutil.which('nvcc') or '/usr/local/cuda/bin/nvcc'
    if not os.path.exists(nvcc):
        pytest.skip('nvcc not available')
    exe = str(tmp_path / 'desc_check')
    src = os.path.join(ROOT, 'tests', 'desc_check.cu')
    inc = os.path.join(ROOT, 'scikit_tt_gb300', 'csrc')
    subprocess.run([nvcc, '-std=c++17', '-O1', '-I', inc, '-o', exe, src], check=True, capture_output=True)
    res = subprocess.run([exe], capture_output=True, text=True)
    assert res.returncode == 0, res.stdout
    assert 'OK' in res.stdout
