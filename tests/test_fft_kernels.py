"""The register butterflies (radix 2, 4, 8, 16; forward and inverse) of the FFT engine, compiled
for the host with nvcc and compared with a naive long-double DFT (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_butterflies_match_naive_dft(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / "dft_check"
    subprocess.run([nvcc, "-std=c++17", "-O2", "-o", str(exe), os.path.join(HERE, "native", "dft_check.cu")],
                   check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
