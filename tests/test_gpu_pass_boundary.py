"""Cost of a pass boundary: a grid-wide barrier in a cooperative persistent kernel against the
boundary between two kernels on one stream (direct launches and CUDA graphs, with and without
programmatic dependent launch), and the capped wait of the barrier: with a zero poll limit the
kernel returns with its error flag set, and the next launch runs normally.

The solver keeps one kernel per pass; these figures are the measured reason (a barrier costs
more than a kernel boundary inside a graph)."""
import os
import re
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.gpu
def test_pass_boundary_costs_and_capped_wait(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    exe = tmp_path / "pass_boundary"
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-o", str(exe),
                    os.path.join(HERE, "native", "pass_boundary.cu")], check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    barriers = [l.split() for l in r.stdout.splitlines() if l.startswith("barrier ")]
    kernels = [l.split() for l in r.stdout.splitlines() if l.startswith("kernel ")]
    assert barriers and kernels
    assert all(b[5] == "0" for b in barriers)
    assert all(float(b[4]) > 0 for b in barriers) and all(float(k[4]) > 0 for k in kernels)
    assert re.search(r"^timeout_status 1$", r.stdout, re.M), r.stdout
    assert re.search(r"^after 0$", r.stdout, re.M), r.stdout
