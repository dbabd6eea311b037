"""Build the reference-equivalent cuFFT baseline ``baseline/_build/librefeq_cufft.so``.

A measurement baseline only: the benchmark times it beside the product to stand in for the
reference's OpenACC + cuFFT build, which needs a Fortran compiler that neither machine has.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_build", "librefeq_cufft.so")
SRC = os.path.join(HERE, "refeq_cufft.cu")


def build(force: bool = False) -> str:
    hdr = os.path.join(HERE, "..", "include", "gturbo.h")
    if not force and os.path.exists(OUT) and os.path.getmtime(OUT) > max(
            os.path.getmtime(SRC), os.path.getmtime(hdr)):
        return OUT
    os.makedirs(os.path.dirname(OUT), exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-std=c++17", "-O3", "-gencode", "arch=compute_103a,code=sm_103a", "-Xcompiler",
           "-fPIC", "-shared", SRC, "-o", OUT + ".tmp", "-lcufft"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"refeq build failed:\n{r.stderr}")
    os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(force=True))
