"""Build the CUDA library ``libgturbo_gb300.so`` in-tree (sm_103a only).

Every grid size is its own translation unit (``csrc/gt_inst_<N>.cu``) so the units compile in
parallel; the host C-ABI is ``csrc/gturbo.cu``. Output: ``gturbo_gb300/_build/``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB_NAME = "libgturbo_gb300.so"
LIB_PATH = os.path.join(BUILD, LIB_NAME)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gturbo_gb300")
    return cand


def sources() -> list[str]:
    units = sorted(f for f in os.listdir(CSRC)
                   if f.startswith(("gt_inst_", "gt_ens_r")) and f.endswith(".cu"))
    return [os.path.join(CSRC, f) for f in units] + [os.path.join(CSRC, "gturbo.cu"),
                                                      os.path.join(CSRC, "gt_ens.cu"),
                                                      os.path.join(CSRC, "gt_adj.cu")]


def _deps() -> list[str]:
    out = []
    for f in os.listdir(CSRC):
        if f.endswith((".cu", ".cuh", ".h", ".inc")):
            out.append(os.path.join(CSRC, f))
    out.append(os.path.join(HERE, "..", "include", "gturbo.h"))
    return out


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, jobs: int | None = None,
          out_dir: str | None = None, extra_flags: list[str] | None = None) -> str:
    """Compile (if stale) and link the library; returns its path.

    ``out_dir`` and ``extra_flags`` (e.g. ``["-DGT_ROW_MINB=3"]``) build a variant elsewhere;
    the environment variable GTURBO_NVCC_FLAGS adds flags to every build.
    """
    bdir = out_dir or BUILD
    lib_path = os.path.join(bdir, LIB_NAME)
    os.makedirs(bdir, exist_ok=True)
    deps = _deps()
    if not force and not _stale(lib_path, deps):
        return lib_path
    nvcc = _nvcc()
    srcs = sources()
    objs = [os.path.join(bdir, os.path.basename(s)[:-3] + ".o") for s in srcs]
    flags = list(NVCC_FLAGS) + list(extra_flags or []) + os.environ.get("GTURBO_NVCC_FLAGS", "").split()

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc, *flags, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    jobs = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(jobs) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    tmp = lib_path + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stderr}")
    os.replace(tmp, lib_path)
    return lib_path


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
