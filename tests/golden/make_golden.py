"""Generate the golden vectors of tests/golden/ from the reference's own statements.

The reference ships no test vectors (its Makefile's ``verify`` target is empty) and cannot be
compiled here (Fortran + OpenACC + cuFFT, no Fortran compiler available). Its library sources are
transliterated mechanically into C by ``oracle/f2c_ref.py`` (the cuFFT calls answered by a shim
that follows cuFFT's documented transform definitions), and every vector below is computed by
those transliterated routines: defk, iniforcing, fft_dir, fft_inv, trunc, nlt, step/step4,
forcing/rann, spectrum/fluxes/glob and writef2. The C oracle and the CUDA path are both checked
against the files. Run from the repository root where the reference checkout is present:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gturbo_gb300.params import Params  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # name: (params, input seed)
    "n32_a2_rk4": (Params(n=32, alpv=2.0, rko=4, k1f=3.0, k2f=5.0, nu=1e-8, alpnu=4.0, mu=0.05,
                          dt=2e-3, famp=0.5), 101),
    "n64_a1_rk2": (Params(n=64, alpv=1.0, rko=2, k1f=6.0, k2f=8.0, nu=1e-20, alpnu=8.0, mu=0.1,
                          dt=1e-3, famp=0.3), 102),
    "n64_a05_rk2_split": (Params(n=64, alpv=0.5, rko=2, k1f=4.0, k2f=6.0, nu=1e-4, alpnu=1.0,
                                 mu=0.0, alpmu=0.0, dt=1e-3, famp=0.2), 103),
    # a non-square grid, NX = 64 by NY = 32 (the reference's transforms planned as NY x NX)
    "n64x32_a2_rk4": (Params(n=64, ny=32, alpv=2.0, rko=4, k1f=3.0, k2f=6.0, nu=1e-12, alpnu=4.0,
                             mu=0.05, dt=1e-3, famp=0.4), 104),
}
# main-loop horizon: steps of src/main.f90:97-137 with diagnostics every HORIZON_IMIX steps
HORIZON_STEPS = 20
HORIZON_IMIX = 10


def make_case(name, p, seed):
    from oracle.refcore import Reference

    r = Reference(p)
    n, ny = p.n, p.rows
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((ny, n))
    out = {"n": p.n, "phys_in": x}
    a = r.zeros()
    a[:, :n] = x
    r.fft_dir(a)
    out["fft_dir"] = a.copy()
    r.trunc(a)
    a *= 20.0
    zk = a
    out["spec_in"] = zk.copy()
    b = zk.copy()
    r.fft_inv(b)
    out["fft_inv"] = b[:, :n].copy()
    b = zk.copy()
    r.nlt(b)
    out["nlt"] = b.copy()
    znl = b
    b = zk.copy()
    r.rk_step(b)
    out["step"] = b.copy()
    b, s = zk.copy(), 481929
    for _ in range(3):
        s = r.forcing(b, s)
    out["forcing3"] = b
    out["forcing3_seed"] = np.array([s], np.int64)
    d = r.diag(zk.copy(), znl)
    for k in ("sp", "sz", "fle", "flz", "glob"):
        out["diag_" + k] = d[k]
        out["diag_written_" + k] = d["written"][k].astype(np.float32)
    ik, jk = r.forcing_modes()
    out["ikxf"], out["ikyf"] = ik, jk
    info = r.info()
    out["inpe"] = np.array([info["inpe"]])
    out["inpz"] = np.array([info["inpz"]])
    t = r.tables()
    out["emk"] = t["emk"]
    # the dump record of fields/w.NNN.MMM (main.f90:119-125: znl = z, fft_inv, writef2)
    with tempfile.TemporaryDirectory() as wd:
        b = zk.copy()
        r.fft_inv(b)
        path = r.writef2(b, 0, 1, wd)
        raw = np.fromfile(path, dtype=np.uint8)
    out["dump_record"] = raw[4:-4].view(np.float32).reshape(ny, n).copy()
    # main-loop horizon from the same field and the reference's seed
    z, s = zk.copy(), 481929
    work = [r.zeros() for _ in range(4)]
    spectra = []
    for ipas in range(1, HORIZON_STEPS + 1):
        s, dd = r.main_step(z, s, ipas, HORIZON_IMIX, work)
        if dd is not None:
            spectra.append(np.stack([dd["sp"], dd["sz"], dd["fle"], dd["flz"]]))
    out["horizon_z"] = z
    out["horizon_seed"] = np.array([s], np.int64)
    out["horizon_spectra"] = np.stack(spectra)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


# the benchmark workloads from their own random-phase initial fields (the reference's forcing and
# seed): steps main-loop iterations each, diagnostics every WORKLOAD_IMIX; a field is summarised by
# sampled retained modes and a checksum (a 2048^2 field is 67 MB)
WORKLOADS = {"c1": 4, "c5": 3, "c2": 3, "c3": 2}  # name: main-loop iterations
WORKLOAD = "c2"  # the headline
WORKLOAD_STEPS = WORKLOADS[WORKLOAD]
WORKLOAD_IMIX = 2
WORKLOAD_MODES = 512


def workload_mode_index(p, z):
    """WORKLOAD_MODES distinct retained (nonzero) modes of z, drawn with a fixed seed: flat
    indices into the complex (NY, NX/2+1) view."""
    from oracle.coracle import spec

    nz = np.flatnonzero(spec(z).ravel())
    return np.sort(np.random.default_rng(7).choice(nz, WORKLOAD_MODES, replace=False))


def make_workload(cfg=WORKLOAD):
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import IC_K0, config
    from oracle.coracle import spec
    from oracle.refcore import Reference

    p = config(cfg)
    r = Reference(p)
    z = random_phase_ic(p, IC_K0[cfg], 0.5, seed=1)
    idx = workload_mode_index(p, z)
    work = [r.zeros() for _ in range(4)]
    s = 481929
    spectra, globs = [], []
    for ipas in range(1, WORKLOADS[cfg] + 1):
        s, d = r.main_step(z, s, ipas, WORKLOAD_IMIX, work)
        if d is not None:
            spectra.append(np.stack([d["sp"], d["sz"], d["fle"], d["flz"]]))
            globs.append(d["glob"])
    zc = spec(z).ravel()
    np.savez_compressed(os.path.join(OUT, f"{cfg}_workload.npz"), mode_index=idx,
                        modes=zc[idx], sum_abs2=np.array([float(np.sum(np.abs(zc) ** 2))]),
                        seed=np.array([s], np.int64), spectra=np.stack(spectra),
                        glob=np.stack(globs))


def make_lcg():
    from oracle.refcore import Reference

    r = Reference(CASES["n32_a2_rk4"][0])
    draws, states = [], []
    s = 481929
    for _ in range(1000):
        d, s = r.rann(s, 1)
        draws.append(d[0])
        states.append(s)
    np.savez_compressed(os.path.join(OUT, "lcg_481929.npz"), draws=np.array(draws, np.float32),
                        states=np.array(states, np.int64))


if __name__ == "__main__":
    from oracle import refcore

    if not refcore.available():
        sys.exit("the reference's sources are needed to generate the golden vectors")
    for name, (p, seed) in CASES.items():
        make_case(name, p, seed)
    make_lcg()
    for cfg in WORKLOADS:
        make_workload(cfg)
    print("written:", sorted(f for f in os.listdir(OUT) if f.endswith(".npz")))
