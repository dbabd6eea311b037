"""Generate the golden vectors of tests/golden/ from the numpy restatement (oracle/np_oracle.py).

The reference publishes no test vectors and cannot be run (Fortran + OpenACC + cuFFT, no Fortran
compiler available), so the fixtures come from the independent numpy restatement of its
routines. The C oracle and the CUDA path are both checked against them. Run from the repo root:

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from gturbo_gb300.params import Params  # noqa: E402
from oracle.np_oracle import NpOracle, to_phys_layout  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # name: (params, input seed)
    "n32_a2_rk4": (Params(n=32, alpv=2.0, rko=4, k1f=3.0, k2f=5.0, nu=1e-8, alpnu=4.0, mu=0.05,
                          dt=2e-3, famp=0.5), 101),
    "n64_a1_rk2": (Params(n=64, alpv=1.0, rko=2, k1f=6.0, k2f=8.0, nu=1e-20, alpnu=8.0, mu=0.1,
                          dt=1e-3, famp=0.3), 102),
    "n64_a05_rk2_split": (Params(n=64, alpv=0.5, rko=2, k1f=4.0, k2f=6.0, nu=1e-4, alpnu=1.0,
                                 mu=0.0, alpmu=0.0, dt=1e-3, famp=0.2), 103),
}


def input_field(q: NpOracle, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    x = rng.standard_normal((q.n, q.n))
    return q.trunc(q.fft_dir(x)) * 20.0, x


def make_case(name, p, seed):
    q = NpOracle(p)
    zk, x = input_field(q, seed)
    out = {"n": p.n}
    out["phys_in"] = x
    out["fft_dir"] = to_phys_layout(q.fft_dir(x))
    out["spec_in"] = to_phys_layout(zk)
    out["fft_inv"] = q.fft_inv(zk)
    out["nlt"] = to_phys_layout(q.nlt(zk))
    out["step"] = to_phys_layout(q.rk_step(zk))
    zf, s = zk, 481929
    for _ in range(3):
        zf, s = q.forcing(zf, s)
    out["forcing3"] = to_phys_layout(zf)
    out["forcing3_seed"] = np.array([s], np.int64)
    d = q.diag(zk, q.nlt(zk))
    for k, v in d.items():
        out["diag_" + k] = v
    ik = np.array([m[0] for m in q.modes], np.int32)
    jk = np.array([m[1] for m in q.modes], np.int32)
    out["ikxf"], out["ikyf"] = ik, jk
    out["inpe"] = np.array([q.inpe])
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def make_lcg():
    s = 481929
    draws, states = [], []
    for _ in range(1000):
        r, s = NpOracle.rann(s)
        draws.append(r)
        states.append(s)
    np.savez_compressed(os.path.join(OUT, "lcg_481929.npz"), draws=np.array(draws, np.float32),
                        states=np.array(states, np.int64))


if __name__ == "__main__":
    for name, (p, seed) in CASES.items():
        make_case(name, p, seed)
    make_lcg()
    print("written:", sorted(f for f in os.listdir(OUT) if f.endswith(".npz")))
