"""ctypes wrapper of the C oracle (``oracle/gturbo_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, the smoke check and the CPU-baseline leg
of ``bench.py``, where results are compared with it; it is never the thing measured for the
GPU path.

Fields are numpy float64 arrays of shape (NY, NX+2): the physical view ``real(8) z(NX+2,NY)``.
``spec(a)`` gives the complex (NY, NX/2+1) view of the same memory (``complex(8) z(NX/2+1,NY)``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from gturbo_gb300.params import GtInfo, GtParams, Params

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc + OpenMP); returns the library path."""
    if force or not os.path.exists(_LIB_PATH):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(_LIB_PATH)
    P = ctypes.c_void_p
    D = ctypes.POINTER(ctypes.c_double)
    I32 = ctypes.POINTER(ctypes.c_int32)
    lib.or_create.restype = P
    lib.or_create.argtypes = [ctypes.POINTER(GtParams), ctypes.POINTER(ctypes.c_int)]
    lib.or_destroy.argtypes = [P]
    lib.or_info.argtypes = [P, ctypes.POINTER(GtInfo)]
    lib.or_forcing_modes.restype = ctypes.c_int
    lib.or_forcing_modes.argtypes = [P, I32, I32]
    lib.or_tables.argtypes = [P, D, D, D]
    for name in ("or_fft_dir", "or_fft_inv", "or_trunc"):
        getattr(lib, name).argtypes = [P, D]
    lib.or_produ.argtypes = [P, D, D, D]
    lib.or_nlt.argtypes = [P, D, D, D]
    lib.or_step.argtypes = [P, D, D, D, D]
    lib.or_step4.argtypes = [P, D, D, D, D, D]
    lib.or_rann.restype = ctypes.c_float
    lib.or_rann.argtypes = [I32]
    lib.or_forcing.argtypes = [P, D, I32]
    lib.or_diag.argtypes = [P, D, D, D, D, D, D, D]
    lib.or_main_step.argtypes = [P, D, D, D, D, D, I32, ctypes.c_int, D, D, D, D, D]
    U64 = ctypes.POINTER(ctypes.c_uint64)
    lib.or_philox4x64_10.argtypes = [U64, U64, U64]
    lib.or_forcing_philox.argtypes = [P, D, ctypes.c_uint64, ctypes.c_uint64]
    lib.or_num_threads.restype = ctypes.c_int
    lib.or_set_num_threads.argtypes = [ctypes.c_int]
    _lib = lib
    return lib


def _dp(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def spec(a: np.ndarray) -> np.ndarray:
    """Complex (NY, NX/2+1) view of an (NY, NX+2) float64 field."""
    return a.view(np.complex128).reshape(a.shape[0], a.shape[1] // 2)


def philox4x64_10(counter, key):
    """Philox4x64-10 block of the oracle (4 uint64 counter words, 2 key words)."""
    lib = _load()
    c = (ctypes.c_uint64 * 4)(*counter)
    k = (ctypes.c_uint64 * 2)(*key)
    o = (ctypes.c_uint64 * 4)()
    lib.or_philox4x64_10(c, k, o)
    return [int(x) for x in o]


def set_num_threads(n: int) -> None:
    _load().or_set_num_threads(int(n))


def num_threads() -> int:
    return int(_load().or_num_threads())


def rann(seed: int, count: int):
    """``count`` draws of the reference's rann from ``seed``; returns (draws, new_seed)."""
    lib = _load()
    s = ctypes.c_int32(seed)
    out = [lib.or_rann(ctypes.byref(s)) for _ in range(count)]
    return np.array(out, dtype=np.float32), s.value


class Oracle:
    """One set of tables (defk + iniforcing) and the routines of the hot path on the CPU."""

    def __init__(self, p: Params):
        self.lib = _load()
        self.p = p
        err = ctypes.c_int(0)
        self._cp = p.to_ctypes()
        self.h = self.lib.or_create(ctypes.byref(self._cp), ctypes.byref(err))
        if not self.h:
            raise ValueError(f"or_create failed with status {err.value}")
        self.n = p.n  # NX
        self.ny = p.rows  # NY
        info = GtInfo()
        self.lib.or_info(self.h, ctypes.byref(info))
        self.info = info

    def close(self):
        if self.h:
            self.lib.or_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def zeros(self) -> np.ndarray:
        return np.zeros((self.ny, self.n + 2), dtype=np.float64)

    def forcing_modes(self):
        ik = np.zeros(2048, np.int32)
        jk = np.zeros(2048, np.int32)
        nf = self.lib.or_forcing_modes(self.h, ik.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                       jk.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)))
        return ik[:nf].copy(), jk[:nf].copy()

    def emk(self) -> np.ndarray:
        e = np.zeros((self.ny, self.n // 2 + 1), np.float64)
        self.lib.or_tables(self.h, _dp(e), None, None)
        return e

    def fft_dir(self, z):
        self.lib.or_fft_dir(self.h, _dp(z))

    def fft_inv(self, z):
        self.lib.or_fft_inv(self.h, _dp(z))

    def trunc(self, z):
        self.lib.or_trunc(self.h, _dp(z))

    def produ(self, z, u, v):
        self.lib.or_produ(self.h, _dp(z), _dp(u), _dp(v))

    def nlt(self, z, u=None, v=None):
        u = self.zeros() if u is None else u
        v = self.zeros() if v is None else v
        self.lib.or_nlt(self.h, _dp(z), _dp(u), _dp(v))

    def step(self, z, znl=None, u=None, v=None):
        znl, u, v = [self.zeros() if a is None else a for a in (znl, u, v)]
        self.lib.or_step(self.h, _dp(z), _dp(znl), _dp(u), _dp(v))

    def step4(self, z, znl=None, znew=None, u=None, v=None):
        znl, znew, u, v = [self.zeros() if a is None else a for a in (znl, znew, u, v)]
        self.lib.or_step4(self.h, _dp(z), _dp(znl), _dp(znew), _dp(u), _dp(v))

    def rk_step(self, z, work=None):
        if self.info.rko == 4:
            self.step4(z)
        else:
            self.step(z)

    def forcing(self, z, seed: int) -> int:
        s = ctypes.c_int32(seed)
        self.lib.or_forcing(self.h, _dp(z), ctypes.byref(s))
        return s.value

    def forcing_philox(self, z, key: int, step: int) -> None:
        self.lib.or_forcing_philox(self.h, _dp(z), ctypes.c_uint64(key), ctypes.c_uint64(step))

    def diag(self, z, znl=None):
        nb = self.n // 2
        sp, sz, fle, flz = (np.zeros(nb) for _ in range(4))
        glob = np.zeros(6)
        self.lib.or_diag(self.h, _dp(z), _dp(znl), _dp(sp), _dp(sz),
                         _dp(fle) if znl is not None else None,
                         _dp(flz) if znl is not None else None, _dp(glob))
        return dict(sp=sp, sz=sz, fle=fle, flz=flz, glob=glob)

    def main_step(self, z, seed: int, diag: bool = False, work=None):
        """One iteration of the reference main loop (step, optional diagnostics, forcing)."""
        if work is None:
            work = [self.zeros() for _ in range(4)]
        znl, znew, u, v = work
        s = ctypes.c_int32(seed)
        nb = self.n // 2
        out = None
        if diag:
            out = dict(sp=np.zeros(nb), sz=np.zeros(nb), fle=np.zeros(nb), flz=np.zeros(nb),
                       glob=np.zeros(6))
            self.lib.or_main_step(self.h, _dp(z), _dp(znl), _dp(znew), _dp(u), _dp(v),
                                  ctypes.byref(s), 1, _dp(out["sp"]), _dp(out["sz"]),
                                  _dp(out["fle"]), _dp(out["flz"]), _dp(out["glob"]))
        else:
            self.lib.or_main_step(self.h, _dp(z), _dp(znl), _dp(znew), _dp(u), _dp(v),
                                  ctypes.byref(s), 0, None, None, None, None, None)
        return s.value, out
