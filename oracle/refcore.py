"""The reference's own routines on the CPU: ctypes wrapper of oracle/_ref.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` (to pin the oracle and to regenerate the golden
vectors) and by the CPU reference arm of ``bench.py``; never by the product package.

``oracle/_ref/gturbo_ref.c`` is the mechanical C transliteration of the reference's Fortran
library sources (``oracle/f2c_ref.py``); it is generated here from the reference checkout and is
not committed. Each grid size is its own library, compiled from that file, the runtime
``f2c_rt.c`` and the cuFFT shim ``cufft_shim.c`` (sizes are compile-time parameters, as in the
reference's modules.f90:4). Where the generated source is absent (a copy of the repository without
the reference) ``available()`` is False and the tests that need it skip.

The set-up follows the reference's main program (src/main.f90:21-33, 58-61): ``inieuler`` reads
``params.dat`` (written here from a Params) and runs defk and iniforcing; the two cuFFT plans are
made as in main.f90:27,32 with the grid's (NY, NX). Fields are numpy float64 arrays of shape
(NY, NX+2), the physical view ``real(8) z(NX+2,NY)``; ``spec(a)`` of oracle.coracle gives the
spectral view.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(_HERE, "_ref")
REF_C = os.path.join(REF_DIR, "gturbo_ref.c")
_SRC = [os.path.join(_HERE, f) for f in ("f2c_rt.c", "f2c_rt.h", "cufft_shim.c")]
CFLAGS = ["-O2", "-std=gnu11", "-fPIC", "-fopenmp", "-fwrapv", "-ffp-contract=off",
          "-Wno-unknown-pragmas"]
SHIM_D2Z, SHIM_Z2D = 1, 2
_LOCK = threading.RLock()
_LIBS: dict[tuple[int, int], ctypes.CDLL] = {}
_OWNER: dict[tuple[int, int], object] = {}


def reference_source_dir() -> str | None:
    """The reference's src/ directory when this checkout has it (only where the fixtures are made)."""
    d = os.environ.get("GTURBO_REF_SRC", "/root/reference/src")
    return d if os.path.isfile(os.path.join(d, "nlt.f90")) else None


def generate(force: bool = False) -> str | None:
    """Transliterate the reference's sources into oracle/_ref/gturbo_ref.c (needs the reference)."""
    src = reference_source_dir()
    if src is None:
        return REF_C if os.path.exists(REF_C) else None
    if force or not os.path.exists(REF_C) or os.path.getmtime(REF_C) < os.path.getmtime(
            os.path.join(_HERE, "f2c_ref.py")):
        subprocess.run(["python3", os.path.join(_HERE, "f2c_ref.py"), "--src", src, "--out", REF_C],
                       check=True, capture_output=True)
    return REF_C


def available() -> bool:
    return generate() is not None


def lib_path(nx: int, ny: int) -> str:
    return os.path.join(REF_DIR, f"libgturbo_ref_{nx}x{ny}.so")


def build(nx: int, ny: int | None = None) -> str:
    """Compile the transliterated reference for an nx x ny grid (gcc, OpenMP); returns the path."""
    ny = nx if ny is None else ny
    if generate() is None:
        raise FileNotFoundError("oracle/_ref/gturbo_ref.c is missing and the reference sources are "
                                "not available to generate it")
    out = lib_path(nx, ny)
    deps = [REF_C] + _SRC
    if not os.path.exists(out) or any(os.path.getmtime(d) > os.path.getmtime(out) for d in deps):
        tmp = out + f".tmp{os.getpid()}"
        cmd = ["gcc", *CFLAGS, f"-DF2C_NX={nx}", f"-DF2C_NY={ny}", "-I", _HERE, "-shared", "-o", tmp,
               REF_C, os.path.join(_HERE, "f2c_rt.c"), os.path.join(_HERE, "cufft_shim.c"), "-lm"]
        subprocess.run(cmd, check=True, capture_output=True)
        os.replace(tmp, out)
    return out


def _load(nx: int, ny: int) -> ctypes.CDLL:
    key = (nx, ny)
    with _LOCK:
        if key in _LIBS:
            return _LIBS[key]
        lib = ctypes.CDLL(build(nx, ny))
        V = ctypes.c_void_p
        for name in ("inieuler", "fft_dir", "fft_inv", "trunc", "produ", "nlt", "step", "step4",
                     "forcing", "spectrum", "fluxes", "glob", "readf", "writef", "writef2", "defk",
                     "iniforcing"):
            fn = getattr(lib, "ref_" + name)
            fn.restype = ctypes.c_int
        lib.f_rann.restype = ctypes.c_float
        lib.f_rann.argtypes = [V]
        lib.f2c_captured.restype = ctypes.c_int
        lib.f2c_captured.argtypes = [ctypes.c_int, V, V, ctypes.c_int]
        lib.f2c_last_stop.restype = ctypes.c_char_p
        lib.f2c_cufft_plan2d.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int,
                                         ctypes.c_int]
        lib.f2c_set_threads.argtypes = [ctypes.c_int]
        lib.f2c_threads.restype = ctypes.c_int
        gnx, gny = ctypes.c_int(), ctypes.c_int()
        lib.ref_grid(ctypes.byref(gnx), ctypes.byref(gny))
        assert (gnx.value, gny.value) == key
        # the two plans of src/main.f90:27,32 (cufftPlan2D with the grid's slow and fast sizes)
        for var, kind in (("f_plan_inv", SHIM_Z2D), ("f_plan_dir", SHIM_D2Z)):
            h = ctypes.c_int(0)
            if lib.f2c_cufft_plan2d(ctypes.byref(h), ny, nx, kind):
                raise RuntimeError("cuFFT shim: plan creation failed")
            ctypes.c_int.in_dll(lib, var).value = h.value
        _LIBS[key] = lib
        return lib


def set_num_threads(n: int, nx: int, ny: int | None = None) -> None:
    _load(nx, nx if ny is None else ny).f2c_set_threads(int(n))


def _ptr(a: np.ndarray):
    assert a.flags.c_contiguous
    return ctypes.c_void_p(a.ctypes.data)


def params_dat(p, imix: int | None = None) -> str:
    """params.dat as src/inieuler.f90:13-20 reads it (6 list-directed records)."""
    r = repr
    return (f"{r(float(p.xlx))} {r(float(p.xly))}\n"
            f"{r(float(p.nu))} {r(float(p.alpnu))} {r(float(p.mu))} {r(float(p.alpmu))} {r(float(p.alpv))}\n"
            f"{r(float(p.dt))} {int(p.rko)}\n"
            f"1 1 {int(imix if imix is not None else p.imix)}\n"
            f"{r(float(p.rtrunc))} {int(p.truncate)}\n"
            f"{r(float(p.famp))} {r(float(p.k1f))} {r(float(p.k2f))}\n")


class Reference:
    """The reference's routines for one set of parameters (grid nx x ny, default p.n x p.n).

    The module state of the reference lives in the library's globals, so instances of one grid
    size take turns: every call first re-runs inieuler when another instance ran last.
    """

    def __init__(self, p, nx: int | None = None, ny: int | None = None, threads: int | None = None):
        self.p = p
        self.nx = nx or p.n
        self.ny = ny or getattr(p, "rows", p.n)
        self.lib = _load(self.nx, self.ny)
        if threads:
            self.lib.f2c_set_threads(int(threads))
        self.threads = self.lib.f2c_threads()
        self._activate(force=True)
        derived = int(ctypes.c_int.in_dll(self.lib, "f_split").value)
        if getattr(p, "split", -1) not in (-1, derived):
            raise ValueError("the reference derives split from alpnu/alpmu (inieuler.f90:22-36); "
                             f"it gives {derived} for these parameters")

    # ---- module state ---------------------------------------------------------------------
    def _activate(self, force=False):
        key = (self.nx, self.ny)
        with _LOCK:
            if not force and _OWNER.get(key) is self:
                return
            z = self.zeros()
            ifr = ctypes.c_int(0)
            with tempfile.TemporaryDirectory() as d:
                with open(os.path.join(d, "params.dat"), "w") as f:
                    f.write(params_dat(self.p))
                cwd = os.getcwd()
                os.chdir(d)
                try:
                    rc = self.lib.ref_inieuler(_ptr(z), ctypes.byref(ifr))
                finally:
                    os.chdir(cwd)
            if rc:
                raise ValueError(f"reference stopped: {self.lib.f2c_last_stop().decode()}")
            _OWNER[key] = self

    def _g(self, ctype, name):
        return ctype.in_dll(self.lib, "f_" + name).value

    def _arr(self, ctype, name, count):
        return np.ctypeslib.as_array((ctype * count).in_dll(self.lib, "f_" + name)).copy()

    @property
    def nh(self):
        return self.nx // 2 + 1

    def zeros(self) -> np.ndarray:
        return np.zeros((self.ny, self.nx + 2), dtype=np.float64)

    def info(self) -> dict:
        self._activate()
        d = {k: self._g(ctypes.c_double, k) for k in ("dkx", "dky", "inpz", "inpe", "fkxsmax",
                                                      "fkysmax", "rtrunc", "sdt", "dt2", "dt3", "dt6")}
        for k in ("nf", "split", "rko", "truncate"):
            d[k] = self._g(ctypes.c_int, k)
        return d

    def tables(self) -> dict:
        self._activate()
        nh, ny = self.nh, self.ny
        return {"emk": self._arr(ctypes.c_double, "emk", nh * ny).reshape(ny, nh),
                "emkx": self._arr(ctypes.c_double, "emkx", nh),
                "emky": self._arr(ctypes.c_double, "emky", ny),
                "fkx": self._arr(ctypes.c_double, "fkx", nh),
                "fky": self._arr(ctypes.c_double, "fky", ny),
                "fkxs": self._arr(ctypes.c_double, "fkxs", nh),
                "fkys": self._arr(ctypes.c_double, "fkys", ny),
                "jc": self._arr(ctypes.c_int, "jc", ny)}

    def forcing_modes(self):
        """(ikxf, ikyf) 0-based, as gt_get_forcing_modes reports them."""
        self._activate()
        nf = self._g(ctypes.c_int, "nf")
        ik = self._arr(ctypes.c_int, "ikxf", 2048)[:nf] - 1
        jk = self._arr(ctypes.c_int, "ikyf", 2048)[:nf] - 1
        return ik.astype(np.int32), jk.astype(np.int32)

    # ---- the routines -----------------------------------------------------------------------
    def _call(self, name, *arrays, ints=()):
        self._activate()
        args = [_ptr(a) for a in arrays] + [ctypes.byref(ctypes.c_int(int(i))) for i in ints]
        rc = getattr(self.lib, "ref_" + name)(*args)
        if rc:
            raise RuntimeError(f"reference stopped in {name}: {self.lib.f2c_last_stop().decode()}")

    def fft_dir(self, z):
        self._call("fft_dir", z, ints=(self._g(ctypes.c_int, "plan_dir"),))

    def fft_inv(self, z):
        self._call("fft_inv", z, ints=(self._g(ctypes.c_int, "plan_inv"),))

    def trunc(self, z):
        self._call("trunc", z)

    def produ(self, z, u, v):
        self._call("produ", z, u, v)

    def nlt(self, z, u=None, v=None):
        u = self.zeros() if u is None else u
        v = self.zeros() if v is None else v
        self._call("nlt", z, u, v)

    def step(self, z, znl=None, u=None, v=None):
        znl, u, v = [self.zeros() if a is None else a for a in (znl, u, v)]
        self._call("step", z, znl, u, v)

    def step4(self, z, znl=None, znew=None, u=None, v=None):
        znl, znew, u, v = [self.zeros() if a is None else a for a in (znl, znew, u, v)]
        self._call("step4", z, znl, znew, u, v)

    def rk_step(self, z):
        (self.step4 if self.p.rko == 4 else self.step)(z)

    def forcing(self, z, seed: int) -> int:
        self._activate()
        s = ctypes.c_int(seed)
        rc = self.lib.ref_forcing(_ptr(z), ctypes.byref(s))
        if rc:
            raise RuntimeError("reference stopped in forcing")
        return s.value

    def rann(self, seed: int, count: int):
        s = ctypes.c_int(seed)
        out = [self.lib.f_rann(ctypes.byref(s)) for _ in range(count)]
        return np.array(out, dtype=np.float32), s.value

    def diag(self, z, znl=None, ifr: int = 0) -> dict:
        """spectrum, fluxes (when znl is given) and glob of src/diagnostics.f90, from the values
        the reference writes. Each key holds the FP64 operands of the real() conversions of its
        write statements; ``written`` holds the real(4) values of the files themselves."""
        self._activate()
        nb = self.nx // 2
        self.lib.f2c_clear_captures()
        out, written = {}, {}

        def grab(unit, count):
            w = np.zeros(count)
            f = np.zeros(count)
            n = self.lib.f2c_captured(unit, _ptr(w), _ptr(f), count)
            assert n == count, (unit, n, count)
            return w, f

        self._call("spectrum", z, ints=(ifr,))
        w, f = grab(20, 3 * nb)
        out["sp"], out["sz"] = f[1::3].copy(), f[2::3].copy()
        written["sp"], written["sz"] = w[1::3].copy(), w[2::3].copy()
        if znl is not None:
            self.lib.f2c_clear_captures()
            self._call("fluxes", z, znl, ints=(ifr,))
            w, f = grab(30, 3 * nb)
            out["fle"], out["flz"] = f[1::3].copy(), f[2::3].copy()
            written["fle"], written["flz"] = w[1::3].copy(), w[2::3].copy()
        self.lib.f2c_clear_captures()
        self._call("glob", z, ints=(ifr,))
        w, f = grab(18, 9)
        # written order (diagnostics.f90:167): t, zz, ee, disz_nu, disz_mu, inpz, dise_nu,
        # dise_mu, inpe -> the gt_diag order ee, zz, disz_nu, disz_mu, dise_nu, dise_mu
        order = [2, 1, 3, 4, 6, 7]
        out["glob"] = f[order].copy()
        written["glob"] = w[order].copy()
        out["written"] = written
        return out

    def main_step(self, z, seed: int, ipas: int, imix: int, work=None):
        """One iteration of src/main.f90:97-137: step/step4, the diagnostics when
        mod(ipas, imix) == 0 (znl = z, nlt, spectrum, fluxes, glob), then the forcing."""
        if work is None:
            work = [self.zeros() for _ in range(4)]
        znl, znew, u, v = work
        if self.p.rko == 4:
            self.step4(z, znl, znew, u, v)
        else:
            self.step(z, znl, u, v)
        out = None
        if ipas % imix == 0:
            znl[...] = z
            self.nlt(znl, u, v)
            out = self.diag(z, znl, ipas)
        seed = self.forcing(z, seed)
        return seed, out

    # ---- restart and dump files (src/read.f90, src/write.f90) ------------------------------
    def readf(self, ifr: int, workdir: str) -> np.ndarray:
        """readf of fields/w.NNN under workdir: the real(4) record widened, padding zeroed."""
        self._activate()
        z = self.zeros()
        cwd = os.getcwd()
        os.chdir(workdir)
        try:
            self._call("readf", z, ints=(ifr,))
        finally:
            os.chdir(cwd)
        return z

    def writef2(self, u, ifr: int, jfr: int, workdir: str) -> str:
        """writef2 of a physical field into workdir/fields/w.NNN.MMM; returns the file path."""
        self._activate()
        os.makedirs(os.path.join(workdir, "fields"), exist_ok=True)
        cwd = os.getcwd()
        os.chdir(workdir)
        try:
            self._call("writef2", u, ints=(ifr, jfr))
        finally:
            os.chdir(cwd)
        return os.path.join(workdir, "fields", f"w.{ifr:03d}.{jfr:03d}")
