"""Run parameters of the solver: the reference's ``params.dat`` plus the grid size.

``Params`` mirrors the ``gt_params`` struct of ``include/gturbo.h`` field by field.
The reference reads the same quantities in ``src/inieuler.f90:13-20``::

    xlx xly / nu alpnu mu alpmu alpv / dt rko / npas iout imix / rtrunc truncate / famp k1f k2f

and takes the grid size NX, NY from the compile-time constants in ``src/modules.f90:4``
(``n`` = NX; ``ny`` = NY, 0 for a square grid).
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
import re

TWO_PI = 2.0 * math.pi  # the reference's params.dat writes 6.2831853071795864769d0


class GtParams(ctypes.Structure):
    """ctypes image of ``gt_params`` (include/gturbo.h)."""

    _fields_ = [
        ("n", ctypes.c_int32),
        ("rko", ctypes.c_int32),
        ("truncate", ctypes.c_int32),
        ("split", ctypes.c_int32),
        ("xlx", ctypes.c_double),
        ("xly", ctypes.c_double),
        ("nu", ctypes.c_double),
        ("alpnu", ctypes.c_double),
        ("mu", ctypes.c_double),
        ("alpmu", ctypes.c_double),
        ("alpv", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("rtrunc", ctypes.c_double),
        ("famp", ctypes.c_double),
        ("k1f", ctypes.c_double),
        ("k2f", ctypes.c_double),
        ("ny", ctypes.c_int32),
        ("ny_pad_", ctypes.c_int32),
    ]


class GtInfo(ctypes.Structure):
    """ctypes image of ``gt_info`` (include/gturbo.h)."""

    _fields_ = [
        ("n", ctypes.c_int32),
        ("nh", ctypes.c_int32),
        ("nbin", ctypes.c_int32),
        ("rko", ctypes.c_int32),
        ("split", ctypes.c_int32),
        ("truncate", ctypes.c_int32),
        ("nf", ctypes.c_int32),
        ("ny", ctypes.c_int32),
        ("field_doubles", ctypes.c_int64),
        ("dkx", ctypes.c_double),
        ("dky", ctypes.c_double),
        ("inpz", ctypes.c_double),
        ("inpe", ctypes.c_double),
        ("fkxsmax", ctypes.c_double),
        ("fkysmax", ctypes.c_double),
        ("rtrunc2", ctypes.c_double),
    ]


@dataclasses.dataclass
class Params:
    """Physical and numerical parameters of one run (one ``params.dat``)."""

    n: int = 256
    xlx: float = TWO_PI
    xly: float = TWO_PI
    nu: float = 1.0e-30
    alpnu: float = 8.0
    mu: float = 0.05
    alpmu: float = 0.0
    alpv: float = 2.0
    dt: float = 1.0e-3
    rko: int = 4
    rtrunc: float = 2.0 / 3.0
    truncate: int = 1
    famp: float = 1.0
    k1f: float = 10.0
    k2f: float = 12.0
    split: int = -1  # -1: derived as src/inieuler.f90:22-36
    ny: int = 0  # NY (rows); 0: NY = NX = n
    # run control (src/inieuler.f90:17); not part of gt_params
    npas: int = 1000
    iout: int = 1000000
    imix: int = 100

    def to_ctypes(self) -> GtParams:
        return GtParams(
            n=int(self.n), rko=int(self.rko), truncate=int(self.truncate), split=int(self.split),
            xlx=float(self.xlx), xly=float(self.xly), nu=float(self.nu), alpnu=float(self.alpnu),
            mu=float(self.mu), alpmu=float(self.alpmu), alpv=float(self.alpv), dt=float(self.dt),
            rtrunc=float(self.rtrunc), famp=float(self.famp), k1f=float(self.k1f), k2f=float(self.k2f),
            ny=int(self.ny),
        )

    def replace(self, **kw) -> "Params":
        return dataclasses.replace(self, **kw)

    @property
    def nx(self) -> int:
        return self.n

    @property
    def rows(self) -> int:
        """NY, the number of rows of a field."""
        return self.ny if self.ny else self.n

    @property
    def square(self) -> bool:
        return self.rows == self.n

    @property
    def nh(self) -> int:
        return self.n // 2 + 1

    @property
    def field_doubles(self) -> int:
        return (self.n + 2) * self.rows

    @property
    def field_shape(self) -> tuple[int, int]:
        """(NY, NX + 2): the physical view real(8) z(NX+2, NY) of a field."""
        return (self.rows, self.n + 2)

    @property
    def spectral_bytes(self) -> int:
        """S = 16 * NY * (NX/2+1): one complex128 spectral field."""
        return 16 * self.rows * self.nh


_FORTRAN_REAL = re.compile(r"([0-9.+-]+)[dD]([+-]?[0-9]+)")


def _fnum(tok: str) -> float:
    return float(_FORTRAN_REAL.sub(r"\1e\2", tok))


def read_params_dat(text: str, n: int) -> Params:
    """Parse a reference ``params.dat`` (list-directed, 6 data lines; src/inieuler.f90:13-20).

    ``n`` is the grid size, a compile-time constant in the reference (src/modules.f90:4).
    """
    lines = [ln.split() for ln in text.splitlines() if ln.strip()]
    if len(lines) < 6:
        raise ValueError("params.dat: expected 6 data lines")
    xlx, xly = (_fnum(t) for t in lines[0][:2])
    nu, alpnu, mu, alpmu, alpv = (_fnum(t) for t in lines[1][:5])
    dt, rko = _fnum(lines[2][0]), int(_fnum(lines[2][1]))
    npas, iout, imix = (int(_fnum(t)) for t in lines[3][:3])
    rtrunc, truncate = _fnum(lines[4][0]), int(_fnum(lines[4][1]))
    famp, k1f, k2f = (_fnum(t) for t in lines[5][:3])
    return Params(n=n, xlx=xlx, xly=xly, nu=nu, alpnu=alpnu, mu=mu, alpmu=alpmu, alpv=alpv, dt=dt,
                  rko=rko, rtrunc=rtrunc, truncate=truncate, famp=famp, k1f=k1f, k2f=k2f,
                  npas=npas, iout=iout, imix=imix)


def nu8_scaled(n: int) -> float:
    """Hyperviscosity scaled to the truncation wavenumber: (2/3 * N/2)^-16."""
    return (2.0 / 3.0 * (n // 2)) ** -16


def forced_inv_sum(p: Params) -> float:
    """Sum over the forced modes of |k|^-alpha, enumerated as src/iniforcing.f90:11-68."""
    n = p.n
    dkx, dky = TWO_PI / p.xlx, TWO_PI / p.xly
    fkx = [i * dkx for i in range(n // 2 + 1)]
    fky = [(j if j <= n // 2 else j - n) * dky for j in range(n)]
    fkxsmax, fkysmax = fkx[-1] ** 2, fky[n // 2] ** 2
    r2 = p.rtrunc * p.rtrunc
    total = 0.0

    def add(i, j):
        nonlocal total
        k2 = fkx[i] ** 2 + fky[j] ** 2
        k2n = fkx[i] ** 2 / fkxsmax + fky[j] ** 2 / fkysmax
        if k2n <= r2 and p.k1f ** 2 < k2 <= p.k2f ** 2:
            total += k2 ** (-p.alpv / 2.0)

    # only |kx|, |ky| <= k2f can be forced: restrict the three loops of iniforcing to them
    kmax = int(math.ceil(p.k2f / min(dkx, dky))) + 1
    rows = sorted({j for j in range(n) if min(j, n - j) <= kmax})
    for j in rows:                                   # i = 1 (kx = 0), j = 2..NY/2+1
        if 1 <= j <= n // 2:
            add(0, j)
    for i in range(1, min(n // 2 - 1, kmax) + 1):     # i = 2..NX/2, all j
        for j in rows:
            add(i, j)
    if n // 2 <= kmax:                               # i = NX/2+1, j = 1..NY/2+1
        for j in rows:
            if j <= n // 2:
                add(n // 2, j)
    return total


def famp_for_injection(p: Params, eps: float = 1.0) -> float:
    """famp such that the reference's mean energy input inpe = sum famp^2 / k^alpha equals eps."""
    s = forced_inv_sum(p)
    if s <= 0.0:
        raise ValueError("no forced modes in the shell")
    return math.sqrt(eps / s)


def config(name: str) -> Params:
    """The benchmark workloads (synthetic; inputs are generated, no dataset is involved).

    ``c1`` plain 256^2 alpha=2 RK4; ``c2`` 2048^2 alpha=1 RK2 (headline); ``c3`` 8192^2 alpha=2
    RK4 (roofline run); ``c5`` 1024^2 alpha=1 RK2 (adjoint workload).

    The two SQG (alpha=1, RK2) workloads use a time step below the one first specified for
    them: with E=0.5 the initial field has u_max ~ 13, so dt=2e-4 at 2048^2 (and 5e-4 at
    1024^2) puts the advective CFL number at the truncation wavenumber near 1.8. RK2's
    stability region excludes the imaginary axis, and the run blows up once the cascade reaches
    k_max (within ~100 steps in the oracle as well as on the GPU). dt=2e-5 (c2) and dt=5e-5 (c5)
    keep that CFL number near 0.2. The cost of a step does not depend on dt.
    """
    if name == "c1":
        p = Params(n=256, nu=1.0e-30, alpnu=8.0, mu=0.05, alpmu=0.0, alpv=2.0, dt=1.0e-3, rko=4,
                   k1f=10.0, k2f=12.0, npas=1000, imix=100)
    elif name == "c2":
        p = Params(n=2048, nu=nu8_scaled(2048), alpnu=8.0, mu=0.1, alpmu=0.0, alpv=1.0, dt=2.0e-5,
                   rko=2, k1f=20.0, k2f=22.0, npas=2000, imix=100)
    elif name == "c3":
        p = Params(n=8192, nu=nu8_scaled(8192), alpnu=8.0, mu=0.02, alpmu=0.0, alpv=2.0, dt=5.0e-5,
                   rko=4, k1f=40.0, k2f=44.0, npas=200, imix=100)
    elif name == "c5":
        p = Params(n=1024, nu=nu8_scaled(1024), alpnu=8.0, mu=0.1, alpmu=0.0, alpv=1.0, dt=5.0e-5,
                   rko=2, k1f=10.0, k2f=12.0, npas=200, imix=100)
    else:
        raise KeyError(name)
    return p.replace(famp=famp_for_injection(p, 1.0))


# initial-condition peak wavenumber k0 of each workload
IC_K0 = {"c1": 5.0, "c2": 10.0, "c3": 20.0, "c5": 6.0}
