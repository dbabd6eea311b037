"""Independent numpy restatement of the hot path: the cross-check of the C oracle.

TEST INFRASTRUCTURE ONLY. Written separately from ``gturbo_oracle.c`` (vectorised numpy,
numpy's pocketfft for the transforms) so that the two restatements check each other. Each
function cites the reference routine it follows. Spectral fields are complex (N, N/2+1)
arrays (``complex(8) z(N/2+1,N)``), physical fields real (N, N) arrays (the N+2 padding of
the reference is dropped here).
"""
from __future__ import annotations

import math

import numpy as np

from gturbo_gb300.params import Params

PI_DEFK = 3.14159265358979323846  # src/defk.f90:19-20
PI_FORC = 3.14159265358979        # src/forcing.f90:10 (truncated in the reference)


class NpOracle:
    def __init__(self, p: Params):
        if p.rows != p.n:
            raise ValueError("the numpy restatement takes square grids only")
        self.p = p
        n = self.n = p.n
        nh = self.nh = n // 2 + 1
        # inieuler.f90:22-36, 78-81
        split = 1 if (0.9995 < p.alpnu < 1.0005 and -0.0005 < p.alpmu < 0.0005) else 0
        if p.rko == 4:
            split = 0
        if p.split in (0, 1):
            split = p.split
        self.split = split
        self.rko = 4 if p.rko == 4 else 2
        self.dt, self.dt2, self.dt3, self.dt6 = p.dt, p.dt / 2.0, p.dt / 3.0, p.dt / 6.0
        self.sdt = math.sqrt(p.dt)
        # defk.f90:12-73
        self.dkx = 2.0 * PI_DEFK / p.xlx
        self.dky = 2.0 * PI_DEFK / p.xly
        self.fkx = np.arange(nh, dtype=np.float64) * self.dkx
        jj = np.arange(n)
        self.fky = np.where(jj <= n // 2, jj, jj - n).astype(np.float64) * self.dky
        self.fkxs = self.fkx * self.fkx
        self.fkys = self.fky * self.fky
        self.jc = np.where(jj == 0, 0, n - jj)
        k2 = self.fkys[:, None] + self.fkxs[None, :]
        self.k2 = k2
        with np.errstate(divide="ignore", invalid="ignore"):
            scra = p.nu * k2 ** p.alpnu + p.mu * k2 ** p.alpmu
            emk = np.exp(-0.5 * p.dt * scra)
        emk[0, 0] = 0.0
        self.emk = emk
        self.emky = np.exp(-0.5 * p.dt * (p.nu * self.fkys ** p.alpnu + p.mu))
        self.emkx = np.exp(-0.5 * p.dt * (p.nu * self.fkxs ** p.alpnu))
        self.fkxsmax = self.fkxs[n // 2]
        self.fkysmax = self.fkys[n // 2]
        self.rtrunc2 = p.rtrunc * p.rtrunc
        k1 = self.fkys / self.fkysmax
        self.trunc_mask = (k1[:, None] + (self.fkxs / self.fkxsmax)[None, :]) > self.rtrunc2
        with np.errstate(divide="ignore", invalid="ignore"):
            ka = k2 ** (p.alpv / 2.0)
        self.ka = ka
        # iniforcing.f90:11-68 (same mode order: kx=0 column, interior columns i-major, Nyquist)
        k2n = self.fkxs[None, :] / self.fkxsmax + self.fkys[:, None] / self.fkysmax
        ok = (k2n <= self.rtrunc2) & (k2 <= p.k2f ** 2) & (k2 > p.k1f ** 2)
        modes = []
        for j in range(1, n // 2 + 1):
            if ok[j, 0]:
                modes.append((0, j))
        cols = np.nonzero(ok[:, 1:n // 2].any(axis=0))[0] + 1
        for i in cols:
            for j in np.nonzero(ok[:, i])[0]:
                modes.append((int(i), int(j)))
        for j in range(0, n // 2 + 1):
            if ok[j, n // 2]:
                modes.append((n // 2, j))
        if len(modes) > 2048:
            raise ValueError("NFORC too small !")
        self.modes = modes
        self.nf = len(modes)
        self.inpz = sum(p.famp ** 2 for _ in modes)
        self.inpe = 0.0
        for i, j in modes:
            self.inpe = self.inpe + p.famp ** 2 / (self.fkxs[i] + self.fkys[j]) ** (p.alpv / 2.0)

    # fft_inv.f90: unnormalised C2R; fft_dir.f90: R2C then /NY/NX
    def fft_inv(self, zk: np.ndarray) -> np.ndarray:
        n = self.n
        return np.fft.irfft2(zk, s=(n, n)) * (n * n)

    def fft_dir(self, x: np.ndarray) -> np.ndarray:
        n = self.n
        return np.fft.rfft2(x) / n / n

    def trunc(self, zk: np.ndarray) -> np.ndarray:  # trunc.f90:10-25
        out = zk.copy()
        out[self.trunc_mask] = 0.0
        out[0, 0] = 0.0
        return out

    def nlt(self, zk: np.ndarray) -> np.ndarray:  # nlt.f90:17-63
        with np.errstate(divide="ignore", invalid="ignore"):
            kx = self.fkx[None, :] / self.ka
            ky = self.fky[:, None] / self.ka
        kx[0, 0] = 0.0
        ky[0, 0] = 0.0
        uk = 1j * ky * zk          # u = -ky*Im z + i ky*Re z
        vk = -1j * kx * zk         # v = +kx*Im z - i kx*Re z
        uk[0, 0] = 0.0
        vk[0, 0] = 0.0
        q = self.fft_inv(zk)
        v = self.fft_inv(vk)
        u = self.fft_inv(uk)
        a = self.fft_dir(q * u)
        b = self.fft_dir(q * v)
        out = (self.fkx[None, :] * a.imag + self.fky[:, None] * b.imag) \
            - 1j * (self.fkx[None, :] * a.real + self.fky[:, None] * b.real)
        if self.p.truncate == 1:
            out = self.trunc(out)
        return out

    def _e(self):
        if self.split:
            return self.emky[:, None] * self.emkx[None, :]
        return self.emk

    def step(self, zk: np.ndarray) -> np.ndarray:  # rkstep.f90:2-76
        e = self._e()
        n1 = self.nlt(zk)
        znl = e * (zk + self.dt2 * n1)
        znl[0, 0] = 0.0
        n2 = self.nlt(znl)
        z = e * (e * zk + self.dt * n2)
        z[0, 0] = 0.0
        return z

    def step4(self, zk: np.ndarray) -> np.ndarray:  # rkstep.f90:82-131
        e = self.emk
        n1 = self.nlt(zk)
        znew = e * e * (zk + self.dt6 * n1)
        n2 = self.nlt(e * (zk + self.dt2 * n1))
        znew = znew + self.dt3 * e * n2
        n3 = self.nlt(e * zk + self.dt2 * n2)
        znew = znew + self.dt3 * e * n3
        n4 = self.nlt(e * (e * zk + self.dt * n3))
        z = znew + self.dt6 * n4
        z[0, 0] = 0.0
        return z

    def rk_step(self, zk):
        return self.step4(zk) if self.rko == 4 else self.step(zk)

    @staticmethod
    def rann(seed: int):  # forcing.f90:40-51
        x = (69069 * (seed & 0xFFFFFFFF) + 1) & 0x7FFFFFFF
        return float(np.float32(x / 2147483647.0)), x

    def forcing(self, zk: np.ndarray, seed: int):  # forcing.f90:16-33
        z = zk.copy()
        sf = self.sdt * self.p.famp
        pi2 = 2.0 * PI_FORC
        for (i, j) in self.modes:
            r, seed = self.rann(seed)
            te = pi2 * r
            cc, cs = math.cos(te), math.sin(te)
            z[j, i] = complex(z[j, i].real + sf * 1.0 * cc, z[j, i].imag + sf * 1.0 * cs)
            if i == 0 or i == self.nh - 1:
                jc = self.jc[j]
                z[jc, i] = complex(z[jc, i].real + sf * 1.0 * cc, z[jc, i].imag - sf * 1.0 * cs)
        return z, seed

    def diag(self, zk: np.ndarray, znl: np.ndarray | None = None):  # diagnostics.f90
        p, n, nh, nb = self.p, self.n, self.nh, self.n // 2
        k2 = self.k2
        k = np.sqrt(k2)
        ib = (k / self.dkx).astype(np.int64)  # 0-based bin = int(k/dk)
        a2 = np.abs(zk) ** 2
        fac = np.ones((n, nh))
        fac[:, 0] = 0.5
        fac[:, nh - 1] = 0.5
        live = np.ones((n, nh), bool)
        live[0, 0] = False
        inb = live & (ib < nb - 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            ka = self.ka
            sp = np.bincount(ib[inb], (fac * a2 / ka)[inb], minlength=nb)[:nb] / self.dkx
            sz = np.bincount(ib[inb], (fac * a2)[inb], minlength=nb)[:nb] / self.dkx
            ee = np.sum((fac * a2 / ka)[live])
            zz = np.sum((fac * a2)[live])
            dnu = np.sum((2 * fac * p.nu * k2 ** p.alpnu * a2)[live])
            dmu = np.sum((2 * fac * p.mu * k2 ** p.alpmu * a2)[live])
            enu = np.sum((2 * fac * p.nu * k2 ** (p.alpnu - p.alpv / 2) * a2)[live])
            emu = np.sum((2 * fac * p.mu * k2 ** (p.alpmu - p.alpv / 2) * a2)[live])
        out = dict(sp=sp, sz=sz, glob=np.array([ee, zz, dnu, dmu, enu, emu]))
        if znl is not None:
            ff = 2.0 * fac
            fz = (zk.real * znl.real + zk.imag * znl.imag)
            with np.errstate(divide="ignore", invalid="ignore"):
                fe = fz / ka
            flzm = np.bincount(ib[inb], (ff * fz)[inb], minlength=nb)[:nb]
            flem = np.bincount(ib[inb], (ff * fe)[inb], minlength=nb)[:nb]
            out["flz"] = np.cumsum(flzm[::-1])[::-1]
            out["fle"] = np.cumsum(flem[::-1])[::-1]
        return out


def to_phys_layout(zk: np.ndarray) -> np.ndarray:
    """Complex (N, N/2+1) -> the (N, N+2) float64 memory image used by the C oracle and the ABI."""
    n = zk.shape[0]
    return np.ascontiguousarray(zk.astype(np.complex128)).view(np.float64).reshape(n, n + 2).copy()


def from_phys_layout(a: np.ndarray) -> np.ndarray:
    n = a.shape[0]
    return a.view(np.complex128).reshape(n, n // 2 + 1).copy()
