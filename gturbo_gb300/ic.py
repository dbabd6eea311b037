"""Initial conditions and the reference's field files.

``random_phase_ic`` draws the random-phase initial vorticity of the benchmark workloads:
energy spectrum E(k) ~ k^4 exp(-(k/k0)^2), uniform random phases, Hermitian on the kx=0 and
Nyquist columns, 2/3-truncated, zero mean, scaled so that the reference's energy
``ee`` (src/diagnostics.f90:150-156, fac=1/2 on the kx=0 and Nyquist columns) equals E0.
The reference itself starts from zero or from a restart file (src/inieuler.f90:90-95); its
noise generator (src/reset.sh:36, gen_noise.py) is not part of its repository.

``write_field`` / ``read_field`` use the reference's unformatted sequential real(4) format of
``fields/w.NNN`` (src/write.f90:3-20, src/read.f90:3-19): one record of NX*NY float32 values,
x fastest, framed by 4-byte record-length markers.
"""
from __future__ import annotations

import numpy as np

from .params import TWO_PI, Params


def wavenumbers(p: Params):
    """fkx over the NX/2+1 columns and fky over the NY rows (src/defk.f90:18-30)."""
    n, ny = p.n, p.rows
    dkx, dky = TWO_PI / p.xlx, TWO_PI / p.xly
    fkx = np.arange(n // 2 + 1) * dkx
    j = np.arange(ny)
    fky = np.where(j <= ny // 2, j, j - ny) * dky
    return fkx, fky


def trunc_mask(p: Params) -> np.ndarray:
    """True where src/trunc.f90:10-20 zeroes a mode (same arithmetic order)."""
    fkx, fky = wavenumbers(p)
    fkxs, fkys = fkx * fkx, fky * fky
    k1 = fkys / fkys[p.rows // 2]
    return (k1[:, None] + (fkxs / fkxs[p.n // 2])[None, :]) > p.rtrunc * p.rtrunc


def energy(p: Params, zk: np.ndarray) -> float:
    """The reference's global energy ee of a spectral field (NY, NX/2+1) complex."""
    fkx, fky = wavenumbers(p)
    k2 = fky[:, None] ** 2 + fkx[None, :] ** 2
    k2[0, 0] = 1.0
    fac = np.ones(k2.shape)
    fac[:, 0] = 0.5
    fac[:, -1] = 0.5
    w = fac * np.abs(zk) ** 2 / k2 ** (p.alpv / 2.0)
    w[0, 0] = 0.0
    return float(w.sum())


def random_phase_ic(p: Params, k0: float, e0: float = 0.5, seed: int = 1) -> np.ndarray:
    """Spectral initial field q_hat as an (NY, NX+2) float64 array (the ABI's memory layout)."""
    n, ny, nh = p.n, p.rows, p.n // 2 + 1
    fkx, fky = wavenumbers(p)
    k2 = fky[:, None] ** 2 + fkx[None, :] ** 2
    k = np.sqrt(k2)
    rng = np.random.default_rng(seed)
    theta = rng.uniform(0.0, 2.0 * np.pi, size=(ny, nh))
    with np.errstate(divide="ignore", invalid="ignore"):
        ek = k ** 4 * np.exp(-(k / k0) ** 2)
        # per-mode |q|^2 so that a shell of ~pi k half-plane modes carries E(k): |q|^2 / k^alpha
        amp2 = np.where(k > 0, ek * k ** p.alpv / (np.pi * k), 0.0)
    zk = np.sqrt(amp2) * np.exp(1j * theta)
    # Hermitian symmetry on the kx=0 and Nyquist columns: q(-ky) = conj q(ky)
    for col in (0, nh - 1):
        zk[ny // 2 + 1:, col] = np.conj(zk[1:ny // 2, col][::-1])
        zk[0, col] = zk[0, col].real
        zk[ny // 2, col] = zk[ny // 2, col].real
    zk[0, 0] = 0.0
    if p.truncate == 1:
        zk[trunc_mask(p)] = 0.0
    e = energy(p, zk)
    if e > 0.0:
        zk *= np.sqrt(e0 / e)
    out = np.ascontiguousarray(zk.astype(np.complex128)).view(np.float64).reshape(ny, n + 2)
    return out.copy()


def write_field(path: str, w: np.ndarray) -> None:
    """Write an N x N physical field as the reference's real(4) unformatted record."""
    w = np.asarray(w)
    n = w.shape[0]
    data = np.ascontiguousarray(w[:, :n], dtype="<f4")
    marker = np.array([data.nbytes], dtype="<i4").tobytes()
    with open(path, "wb") as f:
        f.write(marker)
        f.write(data.tobytes())
        f.write(marker)


def read_field(path: str, n: int) -> np.ndarray:
    """Read a reference real(4) field into an (N, N+2) float64 array, padding zeroed
    (src/read.f90:10-29)."""
    with open(path, "rb") as f:
        raw = f.read()
    nbytes = int(np.frombuffer(raw[:4], "<i4")[0])
    if nbytes != 4 * n * n or len(raw) != nbytes + 8:
        raise ValueError(f"{path}: not a {n}x{n} real(4) field record")
    w = np.frombuffer(raw[4:4 + nbytes], "<f4").reshape(n, n)
    out = np.zeros((n, n + 2))
    out[:, :n] = w
    return out
