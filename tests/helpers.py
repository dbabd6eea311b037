"""Shared helpers of the test suite (fields, comparisons)."""
import numpy as np

from oracle.coracle import Oracle, spec


def rand_field(orc: Oracle, seed: int, truncate: bool = True, hermitian: bool = True) -> np.ndarray:
    """A random spectral field in the (N, N+2) layout, from the oracle's fft_dir of a real field."""
    n = orc.n
    rng = np.random.default_rng(seed)
    a = orc.zeros()
    a[:, :n] = rng.standard_normal((a.shape[0], n))
    orc.fft_dir(a)
    if not hermitian:
        s = spec(a)
        s[:, 0] += 1e-3 * (rng.standard_normal(a.shape[0]) + 1j * rng.standard_normal(a.shape[0]))
    if truncate:
        orc.trunc(a)
    return a


def rel_l2(a, b) -> float:
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    if np.iscomplexobj(a) or np.iscomplexobj(b):
        a, b = a.astype(np.complex128), b.astype(np.complex128)
    else:
        a, b = a.astype(np.float64), b.astype(np.float64)
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def phys(a: np.ndarray) -> np.ndarray:
    """The NY x NX physical values of an (NY, NX+2) field (padding dropped)."""
    return a[:, : a.shape[1] - 2]


def workload_run(step, z, steps, imix):
    """Main-loop iterations through `step(z, seed, ipas, diag)`; the diagnostics and final seed."""
    s, spectra, globs = 481929, [], []
    for ipas in range(1, steps + 1):
        s, d = step(z, s, ipas, ipas % imix == 0)
        if d is not None:
            spectra.append(np.stack([d["sp"], d["sz"], d["fle"], d["flz"]]))
            globs.append(d["glob"])
    return s, np.stack(spectra), np.stack(globs)


def check_workload_fixture(g, z, seed, spectra, globs):
    """A run of the headline workload against the reference's fixture: the LCG seed exactly, the
    spectra and fluxes to 1e-9 and the budgets to 1e-12 (relative to their largest values), the
    sampled retained modes to 1e-12 (relative L2) and the total sum of |q|^2 to 1e-12."""
    assert int(seed) == int(g["seed"][0])
    for k in range(spectra.shape[1]):
        ref = g["spectra"][:, k]
        assert np.abs(spectra[:, k] - ref).max() <= 1e-9 * np.abs(ref).max(), k
    assert np.abs(globs - g["glob"]).max() <= 1e-12 * np.abs(g["glob"]).max()
    zc = spec(z).ravel()
    assert rel_l2(zc[g["mode_index"]], g["modes"]) < 1e-12
    assert abs(float(np.sum(np.abs(zc) ** 2)) - g["sum_abs2"][0]) <= 1e-12 * g["sum_abs2"][0]

