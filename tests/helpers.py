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
