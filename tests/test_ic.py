"""The random-phase initial field and the reference's real(4) field files."""
import numpy as np
import pytest

from gturbo_gb300.ic import energy, random_phase_ic, read_field, trunc_mask, write_field
from gturbo_gb300.params import Params, config
from oracle.coracle import Oracle, spec


@pytest.mark.parametrize("cfg,k0", [("c1", 5.0), ("c2", 10.0)])
def test_ic_energy_symmetry_truncation(cfg, k0):
    p = config(cfg)
    a = random_phase_ic(p, k0, 0.5, seed=1)
    s = spec(a)
    assert energy(p, s) == pytest.approx(0.5, rel=1e-12)
    # the oracle's global energy (src/diagnostics.f90 glob) agrees
    assert Oracle(p).diag(a)["glob"][0] == pytest.approx(0.5, rel=1e-12)
    assert np.all(s[trunc_mask(p)] == 0) and s[0, 0] == 0
    n = p.n
    for col in (0, n // 2):
        assert np.allclose(s[n // 2 + 1:, col], np.conj(s[1:n // 2, col][::-1]))
    # deterministic
    assert np.array_equal(a, random_phase_ic(p, k0, 0.5, seed=1))
    assert not np.array_equal(a, random_phase_ic(p, k0, 0.5, seed=2))


@pytest.mark.parametrize("nx,ny", [(128, 64), (64, 256)])
def test_ic_non_square(nx, ny):
    """NX x NY grids: the field is (NY, NX+2), carries E = 0.5 by the oracle's budgets, is
    truncated as the oracle's trunc truncates it, and is Hermitian on the kx=0 and Nyquist
    columns."""
    p = Params(n=nx, ny=ny, alpv=1.0)
    a = random_phase_ic(p, 6.0, 0.5, seed=4)
    assert a.shape == (ny, nx + 2)
    s = spec(a)
    orc = Oracle(p)
    assert orc.diag(a)["glob"][0] == pytest.approx(0.5, rel=1e-12)
    b = a.copy()
    orc.trunc(b)
    assert np.array_equal(a, b)
    assert np.all(s[trunc_mask(p)] == 0) and s[0, 0] == 0
    for col in (0, nx // 2):
        assert np.allclose(s[ny // 2 + 1:, col], np.conj(s[1:ny // 2, col][::-1]))


def test_ic_spectrum_shape():
    p = config("c1")
    a = random_phase_ic(p, 5.0, 0.5, seed=3)
    sp = Oracle(p).diag(a)["sp"]
    k = np.arange(len(sp)) + 0.5
    model = k ** 4 * np.exp(-(k / 5.0) ** 2)
    sel = slice(2, 12)
    ratio = sp[sel] / model[sel]
    assert ratio.std() / ratio.mean() < 0.25


def test_field_file_round_trip(tmp_path):
    p = Params(n=32)
    rng = np.random.default_rng(0)
    w = np.zeros((32, 34))
    w[:, :32] = rng.standard_normal((32, 32))
    f = tmp_path / "w.001"
    write_field(str(f), w)
    raw = f.read_bytes()
    assert len(raw) == 4 * 32 * 32 + 8
    assert np.frombuffer(raw[:4], "<i4")[0] == 4 * 32 * 32 == np.frombuffer(raw[-4:], "<i4")[0]
    r = read_field(str(f), 32)
    assert np.array_equal(r[:, :32], w[:, :32].astype(np.float32).astype(np.float64))
    assert np.all(r[:, 32:] == 0)
    with pytest.raises(ValueError):
        read_field(str(f), 64)
