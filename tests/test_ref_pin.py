"""The oracle pinned to the reference's own statements (CPU, no GPU).

``oracle/_ref`` is the reference's Fortran library sources transliterated mechanically into C
(``oracle/f2c_ref.py``; the cuFFT calls answered by a shim following cuFFT's documented transform
definitions). These tests compare the C oracle with it routine by routine: bit for bit where no
transform is involved (defk's tables, iniforcing's mode list and inputs, rann/the LCG, trunc,
produ, forcing, the diagnostics of identical inputs), to rounding where two FFT implementations
meet. The committed golden vectors must equal a fresh computation by the reference.

The transliteration needs the reference checkout; where it is absent (a copy of the repository
without it) the tests that need it skip, and the golden-vector tests carry the pin.
"""
import os

import numpy as np
import pytest

from gturbo_gb300.params import Params
from oracle import refcore
from oracle.coracle import Oracle, spec
from tests.helpers import check_workload_fixture, rand_field, rel_l2, workload_run

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
needs_ref = pytest.mark.skipif(not refcore.available(), reason="reference sources not present")


def _p(n, **kw):
    base = dict(n=n, alpv=2.0, rko=4, k1f=3.0, k2f=5.0, nu=1e-10, alpnu=4.0, mu=0.05, dt=1e-3,
                famp=0.4)
    base.update(kw)
    return Params(**base)


CASES = [
    _p(16, alpv=2.0, rko=4),
    _p(32, alpv=1.0, rko=2),
    _p(64, alpv=0.5, rko=4, k1f=6.0, k2f=8.0),
    _p(64, alpv=3.0, rko=2, truncate=0),
    _p(128, alpv=1.0, rko=2, nu=1e-4, alpnu=1.0, mu=0.0, alpmu=0.0),  # split integrator
    _p(256, alpv=2.0, rko=4, k1f=10.0, k2f=12.0, nu=1e-30, alpnu=8.0),
]
IDS = ["n16a2rk4", "n32a1rk2", "n64a05rk4", "n64a3rk2_notrunc", "n128a1rk2_split", "n256a2rk4"]
# non-square grids NX x NY (the reference declares NX and NY separately, modules.f90:4)
CASES += [
    _p(64, ny=32, alpv=1.0, rko=2),
    _p(32, ny=64, alpv=2.0, rko=4),
    _p(128, ny=64, alpv=0.5, rko=4, k1f=6.0, k2f=8.0),
    _p(64, ny=256, alpv=2.0, rko=2, nu=1e-4, alpnu=1.0, mu=0.0, alpmu=0.0),  # split integrator
]
IDS += ["n64x32a1rk2", "n32x64a2rk4", "n128x64a05rk4", "n64x256a2rk2_split"]
# rectangular domains xlx != xly (params.dat carries both, inieuler.f90:13): dkx != dky
import math  # noqa: E402
CASES += [
    _p(64, xly=4.0 * math.pi, alpv=1.0, rko=2, k1f=2.0, k2f=4.0),
    _p(64, ny=128, xlx=math.pi, xly=3.0 * math.pi, alpv=2.0, rko=4, k1f=3.0, k2f=6.0),
]
IDS += ["n64a1rk2_Ly2", "n64x128a2rk4_Lx05_Ly15"]


@needs_ref
@pytest.mark.parametrize("p", CASES, ids=IDS)
def test_tables_modes_and_inputs_bit_exact(p):
    """defk (defk.f90:12-73) and iniforcing (iniforcing.f90:11-68) against the oracle."""
    r, o = refcore.Reference(p), Oracle(p)
    t = r.tables()
    assert np.array_equal(t["emk"], o.emk())
    ik, jk = r.forcing_modes()
    ik2, jk2 = o.forcing_modes()
    assert np.array_equal(ik, ik2) and np.array_equal(jk, jk2)
    info = r.info()
    assert info["nf"] == o.info.nf and info["split"] == o.info.split
    assert info["inpe"] == o.info.inpe and info["inpz"] == o.info.inpz
    assert info["fkxsmax"] == o.info.fkxsmax and info["rtrunc"] == o.info.rtrunc2


@needs_ref
def test_rann_sequence_bit_exact():
    r = refcore.Reference(CASES[0])
    from oracle.coracle import rann
    d1, s1 = r.rann(481929, 2000)
    d2, s2 = rann(481929, 2000)
    assert np.array_equal(d1, d2) and s1 == s2


@needs_ref
@pytest.mark.parametrize("p", CASES, ids=IDS)
def test_routines_against_reference(p):
    r, o = refcore.Reference(p), Oracle(p)
    n = p.n
    z = rand_field(o, 7, truncate=bool(p.truncate))
    # trunc and produ: no transform, bit for bit
    a, b = z.copy(), z.copy()
    spec(a)[:, -3:] += 0.5  # modes beyond the ellipse for trunc to clear
    spec(b)[:, -3:] += 0.5
    r.trunc(a)
    o.trunc(b)
    assert np.array_equal(a, b)
    rng = np.random.default_rng(3)
    q, u, v = (rng.standard_normal((p.rows, n + 2)) for _ in range(3))
    u1, v1, u2, v2 = u.copy(), v.copy(), u.copy(), v.copy()
    r.produ(q, u1, v1)
    o.produ(q, u2, v2)
    assert np.array_equal(u1, u2) and np.array_equal(v1, v2)
    # forcing: bit for bit, seed included
    a, b = z.copy(), z.copy()
    s1 = s2 = 481929
    for _ in range(3):
        s1 = r.forcing(a, s1)
        s2 = o.forcing(b, s2)
    assert s1 == s2 and np.array_equal(a, b)
    # the transforms and everything built on them: to rounding
    x = rng.standard_normal((p.rows, n))
    a, b = r.zeros(), o.zeros()
    a[:, :n] = x
    b[:, :n] = x
    r.fft_dir(a)
    o.fft_dir(b)
    assert rel_l2(a, b) < 2e-15
    for name, tol in (("fft_inv", 2e-15), ("nlt", 1e-13), ("rk_step", 1e-13)):
        a, b = z.copy(), z.copy()
        getattr(r, name)(a)
        getattr(o, name)(b)
        assert rel_l2(a, b) < tol, name


@needs_ref
@pytest.mark.parametrize("p", CASES, ids=IDS)
def test_diagnostics_against_reference(p):
    """spectrum/fluxes/glob (diagnostics.f90:19-166) of identical inputs: the FP64 operands of the
    reference's writes to rounding, the real(4) values it writes within one real(4) rounding."""
    r, o = refcore.Reference(p), Oracle(p)
    z = rand_field(o, 9, truncate=bool(p.truncate))
    znl = z.copy()
    o.nlt(znl)
    dr = r.diag(z, znl)
    do = o.diag(z, znl)
    for k in ("sp", "sz", "fle", "flz", "glob"):
        scale = np.abs(do[k]).max()
        assert np.abs(dr[k] - do[k]).max() <= 1e-13 * scale, k
        w32 = do[k].astype(np.float32).astype(np.float64)
        ulp = np.spacing(np.abs(w32).astype(np.float32)).astype(np.float64)
        assert (np.abs(dr["written"][k] - w32) <= ulp).all(), k


@needs_ref
@pytest.mark.parametrize("p", [CASES[1], CASES[2], CASES[4], CASES[6], CASES[9]],
                         ids=[IDS[1], IDS[2], IDS[4], IDS[6], IDS[9]])
def test_main_loop_horizon_against_reference(p):
    """30 iterations of src/main.f90:97-137 (step, diagnostics every 10, forcing) from the same
    field and seed: the state to 1e-12 and the spectra to 1e-9 (the specification's gates)."""
    r, o = refcore.Reference(p), Oracle(p)
    z1 = rand_field(o, 11)
    z2 = z1.copy()
    s1 = s2 = 481929
    work = [o.zeros() for _ in range(4)]
    for ipas in range(1, 31):
        s1, d1 = r.main_step(z1, s1, ipas, 10)
        s2, d2 = o.main_step(z2, s2, diag=(ipas % 10 == 0), work=work)
        assert s1 == s2
        if d1 is not None:
            for k in ("sp", "sz", "fle", "flz"):
                assert np.abs(d1[k] - d2[k]).max() <= 1e-9 * np.abs(d2[k]).max(), k
    assert rel_l2(z1, z2) < 1e-12


@needs_ref
@pytest.mark.parametrize("cfg,steps", [("c1", 6), ("c5", 3), ("c2", 3)])
def test_workload_configurations_against_reference(cfg, steps):
    """The benchmark workloads' own configurations (256^2 RK4; 1024^2 and 2048^2 alpha=1 RK2),
    from their random-phase initial fields: main-loop iterations with the diagnostics every
    second one, the state to 1e-12 and the spectra to 1e-9 against the reference's statements,
    the LCG seed exactly, and the tables, mode list and forcing inputs bit for bit."""
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import IC_K0, config

    p = config(cfg)
    r, o = refcore.Reference(p), Oracle(p)
    assert np.array_equal(r.tables()["emk"], o.emk())
    ik, jk = r.forcing_modes()
    ik2, jk2 = o.forcing_modes()
    assert np.array_equal(ik, ik2) and np.array_equal(jk, jk2)
    info = r.info()
    assert info["nf"] == o.info.nf and info["inpe"] == o.info.inpe and info["inpz"] == o.info.inpz
    z1 = random_phase_ic(p, IC_K0[cfg], 0.5, seed=1)
    z2 = z1.copy()
    s1 = s2 = 481929
    work = [o.zeros() for _ in range(4)]
    for ipas in range(1, steps + 1):
        s1, d1 = r.main_step(z1, s1, ipas, 2)
        s2, d2 = o.main_step(z2, s2, diag=(ipas % 2 == 0), work=work)
        assert s1 == s2
        if d1 is not None:
            for k in ("sp", "sz", "fle", "flz"):
                assert np.abs(d1[k] - d2[k]).max() <= 1e-9 * np.abs(d2[k]).max(), k
    assert rel_l2(z1, z2) < 1e-12


@needs_ref
def test_restart_files_round_trip_through_reference():
    """writef2 then readf (write.f90:29-51, read.f90:3-27): the real(4) record of the dump and its
    widened restart, against the oracle's fft_inv rounded to real(4)."""
    import tempfile

    p = CASES[2]
    r, o = refcore.Reference(p), Oracle(p)
    n = p.n
    z = rand_field(o, 13)
    a, b = z.copy(), z.copy()
    r.fft_inv(a)
    o.fft_inv(b)
    with tempfile.TemporaryDirectory() as wd:
        path = r.writef2(a, 3, 1, wd)
        raw = np.fromfile(path, dtype=np.uint8)
        assert raw[:4].view(np.int32)[0] == 4 * n * n == raw[-4:].view(np.int32)[0]
        rec = raw[4:-4].view(np.float32).reshape(n, n)
        ulp = np.spacing(np.abs(rec)).astype(np.float64)
        assert (np.abs(rec.astype(np.float64) - b[:, :n]) <= ulp).all()
        os.replace(path, os.path.join(wd, "fields", "w.003"))
        back = r.readf(3, wd)
    assert np.array_equal(back[:, :n], rec.astype(np.float64))
    assert not back[:, n:].any()


@needs_ref
@pytest.mark.parametrize("name", ["n32_a2_rk4", "n64_a1_rk2", "n64_a05_rk2_split", "n64x32_a2_rk4"])
def test_golden_vectors_are_the_reference(name, tmp_path, monkeypatch):
    """The committed fixtures equal a fresh computation by the transliterated reference."""
    from tests.golden import make_golden

    monkeypatch.setattr(make_golden, "OUT", str(tmp_path))
    p, seed = make_golden.CASES[name]
    make_golden.make_case(name, p, seed)
    fresh = np.load(tmp_path / f"{name}.npz")
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    assert sorted(fresh.files) == sorted(g.files)
    for k in g.files:
        assert np.array_equal(fresh[k], g[k]), k


@pytest.mark.parametrize("name", ["n32_a2_rk4", "n64_a1_rk2", "n64_a05_rk2_split", "n64x32_a2_rk4"])
def test_oracle_main_loop_against_golden_horizon(name):
    """The oracle reproduces the reference's 20-step main-loop fixture (no reference needed)."""
    from tests.golden.make_golden import CASES as GC, HORIZON_IMIX, HORIZON_STEPS

    p, _ = GC[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    o = Oracle(p)
    z = g["spec_in"].copy()
    s = 481929
    work = [o.zeros() for _ in range(4)]
    spectra = []
    for ipas in range(1, HORIZON_STEPS + 1):
        s, d = o.main_step(z, s, diag=(ipas % HORIZON_IMIX == 0), work=work)
        if d is not None:
            spectra.append(np.stack([d["sp"], d["sz"], d["fle"], d["flz"]]))
    assert s == int(g["horizon_seed"][0])
    assert rel_l2(z, g["horizon_z"]) < 1e-12
    ref = g["horizon_spectra"]
    got = np.stack(spectra)
    for k in range(4):
        assert np.abs(got[:, k] - ref[:, k]).max() <= 1e-9 * np.abs(ref[:, k]).max()
    assert np.array_equal(o.emk(), g["emk"])


WORKLOADS = ["c1", "c5", "c2", "c3"]


@needs_ref
@pytest.mark.parametrize("cfg", WORKLOADS)
def test_workload_fixture_is_the_reference(cfg, tmp_path, monkeypatch):
    """The committed workload fixtures equal a fresh computation by the reference."""
    from tests.golden import make_golden

    monkeypatch.setattr(make_golden, "OUT", str(tmp_path))
    make_golden.make_workload(cfg)
    fresh = np.load(tmp_path / f"{cfg}_workload.npz")
    g = np.load(os.path.join(GOLDEN, f"{cfg}_workload.npz"))
    assert sorted(fresh.files) == sorted(g.files)
    for k in g.files:
        assert np.array_equal(fresh[k], g[k]), k


@pytest.mark.parametrize("cfg", WORKLOADS)
def test_oracle_against_workload_fixture(cfg):
    """The C oracle runs each benchmark workload (from its random-phase initial field) as the
    reference did for the fixture."""
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import IC_K0, config
    from tests.golden import make_golden as m

    g = np.load(os.path.join(GOLDEN, f"{cfg}_workload.npz"))
    p = config(cfg)
    o = Oracle(p)
    z = random_phase_ic(p, IC_K0[cfg], 0.5, seed=1)
    assert np.array_equal(m.workload_mode_index(p, z), g["mode_index"])
    work = [o.zeros() for _ in range(4)]
    seed, spectra, globs = workload_run(
        lambda zz, s, ipas, dg: o.main_step(zz, s, diag=dg, work=work), z, m.WORKLOADS[cfg],
        m.WORKLOAD_IMIX)
    check_workload_fixture(g, z, seed, spectra, globs)
