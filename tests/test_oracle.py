"""CPU tests of the oracle: C restatement vs numpy restatement, golden vectors, the LCG closed
form and analytic known answers (no GPU)."""
import os

import numpy as np
import pytest

from gturbo_gb300.params import Params, config, famp_for_injection
from oracle.coracle import Oracle, rann, spec
from oracle.np_oracle import NpOracle, from_phys_layout, to_phys_layout
from tests.helpers import rand_field, rel_l2

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _p(n, **kw):
    base = dict(n=n, alpv=2.0, rko=4, k1f=3.0, k2f=5.0, nu=1e-10, alpnu=4.0, mu=0.05, dt=1e-3)
    base.update(kw)
    return Params(**base)


@pytest.mark.parametrize("n,alpv,rko", [(16, 2.0, 4), (32, 1.0, 2), (64, 0.5, 4), (128, 3.0, 2),
                                        (256, 2.0, 4)])
def test_c_oracle_matches_numpy_restatement(n, alpv, rko):
    p = _p(n, alpv=alpv, rko=rko)
    o, q = Oracle(p), NpOracle(p)
    a = rand_field(o, 1)
    zk = from_phys_layout(a)
    b = a.copy()
    o.fft_inv(b)
    assert rel_l2(b[:, :n], q.fft_inv(zk)) < 1e-14
    b = a.copy()
    o.nlt(b)
    assert rel_l2(spec(b), q.nlt(zk)) < 1e-13
    b = a.copy()
    o.rk_step(b)
    assert rel_l2(spec(b), q.rk_step(zk)) < 1e-13
    b = a.copy()
    s1 = o.forcing(b, 481929)
    ref, s2 = q.forcing(zk, 481929)
    assert s1 == s2 and np.abs(spec(b) - ref).max() < 1e-15
    d1 = o.diag(a, to_phys_layout(q.nlt(zk)))
    d2 = q.diag(zk, q.nlt(zk))
    for k in ("sp", "sz", "glob"):
        assert rel_l2(d1[k], d2[k]) < 1e-13, k
    for k in ("fle", "flz"):
        assert np.abs(d1[k] - d2[k]).max() <= 1e-13 * np.abs(d2[k]).max(), k


@pytest.mark.parametrize("name", ["n32_a2_rk4", "n64_a1_rk2", "n64_a05_rk2_split", "n64x32_a2_rk4"])
def test_c_oracle_against_golden(name):
    from tests.golden.make_golden import CASES
    p, _ = CASES[name]
    g = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    o = Oracle(p)
    n = p.n
    ik, jk = o.forcing_modes()
    assert np.array_equal(ik, g["ikxf"]) and np.array_equal(jk, g["ikyf"])
    assert o.info.inpe == pytest.approx(float(g["inpe"][0]), rel=1e-14)
    a = o.zeros()
    a[:, :n] = g["phys_in"]
    o.fft_dir(a)
    assert rel_l2(a, g["fft_dir"]) < 1e-14
    z = g["spec_in"].copy()
    o.fft_inv(z)
    assert rel_l2(z[:, :n], g["fft_inv"]) < 1e-14
    z = g["spec_in"].copy()
    o.nlt(z)
    assert rel_l2(z, g["nlt"]) < 1e-13
    z = g["spec_in"].copy()
    o.rk_step(z)
    assert rel_l2(z, g["step"]) < 1e-13
    z = g["spec_in"].copy()
    s = 481929
    for _ in range(3):
        s = o.forcing(z, s)
    assert s == int(g["forcing3_seed"][0])
    assert np.abs(z - g["forcing3"]).max() < 1e-14
    b = g["spec_in"].copy()
    o.nlt(b)
    d = o.diag(g["spec_in"].copy(), b)
    for k in ("sp", "sz", "glob"):
        assert rel_l2(d[k], g["diag_" + k]) < 1e-13, k


def test_lcg_closed_form_seed_481929():
    """rann (src/forcing.f90:40-51) against x_k = a^k x0 + c (a^k - 1)/(a - 1) mod 2^31."""
    draws, last = rann(481929, 1000)
    g = np.load(os.path.join(GOLDEN, "lcg_481929.npz"))
    assert np.array_equal(draws, g["draws"])
    a, c, m, x0 = 69069, 1, 2 ** 31, 481929
    for k in (1, 2, 10, 137, 1000):
        ak = pow(a, k, m * (a - 1))
        xk = (ak * x0 + c * (ak - 1) // (a - 1)) % m
        assert int(g["states"][k - 1]) == xk
        assert draws[k - 1] == np.float32(xk / (2 ** 31 - 1))
    assert last == int(g["states"][-1])


def test_rann_negative_seed_wraps_like_32bit_fortran():
    draws, s = rann(-5, 3)
    x = -5 & 0xFFFFFFFF
    for d in draws:
        x = (69069 * x + 1) & 0x7FFFFFFF
        assert d == np.float32(x / 2147483647.0)
    assert s == x


@pytest.mark.parametrize("cfg,nf", [("c1", 62), ("c2", 130)])
def test_forced_mode_count_and_injection(cfg, nf):
    p = config(cfg)
    o = Oracle(p)
    assert o.info.nf == nf
    assert o.info.inpe == pytest.approx(1.0, rel=1e-12)  # famp chosen for eps = 1
    assert famp_for_injection(p, 1.0) == pytest.approx(p.famp, rel=1e-15)


def test_nforc_overflow_is_an_error():
    p = _p(512, k1f=0.0, k2f=60.0)
    with pytest.raises(ValueError):
        Oracle(p)


def test_single_mode_decays_exactly():
    """For one Fourier mode (and its conjugate) u.grad q = 0, so a step is the exact decay
    z -> emk^2 z (RK2 and RK4 alike)."""
    for rko in (2, 4):
        p = _p(64, rko=rko, alpv=1.0, nu=1e-6, alpnu=2.0, mu=0.3)
        o = Oracle(p)
        a = o.zeros()
        s = spec(a)
        s[5, 3] = 0.7 - 0.2j
        b = a.copy()
        o.nlt(b)
        assert np.abs(b).max() < 1e-15
        z = a.copy()
        o.rk_step(z)
        e = o.emk()[5, 3]
        assert spec(z)[5, 3] == pytest.approx(e * e * (0.7 - 0.2j), rel=1e-14)


@pytest.mark.parametrize("alpv", [1.0, 2.0])
def test_nonlinear_transfer_conserves_energy_and_enstrophy(alpv):
    """With 2/3 dealiasing the nonlinear term conserves both quadratic invariants: the total
    transfers (fluxes at the first shell) vanish to roundoff."""
    p = _p(128, alpv=alpv)
    o = Oracle(p)
    a = rand_field(o, 3)
    b = a.copy()
    o.nlt(b)
    d = o.diag(a, b)
    scale_z = np.abs(spec(a) * spec(b).conj()).sum()
    assert abs(d["flz"][0]) < 1e-12 * scale_z
    assert abs(d["fle"][0]) < 1e-12 * scale_z


def test_forcing_keeps_hermitian_symmetry_of_edge_columns():
    p = _p(64, k1f=0.0, k2f=6.0)
    o = Oracle(p)
    a = rand_field(o, 4)
    o.forcing(a, 12345)
    s = spec(a)
    n = p.n
    for col in (0, n // 2):
        for j in range(1, n // 2):
            assert s[n - j, col] == pytest.approx(np.conj(s[j, col]), abs=1e-15)


def test_fft_round_trip_and_trunc_idempotent():
    p = _p(64)
    o = Oracle(p)
    rng = np.random.default_rng(5)
    x = np.zeros((64, 66))
    x[:, :64] = rng.standard_normal((64, 64))
    y = x.copy()
    o.fft_dir(y)
    o.fft_inv(y)
    assert rel_l2(y[:, :64], x[:, :64]) < 1e-14
    a = rand_field(o, 6, truncate=False)
    o.trunc(a)
    b = a.copy()
    o.trunc(b)
    assert np.array_equal(a, b)


def test_oracle_philox_matches_numpy_philox():
    """The oracle's Philox4x64-10 block equals numpy.random.Philox (whose first draw uses the
    counter + 1)."""
    from oracle.coracle import philox4x64_10
    M = 2 ** 64
    for ctr, key in [((0, 0, 0, 0), (0, 0)), ((7, 3, 0, 1), (123456789, 42)),
                     ((M - 1, M - 1, 5, 6), (M - 1, 1)), ((M - 1, M - 1, M - 1, M - 1), (5, M - 3))]:
        c = sum(x << (64 * i) for i, x in enumerate(ctr))
        k = sum(x << (64 * i) for i, x in enumerate(key))
        ref = [int(x) for x in np.random.Philox(counter=c, key=k).random_raw(4)]
        v = (c + 1) % 2 ** 256
        assert philox4x64_10([(v >> (64 * i)) & (M - 1) for i in range(4)], key) == ref


def test_philox_forcing_is_order_free_and_hermitian():
    p = _p(64, k1f=0.0, k2f=6.0)
    o = Oracle(p)
    a = o.zeros()
    o.forcing_philox(a, 7, 3)
    b = o.zeros()
    o.forcing_philox(b, 7, 3)
    assert np.array_equal(a, b)
    c = o.zeros()
    o.forcing_philox(c, 8, 3)
    assert not np.array_equal(a, c)
    s = spec(a)
    for col in (0, 32):
        for j in range(1, 32):
            assert s[64 - j, col] == pytest.approx(np.conj(s[j, col]), abs=1e-15)
    # unit-modulus kicks of size sqrt(dt) famp on every forced mode
    ik, jk = o.forcing_modes()
    amp = np.abs(s[jk, ik])
    assert np.allclose(amp[ik > 0], np.sqrt(p.dt) * p.famp, rtol=1e-14)


def test_ensemble_c4_members():
    from gturbo_gb300.ensemble import ensemble_c4
    ms = ensemble_c4()
    assert len(ms) == 64
    assert [m.params.n for m in ms].count(256) == 32 and [m.params.n for m in ms].count(1024) == 8
    assert set(m.params.alpv for m in ms) <= {0.5, 1.0, 2.0, 3.0}
    assert len(set(m.key for m in ms)) == 64
    for m in ms[::9]:
        assert Oracle(m.params).info.inpe == pytest.approx(1.0, rel=1e-12)
        assert m.params.dt == pytest.approx(0.25 / m.params.n)
