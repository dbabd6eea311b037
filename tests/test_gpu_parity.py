"""Parity of every C-ABI routine against the CPU oracle (same seeded inputs).

Tolerance: relative L2 <= 1e-12 (the single-step bound of the specification); integer and
mask work (trunc, forcing's LCG state, forced-mode table) must match exactly.
"""
import os

import numpy as np
import pytest

from gturbo_gb300.params import Params
from oracle.coracle import Oracle, spec
from tests.helpers import phys, rand_field, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12
SIZES = [16, 32, 64, 128, 256, 512]


def _solver(p):
    from gturbo_gb300.solver import Solver
    return Solver(p)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _params(n, **kw):
    base = dict(n=n, alpv=2.0, rko=4, k1f=3.0, k2f=5.0, nu=1e-12, alpnu=4.0, mu=0.05, dt=1e-3)
    base.update(kw)
    return Params(**base)


@pytest.mark.parametrize("n", SIZES + [1024, 2048])
def test_fft_inv(n):
    p = _params(n)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 1)
    ref = a.copy()
    orc.fft_inv(ref)
    z = _dev(a)
    sol.fft_inv(z)
    out = _host(z)
    assert rel_l2(phys(out), phys(ref)) < TOL
    assert np.all(out[:, n:] == 0.0)


@pytest.mark.parametrize("n", SIZES + [1024, 2048])
def test_fft_dir(n):
    p = _params(n)
    orc, sol = Oracle(p), _solver(p)
    rng = np.random.default_rng(2)
    a = np.zeros((n, n + 2))
    a[:, :n] = rng.standard_normal((n, n))
    ref = a.copy()
    orc.fft_dir(ref)
    z = _dev(a)
    sol.fft_dir(z)
    assert rel_l2(_host(z), ref) < TOL


@pytest.mark.parametrize("n", [64, 512, 2048])
def test_dump_real4(n, tmp_path):
    """The real(4) field dump equals the oracle's fft_inv rounded to float32 (src/write.f90)
    and round-trips through the reference's fields/w.NNN record format."""
    from gturbo_gb300.ic import read_field, write_field
    p = _params(n)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 21)
    ref = a.copy()
    orc.fft_inv(ref)
    w = sol.dump_real4(_dev(a))
    assert w.dtype == np.float32 and w.shape == (n, n)
    ref32 = ref[:, :n].astype(np.float32)
    assert np.all(np.abs(w - ref32) <= np.spacing(np.abs(ref32)))
    f = tmp_path / "w.001.001"
    write_field(str(f), w)
    assert np.array_equal(read_field(str(f), n)[:, :n], w.astype(np.float64))


@pytest.mark.parametrize("n,truncate", [(64, 1), (512, 1), (256, 0), (2048, 1)])
def test_load_real4_restart(n, truncate):
    """Restart from a real(4) record: readf's widening + fft_dir + trunc (src/read.f90:3-27,
    src/main.f90:89-92) against the oracle, and the dump -> restart round trip."""
    p = _params(n, truncate=truncate)
    orc, sol = Oracle(p), _solver(p)
    rng = np.random.default_rng(40 + n)
    w = rng.standard_normal((n, n)).astype(np.float32)
    ref = np.zeros((n, n + 2))
    ref[:, :n] = w.astype(np.float64)
    orc.fft_dir(ref)
    if truncate:
        orc.trunc(ref)
    z = sol.load_real4(w)
    assert rel_l2(_host(z), ref) < TOL
    # round trip: a truncated field, dumped as real(4) and restarted, within float rounding
    a = rand_field(orc, 41)
    w2 = sol.dump_real4(_dev(a))
    z2 = sol.load_real4(w2)
    back = _host(z2)
    assert rel_l2(back, a) < 1e-6
    ref2 = np.zeros((n, n + 2))
    ref2[:, :n] = w2.astype(np.float64)
    orc.fft_dir(ref2)
    if truncate:
        orc.trunc(ref2)
    assert rel_l2(back, ref2) < TOL


@pytest.mark.parametrize("n", [16, 64, 256, 1024])
def test_trunc_exact(n):
    p = _params(n)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 3, truncate=False)
    ref = a.copy()
    orc.trunc(ref)
    z = _dev(a)
    sol.trunc(z)
    assert np.array_equal(_host(z), ref)


def test_produ_exact():
    n = 64
    p = _params(n)
    orc, sol = Oracle(p), _solver(p)
    rng = np.random.default_rng(4)
    z, u, v = (rng.standard_normal((n, n + 2)) for _ in range(3))
    ru, rv = u.copy(), v.copy()
    orc.produ(z, ru, rv)
    du, dv = _dev(u), _dev(v)
    sol.produ(_dev(z), du, dv)
    assert np.array_equal(_host(du), ru) and np.array_equal(_host(dv), rv)


@pytest.mark.parametrize("n", SIZES + [1024])
@pytest.mark.parametrize("alpv", [0.5, 1.0, 2.0, 3.0])
def test_nlt(n, alpv):
    p = _params(n, alpv=alpv)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 5)
    ref = a.copy()
    orc.nlt(ref)
    z, u, v = _dev(a), sol.field(), sol.field()
    sol.nlt(z, u, v)
    assert rel_l2(_host(z), ref) < TOL


@pytest.mark.parametrize("n", [32, 256])
def test_nlt_untruncated_input(n):
    """A field with modes outside the 2/3 ellipse must give the reference's result too."""
    p = _params(n)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 6, truncate=False)
    ref = a.copy()
    orc.nlt(ref)
    z, u, v = _dev(a), sol.field(), sol.field()
    sol.nlt(z, u, v)
    assert rel_l2(_host(z), ref) < TOL
    # and a truncated field right after it (the flag must have been cleared)
    b = rand_field(orc, 7)
    ref = b.copy()
    orc.nlt(ref)
    z = _dev(b)
    sol.nlt(z, u, v)
    assert rel_l2(_host(z), ref) < TOL


@pytest.mark.parametrize("n", [32, 256])
def test_nlt_no_dealiasing(n):
    """truncate=0: every column is transformed and kept, in every launch variant."""
    p = _params(n, truncate=0)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 8, truncate=False)
    ref = a.copy()
    orc.nlt(ref)
    for v in sol.supported_variants():
        sol.variant = v
        z, u, vv = _dev(a), sol.field(), sol.field()
        sol.nlt(z, u, vv)
        assert rel_l2(_host(z), ref) < TOL, v


@pytest.mark.parametrize("n,rko,alpv", [(32, 2, 1.0), (64, 4, 2.0), (256, 2, 1.0), (256, 4, 2.0),
                                        (512, 4, 3.0), (1024, 2, 0.5)])
def test_step(n, rko, alpv):
    p = _params(n, rko=rko, alpv=alpv, dt=2e-3)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 9) * 50.0
    ref = a.copy()
    orc.rk_step(ref)
    z = _dev(a)
    sol.rk_step(z, sol.work())
    assert rel_l2(_host(z), ref) < TOL


def test_step_split_rk2():
    """alpnu=1, alpmu=0, RK2: the split integrator emkx(i)*emky(j) (rkstep.f90:21-27, 51-57)."""
    p = _params(128, rko=2, alpnu=1.0, alpmu=0.0, nu=1e-3)
    orc, sol = Oracle(p), _solver(p)
    assert orc.info.split == 1 and sol.info.split == 1
    a = rand_field(orc, 10)
    ref = a.copy()
    orc.rk_step(ref)
    for c in sol.supported_variants():  # every column variant, with each row variant in turn
        for r in sol.supported_row_variants():
            sol.variants = (c, r)
            z = _dev(a)
            sol.rk_step(z, sol.work())
            assert rel_l2(_host(z), ref) < TOL, (c, r)


@pytest.mark.parametrize("n,rko,kw", [(64, 2, {}), (64, 4, {}), (256, 4, dict(k1f=10.0, k2f=12.0)),
                                      (128, 2, dict(alpnu=1.0, alpmu=0.0, nu=1e-3)),
                                      (2048, 2, dict(k1f=20.0, k2f=22.0, alpv=1.0))])
def test_forced_step_equals_step_then_forcing(n, rko, kw):
    """gt_step_rk*_forced (the kick fused into the final stage's store) gives the same bits and
    the same LCG state as gt_step_rk* followed by gt_forcing, in every launch variant, and agrees
    with the oracle's step + forcing."""
    p = _params(n, rko=rko, famp=0.9, dt=2e-3, **kw)
    orc, sol = Oracle(p), _solver(p)
    assert sol.info.nf > 0
    a = rand_field(orc, 23) * 20.0
    ref = a.copy()
    orc.rk_step(ref)
    seed_ref = orc.forcing(ref, 481929)
    for c in sol.supported_variants():
        for r in sol.supported_row_variants():
            sol.variants = (c, r)
            z1, z2 = _dev(a), _dev(a)
            sol.rk_step(z1, sol.work())
            s1 = sol.forcing(z1, 481929)
            s2 = sol.rk_step_forced(z2, sol.work(), 481929)
            assert s1 == s2 == seed_ref, (c, r)
            assert torch.equal(z1, z2), (c, r)
            assert rel_l2(_host(z2), ref) < TOL, (c, r)


@pytest.mark.parametrize("n,rko,variant,truncate", [(512, 4, 2, 1), (512, 2, 1, 1), (1024, 2, 0, 1),
                                                    (1024, 4, 2, 1), (2048, 2, 1, 1), (2048, 2, 0, 1),
                                                    (1024, 2, 2, 0), (512, 4, 1, 0)])
def test_col_split_equals_one_cta_per_column(n, rko, variant, truncate):
    """The field-split column passes (one field of one column per CTA, q in the handle's scratch;
    pass C's epilogue by the column's second CTA, or shared by the column's 2-CTA cluster) agree
    with one CTA per column to rounding, for steps, forced steps, the nonlinear term of an
    untruncated field and the split integrator. The arithmetic is the same, but nvcc may contract
    a stage update into FMAs differently in the kernels, so the bits may differ by an ulp."""
    kw = dict(alpnu=1.0, alpmu=0.0, nu=1e-3) if (rko == 2 and n == 512) else {}
    p = _params(n, rko=rko, dt=1e-3, famp=0.5, truncate=truncate, **kw)
    orc, sol = Oracle(p), _solver(p)
    sol.variants = (variant, 1 if variant == 0 and n >= 2048 else variant)
    a = rand_field(orc, 25, truncate=bool(truncate)) * 20.0
    out = {}
    for split in (2, 1, 0):
        sol.col_split = split
        assert sol.col_split == split
        z = _dev(a)
        sol.rk_step(z, sol.work())
        z2 = _dev(a)
        s2 = sol.rk_step_forced(z2, sol.work(), 777)
        zu = _dev(rand_field(orc, 26, truncate=False))
        u, v = sol.field(), sol.field()
        sol.nlt(zu, u, v)
        out[split] = (_host(z), _host(z2), s2, _host(zu))
    ref = a.copy()
    orc.rk_step(ref)
    for split in (2, 1):
        assert out[split][2] == out[0][2]
        for k in (0, 1, 3):
            assert rel_l2(out[split][k], out[0][k]) < 1e-14, (split, k)
        assert rel_l2(out[split][0], ref) < TOL


@pytest.mark.parametrize("n,rko,cr", [(64, 4, (3, 3)), (256, 4, (3, 2)), (512, 2, (2, 1)), (1024, 2, (0, 0)),
                                     (2048, 2, (1, 1)), (2048, 4, (0, 1))])
def test_pdl_bit_identical(n, rko, cr):
    """Programmatic dependent launch of the pass kernels changes when a launch begins, not what
    it computes: several steps queued back to back (forced and unforced, with and without the
    field-split column passes) give the same bits with it on and off."""
    p = _params(n, rko=rko, dt=1e-3, famp=0.5)
    orc, sol = Oracle(p), _solver(p)
    sol.variants = cr
    a = rand_field(orc, 27) * 20.0
    out = {}
    for pdl in (True, False):
        sol.pdl = pdl
        assert sol.pdl == pdl
        res = []
        for split in (2, 1, 0):
            sol.col_split = split
            z, w = _dev(a), sol.work()
            seed = 4242
            for _ in range(3):
                seed = sol.rk_step_forced(z, w, seed)
                sol.rk_step(z, w)
            res.append((_host(z), seed))
        out[pdl] = res
    for (z1, s1), (z0, s0) in zip(out[True], out[False]):
        assert s1 == s0
        assert np.array_equal(z1, z0)


def test_forced_step_self_conjugate_mode():
    """Without truncation a forced mode can be its own conjugate partner (kx = 0, ky = N/2 or
    the Nyquist column): two kicks on one value. The forced step then runs the step and the
    forcing launch one after the other, with the same result."""
    p = _params(16, rko=2, truncate=0, rtrunc=1.0, k1f=7.5, k2f=8.5, famp=0.8, dt=1e-3)
    orc, sol = Oracle(p), _solver(p)
    ik, jk = sol.forcing_modes()
    assert any((i == 0 and j == 8) or (i == 8 and j in (0, 8)) for i, j in zip(ik, jk))
    a = rand_field(orc, 24, truncate=False)
    ref = a.copy()
    orc.rk_step(ref)
    seed_ref = orc.forcing(ref, 1234)
    z1, z2 = _dev(a), _dev(a)
    sol.rk_step(z1, sol.work())
    s1 = sol.forcing(z1, 1234)
    s2 = sol.rk_step_forced(z2, sol.work(), 1234)
    assert s1 == s2 == seed_ref
    assert torch.equal(z1, z2)
    assert rel_l2(_host(z2), ref) < TOL


@pytest.mark.parametrize("n,k1,k2", [(64, 3.0, 5.0), (256, 10.0, 12.0), (2048, 20.0, 22.0)])
def test_forcing(n, k1, k2):
    p = _params(n, k1f=k1, k2f=k2, famp=0.7)
    orc, sol = Oracle(p), _solver(p)
    ik, jk = orc.forcing_modes()
    gik, gjk = sol.forcing_modes()
    assert np.array_equal(ik, gik) and np.array_equal(jk, gjk)
    assert sol.info.nf == orc.info.nf and sol.info.inpe == pytest.approx(orc.info.inpe, rel=1e-15)
    a = rand_field(orc, 11)
    seed = 481929
    ref = a.copy()
    z = _dev(a)
    for _ in range(3):
        seed_ref = orc.forcing(ref, seed)
        seed_gpu = sol.forcing(z, seed)
        assert seed_ref == seed_gpu
        seed = seed_ref
    out = _host(z)
    assert np.abs(out - ref).max() < 1e-14 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("n,alpv", [(64, 2.0), (256, 1.0), (512, 0.5)])
def test_diag(n, alpv):
    p = _params(n, alpv=alpv, nu=1e-20, alpnu=8.0)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 12)
    b = a.copy()
    orc.nlt(b)
    ref = orc.diag(a, b)
    out = sol.diag(_dev(a), _dev(b))
    for k in ("sp", "sz", "glob"):
        assert rel_l2(out[k], ref[k]) < 1e-13, k
    for k in ("fle", "flz"):
        scale = np.abs(ref[k]).max()
        assert np.abs(out[k] - ref[k]).max() <= 1e-12 * scale, k


@pytest.mark.parametrize("n,alpv", [(128, 1.0), (512, 2.0), (2048, 1.0)])
def test_nonlinear_transfer_conserves_invariants_on_gpu(n, alpv):
    """Known answer: with 2/3 dealiasing the nonlinear term moves energy and enstrophy between
    shells without creating or destroying them, so the fluxes at the first shell (the total
    transfers, computed by the GPU's own nlt and diagnostics) vanish to roundoff."""
    p = _params(n, alpv=alpv)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 13)
    z = _dev(a)
    znl, u, v = z.clone(), sol.field(), sol.field()
    sol.nlt(znl, u, v)
    out = sol.diag(z, znl)
    zs, ns = spec(a), spec(_host(znl))
    scale = np.abs(zs * ns.conj()).sum()
    assert abs(out["flz"][0]) < 1e-12 * scale
    assert abs(out["fle"][0]) < 1e-12 * scale
    assert np.abs(out["flz"]).max() > 1e-6 * scale  # the transfer itself is not trivial


def test_main_loop_10_steps():
    """10 iterations of the main loop (step, diagnostics every 5, forcing) at 256^2, RK4."""
    from gturbo_gb300.params import config
    p = config("c1")
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 13)
    ref = a.copy()
    z = _dev(a)
    work = sol.work()
    s_ref = s_gpu = 481929
    for it in range(1, 11):
        s_ref, d_ref = orc.main_step(ref, s_ref, diag=(it % 5 == 0))
        s_gpu, d_gpu = sol.main_step(z, s_gpu, work, diag=(it % 5 == 0))
        assert s_ref == s_gpu
        if d_ref is not None:
            assert rel_l2(d_gpu["sp"], d_ref["sp"]) < 1e-11
    assert rel_l2(_host(z), ref) < 1e-11


@pytest.mark.parametrize("n,rko", [(4096, 2), (8192, 4)])
def test_step_large_grids(n, rko):
    """One step at the largest grids (512-thread CTAs, the 8192^2 roofline workload's RK4)."""
    p = _params(n, rko=rko, alpv=2.0, k1f=40.0, k2f=44.0, nu=1e-50, alpnu=8.0, dt=5e-5)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 15) * 1e4
    ref = a.copy()
    orc.rk_step(ref)
    z = _dev(a)
    sol.rk_step(z, sol.work())
    assert rel_l2(_host(z), ref) < TOL


@pytest.mark.parametrize("cfg", ["c1", "c5", "c2", "c3"])
def test_workload_against_reference_fixture(cfg):
    """Each benchmark workload (256^2 RK4, 1024^2 and the 2048^2 headline RK2, 8192^2 RK4; the
    reference's forcing and seed, from the workload's random-phase initial field) against the
    reference's own run of it: tests/golden/<cfg>_workload.npz, made by the transliterated
    reference (make_golden.make_workload). Main-loop iterations with the fused kick, diagnostics
    on every second one; seed, spectra, budgets and sampled modes."""
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import IC_K0, config
    from tests.golden import make_golden as m
    from tests.helpers import check_workload_fixture, workload_run

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"{cfg}_workload.npz"))
    p = config(cfg)
    sol = _solver(p)
    z = _dev(random_phase_ic(p, IC_K0[cfg], 0.5, seed=1))
    work = sol.work()
    seed, spectra, globs = workload_run(lambda zz, s, ipas, dg: sol.main_step(zz, s, work, diag=dg), z,
                                        m.WORKLOADS[cfg], m.WORKLOAD_IMIX)
    check_workload_fixture(g, _host(z), seed, spectra, globs)


def test_step_2048_rk2_headline():
    """One RK2 step of the 2048^2 alpha=1 workload against the oracle."""
    from gturbo_gb300.params import config
    p = config("c2")
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 14) * 1e3
    ref = a.copy()
    orc.rk_step(ref)
    z = _dev(a)
    sol.rk_step(z, sol.work())
    assert rel_l2(_host(z), ref) < TOL


@pytest.mark.parametrize("cfg", ["c1", "c2"])
def test_spectra_50_step_horizon(cfg):
    """Spectra, fluxes and budgets within 1e-9 after 50 main-loop steps (forcing from the
    reference's LCG and seed), from the workload's random-phase initial field."""
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import IC_K0, config
    p = config(cfg)
    orc, sol = Oracle(p), _solver(p)
    a = random_phase_ic(p, IC_K0[cfg], 0.5, seed=1)
    ref = a.copy()
    z = _dev(a)
    work = sol.work()
    owork = [orc.zeros() for _ in range(4)]
    s_ref = s_gpu = 481929
    for it in range(1, 51):
        s_ref, d_ref = orc.main_step(ref, s_ref, diag=(it == 50), work=owork)
        s_gpu, d_gpu = sol.main_step(z, s_gpu, work, diag=(it == 50))
    assert s_ref == s_gpu
    assert np.isfinite(ref).all()
    for k in ("sp", "sz", "glob"):
        assert rel_l2(d_gpu[k], d_ref[k]) < 1e-9, k
    for k in ("fle", "flz"):
        assert np.abs(d_gpu[k] - d_ref[k]).max() <= 1e-9 * np.abs(d_ref[k]).max(), k
    assert rel_l2(_host(z), ref) < 1e-10


@pytest.mark.parametrize("name", ["n32_a2_rk4", "n64_a1_rk2", "n64_a05_rk2_split", "n64x32_a2_rk4"])
def test_against_golden_vectors(name):
    """The CUDA path against the committed vectors of the reference's own statements
    (tests/golden/make_golden.py: the transliterated Fortran with the cuFFT shim)."""
    import os
    from tests.golden.make_golden import CASES
    p, _ = CASES[name]
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"{name}.npz"))
    sol = _solver(p)
    n = p.n
    a = np.zeros((p.rows, n + 2))
    a[:, :n] = g["phys_in"]
    z = _dev(a)
    sol.fft_dir(z)
    assert rel_l2(_host(z), g["fft_dir"]) < TOL
    z = _dev(g["spec_in"])
    sol.fft_inv(z)
    assert rel_l2(_host(z)[:, :n], g["fft_inv"]) < TOL
    z, u, v = _dev(g["spec_in"]), sol.field(), sol.field()
    sol.nlt(z, u, v)
    assert rel_l2(_host(z), g["nlt"]) < TOL
    z = _dev(g["spec_in"])
    sol.rk_step(z, sol.work())
    assert rel_l2(_host(z), g["step"]) < TOL
    z = _dev(g["spec_in"])
    s = 481929
    for _ in range(3):
        s = sol.forcing(z, s)
    assert s == int(g["forcing3_seed"][0])
    assert np.abs(_host(z) - g["forcing3"]).max() < 1e-14
    ik, jk = sol.forcing_modes()
    assert np.array_equal(ik, g["ikxf"]) and np.array_equal(jk, g["ikyf"])
    # diagnostics of the fixture's field and its nonlinear term (FP64 operands of the writes)
    d = sol.diag(_dev(g["spec_in"]), _dev(g["nlt"]))
    for k in ("sp", "sz", "fle", "flz", "glob"):
        ref = g["diag_" + k]
        assert np.abs(d[k] - ref).max() <= 1e-12 * np.abs(ref).max(), k
    # the dump record of fields/w.NNN.MMM, within one real(4) rounding
    rec = sol.dump_real4(_dev(g["spec_in"]))
    ulp = np.spacing(np.abs(g["dump_record"])).astype(np.float64)
    assert (np.abs(rec.astype(np.float64) - g["dump_record"]) <= ulp).all()
    # the main loop (step, diagnostics every HORIZON_IMIX, forcing) over the fixture's horizon
    from tests.golden.make_golden import HORIZON_IMIX, HORIZON_STEPS
    z, work, s = _dev(g["spec_in"]), sol.work(), 481929
    spectra = []
    for ipas in range(1, HORIZON_STEPS + 1):
        s, out = sol.main_step(z, s, work, diag=(ipas % HORIZON_IMIX == 0))
        if out is not None:
            spectra.append(np.stack([out["sp"], out["sz"], out["fle"], out["flz"]]))
    assert s == int(g["horizon_seed"][0])
    assert rel_l2(_host(z), g["horizon_z"]) < TOL
    got, ref = np.stack(spectra), g["horizon_spectra"]
    for k in range(4):
        assert np.abs(got[:, k] - ref[:, k]).max() <= 1e-9 * np.abs(ref[:, k]).max()


def test_single_mode_decay_on_gpu():
    p = _params(64, rko=2, alpv=1.0, nu=1e-6, alpnu=2.0, mu=0.3)
    orc, sol = Oracle(p), _solver(p)
    a = orc.zeros()
    spec(a)[5, 3] = 0.7 - 0.2j
    z, u, v = _dev(a), sol.field(), sol.field()
    sol.nlt(z, u, v)
    assert np.abs(_host(z)).max() < 1e-15
    z = _dev(a)
    sol.rk_step(z, sol.work())
    e = orc.emk()[5, 3]
    assert spec(_host(z))[5, 3] == pytest.approx(e * e * (0.7 - 0.2j), rel=1e-14)


# -- launch variants of the nonlinear-term passes and the autotuner ------------------------
@pytest.mark.parametrize("n", [16, 64, 256, 1024, 4096])
def test_nlt_variants(n):
    """Every launch variant gives the oracle's nonlinear term."""
    p = _params(n, alpv=1.0)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 21)
    ref = a.copy()
    orc.nlt(ref)
    assert sol.supported_variants()[0] == 0
    for v in sol.supported_variants():
        sol.variant = v
        z, u, vv = _dev(a), sol.field(), sol.field()
        sol.nlt(z, u, vv)
        assert rel_l2(_host(z), ref) < TOL, f"variant {v}"


@pytest.mark.parametrize("n,rko", [(32, 4), (256, 2), (1024, 4)])
def test_step_variants_untruncated(n, rko):
    """Steps from an untruncated field (every column live in pass B) in every variant."""
    p = _params(n, rko=rko, dt=2e-3)
    orc = Oracle(p)
    a = rand_field(orc, 22, truncate=False) * 20.0
    ref = a.copy()
    orc.rk_step(ref)
    orc.rk_step(ref)
    sol = _solver(p)
    for v in sol.supported_variants():
        sol.variant = v
        z, work = _dev(a), sol.work()
        sol.rk_step(z, work)
        sol.rk_step(z, work)
        assert rel_l2(_host(z), ref) < TOL, f"variant {v}"


@pytest.mark.parametrize("n,rko", [(64, 4), (512, 2), (2048, 2)])
def test_mixed_row_and_column_variants(n, rko):
    """Every (column variant, row variant) pair steps like the oracle."""
    p = _params(n, rko=rko, dt=2e-3 if n <= 512 else 2e-4)
    orc = Oracle(p)
    a = rand_field(orc, 24, truncate=False) * 20.0
    ref = a.copy()
    orc.rk_step(ref)
    sol = _solver(p)
    for c in sol.supported_variants():
        for r in sol.supported_row_variants():
            sol.variants = (c, r)
            assert sol.variants == (c, r)
            z = _dev(a)
            sol.rk_step(z, sol.work())
            assert rel_l2(_host(z), ref) < TOL, (c, r)


def test_variant_rejected_when_unsupported():
    from gturbo_gb300._lib import GturboError
    sol = _solver(_params(2048))
    assert sol.supported_variants() == [0, 1]
    before = sol.variants
    with pytest.raises(GturboError):
        sol.variant = 2
    assert sol.variants == before  # a rejected variant leaves the handle's pair unchanged


def test_autotune_and_cache(tmp_path):
    p = _params(256, rko=2, dt=2e-3)
    sol = _solver(p)
    cache = str(tmp_path / "tune.json")
    res = sol.autotune(steps=5, cache=cache)
    assert not res["cached"]
    assert res["variant"] in sol.supported_variants() and sol.variant == res["variant"]
    assert sol.variants == (res["variant"], res["row_variant"])
    ms = res["ms_per_step"]
    assert all(ms[v] > 0 for v in sol.supported_variants())
    assert ms[res["variant"]] == min(ms[v] for v in sol.supported_variants())
    # a second solver reuses the stored choice without timing
    sol2 = _solver(p)
    res2 = sol2.autotune(steps=5, cache=cache)
    assert res2["cached"] and sol2.variants == (res["variant"], res["row_variant"])
    # and the tuned handle still steps exactly like the oracle
    orc = Oracle(p)
    a = rand_field(orc, 23) * 50.0
    ref = a.copy()
    orc.rk_step(ref)
    z = _dev(a)
    sol2.rk_step(z, sol2.work())
    assert rel_l2(_host(z), ref) < TOL


def test_host_pipeline_matches_serial_loop():
    """HostPipeline (copies on their own streams, two device buffers) gives the results of the
    plain upload -> step -> download loop, bit for bit."""
    from gturbo_gb300.pipeline import HostPipeline
    p = _params(256, rko=4, dt=2e-3)
    sol = _solver(p)
    orc = Oracle(p)
    inputs = [torch.from_numpy(rand_field(orc, 30 + k) * 30.0).pin_memory() for k in range(3)]
    outs = [torch.empty_like(inputs[0]).pin_memory() for _ in range(5)]
    work = sol.work()
    pipe = HostPipeline(sol)
    seed_p = pipe.run(inputs, outs, 5, 481929, work, diag_every=2)
    pipe.sync()
    seed = 481929
    for k in range(5):
        z = inputs[k % 3].cuda()
        seed, _ = sol.main_step(z, seed, work, diag=(k + 1) % 2 == 0)
        torch.cuda.synchronize()
        assert torch.equal(z.cpu(), outs[k]), k
    assert seed == seed_p


@pytest.mark.parametrize("n", [64, 512, 1024])
def test_nlt_partly_untruncated_input(n):
    """Modes beyond the 2/3 ellipse in a few columns only, exact zeros in the columns past them:
    pass A transforms the nonzero columns and raises the flag, stores zeros for the all-zero
    column blocks, and pass B reads every column (in every launch variant)."""
    p = _params(n)
    orc = Oracle(p)
    a = rand_field(orc, 25)
    full = rand_field(orc, 26, truncate=False)
    kx0 = n // 3 + 1
    zs, fs = spec(a), spec(full)
    zs[:, kx0:kx0 + 2] = fs[:, kx0:kx0 + 2]  # two columns just past the ellipse
    ref = a.copy()
    orc.nlt(ref)
    sol = _solver(p)
    for v in sol.supported_variants():
        sol.variant = v
        u, vv = sol.field(), sol.field()
        # stale data in the scratch fields, as a previous evaluation would leave
        u.fill_(7.0)
        vv.fill_(-3.0)
        z = _dev(a)
        sol.nlt(z, u, vv)
        assert rel_l2(_host(z), ref) < TOL, v
