"""Non-square grids NX != NY on the GPU, against the oracle.

The reference declares NX and NY separately (src/modules.f90:4) and carries them through defk,
iniforcing, trunc, fft_dir and the diagnostics; it plans its transforms as NY x NY
(src/main.f90:27,32), so a non-square run of it needs the plan's shape corrected, as the
transliterated reference in oracle/_ref does. The C oracle matches that transliteration on
non-square grids (tests/test_ref_pin.py); here the CUDA path is checked against the oracle:
every routine, both Runge-Kutta orders, alpha 1 and 2, the column variants and split modes that
run on such grids, the fused kick and a main-loop horizon with its spectra.
"""
import numpy as np
import pytest

from gturbo_gb300.params import Params
from oracle.coracle import Oracle, spec
from tests.helpers import rand_field, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-12
GRIDS = [(512, 256), (256, 1024), (64, 32), (32, 128), (128, 2048)]


def _params(nx, ny, **kw):
    base = dict(n=nx, ny=ny, alpv=1.0, rko=2, k1f=4.0, k2f=7.0, nu=1e-12, alpnu=4.0, mu=0.05, dt=1e-3,
                famp=0.3)
    base.update(kw)
    return Params(**base)


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _solver(p):
    from gturbo_gb300.solver import Solver
    return Solver(p)


@pytest.mark.parametrize("nx,ny", [(512, 256), (256, 1024)])
@pytest.mark.parametrize("rko", [2, 4])
@pytest.mark.parametrize("alpv", [1.0, 2.0])
def test_step_against_oracle(nx, ny, rko, alpv):
    p = _params(nx, ny, rko=rko, alpv=alpv)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 1)
    ref = a.copy()
    orc.rk_step(ref)
    z = _dev(a)
    sol.rk_step(z, sol.work())
    assert rel_l2(_host(z), ref) < TOL


@pytest.mark.parametrize("nx,ny", GRIDS)
def test_routines_against_oracle(nx, ny):
    p = _params(nx, ny)
    orc, sol = Oracle(p), _solver(p)
    info = sol.info
    assert (info.n, info.ny, info.nh, info.nbin) == (nx, ny, nx // 2 + 1, nx // 2)
    assert info.field_doubles == (nx + 2) * ny
    rng = np.random.default_rng(2)
    # fft_dir of a physical field
    a = orc.zeros()
    a[:, :nx] = rng.standard_normal((ny, nx))
    z = _dev(a)
    sol.fft_dir(z)
    b = a.copy()
    orc.fft_dir(b)
    assert rel_l2(_host(z), b) < TOL
    zk = rand_field(orc, 3)
    # fft_inv
    z = _dev(zk)
    sol.fft_inv(z)
    b = zk.copy()
    orc.fft_inv(b)
    assert rel_l2(_host(z)[:, :nx], b[:, :nx]) < TOL
    # trunc and produ: bit for bit
    c = zk.copy()
    spec(c)[:, -2:] += 0.25
    z = _dev(c)
    sol.trunc(z)
    orc.trunc(c)
    assert np.array_equal(_host(z), c)
    q, u, v = (rng.standard_normal((ny, nx + 2)) for _ in range(3))
    du, dv = _dev(u), _dev(v)
    sol.produ(_dev(q), du, dv)
    orc.produ(q, u, v)
    assert np.array_equal(_host(du), u) and np.array_equal(_host(dv), v)
    # nlt
    z, u, v = _dev(zk), sol.field(), sol.field()
    sol.nlt(z, u, v)
    b = zk.copy()
    orc.nlt(b)
    assert rel_l2(_host(z), b) < TOL
    znl = b
    # forcing: mode list and state
    ik, jk = sol.forcing_modes()
    ik2, jk2 = orc.forcing_modes()
    assert np.array_equal(ik, ik2) and np.array_equal(jk, jk2) and len(ik) > 0
    z = _dev(zk)
    s = sol.forcing(z, 481929)
    b = zk.copy()
    s2 = orc.forcing(b, 481929)
    assert s == s2 and np.abs(_host(z) - b).max() < 1e-15
    # diagnostics
    d = sol.diag(_dev(zk), _dev(znl))
    do = orc.diag(zk, znl)
    for k in ("sp", "sz", "fle", "flz", "glob"):
        assert np.abs(d[k] - do[k]).max() <= 1e-12 * np.abs(do[k]).max(), k
    # dump (N rows of NX real(4)) and restart
    rec = sol.dump_real4(_dev(zk))
    b = zk.copy()
    orc.fft_inv(b)
    assert rec.shape == (ny, nx)
    assert np.abs(rec.astype(np.float64) - b[:, :nx]).max() <= 1e-6 * np.abs(b[:, :nx]).max()
    back = _host(sol.load_real4(rec))
    w = orc.zeros()
    w[:, :nx] = rec.astype(np.float64)
    orc.fft_dir(w)
    orc.trunc(w)
    assert rel_l2(back, w) < TOL


@pytest.mark.parametrize("nx,ny", [(512, 256), (256, 1024), (128, 2048)])
@pytest.mark.parametrize("rko", [2, 4])
def test_variants_and_split_modes(nx, ny, rko):
    """Every column variant a non-square grid runs (1, 2 where NY allows), every row variant of
    NX, and the three column-split modes agree with the oracle."""
    p = _params(nx, ny, rko=rko, alpv=2.0)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 4)
    ref = a.copy()
    orc.rk_step(ref)
    cols = sol.supported_variants()
    assert cols and set(cols) <= {1, 2}
    for cv in cols:
        for rv in sol.supported_row_variants():
            for split in (0, 1, 2):
                sol.variants = (cv, rv)
                sol.col_split = split
                z = _dev(a)
                sol.rk_step(z, sol.work())
                assert rel_l2(_host(z), ref) < TOL, (cv, rv, split)
    with pytest.raises(Exception):
        sol.variants = (0, sol.supported_row_variants()[0])


@pytest.mark.parametrize("nx,ny", [(512, 256), (256, 1024)])
@pytest.mark.parametrize("rko", [2, 4])
def test_forced_step_equals_step_then_forcing(nx, ny, rko):
    p = _params(nx, ny, rko=rko)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 5)
    z1, z2 = _dev(a), _dev(a)
    s1 = sol.rk_step_forced(z1, sol.work(), 481929)
    sol.rk_step(z2, sol.work())
    s2 = sol.forcing(z2, 481929)
    assert s1 == s2
    assert torch.equal(z1, z2)


@pytest.mark.parametrize("nx,ny,rko,alpv", [(512, 256, 2, 1.0), (256, 1024, 4, 2.0)])
def test_main_loop_horizon(nx, ny, rko, alpv):
    """20 iterations of src/main.f90:97-137 with diagnostics every 10 steps: state to 1e-12,
    spectra to 1e-9."""
    p = _params(nx, ny, rko=rko, alpv=alpv)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 6)
    z, work, s = _dev(a), sol.work(), 481929
    ow = [orc.zeros() for _ in range(4)]
    so = 481929
    for ipas in range(1, 21):
        d = ipas % 10 == 0
        s, out = sol.main_step(z, s, work, diag=d)
        so, od = orc.main_step(a, so, diag=d, work=ow)
        assert s == so
        if d:
            for k in ("sp", "sz", "fle", "flz"):
                assert np.abs(out[k] - od[k]).max() <= 1e-9 * np.abs(od[k]).max(), k
    assert rel_l2(_host(z), a) < TOL


def test_square_only_paths_reject_non_square():
    """The ensemble, the tangent-linear model and the adjoint take square grids only."""
    import ctypes

    from gturbo_gb300 import _lib
    from gturbo_gb300.adjoint import gradient
    from gturbo_gb300.params import GtParams

    p = _params(256, 128)
    sol = _solver(p)
    z = sol.field()
    with pytest.raises(Exception):
        gradient(sol, z, 2, 481929, 4.0, 8.0, checkpoint=1)
    lib = _lib.load()
    arr = (GtParams * 1)(p.to_ctypes())
    keys = (ctypes.c_uint64 * 1)(7)
    h = ctypes.c_void_p()
    assert lib.gt_ens_create(arr, 1, keys, ctypes.byref(h)) == 1


@pytest.mark.parametrize("nx,ny,xlx,xly,rko", [(256, 256, 2.0, 4.0, 2), (256, 256, 2.0, 1.0, 4),
                                               (512, 256, 2.0, 3.0, 4), (128, 512, 1.0, 2.0, 2)])
def test_rectangular_domains(nx, ny, xlx, xly, rko):
    """Box lengths xlx != xly (params.dat's first record, src/inieuler.f90:13), so dkx != dky:
    the nonlinear term, the step, the kick and the diagnostics against the oracle."""
    import math
    p = _params(nx, ny, rko=rko, alpv=2.0, xlx=xlx * math.pi, xly=xly * math.pi, k1f=3.0, k2f=6.0)
    orc, sol = Oracle(p), _solver(p)
    assert sol.info.dkx != sol.info.dky or xlx == xly
    zk = rand_field(orc, 21)
    z, u, v = _dev(zk), sol.field(), sol.field()
    sol.nlt(z, u, v)
    b = zk.copy()
    orc.nlt(b)
    assert rel_l2(_host(z), b) < TOL
    d = sol.diag(_dev(zk), _dev(b))
    do = orc.diag(zk, b)
    for k in ("sp", "sz", "fle", "flz", "glob"):
        assert np.abs(d[k] - do[k]).max() <= 1e-12 * np.abs(do[k]).max(), k
    z = _dev(zk)
    s = sol.rk_step_forced(z, sol.work(), 481929)
    a = zk.copy()
    orc.rk_step(a)
    s2 = orc.forcing(a, 481929)
    assert s == s2
    assert rel_l2(_host(z), a) < TOL


@pytest.mark.parametrize("nx,ny,kw", [
    (512, 256, dict(alpnu=1.0, nu=1e-4, mu=0.0, alpmu=0.0)),  # split integrator (RK2)
    (256, 512, dict(truncate=0)),                             # no dealiasing
    (256, 1024, dict(rko=4, alpv=3.0)),
])
def test_edge_configurations(nx, ny, kw):
    p = _params(nx, ny, **kw)
    orc, sol = Oracle(p), _solver(p)
    if "alpnu" in kw:
        assert sol.info.split == 1
    a = rand_field(orc, 31, truncate=bool(p.truncate))
    ref = a.copy()
    orc.rk_step(ref)
    z = _dev(a)
    sol.rk_step(z, sol.work())
    assert rel_l2(_host(z), ref) < TOL


@pytest.mark.parametrize("nx,ny", [(512, 256), (256, 1024)])
def test_untruncated_input(nx, ny):
    """An input with modes beyond the 2/3 ellipse (the untruncated-input flag path of the column
    passes, with the column count at run time)."""
    p = _params(nx, ny)
    orc, sol = Oracle(p), _solver(p)
    a = rand_field(orc, 32, truncate=False)
    ref = a.copy()
    orc.nlt(ref)
    z, u, v = _dev(a), sol.field(), sol.field()
    sol.nlt(z, u, v)
    assert rel_l2(_host(z), ref) < TOL
