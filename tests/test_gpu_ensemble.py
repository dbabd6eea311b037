"""Batched ensembles (gt_ens_*) and the Philox forcing on the GPU.

A member advanced in the batch must equal the same member advanced alone through the
single-field C-ABI (same tile functions: equal to roundoff), and both must match the oracle
(step/step4 followed by the oracle's Philox kick) within the single-step tolerance.
"""
import numpy as np
import pytest

from gturbo_gb300.params import Params
from oracle.coracle import Oracle
from tests.helpers import rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _members(rko=4):
    from gturbo_gb300.ensemble import Member
    from gturbo_gb300.params import famp_for_injection
    spec = [(128, 1.0), (256, 2.0), (128, 3.0), (512, 0.5), (256, 2.0), (1024, 1.0), (2048, 3.0)]
    out = []
    for m, (n, a) in enumerate(spec):
        p = Params(n=n, alpv=a, rko=rko, dt=0.1 / n, nu=1e-30, alpnu=8.0, mu=0.05,
                   k1f=n / 25.0, k2f=n / 25.0 + 2.0)
        p = p.replace(famp=famp_for_injection(p, 1.0))
        out.append(Member(params=p, key=0xABC0 + m, k0=n / 50.0, ic_seed=77 + m))
    return out


@pytest.mark.parametrize("rko", [4, 2])
@pytest.mark.parametrize("graph", [True, False])
def test_batched_equals_plain_loop(rko, graph):
    from gturbo_gb300.ensemble import Ensemble, PlainLoop
    members = _members(rko)
    ens = Ensemble(members, use_graph=graph)
    ens.load_ic()
    ref = [z.clone() for z in ens.z]
    plain = PlainLoop(members, ref)
    ens.set_step(5)
    plain.step_counter = 5
    ens.step(3)
    plain.step(3)
    torch.cuda.synchronize()
    assert ens.get_step() == 8
    # the batched kernels are separate instantiations of the same tile functions, so the
    # compiler may order FMAs differently: equal to roundoff, not bit for bit
    for a, b in zip(ens.z, ref):
        assert rel_l2(a.cpu().numpy(), b.cpu().numpy()) < 1e-14


def test_batched_members_match_oracle():
    from gturbo_gb300.ensemble import Ensemble
    members = _members(4)
    ens = Ensemble(members)
    ens.load_ic()
    host = [z.cpu().numpy().copy() for z in ens.z]
    ens.set_step(0)
    ens.step(2)
    torch.cuda.synchronize()
    for m, z0, z in zip(members, host, ens.z):
        orc = Oracle(m.params)
        ref = z0.copy()
        for s in range(2):
            orc.rk_step(ref)
            orc.forcing_philox(ref, m.key, s)
        assert rel_l2(z.cpu().numpy(), ref) < 1e-12, m.params.n


def test_forcing_philox_matches_oracle():
    from gturbo_gb300.solver import Solver
    p = Params(n=256, alpv=1.0, k1f=10.0, k2f=12.0, famp=0.3, dt=1e-3)
    orc, sol = Oracle(p), Solver(p)
    a = np.zeros((256, 258))
    ref = a.copy()
    z = torch.from_numpy(a).cuda()
    for step in (0, 1, 12345678901):
        orc.forcing_philox(ref, 99, step)
        sol.forcing_philox(z, 99, step)
    torch.cuda.synchronize()
    assert np.abs(z.cpu().numpy() - ref).max() < 1e-15


def test_ensemble_rejects_mixed_orders_and_sizes():
    from gturbo_gb300 import _lib
    from gturbo_gb300.ensemble import Ensemble, Member
    m4 = _members(4)[:2]
    m2 = _members(2)[:1]
    with pytest.raises(_lib.GturboError):
        Ensemble(m4 + m2)
    bad = [Member(params=Params(n=64, rko=4), key=1, k0=2.0, ic_seed=1)]
    with pytest.raises(_lib.GturboError):
        Ensemble(bad)


@pytest.mark.parametrize("tile", [16, 8, 4])
def test_every_tile_family_matches_oracle(tile):
    """The three tile families (16, 8, 4 values per thread; 128, 256, 512 threads per CTA) differ
    only in the radix decomposition of the transforms: each matches the oracle."""
    from gturbo_gb300.ensemble import Ensemble
    members = _members(4)
    ens = Ensemble(members)
    ens.tile = tile
    assert ens.tile == tile
    ens.load_ic()
    host = [z.cpu().numpy().copy() for z in ens.z]
    ens.set_step(0)
    ens.step(2)
    torch.cuda.synchronize()
    for m, z0, z in zip(members, host, ens.z):
        orc = Oracle(m.params)
        ref = z0.copy()
        for s in range(2):
            orc.rk_step(ref)
            orc.forcing_philox(ref, m.key, s)
        assert rel_l2(z.cpu().numpy(), ref) < 1e-12, (tile, m.params.n)
    with pytest.raises(Exception):
        ens.tile = 32


def test_autotune_restores_members_and_caches(tmp_path):
    """gt_ens_autotune times every family on the members' own fields and puts them back (with the
    Philox step counter): stepping after the autotuner equals stepping without it."""
    from gturbo_gb300.ensemble import Ensemble
    members = _members(2)
    a = Ensemble(members)
    b = Ensemble(members)
    for e in (a, b):
        e.load_ic()
        e.set_step(3)
    cache = str(tmp_path / "tune.json")
    res = a.autotune(steps=2, cache=cache)
    assert res["tile"] in (16, 8, 4) and not res["cached"]
    assert all(v > 0 for v in res["ms_per_step"].values())
    assert a.tile == res["tile"] and a.get_step() == 3
    b.tile = res["tile"]
    a.step(2)
    b.step(2)
    torch.cuda.synchronize()
    for x, y in zip(a.z, b.z):
        assert torch.equal(x, y)
    again = Ensemble(members).autotune(steps=2, cache=cache)
    assert again["cached"] and again["tile"] == res["tile"]
