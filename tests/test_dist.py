"""Multi-process (replica) host logic on CPU with gloo, world_size 2: every rank advances its
own replica with no data-path collective; only the timing is combined."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from gturbo_gb300.replicas import replica_ic_seed, whole_job_rate


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, outdir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import Params
    from oracle.coracle import Oracle

    p = Params(n=32, alpv=1.0, rko=2, k1f=3.0, k2f=5.0, dt=1e-3, nu=1e-10, alpnu=4.0)
    o = Oracle(p)
    z = random_phase_ic(p, 4.0, 0.5, seed=replica_ic_seed(rank))
    seed = 481929
    for _ in range(3):
        seed, _ = o.main_step(z, seed)
    secs = 1.0 + rank  # a deterministic stand-in for the measured time
    units, smax, rate = whole_job_rate(3, secs)
    np.save(os.path.join(outdir, f"z{rank}.npy"), z)
    np.save(os.path.join(outdir, f"r{rank}.npy"), np.array([units, smax, rate]))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_gloo_world2(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    r0 = np.load(tmp_path / "r0.npy")
    r1 = np.load(tmp_path / "r1.npy")
    assert np.array_equal(r0, r1)
    assert r0[0] == 6 and r0[1] == 2.0 and r0[2] == pytest.approx(3.0)
    z0, z1 = np.load(tmp_path / "z0.npy"), np.load(tmp_path / "z1.npy")
    assert not np.allclose(z0, z1)  # independent replicas
    # each replica equals a single-process run with its own seed
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import Params
    from oracle.coracle import Oracle
    p = Params(n=32, alpv=1.0, rko=2, k1f=3.0, k2f=5.0, dt=1e-3, nu=1e-10, alpnu=4.0)
    o = Oracle(p)
    z = random_phase_ic(p, 4.0, 0.5, seed=replica_ic_seed(1))
    s = 481929
    for _ in range(3):
        s, _ = o.main_step(z, s)
    assert np.array_equal(z, z1)


def test_single_process_rate_without_group():
    assert whole_job_rate(10, 2.0) == (10.0, 2.0, 5.0)


def test_member_sharding_partitions_and_balances():
    """The ensemble shards by member: every member on exactly one rank, costs balanced."""
    from gturbo_gb300.ensemble import ensemble_c4
    from gturbo_gb300.replicas import member_cost, shard_members
    members = ensemble_c4()
    costs = [member_cost(m.params.n, m.params.rko) for m in members]
    for world in (1, 2, 3, 4, 8):
        shards = shard_members(costs, world)
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(members)))
        loads = [sum(costs[i] for i in s) for s in shards]
        assert max(loads) - min(loads) <= max(costs) + 1e-9
        assert shards == shard_members(costs, world)  # deterministic: every rank agrees
    with pytest.raises(ValueError):
        shard_members(costs, 0)


def _small_ensemble():
    """Six members of mixed size and alpha (RK4, Philox forcing), small enough for the oracle."""
    from gturbo_gb300.ensemble import Member
    from gturbo_gb300.params import Params, famp_for_injection

    out = []
    for m, (n, a) in enumerate(((32, 0.5), (64, 1.0), (32, 2.0), (64, 3.0), (32, 1.0), (64, 2.0))):
        p = Params(n=n, alpv=a, rko=4, dt=0.25 / n, nu=1e-12, alpnu=4.0, mu=0.05, alpmu=0.0,
                   k1f=n / 16.0, k2f=n / 16.0 + 2.0)
        p = p.replace(famp=famp_for_injection(p, 1.0))
        out.append(Member(params=p, key=0x6774_0000 + m, k0=n / 16.0, ic_seed=1000 + m))
    return out


def _advance(member, steps):
    """One member through the oracle: RK4 step, then the Philox kick at the step counter."""
    from gturbo_gb300.ic import random_phase_ic
    from oracle.coracle import Oracle

    o = Oracle(member.params)
    z = random_phase_ic(member.params, member.k0, 0.5, seed=member.ic_seed)
    for step in range(steps):
        o.step4(z)
        o.forcing_philox(z, member.key, step)
    return z


def _shard_worker(rank, world, port, outdir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from gturbo_gb300.replicas import member_cost, shard_members, whole_job_rate

    members = _small_ensemble()
    mine = shard_members([member_cost(m.params.n, m.params.rko) for m in members], world)[rank]
    # each rank advances its own members (no collective on the data path); only rates combine
    for i in mine:
        np.save(os.path.join(outdir, f"m{i}_r{rank}.npy"), _advance(members[i], 4))
    units, smax, rate = whole_job_rate(len(mine) * 4, 1.0 + 0.5 * rank)
    np.save(os.path.join(outdir, f"u{rank}.npy"), np.array([units, smax, rate]))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_ensemble_gloo_world2_equals_one_process(tmp_path):
    """Two gloo ranks each advance their shard of a mixed-size ensemble (RK4 + Philox kicks)
    through the oracle: every member is advanced by exactly one rank, and the union of the
    shards equals a single-process run of all members bit for bit."""
    world = 2
    mp.spawn(_shard_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    members = _small_ensemble()
    owners = {}
    for f in tmp_path.glob("m*_r*.npy"):
        i, r = (int(x) for x in f.stem[1:].split("_r"))
        assert i not in owners
        owners[i] = r
    assert sorted(owners) == list(range(len(members)))
    assert set(owners.values()) == {0, 1}
    for i, m in enumerate(members):
        got = np.load(tmp_path / f"m{i}_r{owners[i]}.npy")
        assert np.isfinite(got).all()
        assert np.array_equal(got, _advance(m, 4)), i
    u0, u1 = np.load(tmp_path / "u0.npy"), np.load(tmp_path / "u1.npy")
    assert np.array_equal(u0, u1)
    assert u0[0] == 4 * len(members) and u0[1] == 1.5
