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


def _shard_worker(rank, world, port, outdir):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from gturbo_gb300.replicas import shard_members, whole_job_rate
    costs = [4.0, 4.0, 2.0, 1.0, 1.0, 1.0, 1.0]
    mine = shard_members(costs, world)[rank]
    # each rank "advances" its own members (no collective on data); only rates combine
    units, smax, rate = whole_job_rate(len(mine) * 10, 1.0 + 0.5 * rank)
    np.save(os.path.join(outdir, f"s{rank}.npy"), np.array(mine + [-1] * (7 - len(mine))))
    np.save(os.path.join(outdir, f"u{rank}.npy"), np.array([units, smax, rate]))
    dist.barrier()
    dist.destroy_process_group()


def test_sharded_ensemble_rates_gloo_world2(tmp_path):
    world = 2
    mp.spawn(_shard_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    s0 = [i for i in np.load(tmp_path / "s0.npy") if i >= 0]
    s1 = [i for i in np.load(tmp_path / "s1.npy") if i >= 0]
    assert sorted(s0 + s1) == list(range(7)) and not set(s0) & set(s1)
    u0, u1 = np.load(tmp_path / "u0.npy"), np.load(tmp_path / "u1.npy")
    assert np.array_equal(u0, u1)
    assert u0[0] == 70 and u0[1] == 1.5 and u0[2] == pytest.approx(70 / 1.5)
