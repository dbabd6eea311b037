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
