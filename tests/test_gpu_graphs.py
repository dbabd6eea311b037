"""CUDA graphs of the steps (gt_set_graphs) on the GPU.

A replayed step holds the same launches with the same arguments as the direct one, so results
must be bit-identical: for RK2 and RK4, with and without the fused kick (whose LCG state is
rewritten into the graph before every replay), over several steps, after the launch settings
change (a new capture), with more field sets than the handle keeps graphs for (eviction), and
with the graphs bypassed while the handle times its launches.
"""
import numpy as np
import pytest

from gturbo_gb300.params import Params
from oracle.coracle import Oracle
from tests.helpers import rand_field, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _params(n, rko, **kw):
    base = dict(n=n, alpv=2.0, rko=rko, k1f=4.0, k2f=7.0, nu=1e-12, alpnu=4.0, mu=0.05, dt=1e-3, famp=0.5)
    base.update(kw)
    return Params(**base)


def _pair(p):
    from gturbo_gb300.solver import Solver
    a, b = Solver(p), Solver(p)
    b.graphs = False
    assert a.graphs and not b.graphs
    return a, b


@pytest.mark.parametrize("n,rko", [(256, 4), (256, 2), (64, 4), (1024, 2), (512, 4)])
@pytest.mark.parametrize("forced", [False, True])
def test_graph_steps_bit_identical_to_direct(n, rko, forced):
    p = _params(n, rko)
    orc = Oracle(p)
    a, b = _pair(p)
    f0 = rand_field(orc, 7)
    za, zb = torch.from_numpy(f0).cuda(), torch.from_numpy(f0).cuda()
    wa, wb = a.work(), b.work()
    sa = sb = 481929
    for _ in range(5):
        if forced:
            sa = a.rk_step_forced(za, wa, sa)
            sb = b.rk_step_forced(zb, wb, sb)
        else:
            a.rk_step(za, wa)
            b.rk_step(zb, wb)
    torch.cuda.synchronize()
    assert a.graphs  # no fallback to direct launches happened
    assert sa == sb
    assert torch.equal(za, zb)
    # and against the oracle
    ref = f0.copy()
    s = 481929
    for _ in range(5):
        orc.rk_step(ref)
        if forced:
            s = orc.forcing(ref, s)
    assert rel_l2(za.cpu().numpy(), ref) < 1e-12


def test_graphs_follow_settings_fields_and_profiling():
    p = _params(256, 4)
    orc = Oracle(p)
    a, b = _pair(p)
    f0 = rand_field(orc, 8)
    # more field sets than the handle keeps graphs for (8): every step still right
    fields = [(torch.from_numpy(f0).cuda(), a.work()) for _ in range(10)]
    ref = torch.from_numpy(f0).cuda()
    wb = b.work()
    for rnd in range(2):
        for z, w in fields:
            a.rk_step(z, w)
        b.rk_step(ref, wb)
    torch.cuda.synchronize()
    for z, _ in fields:
        assert torch.equal(z, ref)
    a.graphs = True  # cycling through more field sets than it keeps graphs for turned them off
    # a change of launch variants or split mode captures a new graph
    for cv, rv, split in ((2, 2, 0), (3, 2, 0), (2, 1, 2)):
        a.variants = (cv, rv)
        a.col_split = split
        b.variants = (cv, rv)
        b.col_split = split
        z, w = fields[0]
        z.copy_(torch.from_numpy(f0))
        zb = torch.from_numpy(f0).cuda()
        for _ in range(2):
            a.rk_step(z, w)
            b.rk_step(zb, wb)
        torch.cuda.synchronize()
        assert torch.equal(z, zb), (cv, rv, split)
    # while timing its launches the handle launches directly and sees every kernel
    a.profile(True)
    z, w = fields[1]
    a.rk_step(z, w)
    prof = a.profile_read()
    a.profile(False)
    assert sum(v[1] for v in prof.values()) >= 12
    assert a.graphs


def test_handle_cycling_through_many_fields_falls_back_to_direct_launches():
    """A handle stepping more field sets in turn than it keeps graphs for would capture on every
    step; it goes back to direct launches (results unchanged) and gt_set_graphs(h, 1) re-arms it."""
    p = _params(128, 2)
    orc = Oracle(p)
    a, b = _pair(p)
    f0 = rand_field(orc, 9)
    fields = [(torch.from_numpy(f0).cuda(), a.work()) for _ in range(12)]
    ref, wb = torch.from_numpy(f0).cuda(), b.work()
    for _ in range(3):
        for z, w in fields:
            a.rk_step(z, w)
        b.rk_step(ref, wb)
    torch.cuda.synchronize()
    for z, _ in fields:
        assert torch.equal(z, ref)
    assert not a.graphs
    a.graphs = True
    assert a.graphs
