"""gt_diag_static: the diagnostics entry point that allocates no device memory.

It exists for callers that cannot allocate: a driver whose device arrays all belong to OpenACC
data regions or to another runtime's pool sized to fill the GPU, and host code that must not
call cudaMalloc/cudaFree between time steps because they synchronise the whole device. It keeps
its scratch in a static device array and takes only the caller's fields and output arrays.

This file sorts last so that a run stopping at the first failure has already run every other
test. It calls the entry point through the C-ABI twice in a row (the second call on a smaller
grid, so stale scratch from the first call would show) and checks each result against
gt_diag and against the oracle, with the tolerances of the other diagnostics tests; a third call
asks for one output only.
"""
import ctypes

import numpy as np
import pytest

from gturbo_gb300.params import Params
from oracle.coracle import Oracle
from tests.helpers import rand_field, rel_l2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _params(n, alpv):
    return Params(n=n, alpv=alpv, rko=2, k1f=3.0, k2f=5.0, nu=1e-20, alpnu=8.0, mu=0.05, dt=1e-3)


def _static_diag(lib, p, z, znl):
    nb = p.n // 2
    dev = z.device
    out = {k: torch.full((nb,), float("nan"), dtype=torch.float64, device=dev)
           for k in ("sp", "sz", "fle", "flz")}
    glob = torch.full((6,), float("nan"), dtype=torch.float64, device=dev)
    cp = p.to_ctypes()
    stream = torch.cuda.current_stream(dev).cuda_stream
    rc = lib.gt_diag_static(ctypes.byref(cp), z.data_ptr(), znl.data_ptr(),
                            out["sp"].data_ptr(), out["sz"].data_ptr(), out["fle"].data_ptr(),
                            out["flz"].data_ptr(), glob.data_ptr(), ctypes.c_void_p(stream))
    assert rc == 0, lib.gt_last_error(None)
    torch.cuda.synchronize()
    res = {k: v.cpu().numpy() for k, v in out.items()}
    res["glob"] = glob.cpu().numpy()
    return res


def test_diag_static_matches_gt_diag_on_two_calls():
    from gturbo_gb300 import _lib
    from gturbo_gb300.solver import Solver

    lib = _lib.load()
    for n, alpv, seed in ((256, 1.0, 31), (128, 2.0, 32)):
        p = _params(n, alpv)
        orc = Oracle(p)
        a = rand_field(orc, seed)
        b = a.copy()
        orc.nlt(b)
        z = torch.from_numpy(a).cuda()
        znl = torch.from_numpy(b).cuda()
        ref = Solver(p).diag(z, znl)
        direct = orc.diag(a, b)
        got = _static_diag(lib, p, z, znl)
        for k in ("sp", "sz", "glob"):
            assert np.isfinite(got[k]).all(), k
            assert rel_l2(got[k], ref[k]) < 1e-13, k
            assert rel_l2(got[k], direct[k]) < 1e-12, k
        for k in ("fle", "flz"):
            assert np.isfinite(got[k]).all(), k
            assert np.abs(got[k] - ref[k]).max() <= 1e-12 * np.abs(ref[k]).max(), k
            assert np.abs(got[k] - direct[k]).max() <= 1e-12 * np.abs(direct[k]).max(), k


def test_diag_static_subset_of_outputs_leaves_the_others_untouched():
    """znl = NULL with only sp requested (no fluxes, no budgets): sp matches the oracle and the
    output arrays that were not passed keep their NaN contents."""
    from gturbo_gb300 import _lib

    lib = _lib.load()
    p = _params(128, 1.0)
    orc = Oracle(p)
    a = rand_field(orc, 33)
    z = torch.from_numpy(a).cuda()
    nb = p.n // 2
    sp = torch.full((nb,), float("nan"), dtype=torch.float64, device="cuda")
    others = [torch.full((nb,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(3)]
    glob = torch.full((6,), float("nan"), dtype=torch.float64, device="cuda")
    cp = p.to_ctypes()
    rc = lib.gt_diag_static(ctypes.byref(cp), z.data_ptr(), None, sp.data_ptr(), None, None, None,
                            None, None)
    assert rc == 0, lib.gt_last_error(None)
    torch.cuda.synchronize()
    assert rel_l2(sp.cpu().numpy(), orc.diag(a)["sp"]) < 1e-12
    for t in others + [glob]:
        assert torch.isnan(t).all()
    # fluxes without znl are refused
    rc = lib.gt_diag_static(ctypes.byref(cp), z.data_ptr(), None, None, None, others[0].data_ptr(),
                            None, None, None)
    assert rc == 1  # GT_ERR_ARG


def test_diag_static_rejects_grid_beyond_its_scratch():
    from gturbo_gb300 import _lib

    lib = _lib.load()
    p = _params(4096, 1.0)
    z = torch.zeros((16,), dtype=torch.float64, device="cuda")
    cp = p.to_ctypes()
    rc = lib.gt_diag_static(ctypes.byref(cp), z.data_ptr(), None, None, None, None, None,
                            z.data_ptr(), None)
    assert rc == 1  # GT_ERR_ARG
    assert b"GT_DIAG_STATIC_MAX_N" in lib.gt_last_error(None)
