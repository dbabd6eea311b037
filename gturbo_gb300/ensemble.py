"""Batched ensembles: many independent fields of mixed size and parameters in one launch per
pass (``gt_ens_*`` of include/gturbo.h), with per-member Philox forcing streams.

``ensemble_c4()`` builds the benchmark ensemble: 64 members, 32 x 256^2, 24 x 512^2 and
8 x 1024^2, alpha drawn per member from {0.5, 1, 2, 3}, FP64, Lawson RK4, hyperviscosity scaled
to the truncation wavenumber, drag 0.05, forcing on the shell N/25 < |k| <= N/25 + 2 with
injection rate 1, a random-phase initial field with k0 = N/50 and E = 0.5, and an independent
Philox stream per member. The time step is dt = 0.25/N (1e-3 at 256^2, the plain 256^2 run's
step): the literal 0.25 * 256 / N gives dt = 0.25 at 256^2, 250 times the RK4 stability limit
of these fields.
"""
from __future__ import annotations

import ctypes
import dataclasses

import numpy as np
import torch

from . import _lib
from .ic import random_phase_ic
from .params import GtParams, Params, famp_for_injection, nu8_scaled


@dataclasses.dataclass
class Member:
    params: Params
    key: int
    k0: float
    ic_seed: int


def ensemble_c4(seed: int = 4) -> list[Member]:
    rng = np.random.default_rng(seed)
    sizes = [256] * 32 + [512] * 24 + [1024] * 8
    alphas = rng.choice([0.5, 1.0, 2.0, 3.0], size=len(sizes))
    out = []
    for m, (n, a) in enumerate(zip(sizes, alphas)):
        p = Params(n=n, alpv=float(a), rko=4, dt=0.25 / n, nu=nu8_scaled(n), alpnu=8.0, mu=0.05,
                   alpmu=0.0, k1f=n / 25.0, k2f=n / 25.0 + 2.0)
        p = p.replace(famp=famp_for_injection(p, 1.0))
        out.append(Member(params=p, key=0x6774_0000 + m, k0=n / 50.0, ic_seed=1000 + m))
    return out


class Ensemble:
    """The members' fields (torch, float64 (N, N+2) each) and the batched C-ABI handle."""

    def __init__(self, members: list[Member], device=None, use_graph: bool = True):
        self.lib = _lib.load()
        self.members = members
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        nm = len(members)
        arr = (GtParams * nm)(*[m.params.to_ctypes() for m in members])
        keys = (ctypes.c_uint64 * nm)(*[m.key for m in members])
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            rc = self.lib.gt_ens_create(arr, nm, keys, ctypes.byref(h))
        if rc:
            raise _lib.GturboError(rc, self.lib.gt_last_error(None).decode())
        self.h = h
        self.stream = torch.cuda.current_stream(self.device)
        self._check(self.lib.gt_ens_set_stream(self.h, ctypes.c_void_p(self.stream.cuda_stream)))
        self._check(self.lib.gt_ens_use_graph(self.h, 1 if use_graph else 0))
        rk4 = members[0].params.rko == 4
        mk = lambda m: torch.zeros((m.params.n, m.params.n + 2), dtype=torch.float64,  # noqa: E731
                                   device=self.device)
        self.z = [mk(m) for m in members]
        self.work = [[mk(m) for _ in range(4 if rk4 else 3)] for m in members]
        ptr = lambda ts: (ctypes.c_void_p * nm)(*[t.data_ptr() for t in ts])  # noqa: E731
        znl = [w[0] for w in self.work]
        znew = [w[1] for w in self.work] if rk4 else None
        u = [w[-2] for w in self.work]
        v = [w[-1] for w in self.work]
        self._keep = (znl, znew, u, v)
        self._check(self.lib.gt_ens_set_fields(self.h, ptr(self.z), ptr(znl), ptr(znew) if znew else None,
                                               ptr(u), ptr(v)))

    def _check(self, rc):
        if rc:
            msg = self.lib.gt_ens_last_error(self.h)
            raise _lib.GturboError(rc, msg.decode() if msg else "")

    def load_ic(self) -> None:
        for m, z in zip(self.members, self.z):
            z.copy_(torch.from_numpy(random_phase_ic(m.params, m.k0, 0.5, seed=m.ic_seed)))

    def set_step(self, step: int) -> None:
        self._check(self.lib.gt_ens_set_step(self.h, int(step)))

    def get_step(self) -> int:
        s = ctypes.c_uint64()
        self._check(self.lib.gt_ens_get_step(self.h, ctypes.byref(s)))
        return s.value

    def step(self, nsteps: int = 1) -> None:
        self._check(self.lib.gt_ens_step(self.h, int(nsteps)))

    TILES = (16, 8, 4)

    @property
    def tile(self) -> int:
        """Values per thread of the pass kernels' tile family (16, 8 or 4; gt_ens_get_tile)."""
        r = ctypes.c_int32()
        self._check(self.lib.gt_ens_get_tile(self.h, ctypes.byref(r)))
        return r.value

    @tile.setter
    def tile(self, values_per_thread: int) -> None:
        self._check(self.lib.gt_ens_set_tile(self.h, int(values_per_thread)))

    def autotune(self, steps: int = 10, cache: str | None = "default") -> dict:
        """Pick the fastest tile family for these members (gt_ens_autotune: each family timed on
        the members' own fields, which are restored afterwards) and cache the choice in the JSON
        file of Solver.autotune, keyed by device, member sizes, RK order and library build.
        Returns {"tile": R, "ms_per_step": {R: ms} or None, "cached": bool}."""
        import collections
        import os

        from .solver import _read_cache, _tune_cache_default, _write_cache

        if cache == "default":
            cache = _tune_cache_default()
        st = os.stat(getattr(self.lib, "_gt_path", _lib.LIB_PATH))
        sizes = collections.Counter(m.params.n for m in self.members)
        key = (f"{torch.cuda.get_device_name(self.device)}|ensemble|"
               + ",".join(f"{c}x{n}" for n, c in sorted(sizes.items()))
               + f"|rko={self.members[0].params.rko}|lib={st.st_size}-{int(st.st_mtime)}")
        table = _read_cache(cache)
        hit = table.get(key)
        if hit and hit.get("tile") in self.TILES:
            self.tile = hit["tile"]
            return {"tile": hit["tile"], "ms_per_step": hit.get("ms_per_step"), "cached": True}
        ms = (ctypes.c_double * 3)()
        best = ctypes.c_int32()
        self._check(self.lib.gt_ens_autotune(self.h, int(steps), ms, ctypes.byref(best)))
        res = {"tile": best.value, "ms_per_step": {str(r): ms[q] for q, r in enumerate(self.TILES)}}
        if cache:
            table[key] = res
            _write_cache(cache, table)
        res["cached"] = False
        return res

    def close(self):
        if getattr(self, "h", None):
            self.lib.gt_ens_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PlainLoop:
    """The same members advanced one at a time through the single-field C-ABI (the baseline
    of the batched path): gt_step_rk4 / gt_step_rk2 then gt_forcing_philox, member by member."""

    def __init__(self, members: list[Member], z: list[torch.Tensor]):
        from .solver import Solver
        self.members = members
        self.z = z
        cache = {}
        self.solvers = []
        for m in members:
            key = dataclasses.astuple(m.params)
            if key not in cache:
                cache[key] = Solver(m.params)
            self.solvers.append(cache[key])
        self.work = [s.work() for s in self.solvers]
        self.step_counter = 0

    def step(self, nsteps: int = 1) -> None:
        for _ in range(nsteps):
            for m, s, z, w in zip(self.members, self.solvers, self.z, self.work):
                s.rk_step(z, w)
                s.forcing_philox(z, m.key, self.step_counter)
            self.step_counter += 1
