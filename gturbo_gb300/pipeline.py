"""Main-loop steps on fields that arrive from and return to pinned host memory.

A field-in / field-out service (or a driver that keeps its fields on the host between steps)
pays one host-to-device and one device-to-host copy of the field per step: 2·(N+2)·N·8 bytes,
67 MB at 2048². ``HostPipeline`` runs those copies on two copy streams of their own, so that
the upload of step k+1's input and the download of step k-1's result go through the copy
engines while step k computes on the solver's stream. Two device buffers alternate; events
order each buffer's upload → step → download, and an upload waits for the download that last
read its buffer.
"""
from __future__ import annotations

from typing import Sequence

import torch

from .solver import Solver


class HostPipeline:
    """Double-buffered upload → step → download of host fields through a ``Solver``."""

    def __init__(self, sol: Solver, nbuf: int = 2):
        self.sol = sol
        self.dev = [sol.field() for _ in range(nbuf)]
        self.h2d = torch.cuda.Stream(sol.device)
        self.d2h = torch.cuda.Stream(sol.device)
        self.ev_in = [torch.cuda.Event() for _ in range(nbuf)]
        self.ev_step = [torch.cuda.Event() for _ in range(nbuf)]
        self.ev_out = [torch.cuda.Event() for _ in range(nbuf)]
        self._used = [False] * nbuf

    def run(self, host_in: Sequence[torch.Tensor], host_out: Sequence[torch.Tensor], nsteps: int,
            seed: int, work: list[torch.Tensor], diag_every: int = 0, first_step: int = 1) -> int:
        """``nsteps`` main-loop steps (``Solver.main_step``). Step k starts from a copy of
        ``host_in[k % len(host_in)]`` and its result is copied to ``host_out[k % len(host_out)]``.
        Host tensors must be pinned float64 fields. Returns the LCG state after the last kick;
        the downloads are complete when ``sync()`` returns."""
        sol, nb = self.sol, len(self.dev)
        for k in range(nsteps):
            b = k % nb
            buf = self.dev[b]
            if self._used[b]:
                self.h2d.wait_event(self.ev_out[b])   # the last download of buf is done
            with torch.cuda.stream(self.h2d):
                buf.copy_(host_in[k % len(host_in)], non_blocking=True)
                self.ev_in[b].record(self.h2d)
            sol.stream.wait_event(self.ev_in[b])
            ipas = first_step + k
            seed, _ = sol.main_step(buf, seed, work, diag=bool(diag_every) and ipas % diag_every == 0)
            self.ev_step[b].record(sol.stream)
            self.d2h.wait_event(self.ev_step[b])
            with torch.cuda.stream(self.d2h):
                host_out[k % len(host_out)].copy_(buf, non_blocking=True)
                self.ev_out[b].record(self.d2h)
            self._used[b] = True
        return seed

    def sync(self) -> None:
        self.d2h.synchronize()
        self.h2d.synchronize()
        self.sol.stream.synchronize()
