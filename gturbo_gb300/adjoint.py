"""Gradients of a final-time spectral objective: tangent-linear model and discrete adjoint of
the Lawson RK2 step, discrete adjoint of the Lawson RK4 step, each with the LCG forcing kick
(``gt_objective``, ``gt_tlm_*``, ``gt_adj_*`` of include/gturbo.h).

The objective is the energy in the shells kmin <= |k| <= kmax of the final field, with the
reference's weights: J = sum fac |q|^2 / |k|^alpha (fac = 1/2 on the kx=0 and Nyquist columns).
The parameters are the initial spectral field (real and imaginary parts of every stored value)
and the forcing amplitude famp; the forcing phases are the reference's LCG sequence from a seed.
"""
from __future__ import annotations

import ctypes

import torch

from .solver import Solver


def objective(sol: Solver, z: torch.Tensor, kmin: float, kmax: float, grad: bool = False):
    """J(z) and, when ``grad``, dJ/dz (a field of z's shape)."""
    J = ctypes.c_double()
    g = sol.field() if grad else None
    sol._check(sol.lib.gt_objective(sol.h, sol._ptr(z), kmin, kmax, ctypes.byref(J),
                                    sol._ptr(g) if grad else None))
    return (J.value, g) if grad else J.value


def forward_objective(sol: Solver, z0: torch.Tensor, nsteps: int, seed: int, kmin: float,
                      kmax: float) -> float:
    """J after nsteps of the handle's integrator + kick (the plain forward path,
    gt_step_rk2 or gt_step_rk4, then gt_forcing)."""
    z = z0.clone()
    work = sol.work(4)
    s = seed
    for _ in range(nsteps):
        sol.rk_step(z, work)
        s = sol.forcing(z, s)
    return objective(sol, z, kmin, kmax)


def tlm_run(sol: Solver, z0, dz0, dfamp: float, nsteps: int, seed: int, kmin: float, kmax: float):
    """(J, dJ): the objective and its derivative along (dz0, dfamp) by the tangent-linear model."""
    J, dJ = ctypes.c_double(), ctypes.c_double()
    sol._check(sol.lib.gt_tlm_run(sol.h, sol._ptr(z0), sol._ptr(dz0), float(dfamp), int(nsteps),
                                  int(seed), kmin, kmax, ctypes.byref(J), ctypes.byref(dJ)))
    return J.value, dJ.value


def gradient(sol: Solver, z0, nsteps: int, seed: int, kmin: float, kmax: float, checkpoint: int = 20,
             memory: int | None = None):
    """(J, dJ/dz0, dJ/dfamp, z_T, (forward ms, backward ms)) by the checkpointed adjoint.

    ``memory`` (bytes), when given, sets the handle's budget for whole kept segments
    (``Solver.adj_memory``): the forward sweep keeps as many of its last segments as fit, and only
    the earlier ones are recomputed from their checkpoints."""
    if memory is not None:
        sol.adj_memory = memory
    J, gf = ctypes.c_double(), ctypes.c_double()
    gz, zT = sol.field(), sol.field()
    t = (ctypes.c_double * 2)()
    sol._check(sol.lib.gt_adj_gradient(sol.h, sol._ptr(z0), int(nsteps), int(seed), int(checkpoint),
                                       kmin, kmax, ctypes.byref(J), sol._ptr(gz), ctypes.byref(gf),
                                       sol._ptr(zT), t))
    return J.value, gz, gf.value, zT, (t[0], t[1])
