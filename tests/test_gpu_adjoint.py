"""Tangent-linear model and discrete adjoint of the RK2 step + LCG kick, on the GPU.

Checks, for J = energy in the shells 4 <= |k| <= 8 of the final field:
  * dot-product test: <dJ/dz0, dz0> + dJ/dfamp dfamp == the tangent-linear dJ (same discrete
    map, both exact derivatives: agreement to roundoff);
  * FP64 central finite differences (relative step 1e-6) along random directions agree with
    the tangent-linear dJ to 1e-6;
  * the adjoint's J equals the plain forward path's J;
  * a torch.autograd.Function wrapping the C-ABI gradient (test harness only) passes
    torch.autograd.gradcheck-style directional checks.
"""
import numpy as np
import pytest

from gturbo_gb300.params import Params

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

KMIN, KMAX = 4.0, 8.0
SEED = 481929


def _setup(n=128, nsteps=12):
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import famp_for_injection, nu8_scaled
    from gturbo_gb300.solver import Solver
    p = Params(n=n, alpv=1.0, rko=2, dt=5e-4, nu=nu8_scaled(n), alpnu=8.0, mu=0.1, k1f=10.0, k2f=12.0)
    p = p.replace(famp=famp_for_injection(p, 1.0))
    sol = Solver(p)
    z0 = torch.from_numpy(random_phase_ic(p, 6.0, 0.5, seed=5)).cuda()
    return p, sol, z0, nsteps


def _direction(z0, seed, truncated_only=False):
    g = torch.Generator(device="cpu").manual_seed(seed)
    d = torch.randn(z0.shape, generator=g, dtype=torch.float64).cuda()
    if truncated_only:
        d = d * (z0 != 0).to(torch.float64)
    return d * (z0.abs().max() / d.abs().max())


def test_adjoint_forward_matches_plain_forward():
    from gturbo_gb300.adjoint import forward_objective, gradient
    p, sol, z0, ns = _setup()
    J_plain = forward_objective(sol, z0, ns, SEED, KMIN, KMAX)
    J, gz, gf, zT, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=5)
    assert J == pytest.approx(J_plain, rel=1e-14)
    assert torch.isfinite(gz).all()


@pytest.mark.parametrize("k", [1, 5, 12])
def test_dot_product_adjoint_vs_tlm(k):
    from gturbo_gb300.adjoint import gradient, tlm_run
    p, sol, z0, ns = _setup()
    J, gz, gf, _, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=k)
    for seed in (1, 2):
        dz = _direction(z0, seed)
        dfamp = 0.3 * seed
        J2, dJ = tlm_run(sol, z0, dz, dfamp, ns, SEED, KMIN, KMAX)
        adj = float((gz * dz).sum().item()) + gf * dfamp
        assert J2 == pytest.approx(J, rel=1e-14)
        assert adj == pytest.approx(dJ, rel=1e-11, abs=1e-14 * abs(J))


def test_tlm_against_central_differences():
    from gturbo_gb300.adjoint import forward_objective, tlm_run
    p, sol, z0, ns = _setup()
    for seed in range(1, 9):
        dz = _direction(z0, 100 + seed, truncated_only=(seed % 2 == 0))
        dfamp = 0.0 if seed % 3 else 0.5
        _, dJ = tlm_run(sol, z0, dz, dfamp, ns, SEED, KMIN, KMAX)
        h = 1e-6
        if dfamp:
            from gturbo_gb300.solver import Solver
            sp = Solver(p.replace(famp=p.famp + h * dfamp))
            sm = Solver(p.replace(famp=p.famp - h * dfamp))
            Jp = forward_objective(sp, z0 + h * dz, ns, SEED, KMIN, KMAX)
            Jm = forward_objective(sm, z0 - h * dz, ns, SEED, KMIN, KMAX)
        else:
            Jp = forward_objective(sol, z0 + h * dz, ns, SEED, KMIN, KMAX)
            Jm = forward_objective(sol, z0 - h * dz, ns, SEED, KMIN, KMAX)
        fd = (Jp - Jm) / (2 * h)
        assert fd == pytest.approx(dJ, rel=1e-6, abs=1e-9 * abs(Jp)), seed


class _AdjointJ(torch.autograd.Function):
    """J(z0) after nsteps, with the C-ABI adjoint as its backward (test harness only)."""

    @staticmethod
    def forward(ctx, z0, sol, nsteps, seed):
        from gturbo_gb300.adjoint import gradient
        J, gz, gf, _, _ = gradient(sol, z0.detach(), nsteps, seed, KMIN, KMAX, checkpoint=4)
        ctx.save_for_backward(gz)
        return torch.tensor(J, dtype=torch.float64, device=z0.device)

    @staticmethod
    def backward(ctx, gout):
        (gz,) = ctx.saved_tensors
        return gout * gz, None, None, None


def test_autograd_function_wrapper():
    from gturbo_gb300.adjoint import tlm_run
    p, sol, z0, ns = _setup(n=128, nsteps=6)
    z = z0.clone().requires_grad_(True)
    J = _AdjointJ.apply(z, sol, ns, SEED)
    J.backward()
    dz = _direction(z0, 7)
    _, dJ = tlm_run(sol, z0, dz, 0.0, ns, SEED, KMIN, KMAX)
    assert float((z.grad * dz).sum()) == pytest.approx(dJ, rel=1e-11)


def test_adjoint_limits():
    """The single-step tangent-linear / adjoint calls are RK2 only (RK4 goes through
    gt_tlm_run and gt_adj_gradient, tested below)."""
    import ctypes
    from gturbo_gb300 import _lib
    from gturbo_gb300.solver import Solver
    sol = Solver(Params(n=64, rko=4))
    work = [sol.field() for _ in range(8)]
    wk = (ctypes.c_void_p * 8)(*[w.data_ptr() for w in work])
    s = ctypes.c_int32(SEED)
    rc = sol.lib.gt_tlm_step_rk2(sol.h, sol._ptr(work[0]), sol._ptr(work[1]), 0.0, ctypes.byref(s), wk)
    assert rc == 1
    with pytest.raises(_lib.GturboError):
        sol._check(rc)


@pytest.mark.parametrize("n", [128, 1024])
def test_adjoint_in_every_launch_variant(n):
    """The gradient and the tangent-linear dJ in each launch variant: dot-product test per
    variant, and the same gradient (to rounding) from every variant."""
    from gturbo_gb300.adjoint import gradient, tlm_run
    p, sol, z0, ns = _setup(n=n, nsteps=6)
    dz = _direction(z0, 3)
    grads = []
    for v in sol.supported_variants():
        sol.variant = v
        J, gz, gf, _, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=3)
        J2, dJ = tlm_run(sol, z0, dz, 0.4, ns, SEED, KMIN, KMAX)
        adj = float((gz * dz).sum().item()) + gf * 0.4
        assert J2 == pytest.approx(J, rel=1e-14), v
        assert adj == pytest.approx(dJ, rel=1e-11, abs=1e-14 * abs(J)), v
        grads.append((J, gz, gf))
    J0, g0, f0 = grads[0]
    for J, gz, gf in grads[1:]:
        assert J == pytest.approx(J0, rel=1e-12)
        assert float((gz - g0).norm() / g0.norm()) < 1e-12
        assert gf == pytest.approx(f0, rel=1e-11)


@pytest.mark.parametrize("n,variant,rko", [(512, 2, 2), (1024, 1, 2), (1024, 0, 4)])
def test_gradient_with_and_without_col_split(n, variant, rko):
    """The field-split column passes (forward, recomputed and transposed; pass C in its counter
    form and as clusters) give the gradient of one CTA per column to rounding, for RK2 and RK4."""
    from gturbo_gb300.adjoint import gradient
    p, sol, z0, ns = _setup(n=n, nsteps=4)
    if rko == 4:
        from gturbo_gb300.solver import Solver
        p = p.replace(rko=4)
        sol = Solver(p)
    sol.variant = variant
    res = {}
    for split in (2, 1, 0):
        sol.col_split = split
        assert sol.col_split == split
        res[split] = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=2)
    J0, gz0, gf0, zT0, _ = res[0]
    for split in (2, 1):
        J1, gz1, gf1, zT1, _ = res[split]
        assert J1 == pytest.approx(J0, rel=1e-13), split
        assert gf1 == pytest.approx(gf0, rel=1e-11, abs=1e-20), split
        assert (torch.linalg.norm(gz1 - gz0) / torch.linalg.norm(gz0)).item() < 1e-12, split
        assert (torch.linalg.norm(zT1 - zT0) / torch.linalg.norm(zT0)).item() < 1e-13, split


@pytest.mark.parametrize("n,variant", [(256, 2), (1024, 2)])
def test_gradient_with_and_without_pdl(n, variant):
    """Programmatic dependent launch of the forward, tangent and transposed pass kernels leaves
    the gradient and the tangent-linear run bit for bit the same."""
    from gturbo_gb300.adjoint import gradient, tlm_run
    p, sol, z0, ns = _setup(n=n, nsteps=5)
    sol.variant = variant
    dz = torch.randn_like(z0) * 1e-3
    res = {}
    for pdl in (True, False):
        sol.pdl = pdl
        J, gz, gf, zT, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=2)
        J2, dJ = tlm_run(sol, z0, dz, 0.4, ns, SEED, KMIN, KMAX)
        res[pdl] = (J, gz.cpu(), gf, zT.cpu(), J2, dJ)
    a, b = res[True], res[False]
    assert a[0] == b[0] and a[2] == b[2] and a[4] == b[4] and a[5] == b[5]
    assert torch.equal(a[1], b[1]) and torch.equal(a[3], b[3])


@pytest.mark.parametrize("n,variant", [(128, 0), (128, 2), (256, 1)])
def test_gradient_driver_matches_step_by_step_adjoint(n, variant):
    """gt_adj_gradient (whose adjoint passes read the physical fields that the recomputed
    forward stages kept) against a step-by-step backward sweep through gt_adj_step_rk2 (whose
    passes transform the linearisation points themselves)."""
    import ctypes
    from gturbo_gb300.adjoint import gradient, objective
    p, sol, z0, ns = _setup(n=n, nsteps=7)
    sol.variant = variant
    J, gz, gf, zT, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=3)
    # forward: states z_s, stage states w_s, LCG states
    work = sol.work(6)
    P = ctypes.c_void_p
    wk = (P * 6)(*[w.data_ptr() for w in work])
    zs, ws, seeds = [], [], []
    z, sd = z0.clone(), SEED
    for _ in range(ns):
        w = sol.field()
        sol._check(sol.lib.gt_adj_stage(sol.h, sol._ptr(z), sol._ptr(w), wk))
        zs.append(z.clone())
        ws.append(w)
        seeds.append(sd)
        sol.step(z, *work[:3])
        sd = sol.forcing(z, sd)
    J2, lam = objective(sol, z, KMIN, KMAX, grad=True)
    assert J2 == pytest.approx(J, rel=1e-14)
    gfamp = ctypes.c_double(0.0)
    for st in reversed(range(ns)):
        sol._check(sol.lib.gt_adj_step_rk2(sol.h, sol._ptr(zs[st]), sol._ptr(ws[st]), sol._ptr(lam),
                                           int(seeds[st]), ctypes.byref(gfamp), wk))
    torch.cuda.synchronize()
    assert float((gz - lam).norm() / lam.norm()) < 1e-13
    assert gf == pytest.approx(gfamp.value, rel=1e-12)


def _setup_rk4(n=128, nsteps=8):
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import famp_for_injection, nu8_scaled
    from gturbo_gb300.solver import Solver
    p = Params(n=n, alpv=2.0, rko=4, dt=1e-3, nu=nu8_scaled(n), alpnu=8.0, mu=0.05, k1f=10.0, k2f=12.0)
    p = p.replace(famp=famp_for_injection(p, 1.0))
    sol = Solver(p)
    z0 = torch.from_numpy(random_phase_ic(p, 5.0, 0.5, seed=9)).cuda()
    return p, sol, z0, nsteps


def test_rk4_gradient_against_central_differences():
    """The RK4 adjoint (gt_adj_gradient on an RK4 handle) against FP64 central differences
    (h = 1e-6) along random directions, in z0 and in famp; J equals the plain RK4 run's."""
    from gturbo_gb300.adjoint import forward_objective, gradient
    from gturbo_gb300.solver import Solver
    p, sol, z0, ns = _setup_rk4()
    J, gz, gf, _, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=3)
    assert J == pytest.approx(forward_objective(sol, z0, ns, SEED, KMIN, KMAX), rel=1e-14)
    h = 1e-6
    for seed in range(1, 5):
        dz = _direction(z0, 300 + seed, truncated_only=(seed % 2 == 0))
        Jp = forward_objective(sol, z0 + h * dz, ns, SEED, KMIN, KMAX)
        Jm = forward_objective(sol, z0 - h * dz, ns, SEED, KMIN, KMAX)
        fd = (Jp - Jm) / (2 * h)
        adj = float((gz * dz).sum().item())
        assert adj == pytest.approx(fd, rel=1e-6, abs=1e-9 * abs(J)), seed
    sp, sm = Solver(p.replace(famp=p.famp + h)), Solver(p.replace(famp=p.famp - h))
    fd = (forward_objective(sp, z0, ns, SEED, KMIN, KMAX) - forward_objective(sm, z0, ns, SEED, KMIN, KMAX)) / (2 * h)
    assert gf == pytest.approx(fd, rel=1e-6, abs=1e-9 * abs(J))


@pytest.mark.parametrize("n", [64, 256])
def test_rk4_gradient_independent_of_checkpointing(n):
    """Checkpoint interval and launch variant change the schedule, not the RK4 gradient."""
    from gturbo_gb300.adjoint import gradient
    p, sol, z0, ns = _setup_rk4(n=n, nsteps=7)
    ref = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=1)
    for k in (2, 3, 7, 20):
        J, gz, gf, _, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=k)
        assert J == ref[0]
        assert float((gz - ref[1]).norm() / ref[1].norm()) < 1e-14, k
        assert gf == pytest.approx(ref[2], rel=1e-13)
    for v in sol.supported_variants():
        sol.variant = v
        J, gz, gf, _, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=3)
        assert float((gz - ref[1]).norm() / ref[1].norm()) < 1e-12, v


@pytest.mark.parametrize("k", [1, 4])
def test_rk4_dot_product_adjoint_vs_tlm(k):
    """RK4: <dJ/dz0, dz0> + dJ/dfamp dfamp from the adjoint equals the tangent-linear dJ
    (the same discrete map differentiated two ways: agreement to roundoff)."""
    from gturbo_gb300.adjoint import gradient, tlm_run
    p, sol, z0, ns = _setup_rk4(nsteps=6)
    J, gz, gf, _, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=k)
    for seed in (1, 2):
        dz = _direction(z0, 400 + seed)
        dfamp = 0.2 * seed
        J2, dJ = tlm_run(sol, z0, dz, dfamp, ns, SEED, KMIN, KMAX)
        adj = float((gz * dz).sum().item()) + gf * dfamp
        assert J2 == pytest.approx(J, rel=1e-14)
        assert adj == pytest.approx(dJ, rel=1e-11, abs=1e-14 * abs(J))


@pytest.mark.parametrize("rko", [2, 4])
def test_gradient_with_kept_segments_matches_recomputation(rko):
    """gt_adj_set_memory: keeping more whole segments (less recomputation) changes only where the
    adjoint reads the stage states and physical fields from, not the gradient."""
    from gturbo_gb300.adjoint import gradient
    p, sol, z0, ns = _setup(n=128, nsteps=12)
    if rko == 4:
        from gturbo_gb300.solver import Solver
        sol = Solver(p.replace(rko=4))
    J0, g0, f0, _, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=4, memory=0)
    for mem in (1, 10 ** 7, 1 << 40):  # one segment, two of three, everything (capped by free memory)
        J, g, f, _, _ = gradient(sol, z0, ns, SEED, KMIN, KMAX, checkpoint=4, memory=mem)
        assert J == J0
        assert float((g - g0).norm() / g0.norm()) < 1e-13
        assert f == pytest.approx(f0, rel=1e-12)
    sol.adj_memory = 0
    assert sol.adj_memory == 0


def test_c5_configuration_fd_tlm_and_dot_product():
    """The gradient workload at its own configuration: 1024^2, alpha=1, Lawson RK2, 200 steps with
    the LCG kick, checkpoint every 20, J = energy in 4 <= |k| <= 8. Along 8 random directions of
    the initial field and along the forcing amplitude, FP64 central differences (h = 1e-6) agree
    with the tangent-linear run to 1e-6, and the adjoint gradient's directional derivatives equal
    the tangent's (dot-product test)."""
    from gturbo_gb300.adjoint import forward_objective, gradient, tlm_run
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import IC_K0, config
    from gturbo_gb300.solver import Solver

    p = config("c5")
    nsteps, K, h = 200, 20, 1e-6
    sol = Solver(p)
    z0 = torch.from_numpy(random_phase_ic(p, IC_K0["c5"], 0.5, seed=1)).cuda()
    J, gz, gf, _, _ = gradient(sol, z0, nsteps, SEED, KMIN, KMAX, checkpoint=K)
    assert J == pytest.approx(forward_objective(sol, z0, nsteps, SEED, KMIN, KMAX), rel=1e-14)
    for d in range(8):
        dz = _direction(z0, 500 + d, truncated_only=(d % 2 == 1))
        J2, dJ = tlm_run(sol, z0, dz, 0.0, nsteps, SEED, KMIN, KMAX)
        assert J2 == pytest.approx(J, rel=1e-14)
        adj = float((gz * dz).sum().item())
        assert adj == pytest.approx(dJ, rel=1e-11, abs=1e-14 * abs(J)), d
        fd = (forward_objective(sol, z0 + h * dz, nsteps, SEED, KMIN, KMAX)
              - forward_objective(sol, z0 - h * dz, nsteps, SEED, KMIN, KMAX)) / (2 * h)
        assert fd == pytest.approx(dJ, rel=1e-6), d
    # the forcing-amplitude direction
    _, dJf = tlm_run(sol, z0, torch.zeros_like(z0), 1.0, nsteps, SEED, KMIN, KMAX)
    assert gf == pytest.approx(dJf, rel=1e-11)
    hf = h * p.famp
    fd = (forward_objective(Solver(p.replace(famp=p.famp + hf)), z0, nsteps, SEED, KMIN, KMAX)
          - forward_objective(Solver(p.replace(famp=p.famp - hf)), z0, nsteps, SEED, KMIN, KMAX)) / (2 * hf)
    assert fd == pytest.approx(dJf, rel=1e-6)


@pytest.mark.parametrize("rko", [2, 4])
def test_tlm_cluster_pass_c_matches_counter_form(rko):
    """The tangent pass C as 4-CTA clusters (split mode 2, the default) against its per-column
    counter form (mode 1): the same arithmetic per value, so J and dJ agree to rounding."""
    from gturbo_gb300.adjoint import tlm_run
    from gturbo_gb300.solver import Solver
    p, sol, z0, ns = _setup(n=256, nsteps=6)
    if rko == 4:
        sol = Solver(p.replace(rko=4))
    dz = _direction(z0, 11)
    out = {}
    for mode in (2, 1):
        sol.col_split = mode
        out[mode] = tlm_run(sol, z0, dz, 0.2, ns, SEED, KMIN, KMAX)
    assert out[2][0] == pytest.approx(out[1][0], rel=1e-14)
    assert out[2][1] == pytest.approx(out[1][1], rel=1e-12)
