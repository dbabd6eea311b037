#!/usr/bin/env python3
"""Benchmark of the Gturbo time-stepping hot path on GB300.

Workload (default ``--config c2``): the 2048^2 SQG-like run -- alpha=1, Lawson RK2, dt=2e-5
(the dt=2e-4 first specified for it is CFL-unstable for RK2 at E=0.5; see gturbo_gb300.params.config),
hyperviscosity (2/3 N/2)^-16 k^16, drag mu=0.1, stochastic forcing on 20 < |k| <= 22 with
injection rate 1 (the reference's LCG, seed 481929), diagnostics (spectra, fluxes, budgets) every
100 steps, random-phase initial field with E(k) ~ k^4 exp(-(k/10)^2), E=0.5. Inputs are synthetic
and resident in HBM; the working set (4 fields + 2 tables + the q scratch, ~202 MB) exceeds the 126 MB L2, so no
flush is needed between steps.

A "step" is one iteration of the reference's main loop (src/main.f90:97-137): the RK step,
the diagnostics when ipas % imix == 0, and the forcing kick.

Arms:
  default            the CUDA path (gturbo_gb300) -> one JSON line on rank 0
  --impl reference   the reference on the host cores, all threads: its Fortran library
                     transliterated into C (oracle/_ref), or the C oracle port where that is absent
Multi-GPU (torchrun): every rank advances its own independent replica (no collective on the
data path); the barrier + max-over-ranks timing gives the whole-job throughput.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "steps/s @2048² FP64 vs ref; batched member-steps/s vs plain; adjoint/fwd time"
SEED = 481929  # src/seed.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="c2")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="CPU-baseline sample budget")
    ap.add_argument("--no-extras", action="store_true", help="skip e2e / cpu / ref-equivalent legs")
    ap.add_argument("--variant", type=int, default=None,
                    help="launch variant of the nonlinear-term passes (default: autotuned)")
    ap.add_argument("--row-variant", type=int, default=None,
                    help="with --variant: the row passes' own launch variant (default: the same)")
    ap.add_argument("--col-split", type=int, choices=[0, 1, 2], default=None,
                    help="field-split column passes: 0 off, 1 counter epilogue, 2 2-CTA clusters")
    ap.add_argument("--no-pdl", action="store_true",
                    help="launch the pass kernels without programmatic dependent launch")
    ap.add_argument("--adjoint-rk", type=int, choices=[2, 4], default=2,
                    help="integrator of the --only adjoint leg (the bench's own leg is RK2)")
    ap.add_argument("--only", choices=["ensemble", "adjoint", "next"], default=None,
                    help="run one secondary leg alone and print its JSON object (profiling)")
    return ap.parse_args()


def workload(name):
    from gturbo_gb300.params import IC_K0, config

    p = config(name)
    desc = (f"{name}: {p.n}^2 alpha={p.alpv:g} RK{p.rko} dt={p.dt:g} nu={p.nu:.3e} k^{2 * p.alpnu:g} "
            f"mu={p.mu:g} forcing {p.k1f:g}<|k|<={p.k2f:g} eps=1 (famp={p.famp:.6f}) "
            f"IC k0={IC_K0[name]:g} E=0.5, diagnostics every {p.imix} steps")
    return p, IC_K0[name], desc


def run_config(args):
    """The JSON line's `config`, built the same way by both arms from the workload alone (the
    GPU arm's launch settings go to its own `settings` object)."""
    p, _, desc = workload(args.config)
    # fields of the integrator, the emk and kainv tables (S together), and the q scratch of the
    # field-split column passes (N <= 2048)
    s = 16 * p.n * (p.n // 2 + 1)
    ws = s * ((4 if p.rko == 2 else 5) + 1 + (1 if p.n <= 2048 else 0))
    l2 = (f"no flush: working set ~{ws / 1e6:.0f} MB > 126 MB L2" if ws > 126e6 else
          f"no flush: the working set (~{ws / 1e6:.0f} MB) fits in L2 (small grid)")
    return {"workload": desc, "n": p.n, "alpha": p.alpv, "rk": p.rko, "dt": p.dt,
            "imix": p.imix,
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single",
            "l2": l2}


# ---------------------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception as e:  # nvidia-smi missing: report no clocks
            log("clock sampler unavailable:", e)
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------------------
# CPU baseline: the C oracle (the reference's algorithm restated) on the host cores
# ---------------------------------------------------------------------------------------
def cpu_oracle_run(p, k0, steps, budget_s, threads=None):
    """Times up to `steps` main-loop iterations of the oracle within ~budget_s seconds."""
    import numpy as np

    from gturbo_gb300.ic import random_phase_ic
    from oracle import coracle

    if threads:
        coracle.set_num_threads(threads)
    orc = coracle.Oracle(p)
    z = random_phase_ic(p, k0, 0.5, seed=1)
    work = [orc.zeros() for _ in range(4)]
    seed = SEED
    t0 = time.perf_counter()
    seed, _ = orc.main_step(z, seed, work=work)  # warm-up + calibration
    t1 = time.perf_counter() - t0
    k = max(1, min(steps, int(budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    for ipas in range(1, k + 1):
        seed, _ = orc.main_step(z, seed, diag=(ipas % p.imix == 0), work=work)
    dt = time.perf_counter() - t0
    assert np.isfinite(z).all()
    return {"value": k / dt, "unit": "steps/s", "cores": coracle.num_threads(), "kind": "port",
            "sample": f"{k} main-loop steps of the {p.n}^2 workload (RK{p.rko} + forcing"
                      f"{', diagnostics every ' + str(p.imix) if k >= p.imix else ''}), "
                      f"C oracle with OpenMP"}


def cpu_reference_run(p, k0, steps, budget_s):
    """Main-loop steps/s of the reference's own statements on the host cores: its Fortran library
    transliterated into C (oracle/_ref; the acc parallel loops as OpenMP loops, cuFFT answered by
    the shim), driven in the order of src/main.f90:97-137. None where oracle/_ref is absent."""
    import numpy as np

    from gturbo_gb300.ic import random_phase_ic
    from oracle import refcore

    if not refcore.available():
        return None
    ref = refcore.Reference(p)
    z = random_phase_ic(p, k0, 0.5, seed=1)
    work = [ref.zeros() for _ in range(4)]
    seed = SEED
    t0 = time.perf_counter()
    seed, _ = ref.main_step(z, seed, 1, p.imix, work)  # warm-up + calibration
    t1 = time.perf_counter() - t0
    k = max(1, min(steps, int(budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    for ipas in range(1, k + 1):
        seed, _ = ref.main_step(z, seed, ipas, p.imix, work)
    dt = time.perf_counter() - t0
    assert np.isfinite(z).all()
    return {"value": k / dt, "unit": "steps/s", "cores": ref.threads, "kind": "reference",
            "sample": f"{k} main-loop steps of the {p.n}^2 workload (RK{p.rko} + forcing"
                      f"{', diagnostics every ' + str(p.imix) if k >= p.imix else ''}): the "
                      "reference's Fortran library transliterated into C (acc parallel loops as "
                      "OpenMP loops, cuFFT calls answered by a CPU FFT)"}


def numpy_run(p, k0, budget_s):
    """Main-loop steps/s of the single-threaded numpy restatement (pocketfft) within ~budget_s."""
    import numpy as np

    from gturbo_gb300.ic import random_phase_ic
    from oracle.np_oracle import NpOracle, from_phys_layout

    orc = NpOracle(p)
    zk = from_phys_layout(random_phase_ic(p, k0, 0.5, seed=1))
    seed = SEED
    t0 = time.perf_counter()
    zk = orc.rk_step(zk)
    zk, seed = orc.forcing(zk, seed)
    t1 = time.perf_counter() - t0
    k = max(1, int(budget_s / max(t1, 1e-6)))
    t0 = time.perf_counter()
    for _ in range(k):
        zk = orc.rk_step(zk)
        zk, seed = orc.forcing(zk, seed)
    dt = time.perf_counter() - t0
    assert np.isfinite(zk).all()
    return {"value": k / dt, "unit": "steps/s", "cores": 1, "steps": k,
            "sample": f"{k} steps (RK{p.rko} + forcing, no diagnostics) of the {p.n}^2 workload, "
                      "numpy restatement, pocketfft"}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    p, k0, desc = workload(args.config)
    budget = max(10.0, min(120.0, args.cpu_seconds * 3))
    try:
        res = cpu_reference_run(p, k0, args.steps, budget)
    except Exception as e:  # the transliterated reference failed to build or run: the port
        log("reference statements unavailable:", e)
        res = None
        why = str(e)[:200]
    else:
        why = None
    if res is None:
        res = cpu_oracle_run(p, k0, args.steps, budget)
        if why:
            res["reference_unavailable"] = why
    line = {"metric": METRIC, "value": res["value"], "unit": "steps/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 / res["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": run_config(args),
            "cpu_baseline": res,
            "e2e": {"value": res["value"], "unit": "steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------
# the CUDA path
# ---------------------------------------------------------------------------------------
def fp64_gemm_tflops(torch, dev):
    """Measured FP64 peak proxy: cuBLAS DGEMM 4096^3, best of 3."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    del a, b
    return 2.0 * n ** 3 / best / 1e12


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def pass_model(p, kind):
    """Algorithmic FLOPs and HBM bytes of one launch of a pass of the nonlinear term.

    FLOPs follow the FFT convention 5 L log2 L per complex length-L transform (2.5 L log2 L per
    real one) and count the unpruned work of the reference's 5 cuFFT transforms per nlt.
    Bytes count every field touched once (S = 16 N (N/2+1)): A reads q and writes 3 fields,
    B reads 3 and writes 2, C reads 2 fields and the RK2 stage reads z and writes one field.
    """
    n = p.n
    nh = n // 2 + 1
    S = 16 * n * nh
    lg = math.log2(n)
    if kind == "nlt_colinv":
        return 3 * nh * 5 * n * lg, 4 * S
    if kind == "nlt_row":
        return 5 * n * 2.5 * n * lg, 5 * S
    if kind == "nlt_colfwd":
        return 2 * nh * 5 * n * lg, 4 * S
    if kind == "nlt_colfwd_inv":  # pass C of a stage + pass A of the next
        return 5 * nh * 5 * n * lg, 7 * S
    return None, None


# DRAM bytes (read + write) per launch of a pass, from single-kernel ncu captures
# (dram__bytes_read.sum + dram__bytes_write.sum) of the same launch variant:
#   2048^2, variant 0: ncu --set full --clock-control none -k "regex:k_nlt_(row|colfwd_inv|colinv)" -s 4 -c 3
#                      python bench.py --steps 2 --warmup 3 --no-extras --variant 0
#   2048^2, variant 1: ncu --set full --clock-control none -k "regex:k_nltv_(row|colfwd_inv|colinv)" -s 4 -c 3
#                      python bench.py --steps 2 --warmup 3 --no-extras --variant 1
#   256^2, column variant 3, row variant 2:
#                      ncu --set full --clock-control none --kernel-name-base demangled -k "regex:k_nltv_(row<\(int\)256,
#                      \(int\)2>|colfwd_inv<\(int\)256, \(int\)3>|colinv<\(int\)256, \(int\)3>)" -s 8 -c 3
#                      python bench.py --config c1 --steps 2 --warmup 3 --no-extras --variant 3
# Keyed by (N, the launch variant of that kernel: the row variant for the row pass, the column
# variant otherwise, pass).
# FP64 instructions (thread level) per launch of a pass, from ncu's
# smsp__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum of the same launch variant:
#   2048^2, variant 1: ncu --metrics <those> --clock-control none -k "regex:k_nltv_(row|colfwd_inv|colinv)" -s 4 -c 3
#                      python bench.py --steps 2 --warmup 3 --no-extras --variant 1
# The FP64 pipe issues 2 such operations per clock per SM (152 SMs).
NCU_FP64_OPS = {
    (2048, 1, "nlt_colinv"): 23.080e6 + 92.320e6 + 8.393e6,
    (2048, 1, "nlt_row"): 65.704e6 + 247.464e6 + 4.194e6,
    (2048, 1, "nlt_colfwd_inv"): 44.064e6 + 159.461e6 + 17.137e6,
}

NCU_TRAFFIC = {
    (2048, 0, "nlt_colinv"): 50.01e6 + 47.65e6,
    (2048, 0, "nlt_row"): 68.00e6 + 1.50e6,
    (2048, 0, "nlt_colfwd_inv"): 111.96e6 + 55.95e6,
    (2048, 1, "nlt_colinv"): 58.38e6 + 55.84e6,
    (2048, 1, "nlt_row"): 67.95e6 + 1.47e6,
    (2048, 1, "nlt_colfwd_inv"): 114.65e6 + 52.83e6,
    (256, 3, "nlt_colinv"): 0.757e6,
    (256, 2, "nlt_row"): 1.177e6,
    (256, 3, "nlt_colfwd_inv"): 1.828e6,
}


def ours_arm(args):
    import numpy as np
    import torch
    import torch.distributed as dist

    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.replicas import replica_ic_seed, whole_job_rate
    from gturbo_gb300.solver import Solver

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        dist.init_process_group("nccl", device_id=dev)

    def barrier():
        if world > 1:
            dist.barrier()

    p, k0, desc = workload(args.config)
    K, W = args.steps, max(3, args.warmup)
    sol = Solver(p, device=local)
    sol.pdl = not args.no_pdl
    # launch variant of the nonlinear-term passes: timed per variant before the run (like a
    # cuFFT plan, outside the timed region)
    if args.variant is None:
        tune = sol.autotune(steps=50 if p.n <= 1024 else 10, cache=None)
    else:
        sol.variant = args.variant
        if args.row_variant is not None:
            sol.variants = (args.variant, args.row_variant)
        tune = {"variant": args.variant, "ms_per_step": None}
    if args.col_split is not None:
        sol.col_split = args.col_split
    stream = sol.stream
    work = sol.work()
    z0 = torch.from_numpy(random_phase_ic(p, k0, 0.5, seed=replica_ic_seed(rank))).to(dev)
    z = z0.clone()
    seed = SEED
    # warm-up (including one diagnostics pass)
    for it in range(W):
        seed, _ = sol.main_step(z, seed, work, diag=(it == W - 1))
    torch.cuda.synchronize()

    # ---- timed region: K main-loop steps, diagnostics every imix ----------------------
    z.copy_(z0)
    seed = SEED
    torch.cuda.synchronize()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    ndiag = 0
    for ipas in range(1, K + 1):
        d = ipas % p.imix == 0
        ndiag += d
        seed, out = sol.main_step(z, seed, work, diag=d)
    e1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    t = e0.elapsed_time(e1) / 1e3
    _, t_all, value = whole_job_rate(K, t)
    barrier()
    finite = bool(torch.isfinite(z).all().item())
    stages = 4 if p.rko == 4 else 2
    # per step: pass A of stage 1, then per stage pass B and pass C (fused with the next
    # stage's pass A) -> 2 * stages + 1; with the field-split column passes, pass C and the next
    # pass A are separate launches -> 3 * stages. One more launch per step computes the kick
    # increments (side stream) that the last pass C adds, or, on a diagnostics step, applies
    # the kick after the diagnostics, which add one nonlinear term (3 passes) and 5 kernels
    per_step = 3 * stages if sol.col_split else 2 * stages + 1
    launches = K * (per_step + 1) + ndiag * (3 + 5)

    # ---- diagnostics stated explicitly: the timed region holds ndiag diagnostics steps (one
    # every imix); here one diagnostics step is timed against a plain step, and the rate with
    # diagnostics every imix steps is derived from the two ------------------------------------
    diag = {}
    if rank == 0:
        nd = 10
        t_kind = {}
        for with_diag in (False, True):
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(nd):
                seed, _ = sol.main_step(z, seed, work, diag=with_diag)
            e1.record(stream)
            torch.cuda.synchronize()
            t_kind[with_diag] = e0.elapsed_time(e1) / nd
        extra = t_kind[True] - t_kind[False]
        diag = {"imix": p.imix, "ms_per_plain_step": t_kind[False],
                "ms_per_diag_step": t_kind[True], "ms_extra_per_diag_step": extra,
                "steps_per_s_diag_every_imix": 1e3 / (t_kind[False] + extra / p.imix),
                "note": "a diagnostics step adds one nonlinear term (3 passes) and the spectra, "
                        "fluxes and budgets of src/diagnostics.f90 to a plain step"}

    extras = {}
    if rank == 0:
        # ---- per-kernel CUDA-event timing (same workload, separate pass) ---------------
        kp = min(K, 100)
        sol.profile(True)
        for ipas in range(1, kp + 1):
            seed, _ = sol.main_step(z, seed, work, diag=(ipas % p.imix == 0))
        prof = sol.profile_read()
        sol.profile(False)
        tot = sum(v[0] for v in prof.values())
        kernels = {k: {"ms_per_launch": (v[0] / v[1]) if v[1] else None, "launches": v[1],
                       "share": v[0] / tot if tot else None} for k, v in prof.items() if v[1]}
        top = max(kernels, key=lambda k: kernels[k]["share"])
        peaks, src = measured_peaks()
        fp64 = fp64_gemm_tflops(torch, dev)
        fl, by = pass_model(p, top)
        ms = kernels[top]["ms_per_launch"]
        roof = {"kernel": top, "bound": "fp64",
                "achieved": fl / (ms / 1e3) / 1e12 if fl else None, "unit": "TFLOP/s",
                "peak": fp64, "peak_source": "cuBLAS DGEMM 4096^3 measured in this run "
                "(FP64 pipe; MEASURED_PEAKS.json has no FP64 figure)",
                "traffic": NCU_TRAFFIC.get((p.n, sol.variants[1] if top == "nlt_row" else sol.variants[0], top)),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch "
                                  "(capture of the same kernel and launch variant)",
                "hbm_achieved_gbs": by / (ms / 1e3) / 1e9 if by else None,
                "hbm_peak_gbs": peaks.get("hbm_gbs"), "hbm_peak_source": src}
        roof["frac"] = roof["achieved"] / fp64 if roof["achieved"] else None
        if roof["hbm_achieved_gbs"] and roof["hbm_peak_gbs"]:
            roof["hbm_frac"] = roof["hbm_achieved_gbs"] / roof["hbm_peak_gbs"]
        # the same kernel against the FP64 pipe itself: counted instructions per launch over
        # 2 per clock per SM at the SM clock sampled during the timed region
        ops = NCU_FP64_OPS.get((p.n, sol.variants[1] if top == "nlt_row" else sol.variants[0], top))
        mhz = clk.get("sm_mhz") if isinstance(clk, dict) else None
        if ops and mhz:
            pipe_peak = 2.0 * torch.cuda.get_device_properties(dev).multi_processor_count * mhz * 1e6
            roof["fp64_pipe"] = {"ops_per_launch": ops, "ops_source": "ncu smsp__sass_thread_inst_executed_op_"
                                 "{dfma,dadd,dmul}_pred_on.sum (same kernel and launch variant)",
                                 "achieved_gops": ops / (ms / 1e3) / 1e9, "peak_gops": pipe_peak / 1e9,
                                 "frac": ops / (ms / 1e3) / pipe_peak}
        extras["roofline"] = roof
        extras["kernels"] = kernels
        step_bytes = (26 if p.rko == 2 else 57) * 16 * p.n * (p.n // 2 + 1)
        extras["step_hbm_gbs"] = step_bytes * value / world / 1e9

        if not args.no_extras:
            # ---- no-diagnostics throughput (the comparison with the cuFFT baseline) ----
            z.copy_(z0)
            torch.cuda.synchronize()
            kn = min(K, 100)
            e0.record(stream)
            for _ in range(kn):
                seed, _ = sol.main_step(z, seed, work, diag=False)
            e1.record(stream)
            torch.cuda.synchronize()
            ours_nodiag = kn / (e0.elapsed_time(e1) / 1e3)

            # ---- end to end through the public API, host buffers every step ------------
            from gturbo_gb300.pipeline import HostPipeline
            host = torch.from_numpy(random_phase_ic(p, k0, 0.5, seed=1)).pin_memory()
            res_host = [torch.empty_like(host).pin_memory() for _ in range(2)]
            ke = min(K, 100)
            pipe = HostPipeline(sol)
            pipe.run([host], res_host, 3, seed, work)  # warm-up of the copy streams
            pipe.sync()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e0.record(pipe.h2d)
            seed = pipe.run([host], res_host, ke, seed, work, diag_every=p.imix)
            e1.record(pipe.d2h)
            pipe.sync()
            torch.cuda.synchronize()
            te = max(e0.elapsed_time(e1) / 1e3, 0.0)
            te_wall = time.perf_counter() - t0
            nbytes = host.numel() * 8
            extras["e2e"] = {"value": ke / max(te, te_wall), "unit": "steps/s",
                             "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                             "steps": ke, "note": "per step: pinned H2D of the step's input field, "
                             "main-loop step through gturbo_gb300.Solver (C-ABI), D2H of the result "
                             "field; copies on two copy streams overlap the neighbouring steps' "
                             "compute (gturbo_gb300.pipeline.HostPipeline)"}

            # ---- reference-equivalent GPU build (cuFFT + unfused kernels) --------------
            try:
                extras["ref_gpu_equivalent"] = refeq_run(p, k0, kn, W, dev, torch)
                extras["ref_gpu_equivalent"]["ours_nodiag_steps_s"] = ours_nodiag
                extras["ref_gpu_equivalent"]["speedup_nodiag"] = (
                    ours_nodiag / extras["ref_gpu_equivalent"]["value"])
            except Exception as e:  # reported, never fatal
                extras["ref_gpu_equivalent"] = {"unavailable": str(e)[:200]}

            # ---- batched ensemble (64 members of mixed size) vs the plain member loop ----
            try:
                extras["ensemble"] = ensemble_run(min(K, 100), W, torch, pdl=not args.no_pdl)
            except Exception as e:
                extras["ensemble"] = {"unavailable": str(e)[:300]}

            # ---- adjoint gradient (1024^2, 200 steps, checkpoints) vs the forward run ---
            try:
                extras["adjoint"] = adjoint_run(torch)
            except Exception as e:
                extras["adjoint"] = {"unavailable": str(e)[:300]}

            # ---- dumps and restarts, the split integrator, a non-square grid ------------
            try:
                extras["next_rows"] = next_rows_run(torch, fp64)
            except Exception as e:
                extras["next_rows"] = {"unavailable": str(e)[:300]}

            # ---- CPU baseline: the reference's statements on the host cores (the oracle
            # port where they are absent), and the oracle port beside it --------------------
            try:
                extras["cpu_baseline"] = (cpu_reference_run(p, k0, 10 ** 6, args.cpu_seconds)
                                          or cpu_oracle_run(p, k0, 10 ** 6, args.cpu_seconds))
            except Exception as e:
                extras["cpu_baseline"] = {"unavailable": str(e)[:200]}
            if extras["cpu_baseline"].get("kind") == "reference":
                try:
                    extras["cpu_baseline"]["port"] = cpu_oracle_run(p, k0, 10 ** 6, args.cpu_seconds / 2)
                except Exception as e:
                    extras["cpu_baseline"]["port"] = {"unavailable": str(e)[:200]}
            # ---- numpy, one thread, at 256^2 (c1) and at the bench's own size --------
            try:
                from gturbo_gb300.params import IC_K0, config
                np1 = {"c1": numpy_run(config("c1"), IC_K0["c1"], 3.0)}
                if args.config != "c1":
                    np1[args.config] = numpy_run(p, k0, 5.0)
                extras["cpu_baseline"]["numpy_1thread"] = np1
            except Exception as e:
                extras["cpu_baseline"]["numpy_1thread"] = {"unavailable": str(e)[:200]}
        if "e2e" not in extras:
            extras["e2e"] = {"value": None, "unit": "steps/s", "h2d_bytes_per_step": 0,
                             "d2h_bytes_per_step": 0, "note": "skipped (--no-extras)"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world, "steps": K,
                "warmup": W, "ms_per_step": 1e3 * t_all / K, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic (random-phase IC, reference LCG forcing, seed 481929)",
                "config": run_config(args),
                "settings": {"launch_variant": tune["variant"], "row_variant": sol.variants[1],
                             "col_split": sol.col_split, "pdl": sol.pdl,
                             "autotune_ms_per_step": tune["ms_per_step"]},
                "gpu_launches": launches, "finite": finite, "clocks": clk}
        diag["calls_timed"] = ndiag
        line["diagnostics"] = diag
        line.update(extras)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def step_flops(p):
    """FFT-convention FLOPs of the transforms one RK step of an NX x NY grid runs: per nonlinear
    term 5 column transforms of length NY over the columns up to the 2/3 cut (kx <= rtrunc NX/2;
    the others hold no retained mode and are not transformed) and 5 real row transforms of
    length NX over the NY rows."""
    nx, ny = p.n, p.rows
    cols = int(p.rtrunc * (nx // 2) + 1e-9) + 1
    per_nlt = 5 * cols * 5 * ny * math.log2(ny) + 5 * ny * 2.5 * nx * math.log2(nx)
    return (4 if p.rko == 4 else 2) * per_nlt


def _gpu_rate(sol, z, steps, torch):
    """Main-loop steps/s (forced, no diagnostics) of sol on z, CUDA events on its stream."""
    work = sol.work()
    seed = SEED
    for _ in range(3):
        seed, _ = sol.main_step(z, seed, work)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(sol.stream)
    for _ in range(steps):
        seed, _ = sol.main_step(z, seed, work)
    e1.record(sol.stream)
    torch.cuda.synchronize()
    assert bool(torch.isfinite(z).all().item())
    return steps / (e0.elapsed_time(e1) / 1e3)


def _cpu_ref_rate(p, z, budget_s):
    """Main-loop steps/s of the reference's statements (oracle/_ref, all host cores) on z."""
    import numpy as np

    from oracle import refcore

    if not refcore.available():
        return None
    ref = refcore.Reference(p)
    z = np.array(z, copy=True)
    work = [ref.zeros() for _ in range(4)]
    t0 = time.perf_counter()
    seed, _ = ref.main_step(z, SEED, 1, 10 ** 9, work)
    k = max(1, int(budget_s / max(time.perf_counter() - t0, 1e-6)))
    t0 = time.perf_counter()
    for ipas in range(2, k + 2):
        seed, _ = ref.main_step(z, seed, ipas, 10 ** 9, work)
    dt = time.perf_counter() - t0
    return {"value": k / dt, "unit": "steps/s", "cores": ref.threads, "steps": k, "kind": "reference"}


def next_rows_run(torch, fp64_tflops, cpu_budget_s=4.0):
    """The paths beside the main-loop step, each timed on the GPU against the FP64 roofline of
    its transforms and beside the reference's statements on the host cores (oracle/_ref):
      * dump and restart at 2048^2: gt_dump_real4 (inverse 2D transform with the real(4)
        conversion of src/write.f90:29-51 fused into its row pass, then the N x N floats to the
        host) and gt_load_real4 (the floats to the device, widening fused into the forward
        transform, trunc: src/read.f90 + src/main.f90:89-92), against the reference's
        fft_inv / fft_dir of the same field;
      * the split integrator emkx(i) emky(j) (src/rkstep.f90:21-27, 51-57) at 2048^2, RK2,
        alpha=2 with Laplacian viscosity and linear drag, against the emk table on the same run;
      * a non-square 4096 x 2048 (NX x NY) grid, the c2 workload's alpha=1 RK2 step."""
    import numpy as np

    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import IC_K0, config
    from gturbo_gb300.solver import Solver
    from oracle import refcore

    out = {}
    dev = torch.device("cuda", torch.cuda.current_device())
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    # ---- dump and restart -----------------------------------------------------------------
    p = config("c2")
    n = p.n
    sol = Solver(p)
    z = torch.from_numpy(random_phase_ic(p, IC_K0["c2"], 0.5, seed=1)).to(dev)
    fl2d = (n // 2 + 1) * 5 * n * math.log2(n) + n * 2.5 * n * math.log2(n)
    work = z.clone()
    wdev = torch.empty((n, n), dtype=torch.float32, device=dev)
    zr = sol.field()
    reps = 20
    t_dump = t_load = 0.0
    for it in range(reps + 2):  # device time of the kernels of one call (first two: warm-up)
        work.copy_(z)
        e0.record(sol.stream)
        sol._check(sol.lib.gt_dump_real4(sol.h, sol._ptr(work), wdev.data_ptr()))
        e1.record(sol.stream)
        torch.cuda.synchronize()
        t_dump += e0.elapsed_time(e1) if it >= 2 else 0.0
        e0.record(sol.stream)
        sol._check(sol.lib.gt_load_real4(sol.h, wdev.data_ptr(), sol._ptr(zr)))
        e1.record(sol.stream)
        torch.cuda.synchronize()
        t_load += e0.elapsed_time(e1) if it >= 2 else 0.0
    t_dump, t_load = t_dump / reps, t_load / reps
    w = sol.dump_real4(z)
    t0 = time.perf_counter()
    for _ in range(reps):
        w = sol.dump_real4(z)
    t_dump_e2e = (time.perf_counter() - t0) / reps * 1e3
    sol.load_real4(w, zr)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        sol.load_real4(w, zr)
    torch.cuda.synchronize()
    t_load_e2e = (time.perf_counter() - t0) / reps * 1e3
    dump = {"grid": f"{n}^2", "dump_ms": t_dump, "restart_ms": t_load,
            "dump_e2e_ms": t_dump_e2e, "restart_e2e_ms": t_load_e2e,
            "e2e_note": "Solver.dump_real4 / load_real4 from and to pageable host numpy arrays "
                        f"({n * n * 4} bytes of real(4) per call), host wall clock",
            "transform_tflops": {"dump": fl2d / (t_dump / 1e3) / 1e12,
                                 "restart": fl2d / (t_load / 1e3) / 1e12,
                                 "peak": fp64_tflops, "unit": "TFLOP/s (FFT convention)"}}
    try:
        if refcore.available():
            ref = refcore.Reference(p)
            a = z.cpu().numpy()
            for name in ("fft_inv", "fft_dir"):
                b = a.copy()
                t0 = time.perf_counter()
                getattr(ref, name)(b)
                k = max(1, int(cpu_budget_s / 2 / max(time.perf_counter() - t0, 1e-6)))
                t0 = time.perf_counter()
                for _ in range(k):
                    b[:] = a
                    getattr(ref, name)(b)
                dump["reference_" + name + "_ms"] = (time.perf_counter() - t0) / k * 1e3
            dump["reference_cores"] = ref.threads
    except Exception as e:
        dump["reference"] = {"unavailable": str(e)[:200]}
    out["dump_restart"] = dump
    sol.close()
    del work, wdev, zr

    # ---- split integrator -------------------------------------------------------------------
    pe = config("c2").replace(alpv=2.0, alpnu=1.0, nu=1e-5, alpmu=0.0, mu=0.1)
    ze = random_phase_ic(pe, IC_K0["c2"], 0.5, seed=2)
    rates = {}
    for split in (1, 0):
        s2 = Solver(pe.replace(split=split))
        rates[split] = _gpu_rate(s2, torch.from_numpy(ze).to(dev), 100, torch)
        s2.close()
    split_row = {"grid": f"{n}^2 RK2, alpha=2, nu k^2, mu (Ekman-NS)",
                 "split_steps_s": rates[1], "table_steps_s": rates[0],
                 "split_tflops": step_flops(pe) * rates[1] / 1e12, "peak": fp64_tflops}
    try:
        split_row["cpu_reference"] = _cpu_ref_rate(pe, ze, cpu_budget_s)
    except Exception as e:
        split_row["cpu_reference"] = {"unavailable": str(e)[:200]}
    out["split_integrator"] = split_row

    # ---- non-square grid ----------------------------------------------------------------------
    pn = config("c2").replace(n=2 * n, ny=n)
    zn = random_phase_ic(pn, IC_K0["c2"], 0.5, seed=3)
    s3 = Solver(pn)
    r = _gpu_rate(s3, torch.from_numpy(zn).to(dev), 50, torch)
    s3.close()
    ns_row = {"grid": f"{pn.n} x {pn.rows} (NX x NY), alpha=1 RK2 (the c2 step)", "steps_s": r,
              "tflops": step_flops(pn) * r / 1e12, "peak": fp64_tflops,
              "square_2048_step_flops_ratio": step_flops(pn) / step_flops(p)}
    try:
        ns_row["cpu_reference"] = _cpu_ref_rate(pn, zn, cpu_budget_s)
    except Exception as e:
        ns_row["cpu_reference"] = {"unavailable": str(e)[:200]}
    out["non_square"] = ns_row
    return out


# Device memory the adjoint leg lets the gradient hold for whole kept segments (gt_adj_set_memory):
# at 1024^2 RK2 (K = 20) a segment's stage states and physical fields take 1.34 GB, so 4 GiB keeps
# the last 3 of the 10 segments and the other 7 are recomputed from their checkpoints.
ADJ_MEMORY_BUDGET = 4 << 30


def adjoint_run(torch, rko=2):
    """The 1024^2 gradient workload: 200 RK2 (or, with rko=4, RK4) steps with the LCG kick
    (alpha=1, dt=5e-5), J =
    energy in the shells 4 <= |k| <= 8 at the final time, gradients with respect to the initial
    field and famp by the checkpointed adjoint (checkpoint every 20 steps). Reports the backward
    sweep against the plain forward run, and checks the gradient against the tangent-linear
    model (dot-product test) and a central finite difference along one random direction."""
    from gturbo_gb300.adjoint import forward_objective, gradient, tlm_run
    from gturbo_gb300.ic import random_phase_ic
    from gturbo_gb300.params import IC_K0, config
    from gturbo_gb300.solver import Solver

    p = config("c5")
    if rko == 4:
        p = p.replace(rko=4)
    nsteps, K, kmin, kmax = 200, 20, 4.0, 8.0
    sol = Solver(p)
    z0 = torch.from_numpy(random_phase_ic(p, IC_K0["c5"], 0.5, seed=1)).cuda()
    forward_objective(sol, z0, 3, SEED, kmin, kmax)  # warm-up
    torch.cuda.synchronize()
    s = sol.stream
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    J_fwd = forward_objective(sol, z0, nsteps, SEED, kmin, kmax)
    e1.record(s)
    torch.cuda.synchronize()
    t_fwd = e0.elapsed_time(e1)
    gradient(sol, z0, 2, SEED, kmin, kmax, checkpoint=K)  # warm-up
    # minimum memory: only the last segment kept whole, every other one recomputed
    _, _, _, _, (tf0, tb0) = gradient(sol, z0, nsteps, SEED, kmin, kmax, checkpoint=K, memory=0)
    # with a device-memory budget for whole kept segments: the forward sweep keeps its last
    # segments within it, and only the earlier ones are recomputed from their checkpoints
    budget = ADJ_MEMORY_BUDGET
    nfield = 8 * (p.n + 2) * p.n
    per_step = (2 if p.rko == 2 else 4) * (nfield + 24 * p.n * p.n)
    kept = max(1, min(-(-nsteps // K), budget // (K * per_step)))
    J, gz, gf, _, (tf, tb) = gradient(sol, z0, nsteps, SEED, kmin, kmax, checkpoint=K, memory=budget)
    sol.adj_memory = 0
    g = torch.Generator(device="cpu").manual_seed(3)
    dz = torch.randn(z0.shape, generator=g, dtype=torch.float64).cuda() * (z0.abs().max() / 4)
    torch.cuda.synchronize()
    e0.record(s)
    _, dJ = tlm_run(sol, z0, dz, 0.0, nsteps, SEED, kmin, kmax)
    e1.record(s)
    torch.cuda.synchronize()
    t_tlm = e0.elapsed_time(e1)
    adj = float((gz * dz).sum().item())
    h = 1e-6
    fd = (forward_objective(sol, z0 + h * dz, nsteps, SEED, kmin, kmax)
          - forward_objective(sol, z0 - h * dz, nsteps, SEED, kmin, kmax)) / (2 * h)
    return {"workload": f"{p.n}^2 alpha={p.alpv:g} RK{p.rko} dt={p.dt:g}, {nsteps} steps, LCG kick, "
                        f"J = energy in {kmin:g}<=|k|<={kmax:g}, checkpoint every {K}",
            "forward_ms": t_fwd, "adjoint_forward_sweep_ms": tf, "adjoint_backward_sweep_ms": tb,
            "backward_over_forward": tb / t_fwd, "gradient_over_forward": (tf + tb) / t_fwd,
            "memory_budget_bytes": budget, "segments_kept": kept, "segments": -(-nsteps // K),
            "min_memory": {"segments_kept": 1, "adjoint_forward_sweep_ms": tf0,
                           "adjoint_backward_sweep_ms": tb0,
                           "gradient_over_forward": (tf0 + tb0) / t_fwd},
            "tlm_ms": t_tlm, "tlm_over_forward": t_tlm / t_fwd,
            "J": J, "J_plain_forward": J_fwd, "dJdfamp": gf,
            "dot_test_rel": abs(adj - dJ) / abs(dJ), "fd_vs_tlm_rel": abs(fd - dJ) / abs(dJ),
            "fd_step": h}


def ensemble_run(steps, warm, torch, shard=False, pdl=True):
    """Member-steps/s of the 64-member mixed-size ensemble: batched (one launch per pass, CUDA
    graph) against the plain loop over members through the single-field C-ABI. With
    ``shard`` (every rank of the process group calls it) the members are split over the ranks
    by cost and the rates are whole-job: all ranks' member-steps over the slowest rank's time."""
    from gturbo_gb300.ensemble import Ensemble, PlainLoop, ensemble_c4

    import torch.distributed as dist

    from gturbo_gb300.replicas import member_cost, shard_members, whole_job_rate

    members = ensemble_c4()
    # sharded: each rank advances its own members (no data-path collective)
    world = dist.get_world_size() if shard and dist.is_available() and dist.is_initialized() else 1
    rank = dist.get_rank() if world > 1 else 0
    mine = shard_members([member_cost(m.params.n, m.params.rko) for m in members], world)[rank]
    members = [members[i] for i in mine]
    ens = Ensemble(members)
    ens.load_ic()
    z0 = [z.clone() for z in ens.z]
    ens.set_step(0)
    # tile family of the pass kernels: timed per family on these members (outside the timed
    # region, like a cuFFT plan), fields restored afterwards
    tune = ens.autotune(steps=5, cache=None)
    ens.step(warm)
    torch.cuda.synchronize()
    for z, a in zip(ens.z, z0):
        z.copy_(a)
    ens.set_step(0)
    s = ens.stream
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    ens.step(steps)
    e1.record(s)
    torch.cuda.synchronize()
    tb = e0.elapsed_time(e1) / 1e3
    finite = all(bool(torch.isfinite(z).all().item()) for z in ens.z)
    # plain loop on copies of the same initial fields
    zp = [a.clone() for a in z0]
    plain = PlainLoop(members, zp)
    for ps in plain.solvers:
        ps.pdl = pdl
    plain.step(min(warm, 2))
    kp = max(5, steps // 4)
    torch.cuda.synchronize()
    e0.record(s)
    plain.step(kp)
    e1.record(s)
    torch.cuda.synchronize()
    tp = e0.elapsed_time(e1) / 1e3
    nm = len(members)
    if world > 1:
        _, _, rate_b = whole_job_rate(nm * steps, tb)
        _, _, rate_p = whole_job_rate(nm * kp, tp)
    else:
        rate_b, rate_p = nm * steps / tb, nm * kp / tp
    return {"members": 64, "members_per_rank": nm, "ranks": world,
            "sizes": "32x256^2 + 24x512^2 + 8x1024^2", "rk": 4,
            "alphas": "drawn from {0.5,1,2,3}", "dt": "0.25/N", "forcing": "Philox per member",
            "batched_member_steps_s": rate_b, "batched_steps": steps,
            "plain_member_steps_s": rate_p, "plain_steps": kp,
            "speedup": rate_b / rate_p, "graph": True, "finite": finite,
            "tile_values_per_thread": tune["tile"], "autotune_ms_per_step": tune["ms_per_step"]}


def refeq_run(p, k0, steps, warm, dev, torch):
    """The reference-equivalent cuFFT build: steps/s of step + forcing (no diagnostics)."""
    import ctypes

    from baseline import build as bb
    from gturbo_gb300.ic import random_phase_ic

    lib = ctypes.CDLL(bb.build())
    P = ctypes.c_void_p
    lib.re_create.argtypes = [ctypes.c_void_p, ctypes.POINTER(P)]
    lib.re_set_stream.argtypes = [P, P]
    lib.re_step.argtypes = [P, P, P, P, P, P]
    lib.re_forcing.argtypes = [P, P]
    lib.re_set_seed.argtypes = [P, ctypes.c_int32]
    lib.re_destroy.argtypes = [P]
    cp = p.to_ctypes()
    h = P()
    rc = lib.re_create(ctypes.byref(cp), ctypes.byref(h))
    if rc:
        raise RuntimeError(f"re_create failed: {rc}")
    stream = torch.cuda.current_stream(dev)
    lib.re_set_stream(h, P(stream.cuda_stream))
    z = torch.from_numpy(random_phase_ic(p, k0, 0.5, seed=1)).to(dev)
    w = [torch.zeros_like(z) for _ in range(4)]
    ptr = lambda t: P(t.data_ptr())  # noqa: E731
    lib.re_set_seed(h, SEED)
    for _ in range(warm):
        lib.re_step(h, ptr(z), ptr(w[0]), ptr(w[1]), ptr(w[2]), ptr(w[3]))
        lib.re_forcing(h, ptr(z))
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        lib.re_step(h, ptr(z), ptr(w[0]), ptr(w[1]), ptr(w[2]), ptr(w[3]))
        lib.re_forcing(h, ptr(z))
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    finite = bool(torch.isfinite(z).all().item())
    lib.re_destroy(h)
    return {"value": steps / t, "unit": "steps/s", "steps": steps, "finite": finite,
            "what": "cuFFT in-place D2Z/Z2D + one kernel per OpenACC region of the reference "
                    "(no diagnostics), same GPU, same run"}


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    if args.only is not None:
        import torch
        import torch.distributed as dist
        world = int(os.environ.get("WORLD_SIZE", "1"))
        rank = int(os.environ.get("RANK", "0"))
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        if args.only == "ensemble":
            if world > 1:  # members sharded over the ranks
                dist.init_process_group("nccl", device_id=torch.device("cuda", torch.cuda.current_device()))
            res = ensemble_run(args.steps, max(3, args.warmup), torch, shard=world > 1, pdl=not args.no_pdl)
            if world > 1:
                dist.destroy_process_group()
        elif rank == 0 and args.only == "next":
            res = next_rows_run(torch, fp64_gemm_tflops(torch, torch.device("cuda", torch.cuda.current_device())))
        elif rank == 0:
            res = adjoint_run(torch, args.adjoint_rk)
        else:
            return 0
        if rank == 0:
            print(json.dumps(res), flush=True)
        return 0
    return ours_arm(args)


if __name__ == "__main__":
    sys.exit(main())
