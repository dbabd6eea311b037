"""bench.py's command line and the JSON line of its reference arm, on the CPU.

The reference arm times the C oracle on the host cores (the reference itself has no CPU build),
so it runs without a GPU; the CUDA arm is exercised by the GPU runs of bench.py itself.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _bench_module():
    sys.path.insert(0, ROOT)
    try:
        import bench
    finally:
        sys.path.remove(ROOT)
    return bench


def _parse(argv, monkeypatch):
    bench = _bench_module()
    monkeypatch.setattr(sys, "argv", ["bench.py", *argv])
    return bench.parse()


def test_defaults(monkeypatch):
    """With no flags: one GPU, the c2 workload, the CUDA arm, every switch at its default."""
    a = _parse([], monkeypatch)
    assert (a.gpus, a.impl, a.config) == (1, "ours", "c2")
    assert a.steps >= 1 and a.warmup >= 3
    assert a.variant is None and a.row_variant is None and a.col_split is None
    assert not a.no_pdl and not a.no_extras and a.only is None


def test_switches(monkeypatch):
    a = _parse(["--variant", "1", "--row-variant", "2", "--col-split", "2", "--no-pdl", "--config", "c3",
                "--no-extras"], monkeypatch)
    assert (a.variant, a.row_variant, a.col_split, a.no_pdl, a.config) == (1, 2, 2, True, "c3")
    with pytest.raises(SystemExit):
        _parse(["--col-split", "3"], monkeypatch)


def test_reference_arm_line():
    """The reference arm prints one JSON line with the contract's keys: impl "reference", its
    own cpu_baseline and an e2e object without host-device copies."""
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", "c1", "--steps", "2",
                          "--warmup", "1", "--cpu-seconds", "1"], cwd=ROOT, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "dtype", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "steps/s" and line["higher_is_better"] is True
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
    from oracle import refcore
    if refcore.available():  # the reference's own statements, transliterated (oracle/_ref)
        assert line["cpu_baseline"]["kind"] == "reference"
    assert line["cpu_baseline"]["cores"] >= 1 and line["cpu_baseline"]["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_both_arms_share_one_config(monkeypatch):
    """Both arms build `config` with the same helper from the workload alone, so the two lines'
    configs are equal; launch settings of the CUDA arm live in its own `settings` object."""
    bench = _bench_module()
    a = _parse(["--config", "c1"], monkeypatch)
    cfg = bench.run_config(a)
    assert cfg == bench.run_config(_parse(["--config", "c1", "--impl", "reference"], monkeypatch))
    for k in ("workload", "n", "alpha", "rk", "dt", "imix", "parallelism", "l2"):
        assert k in cfg, k
    assert cfg["n"] == 256 and cfg["rk"] == 4
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--config", "c1", "--steps", "1",
                          "--warmup", "1", "--cpu-seconds", "1"], cwd=ROOT, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert json.loads(out.stdout.strip().splitlines()[-1])["config"] == cfg
