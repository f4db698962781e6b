"""bench.py on the CPU.

- The reference arm runs on the host cores only: its JSON line carries the
  main line's metric, unit and workload with impl "reference", a
  cpu_baseline and an e2e object; under torchrun every rank but 0 exits 0
  without output.
- The clocks summary and the roofline arithmetic of the main line."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def _run(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", *args],
                          cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_line():
    import bench
    p = _run({}, "--steps", "1", "--warmup", "0")
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True
    assert d["config"]["workload"] == bench.WORKLOAD
    assert d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == d["value"]
    # the CPU model and the seed; the step's system solves are spread over
    # the workload's cells (a fixed cost per step and a cost per cell)
    assert cb["cpu_model"] and cb["seed"] == bench.SEED
    # (the fixed cost is fitted from two timings and clipped at 0: on a
    # loaded host it can come out as 0)
    assert cb["fixed_s_per_step"] >= 0 and cb["ms_per_cell"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    p = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--steps", "1", "--warmup", "0")
    assert p.returncode == 0, p.stderr[-2000:]
    assert not [ln for ln in p.stdout.splitlines() if ln.startswith("{")]


def test_clock_summary_reads_throttle_reasons():
    """The clocks object of the bench line: median SM clock under load, the
    maximum, and the throttle reasons nvidia-smi reports as Active."""
    import bench
    c = bench.Clocks()
    c.out = ["2070, 2070, 900.5, Not Active, Not Active, Not Active, Not Active",
             "2055, 2070, 1010.0, Not Active, Not Active, Not Active, Active",
             "1980, 2070, 1390.0, Active, Not Active, Not Active, Active",
             "garbage line", "[N/A], 2070, 0, Not Active, Not Active, Not Active, Not Active"]
    s = c.summary()
    assert s["sm_mhz"] == 2055.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]


def test_roofline_arithmetic(monkeypatch):
    """achieved / peak with the peak taken by bound: tensor from the measured
    bf16 figure, FP64 and FP32 from the measured FMA rates."""
    import bench
    monkeypatch.setattr(bench, "measured_peaks", lambda: (1900.0, 6800.0, "measured"))
    monkeypatch.setattr(bench, "fma_peak_tflops", lambda f64: 1.0 if f64 else 80.0)
    k = {"ms": 100.0, "launches": 4, "achieved_tflops": 0.5}
    r = bench.roofline_for("cells_fp64", k)
    assert r["bound"] == "fp64" and r["peak"] == 1.0 and r["frac"] == 0.5
    assert r["per_launch_ms"] == 25.0 and r["unit"] == "TFLOP/s"
    r = bench.roofline_for("var_tc", k)
    assert r["bound"] == "tensor" and r["peak"] == 1900.0
    r = bench.roofline_for("idw", k)
    assert r["bound"] == "fp32" and r["peak"] == 80.0
    assert bench.max_over_ranks(12.5, 1, "cpu") == 12.5
