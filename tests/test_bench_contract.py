"""The bench's JSON line keeps its contract: the keys, their types and their
consistency, for both arms (a short run of each)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                         cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


def test_our_arm_line():
    d = _run("--steps", "20", "--warmup", "3", "--cpu-seconds", "2", "--no-batched", "--no-adjoint",
             "--no-other-workloads")
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks"):
        assert k in d, k
    assert d["n_gpus"] == 1 and d["steps"] == 20 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["unit"] == "particle-updates/s" and d["dtype"] == "f32" and d["scaling"] == "weak"
    assert d["config"]["workload"] == "double_dambreak_1m" and d["config"]["particles"] == 1048576
    n = d["config"]["particles"]
    assert d["value"] == pytest.approx(n / (d["ms_per_step"] * 1e-3), rel=1e-6)
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"], rel=1e-9)
    e = d["e2e"]
    assert e["unit"] == d["unit"] and e["h2d_bytes_per_step"] == 2 * n * 12 and e["d2h_bytes_per_step"] == 2 * n * 12
    assert 0 < e["value"] < d["value"] and e["state_finite"]
    parts = e["parts_ms"]
    assert 0 < parts["set_state_return"] <= parts["set_state"] and parts["advance_frame"] > 0
    assert parts["get_state"] > 0
    c = d["cpu_baseline"]
    assert c["kind"] == "port" and c["cores"] >= 1 and c["value"] > 0
    assert d["gpu_launches"] == 5 * d["steps"]
    assert d["clocks"]["sm_max_mhz"] is None or d["clocks"]["sm_max_mhz"] > 0


def test_reference_arm_line():
    """The reference arm reports the GPU arm's metric, unit, config, steps and
    warm-up, and loads nothing of the product library."""
    d = _run("--impl", "reference", "--steps", "3", "--warmup", "3")
    assert d["impl"] == "reference" and d["unit"] == "particle-updates/s" and d["value"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["steps"] == 3 and d["warmup"] == 3 and d["gpu_launches"] == 0
    ours = _run("--steps", "3", "--warmup", "3", "--no-cpu-baseline", "--no-batched", "--no-adjoint",
                "--no-other-workloads")
    assert d["config"] == ours["config"] and d["metric"] == ours["metric"]
    code = ("import sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '3']; "
            "import runpy; runpy.run_path('bench.py', run_name='__main__'); "
            "print('LOADED', [l for l in open('/proc/self/maps') if 'libsimplefluid_gb300' in l])")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert "LOADED []" in out.stdout


def test_batched_and_adjoint_sections():
    """The batched section (sharding, autotuning, sequential and interleaved
    comparisons, CPU sample) and the adjoint section run from their workload
    configurations and report their records."""
    d = _run("--steps", "5", "--warmup", "3", "--cpu-seconds", "1", "--batch-steps", "3", "--no-other-workloads")
    b = d["batched"]
    assert b["scenes"] == 256 and b["steps"] == 3 and b["value"] > 0 and b["ratio_vs_sequential"] > 1
    assert b["ratio_vs_interleaved_streams"] == pytest.approx(b["value"] / b["interleaved_streams_value"])
    assert set(b["variants"]) == {"five_launches", "persistent_cluster4_block256", "persistent_cluster4_block1024",
                                  "persistent_cluster8_block256", "persistent_cluster8_block1024"}
    assert all(v > 0 for v in b["variants"].values()) and b["device_time_value"] > 0
    assert b["cpu_baseline"]["value"] > 0 and b["cpu_baseline"]["kind"] == "port"
    a = d["adjoint"]
    assert a["particles"] == 65536 and a["steps"] == 200 and a["ckpt_every"] == 20
    assert 0 < a["ratio_adjoint_over_forward"] < 10 and a["loss"] > 0
    assert set(a["passes_ms_per_step"]) == {"adj_integrate", "adj_forces", "adj_density"}
    r = a["roofline"]
    assert r["kernel"] == "k_adj_forces" and r["frac"] == pytest.approx(r["achieved"] / r["peak"])


def test_only_batched_prints_its_record():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--only", "batched", "--batch-steps", "2"],
                         capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    rec = json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("{")][-1])
    assert rec["section"] == "batched" and rec["scenes"] == 256 and rec["value"] > 0


def test_only_adjoint_prints_its_record():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--only", "adjoint"], capture_output=True,
                         text=True, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    rec = json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("{")][-1])
    assert rec["section"] == "adjoint" and rec["adjoint_ms"] > 0
