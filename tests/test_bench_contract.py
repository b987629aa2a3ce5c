"""The bench's reference arm on the CPU: one JSON line with the contract's keys (the GPU arm's
line is checked by the GPU runs of bench.py itself)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "2", "--warmup", "1", "--cell", "1e-3", "--start", "40"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference"
    assert line["value"] > 0.0 and line["unit"] == "element-cycles/s"
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    # the arms time the same window of the same scene: the reference's config is the dict the
    # GPU arm builds for the same flags
    sys.path.insert(0, ROOT)
    import argparse
    import bench
    args = argparse.Namespace(cell=1e-3, start=40, warmup=1, steps=2)
    cfg = line["config"]
    assert cfg == bench.bench_config(args, cfg["elements"], cfg["nodes"])
    assert line["window_state"]["t_start_us"] > 0.0
    assert line["ms_per_step"] > 0.0
