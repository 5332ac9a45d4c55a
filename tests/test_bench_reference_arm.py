"""The reference arm of bench.py on the CPU (the oracle standing in for the
reference, which cannot be built): one JSON line with the contract's keys,
on the 128x128x150 box so that it runs in seconds."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--small",
                          "--steps", "1", "--warmup", "0"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "Mpoint-steps/s"
    for key in ("metric", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling", "dtype",
                "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert cb["production"]["value"] > 0 and cb["production"]["cores"] >= 1
    # the line's labels agree with each other: value = point-steps of one
    # bench step of the named workload / ms_per_step
    pts = line["config"]["point_steps_per_step"]
    assert abs(pts / (line["ms_per_step"] * 1e-3) / 1e6 - line["value"]) <= 1e-9 * line["value"]
    assert line["sample"]["kernel_accumulation_ms"] > 0 and line["sample"]["forward_step_ms"] > 0
