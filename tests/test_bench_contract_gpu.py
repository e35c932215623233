"""The bench's JSON line: every key a driver reads, with consistent values.

Runs `bench.py --small` (96x80x128) with the optional sections off and checks
the contract: metric/value/unit, step counts, timing keys, the roofline and
end-to-end objects, the sampled clocks and the kernel-launch count.
"""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_json_line_contract():
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--small", "--steps", "2", "--warmup", "3",
           "--no-cpu-baseline", "--no-batched", "--no-soft", "--no-linear"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "clocks", "e2e", "gpu_launches", "roofline"):
        assert key in d, key
    assert d["n_gpus"] == 1 and d["steps"] == 2 and d["warmup"] == 3
    assert d["higher_is_better"] is True and d["scaling"] == "weak" and d["unit"] == "pairs/s"
    assert d["value"] > 0 and abs(d["ms_per_step"] - 1000.0 / d["value"]) < 0.05 * d["ms_per_step"]
    assert "workload" in d["config"]
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 2 * 96 * 80 * 128 * 4 and e2e["d2h_bytes_per_step"] > 0
    roof = d["roofline"]
    for key in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert key in roof, key
    assert 0 < roof["frac"] < 1.5 and abs(roof["frac"] - roof["achieved"] / roof["peak"]) < 1e-6
    assert d["gpu_launches"] > 0
    assert "sm_mhz" in d["clocks"] and "reasons" in d["clocks"]
