"""bench.py's reference arm (the reference's algorithm on the host cores)
runs without a GPU and without loading the product's library; its JSON line
carries the contract's keys, on the same metric and config as the GPU arm."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROBE = r"""
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--cells", "64", "--steps", "1", "--warmup", "3"]
try:
    runpy.run_path("bench.py", run_name="__main__")
finally:
    maps = open("/proc/self/maps").read()
    print("PRODUCT_SO_LOADED" if "_solver.so" in maps else "PRODUCT_SO_ABSENT")
"""


def test_reference_arm_line():
    out = subprocess.run([sys.executable, "-c", PROBE], capture_output=True, text=True,
                         timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    assert "PRODUCT_SO_ABSENT" in out.stdout
    d = json.loads(lines[0])
    sys.path.insert(0, ROOT)
    import bench

    class A:
        cells, config, steps, max_substeps = 64, "config2", 1, 50000
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC
    assert d["config"] == json.loads(json.dumps(bench.config_dict(A)))
    for k in ("value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["value"] > 0 and d["higher_is_better"] is True and d["unit"] == "cells/s"
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
