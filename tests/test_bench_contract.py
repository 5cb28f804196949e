"""The reference arm of bench.py runs on the host cores alone: one JSON line
with the contract's keys, the CPU restatement timed on the same workload and
config object as the GPU arm, and an e2e entry without copies."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_contract():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    sys.path.insert(0, ROOT)
    import bench
    assert d["config"] == bench.workload_config(4, 64)
    assert d["cpu_baseline"]["build"].startswith("gcc -O3")


def test_headline_algorithmic_bytes():
    """p=4 on 64^3 deformed cells in FP32: x read and y written once (16.97 M
    nodes) plus 6 geometry entries per Gauss point of 262,144 cells:
    922,228,744 bytes per apply, the roofline's numerator"""
    import sys
    sys.path.insert(0, ROOT)
    import bench
    cfg = bench.workload_config(4, 64)
    assert cfg["n_dofs"] == 257 ** 3 == 16974593
    assert bench.algorithmic_bytes(4, cfg["n_dofs"], 64 ** 3, 4) == 922228744
