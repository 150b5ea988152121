"""bench.py's reference arm (the oracle's OpenMP eigenvalue cycle on the host cores) prints one JSON
line with the fields the bench contract asks of it, and names the same workload and step as the GPU
arm's config; a small population keeps it to seconds.  No GPU is used."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "3", "--pop", "20000"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == "histories/s" and d["value"] > 0
    assert d["steps"] == 2 and d["warmup"] == 3 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    assert d["config"]["workload"] == "lattice_17x17_7g_eigen"
    # the GPU arm prints the same config dict for the same arguments
    sys.path.insert(0, ROOT)
    import bench
    ns = type("A", (), {"pop": 20000, "transport": "dt"})()
    assert d["config"] == bench.workload_config(ns, 1)
