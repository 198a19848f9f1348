"""CPU: the reference arm's JSON line (bench.py --impl reference) describes
the same workload as the GPU arm's: one ``config`` dict built by
``bench.workload_config`` for both, and exactly the K timed and W warm-up
steps asked for."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_line_carries_the_shared_config():
    sys.path.insert(0, ROOT)
    import bench

    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2", "--warmup", "3",
                          "--n-systems", "8"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert (line["steps"], line["warmup"]) == (2, 3)
    assert line["config"] == bench.workload_config("ensemble8", 8, 8, 1)
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_reference_arm_names_workloads_it_does_not_time():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "large", "--steps", "2",
                          "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and "unavailable" in line
