"""The benchmark's CPU arm (bench.py --impl reference) on a small case: one
JSON line in the GPU arm's metric and unit, accepted EXPREM steps as its
steps, and nothing of the GB300 library mapped into the process -- its
geometry comes from the oracle's own mesh preprocessing."""
import json
import os
import subprocess
import sys

from tests.helpers import ROOT


def test_reference_arm_loads_only_the_oracle():
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                          "--n-macro", "11", "--n-micro", "5", "--steps", "3", "--warmup", "2"],
                         capture_output=True, text=True, env=env, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"].startswith("G-evals/s") and line["unit"] == "G-evals/s"
    assert line["value"] > 0 and line["steps"] == 3 and line["warmup"] == 2
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["repo_libraries_loaded"] == ["oracle/libtsr_oracle_libm.so"]
