"""The bench's reference arm on the CPU: one JSON line with the GPU arm's metric, unit and workload,
its CPU baseline and end-to-end blocks; under several ranks only rank 0 works and prints."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def run_bench(args, env_extra=None):
    env = dict(os.environ, EMLAB_REFERENCE_BUDGET_S="20", **(env_extra or {}))
    p = subprocess.run([sys.executable, "bench.py", *args], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return [ln for ln in p.stdout.splitlines() if ln.startswith("{")]


@pytest.mark.timeout(600)
def test_reference_arm_line():
    import bench

    lines = run_bench(["--impl", "reference", "--workload", "plain_small", "--steps", "2", "--warmup", "3"])
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "Mcells/s"
    assert d["higher_is_better"] is True and d["n_gpus"] == 1 and d["steps"] >= 1 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] in ("reference", "port") and d["cpu_baseline"]["value"] == d["value"]
    assert d["cpu_baseline"]["cores"] >= 1 and d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "Mcells/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["cells"] == 128 ** 3 and d["config"]["workload"].startswith("plain_small 128x128x128")


def test_reference_arm_other_ranks_exit_without_work():
    lines = run_bench(["--impl", "reference", "--workload", "plain_small", "--steps", "2", "--warmup", "3"],
                      {"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert lines == []
