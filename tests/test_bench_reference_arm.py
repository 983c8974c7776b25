"""bench.py --impl reference on the host: one JSON line with the contract's keys (the oracle restatement timed
on host cores), and the 'unavailable' line for workloads it does not time."""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def _run(*args):
    env = dict(os.environ, PYTHONPATH=str(ROOT))
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", *args], cwd=ROOT,
                         capture_output=True, text=True, timeout=600, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, res.stdout
    return json.loads(lines[0])


def test_reference_arm_line():
    d = _run("--workload", "tfim4x4_D2_chi4", "--steps", "1", "--warmup", "0", "--ref-chains-per-core", "1")
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"] == d["e2e"]["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["config"]["workload"] == "tfim4x4_D2_chi4"


def test_reference_arm_unavailable_workload():
    d = _run("--workload", "uneven")
    assert d["impl"] == "reference" and "unavailable" in d


def test_reference_arm_gi_workload_times_the_gi_oracle():
    """gi9x9: the FP64 GI oracle over the host cores, one chain per core (about half a minute)."""
    d = _run("--workload", "gi9x9", "--steps", "1", "--warmup", "0")
    assert d["impl"] == "reference" and "unavailable" not in d and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"] == d["e2e"]["value"]
    assert d["config"]["workload"] == "gi9x9"


def test_reference_arm_other_ranks_exit_without_work():
    """Under torchrun with N > 1 only rank 0 times the reference and prints; the others exit 0 at once."""
    env = dict(os.environ, PYTHONPATH=str(ROOT), RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload",
                          "tfim4x4_D2_chi4", "--steps", "1", "--warmup", "0"], cwd=ROOT, capture_output=True,
                         text=True, timeout=120, env=env)
    assert res.returncode == 0, res.stderr[-2000:]
    assert not [l for l in res.stdout.splitlines() if l.startswith("{")]
