"""The CPU reference arm of bench.py.  The reference's CPU path cannot solve
one point of the headline workload (300 x 192) within the step budget, so
the arm prints the reason and no value (so no ratio across sizes is formed),
with one measured 60 x 32 sample of the same physics through the oracle's
CPU path (C assembly, LAPACK boundary rows, SuperLU + ARPACK).  Needs no
GPU."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]

pytestmark = pytest.mark.timeout(600)


def _run(env_extra):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                           "--warmup", "0"], cwd=ROOT, env=env, capture_output=True, text=True,
                          timeout=540)


def test_reference_arm_line():
    r = _run({})
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert "300x192" in d["unavailable"] and "value" not in d
    assert d["metric"].startswith("eigenpairs/s at resid<=1e-10") and d["unit"] == "eigenpairs/s"
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["n_gpus"] == 1
    smp = d["sample"]
    assert smp["kind"] == "port" and smp["cores"] >= 1 and smp["value"] > 0
    # every pair of the 60 x 32 sample converged to the residual bar
    assert smp["eigenpairs"] == 8


def test_reference_arm_other_ranks_are_silent():
    r = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
