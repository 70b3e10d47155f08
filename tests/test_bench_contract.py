"""bench.py's reference arm runs on the host cores (no GPU): its JSON line
keeps the contract's keys for the headline workload and under --sim."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--sets", "3000",
                          "--steps", "1", "--warmup", "0", *args], capture_output=True, text=True, timeout=600,
                         env={**os.environ, "WORLD_SIZE": "1", "RANK": "0"})
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [json.loads(l) for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    return lines[0]


@pytest.mark.parametrize("sim", ["jaccard", "cosine"])
def test_reference_arm_line(sim):
    d = _run("--sim", sim)
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["sim"] == sim and d["config"]["result_pairs"] >= 0
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
