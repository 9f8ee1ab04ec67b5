"""The bench's reference arm on CPU: `bench.py --impl reference` prints one JSON line
timing the reference's own integrator (its src/ built for the host, oracle/_ref) where
the reference sources or their staged copy are present, else the CPU restatement of it
(oracle/), with the keys the bench line carries."""
import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT


def _run(extra_env=None, *args):
    env = dict(os.environ, **(extra_env or {}))
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--res", "48", "--steps", "2",
           "--warmup", "1", "--tris", "2000", "--depth", "6", *args]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout[-2000:]          # one JSON line and nothing else on stdout
    return json.loads(lines[0])


def _check_common(line):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "config",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "Mrays/s" and line["higher_is_better"] is True
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"] == {"value": line["value"], "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_times_the_reference_integrator(native_lib):
    from oracle import build_ref
    if not (build_ref.available() or build_ref.staged_available()):
        pytest.skip("no reference sources or staged copy here")
    line = _run()
    _check_common(line)
    assert line["cpu_baseline"]["kind"] == "reference"
    assert line["config"]["pixels_per_step"] == 48 * 48


def test_reference_arm_falls_back_to_the_restatement_off_the_traversal_workload(native_lib):
    line = _run(None, "--workload", "cornell")
    _check_common(line)
    assert line["cpu_baseline"]["kind"] == "port"
    assert "traversal workload only" in line["config"]["reference_integrator"]
