"""bench.py's CPU arms, which run without a GPU: `--impl reference` prints one
JSON line with the reference integrator's rate (the oracle's C restatement for a
workload the reference's scene JSON cannot state), its own cpu_baseline block
and an e2e block without host-device copies."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_arm(workload):
    env = dict(os.environ, LT_REF_THREADS=str(min(8, os.cpu_count() or 1)))
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", workload,
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT,
                       env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def _check_line(d, workload, kind):
    assert d["impl"] == "reference" and "unavailable" not in d
    assert d["value"] > 0 and d["unit"] == "Msamples/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] >= 3
    assert d["config"]["workload"] == workload
    cb = d["cpu_baseline"]
    assert cb["kind"] == kind and cb["value"] == d["value"] and cb["cores"] >= 1
    assert d["e2e"] == {"value": d["value"], "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm(reference_available):
    if not reference_available:
        pytest.skip("reference integrator not built (its sources are not staged here)")
    _check_line(_reference_arm("nine-spheres"), "nine-spheres", "reference")


def test_reference_arm_of_a_workload_only_the_oracle_states():
    d = _reference_arm("medium-c2")
    _check_line(d, "medium-c2", "port")
    assert d["config"]["max_depth"] == 32 and d["config"]["width"] == 512
