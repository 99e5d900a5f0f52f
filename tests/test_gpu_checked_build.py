"""The kernels with their device-side bound checks compiled in
(liblantern_gpu_checked.so, -DLT_CHECKS=1), in a process of their own
(tests/checked_worker.py). The stand-in for compute-sanitizer, which the test
machines cannot run: every queue slot, connection record, BVH node, leaf range,
traversal stack entry, hit primitive, scene slot, light, medium, mesh,
material and film pixel index that the wavefront kernels form is checked
before the access.

* No check fails on the parity scenes (three BVH widths on some), a render
  whose wavefront refills from work items, a three-scene batch, the
  fixed-scratch render and the differentiable forward and adjoint; the
  checked renders still match the oracle and the single-scene renders.
* A failed check is reported: a test-only film pixel limit below the film's
  size makes a normal render return LT_ERR_CHECK naming the film pixel check
  (the skipped accesses were in bounds), and the context renders cleanly once
  the limit is lifted.
"""
import json
import os
import subprocess
import sys

import pytest

from lantern_gb300 import build

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def result():
    build.build()
    env = dict(os.environ, LANTERN_GPU_CHECKED="1")
    r = subprocess.run([sys.executable, os.path.join(HERE, "checked_worker.py")], env=env, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_the_checked_library_ran(result):
    assert result["library"] == "liblantern_gpu_checked.so"
    assert "errors" not in result, result.get("errors")


def test_parity_scenes_pass_their_checks_and_match_the_oracle(result):
    assert len(result["parity"]) == 11
    for r in result["parity"]:
        assert r["counts"], r
        assert r["bounces"] > 0.97 and r["colour"] > 0.97, r


def test_refills_batch_noalloc_and_gradients_pass_their_checks(result):
    assert result["refills"] == {"min": 16, "max": 16}
    assert result["batch"] and result["noalloc"]
    assert result["diff"]["counts"] == 4 and result["diff"]["grad_finite"]


def test_a_failed_check_is_reported_and_the_context_recovers(result):
    assert result["planted"]["status"] == "LT_ERR_CHECK", result["planted"]
    assert "film pixel" in result["planted"]["message"]
    assert result["after_planted"] == {"min": 2, "max": 2}
