"""The context's work-ordering rules (lantern_gb300/csrc/lt_order.h) on the CPU:
a stream switch makes the new stream wait for the old one's work, and a host
rewrite of the pinned scene table waits for the last queued reader of the
table (the batched loop or a batched differentiable kernel, which return once
queued), whichever stream it was queued on. tests/native/order_check.cpp runs
the rules over a runtime that records its calls."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_work_order_rules(tmp_path):
    cxx = os.environ.get("CXX", shutil.which("g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "order_check")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-I" + os.path.join(ROOT, "lantern_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "native", "order_check.cpp"), "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr
