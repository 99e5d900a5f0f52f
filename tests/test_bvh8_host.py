"""The compressed 8-wide BVH builder (lantern_gb300/csrc/lt_bvh8.cpp), checked
on the host by tests/native/bvh8_check.cpp: index ranges, one copy of every
triangle, conservative quantised boxes, and a host emulation of the device
traversal against brute-force closest hits on seeded rays."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bvh8_builder_and_traversal_on_host(tmp_path):
    cxx = os.environ.get("CXX", shutil.which("g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "bvh8_check")
    csrc = os.path.join(ROOT, "lantern_gb300", "csrc")
    cmd = [cxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + csrc,
           "-I/usr/local/cuda/include", os.path.join(ROOT, "tests", "native", "bvh8_check.cpp"),
           os.path.join(csrc, "lt_bvh8.cpp"), os.path.join(csrc, "lt_scene.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout[-2000:]
