"""Scene loading on the host, before anything reaches the GPU: the loader and
the host scene build (tests/native/scene_check.cpp over lt_json.cpp and
lt_scene.cpp) accept the reference's scene JSON and LMF files and turn every
malformed input into a status instead of a crash -- missing files (LT_ERR_IO),
broken JSON and truncated LMF (LT_ERR_PARSE), and indices that point outside
their arrays (LT_ERR_INVALID). The light's radiance follows AreaLight's
constructor, color * radiant_power / (pi * area) (area_light.h:16-21)."""
import json
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

import lantern_gb300.scenes as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    cxx = os.environ.get("CXX", shutil.which("g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path_factory.mktemp("scene_check") / "scene_check")
    csrc = os.path.join(ROOT, "lantern_gb300", "csrc")
    cmd = [cxx, "-std=c++17", "-O1", "-ffp-contract=off", "-I" + os.path.join(ROOT, "include"), "-I" + csrc,
           "-I/usr/local/cuda/include", os.path.join(ROOT, "tests", "native", "scene_check.cpp"),
           os.path.join(csrc, "lt_json.cpp"), os.path.join(csrc, "lt_scene.cpp"), os.path.join(csrc, "lt_image.cpp"),
           "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def _run(exe, paths):
    r = subprocess.run([exe] + list(paths), capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    out = []
    for line in r.stdout.strip().splitlines():
        a, b, t, l, rad = line.split()
        out.append((int(a), int(b), int(t), int(l), float(rad)))
    return out


def _tiny(tmp_path, name):
    sc = S.tiny_scene(width=8, height=8, name=name)
    path = sc.write(str(tmp_path))
    return path, json.load(open(path)), sc


def test_valid_scene_and_light_radiance(checker, tmp_path):
    path, _, sc = _tiny(tmp_path, "ok")
    (a, b, tris, lights, rad), = _run(checker, [path])
    assert (a, b) == (0, 0) and tris == sc.num_triangles and lights == 1
    assert rad == pytest.approx(15.0 * np.pi * 4.0 / (np.pi * 4.0), rel=1e-6)  # L = 15 for the 2x2 quad


def test_malformed_inputs_are_statuses(checker, tmp_path):
    path, doc, sc = _tiny(tmp_path, "base")
    cases = {}
    cases["missing"] = (str(tmp_path / "no_such.json"), (5, -1))
    bad = tmp_path / "bad.json"
    bad.write_text('{"camera": {"client_width": 8, ')
    cases["bad_json"] = (str(bad), (6, -1))
    # a truncated LMF (half of the first mesh's file)
    lmf = os.path.join(str(tmp_path), doc["primitives"][0]["file_path"])
    data = open(lmf, "rb").read()
    trunc = tmp_path / "trunc.lmf"
    trunc.write_bytes(data[: len(data) // 2])
    d2 = json.loads(json.dumps(doc))
    d2["primitives"][0]["file_path"] = "trunc.lmf"
    p2 = tmp_path / "trunc.json"
    p2.write_text(json.dumps(d2))
    cases["truncated_lmf"] = (str(p2), (6, -1))
    # an LMF whose index points past its vertices
    m = sc.meshes[0]
    idx = m.indices.copy()
    idx[0, 0] = m.positions.shape[0] + 5
    S.write_lmf(str(tmp_path / "oob.lmf"), m.positions, idx, m.normals)
    d3 = json.loads(json.dumps(doc))
    d3["primitives"][0]["file_path"] = "oob.lmf"
    p3 = tmp_path / "oob.json"
    p3.write_text(json.dumps(d3))
    # a primitive naming a material that does not exist
    d4 = json.loads(json.dumps(doc))
    d4["primitives"][0]["material"] = "no_such_material"
    p4 = tmp_path / "nomat.json"
    p4.write_text(json.dumps(d4))
    names = list(cases)
    res = dict(zip(names, _run(checker, [cases[k][0] for k in names])))
    for k in names:
        assert res[k][:2] == cases[k][1], (k, res[k])
    (a, b, *_), (a4, b4, *_) = _run(checker, [str(p3), str(p4)])
    assert a == 0 and b == 1                  # loads, then LT_ERR_INVALID: index out of range
    assert (a4, b4) == (6, -1)                # an unknown material: LT_ERR_PARSE


def test_malformed_media_are_statuses(checker, tmp_path):
    """A medium missing a field its type needs is LT_ERR_PARSE (the reference
    reads absorption_color, absorption_at_distance and, for isotropic media,
    scattering_distance: scene.cpp:322-334); each well-formed kind loads."""
    paths, want = [], []
    for kind, kw in (("iso", {"reference_expressible": True}), ("absorb", {"non_scattering": True}), ("hg", {})):
        sc = S.medium_sphere_scene(width=8, height=8, name=f"med_{kind}", **kw)
        path = sc.write(str(tmp_path))
        paths.append(path)
        want.append((0, 0))
        doc = json.load(open(path))
        drop = {"iso": "scattering_distance", "absorb": "absorption_at_distance", "hg": "sigma_s"}[kind]
        del doc["media"][0][drop]
        bad = tmp_path / f"med_{kind}_bad.json"
        bad.write_text(json.dumps(doc))
        paths.append(str(bad))
        want.append((6, -1))
    res = _run(checker, paths)
    assert [r[:2] for r in res] == want, res
