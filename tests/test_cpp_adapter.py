"""The C++ drop-in for the reference's Integrator (tests/native/cpp_adapter.cpp:
GpuIntegrator over lt_render with the reference's FrameBuffer, two films
swapped per RenderFrame as the reference's render loop does). It compiles and
links against include/lantern_gpu.h and liblantern_gpu.so; where the reference
sources are staged (oracle/_ref/src) it uses the reference's own
camera/frame_buffer.{h,cpp}, else a stand-in of the same layout. On a GPU its
films, summed, equal the Python path's render of the same frames."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_DIR = os.path.join(ROOT, "lantern_gb300", "_build")
REF_SRC = os.path.join(ROOT, "oracle", "_ref", "src")


def reference_frame_buffer() -> bool:
    return os.path.exists(os.path.join(REF_SRC, "core", "camera", "frame_buffer.h"))


def _build(tmp_path):
    cxx = os.environ.get("CXX", shutil.which("g++"))
    if not cxx:
        pytest.skip("no C++ compiler")
    if not os.path.exists(os.path.join(LIB_DIR, "liblantern_gpu.so")):
        pytest.skip("liblantern_gpu.so not built")
    exe = str(tmp_path / "cpp_adapter")
    srcs = [os.path.join(ROOT, "tests", "native", "cpp_adapter.cpp")]
    flags = ["-std=c++17", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include")]
    if reference_frame_buffer():
        # the reference's FrameBuffer with the scalar stand-ins of Embree's vector
        # headers that oracle/build_ref.sh compiles the reference with
        flags += ["-DLT_REFERENCE_FRAME_BUFFER", "-include", "cstring", "-DEMBREE_STATIC_LIB",
                  "-I" + os.path.join(ROOT, "oracle", "ref_shim"), "-I" + os.path.join(REF_SRC, "core"),
                  "-I" + os.path.join(REF_SRC, "embree", "include")]
        srcs.append(os.path.join(REF_SRC, "core", "camera", "frame_buffer.cpp"))
    cmd = [cxx] + flags + srcs + ["-L" + LIB_DIR, "-llantern_gpu", "-Wl,-rpath," + LIB_DIR, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    return exe


def test_cpp_adapter_builds_against_the_c_abi(tmp_path):
    assert os.path.exists(_build(tmp_path))


def test_cpp_adapter_uses_the_reference_frame_buffer(tmp_path):
    if not reference_frame_buffer():
        pytest.skip("reference sources not staged (oracle/_ref/src)")
    exe = _build(tmp_path)
    r = subprocess.run(["nm", "-C", exe], capture_output=True, text=True)
    assert "Lantern::FrameBuffer::FrameBuffer(unsigned int, unsigned int)" in r.stdout


@pytest.mark.gpu
def test_cpp_adapter_renders_as_the_python_path(tmp_path, scene_dir):
    import torch

    import lantern_gb300.scenes as S
    from lantern_gb300.integrator import FrameBuffer, Integrator, Scene
    exe = _build(tmp_path)
    path = S.tiny_scene(width=24, height=20, name="cpp_adapter").write(scene_dir)
    out = str(tmp_path / "film.bin")
    frames = 6
    r = subprocess.run([exe, path, str(frames), out], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    raw = np.fromfile(out, dtype=np.uint32)
    w, h = int(raw[0]), int(raw[1])
    n = w * h
    rgb = raw[2:2 + 3 * n].view(np.float32).reshape(h, w, 3)
    bounces = raw[2 + 3 * n:2 + 4 * n].reshape(h, w)
    counts = raw[2 + 4 * n:2 + 5 * n].reshape(h, w)
    sc = Scene(0)
    sc.LoadSceneFromJSON(path)
    fb = FrameBuffer(sc.width, sc.height, "cuda:0")
    Integrator(sc, fb, max_depth=8, rr_depth=3).RenderFrame(frames)
    torch.cuda.synchronize()
    assert (w, h) == (sc.width, sc.height)
    assert np.array_equal(counts, fb.ColorSampleCount.cpu().numpy().astype(np.uint32))
    assert np.all(counts == frames)
    assert np.array_equal(bounces, fb.Bounces.cpu().numpy().astype(np.uint32))
    assert np.allclose(rgb, fb.ColorData.cpu().numpy(), rtol=1e-5, atol=1e-6)
