"""Failure handling without a GPU fault: injected allocation failures surface as
LT_ERR_OOM and leave the context usable; non-finite film contributions are
counted (the reference's NaN shading of a mesh without normals,
integrator.cpp:179-183, reproduced and reported)."""
import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.integrator import FrameBuffer, Integrator, Scene
from lantern_gb300.native import Context, LanternError, load

pytestmark = pytest.mark.gpu


def test_injected_allocation_failure_is_reported_and_recoverable(scene_dir):
    L = load()
    path = S.tiny_scene(width=24, height=24, name="fail_alloc").write(scene_dir)
    ctx = Context(0)
    try:
        L.lt_debug_fail_allocations(2)  # the scene upload needs more than two buffers
        with pytest.raises(LanternError, match="LT_ERR_OOM"):
            ctx.load_scene_json(path)
        L.lt_debug_fail_allocations(0xFFFFFFFF)
        ctx.load_scene_json(path)  # the same context loads the scene afterwards
        fb = FrameBuffer(24, 24, "cuda:0")
        ctx.set_stream(torch.cuda.current_stream().cuda_stream)
        L.lt_debug_fail_allocations(0)  # the first render allocates its wavefront
        with pytest.raises(LanternError, match="LT_ERR_OOM"):
            ctx.render(fb.film(), 2, 0, 8, 3)
        L.lt_debug_fail_allocations(0xFFFFFFFF)
        fb.Reset()
        ctx.render(fb.film(), 2, 0, 8, 3)
        torch.cuda.synchronize()
        assert int(fb.ColorSampleCount.min()) == 2 and float(fb.ColorData.sum()) > 0
    finally:
        L.lt_debug_fail_allocations(0xFFFFFFFF)
        ctx.close()


def test_nonfinite_contributions_are_counted(scene_dir):
    sc = S.tiny_scene(width=32, height=32, name="nan_normals")
    sc.meshes[0].normals = np.zeros((0, 3), np.float32)  # the Lambert sphere: no normals
    s = Scene(0)
    s.LoadSceneFromJSON(sc.write(scene_dir))
    fb = FrameBuffer(s.width, s.height, "cuda:0")
    it = Integrator(s, fb, max_depth=8)
    it.RenderFrame(2)
    torch.cuda.synchronize()
    assert it.stats().nonfinite_samples > 0
    assert not torch.isfinite(fb.ColorData).all()
    ok = Scene(0)
    ok.LoadSceneFromJSON(S.tiny_scene(width=32, height=32, name="finite_normals").write(scene_dir))
    it2 = Integrator(ok, FrameBuffer(ok.width, ok.height, "cuda:0"), max_depth=8)
    it2.RenderFrame(2)
    torch.cuda.synchronize()
    assert it2.stats().nonfinite_samples == 0
