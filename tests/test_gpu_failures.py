"""Failure handling without a GPU fault: injected allocation failures surface as
LT_ERR_OOM and leave the context usable; a render that runs out of its
iteration bound returns LT_ERR_TIMEOUT (lt_debug_set_iteration_limit lowers the
bound, nothing hangs: the loops are bounded on the host or by the captured
loop's condition kernel) and the contexts render correctly afterwards;
non-finite film contributions are counted (the reference's NaN shading of a
mesh without normals, integrator.cpp:179-183, reproduced and reported)."""
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


def test_iteration_limit_returns_timeout_and_contexts_recover(scene_dir):
    L = load()
    a = Scene(0)
    a.LoadSceneFromJSON(S.tiny_scene(width=32, height=32, name="timeout_a").write(scene_dir))
    b = Scene(0)
    b.LoadSceneFromJSON(S.nine_spheres(width=24, height=16, slices=12, stacks=6, name="timeout_b").write(scene_dir))
    stream = torch.cuda.current_stream().cuda_stream
    for s in (a, b):
        s.ctx.set_stream(stream)

    def films():
        return FrameBuffer(a.width, a.height, "cuda:0"), FrameBuffer(b.width, b.height, "cuda:0")

    spp, depth = 4, 8
    fa, fb = films()
    try:
        # two iterations cannot finish paths of up to 8 bounces
        L.lt_debug_set_iteration_limit(2)
        with pytest.raises(LanternError, match="LT_ERR_TIMEOUT"):
            a.ctx.render(fa.film(), spp, 0, depth, 3)
        with pytest.raises(LanternError, match="LT_ERR_TIMEOUT"):
            a.ctx.render_noalloc(fa.film(), spp, 1024, 0, depth, 3)
        with pytest.raises(LanternError, match="LT_ERR_TIMEOUT"):
            a.ctx.render_batch([a.ctx, b.ctx], [(spp, 0, depth, 3), (spp, 0, depth, 3)], [fa.film(), fb.film()])
    finally:
        L.lt_debug_set_iteration_limit(0)
    # at the library's own bound every context renders correctly again
    ra, rb = films()
    a.ctx.render(ra.film(), spp, 0, depth, 3)
    b.ctx.render(rb.film(), spp, 0, depth, 3)
    na, _ = films()
    a.ctx.render_noalloc(na.film(), spp, 1024, 0, depth, 3)
    ba, bb = films()
    a.ctx.render_batch([a.ctx, b.ctx], [(spp, 0, depth, 3), (spp, 0, depth, 3)], [ba.film(), bb.film()])
    torch.cuda.synchronize()
    for want, got in ((ra, na), (ra, ba), (rb, bb)):
        assert int(got.ColorSampleCount.min()) == spp and int(got.ColorSampleCount.max()) == spp
        assert torch.equal(got.Bounces, want.Bounces)
        assert torch.allclose(got.ColorData, want.ColorData, rtol=1e-5, atol=1e-6)
