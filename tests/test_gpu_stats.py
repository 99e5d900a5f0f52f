"""lt_render_stats: with stage timing on, the kernel times of the stages
(events around every launch), the device time of the whole render and the
time between its kernels are consistent; with it off (the default) the stage
times stay 0 and the render is the same; the ray counts add up to what was
traced."""
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.integrator import FrameBuffer, Integrator, Scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("paths", [0, 4096])  # the whole render in flight, and refills from work items
def test_stage_times_and_counts(scene_dir, paths):
    s = Scene(0)
    s.LoadSceneFromJSON(S.nine_spheres(width=64, height=48, slices=16, stacks=8, name="stats_nine").write(scene_dir))
    if paths:
        s.ctx.set_tuning(paths_in_flight=paths)
    s.ctx.set_stage_timing(True)
    fb = FrameBuffer(s.width, s.height, "cuda:0")
    it = Integrator(s, fb, max_depth=8, rr_depth=3)
    it.RenderFrame(8)
    torch.cuda.synchronize()
    st = it.stats()
    assert st.samples == 64 * 48 * 8
    assert st.init_ms > 0 and st.trace_ms > 0 and st.shade_ms > 0
    busy = st.init_ms + st.trace_ms + st.shade_ms
    assert busy <= st.gpu_ms * 1.001 + 1e-3
    assert st.idle_ms >= 0 and abs(busy + st.idle_ms - st.gpu_ms) <= 1e-3 * st.gpu_ms + 1e-3
    assert st.kernel_launches == 1 + 3 * st.iterations  # camera rays; trace, small-iteration trace, shade
    assert st.main_rays >= st.samples  # every sample traces its camera ray
    assert st.light_traversals <= st.light_rays + st.bsdf_rays
    assert int(fb.ColorSampleCount.min()) == 8
    # stage timing off: no stage times, the same samples
    s.ctx.set_stage_timing(False)
    fb2 = FrameBuffer(s.width, s.height, "cuda:0")
    Integrator(s, fb2, max_depth=8, rr_depth=3).RenderFrame(8)
    torch.cuda.synchronize()
    st2 = s.ctx.stats()
    assert st2.trace_ms == 0 and st2.shade_ms == 0 and st2.init_ms == 0 and st2.gpu_ms > 0
    assert st2.kernel_launches == st.kernel_launches and st2.main_rays == st.main_rays
    assert torch.equal(fb.ColorSampleCount, fb2.ColorSampleCount) and torch.equal(fb.Bounces, fb2.Bounces)


def test_launch_shapes_render_the_same_samples(scene_dir):
    """Threads per block of both stage kernels (64 to 256, 512 for the shade
    kernel) change the order of the queues and of the film additions, not the
    samples: counts and path lengths are equal, colours equal up to the order
    of float additions."""
    s = Scene(0)
    s.LoadSceneFromJSON(S.medium_sphere_scene(width=48, height=40, name="stats_shapes").write(scene_dir))
    films = []
    for tt, st in ((128, 256), (64, 512), (256, 64), (128, 128)):
        s.ctx.set_tuning(trace_threads=tt, shade_threads=st, paths_in_flight=2048)
        fb = FrameBuffer(s.width, s.height, "cuda:0")
        Integrator(s, fb, max_depth=16, rr_depth=3).RenderFrame(6)
        films.append(fb)
    torch.cuda.synchronize()
    a = films[0]
    for b in films[1:]:
        assert torch.equal(a.ColorSampleCount, b.ColorSampleCount) and torch.equal(a.Bounces, b.Bounces)
        assert torch.allclose(a.ColorData, b.ColorData, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("paths", [0, 4096])
def test_queue_trace_adds_up_to_the_ray_counts(scene_dir, paths):
    """lt_set_queue_trace / lt_queue_trace_get: one row per iteration; the path
    and camera rays sum to main_rays and the connection records to
    light_traversals. With every sample in flight the first row holds all
    camera rays as path rays and the paths only end; with a 4,096-path
    wavefront the later rows start paths from work items (camera rays)."""
    from lantern_gb300.native import LanternError
    s = Scene(0)
    s.LoadSceneFromJSON(S.nine_spheres(width=64, height=48, slices=16, stacks=8, name="qtrace_nine").write(scene_dir))
    if paths:
        s.ctx.set_tuning(paths_in_flight=paths)
    s.ctx.set_queue_trace(4096)
    fb = FrameBuffer(s.width, s.height, "cuda:0")
    it = Integrator(s, fb, max_depth=8, rr_depth=3)
    it.RenderFrame(8)
    torch.cuda.synchronize()
    st = it.stats()
    q = s.ctx.queue_trace().astype("int64")
    assert q.shape == (st.iterations, 3)
    assert int(q[:, 0].sum() + q[:, 1].sum()) == st.main_rays
    assert int(q[:, 2].sum()) == st.light_traversals
    assert q[0, 2] == 0  # no connection record before the first shade
    if paths == 0:
        assert q[0, 0] == 64 * 48 * 8 and q[:, 1].sum() == 0 and (q[1:, 0] <= q[:-1, 0]).all()
    else:
        assert q[0, 0] == paths and q[:, 1].sum() == 64 * 48 * 8 - paths
    with pytest.raises(LanternError, match="LT_ERR_INVALID"):
        s.ctx.set_queue_trace(1 << 20)
    s.ctx.set_queue_trace(0)  # off: the next render records nothing
    Integrator(s, FrameBuffer(s.width, s.height, "cuda:0"), max_depth=8, rr_depth=3).RenderFrame(1)
    assert s.ctx.queue_trace().shape == (0, 3)
