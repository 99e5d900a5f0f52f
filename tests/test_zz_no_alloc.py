"""lt_render_noalloc, the render entry point that allocates nothing.

It is for callers that cannot have the library allocate GPU memory while they
run -- an application that hands the library a fixed memory budget at start-up
and forbids later allocations, or an interactive loop where cudaMalloc/cudaFree
(which may synchronise the whole device) would stall other work. Its wavefront
state lives in a fixed array inside the library (LT_NOALLOC_MAX_PATHS path
slots). Called through the C ABI, two calls in a row must give what lt_render
gives for the same samples: identical sample counts and path lengths, and
colour sums equal up to float atomic-add order (rtol 1e-5). The array keeps
the previous call's contents, so the second call also checks that a call
starts from a clean state. A fresh context's first call leaves the device's
free memory unchanged, and its statistics count what lt_render's count. This
file is named to be collected last.
"""
import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.integrator import FrameBuffer
from lantern_gb300.native import NOALLOC_MAX_PATHS, Context, Film, LanternError

pytestmark = pytest.mark.gpu

DEPTH, RR = 12, 3
CALLS = [(0, 6, 4096), (100, 3, NOALLOC_MAX_PATHS)]  # (first frame, spp, paths in flight)


@pytest.mark.parametrize("bvh_width", [2, 8])
def test_noalloc_render_matches_render(scene_dir, bvh_width):
    path = S.tiny_scene(width=48, height=40, name="noalloc_tiny").write(scene_dir)
    ctx = Context(0)
    ctx.load_scene_json(path)
    ctx.set_tuning(bvh_width=bvh_width)
    info = ctx.scene_info()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    expected = []
    for first, spp, _ in CALLS:
        fb = FrameBuffer(info.width, info.height, "cuda:0")
        ctx.render(fb.film(), spp, first, DEPTH, RR)
        expected.append(fb)
    got = []
    for first, spp, paths in CALLS:  # two lt_render_noalloc calls in a row
        fb = FrameBuffer(info.width, info.height, "cuda:0")
        ctx.render_noalloc(fb.film(), spp, paths, first, DEPTH, RR)
        got.append(fb)
    torch.cuda.synchronize()
    for (first, spp, _), e, g in zip(CALLS, expected, got):
        assert int(g.ColorSampleCount.min()) == spp and int(g.ColorSampleCount.max()) == spp
        assert torch.equal(g.ColorSampleCount, e.ColorSampleCount)
        assert torch.equal(g.Bounces, e.Bounces)
        assert torch.allclose(g.ColorData, e.ColorData, rtol=1e-5, atol=1e-6)
        assert float(g.ColorData.sum()) > 0.0
    ctx.close()


def test_noalloc_rejects_sizes_beyond_its_limit(scene_dir):
    path = S.tiny_scene(width=8, height=8, name="noalloc_limits").write(scene_dir)
    ctx = Context(0)
    ctx.load_scene_json(path)
    fb = FrameBuffer(8, 8, "cuda:0")
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    for bad in (0, NOALLOC_MAX_PATHS + 1):
        with pytest.raises(LanternError) as e:
            ctx.render_noalloc(fb.film(), 1, bad)
        assert e.value.status == 1 and "paths_in_flight" in str(e.value)
    host = np.zeros((8, 8, 3), np.float32), np.zeros((8, 8), np.uint32), np.zeros((8, 8), np.uint32)
    with pytest.raises(LanternError) as e:
        ctx.render_noalloc(Film(host[0].ctypes.data, host[1].ctypes.data, host[2].ctypes.data, 8, 8, 0), 1, 64)
    assert e.value.status == 1
    ctx.close()


def test_noalloc_first_call_on_a_fresh_context_allocates_nothing(scene_dir):
    """lt_ctx_create did the set-up (loaded the module holding the fixed array
    and the wavefront kernels, looked up the array's address): the first
    lt_render_noalloc of a new context changes nothing in device memory."""
    path = S.tiny_scene(width=32, height=24, name="noalloc_fresh").write(scene_dir)
    ctx = Context(0)
    ctx.load_scene_json(path)
    info = ctx.scene_info()
    fb = FrameBuffer(info.width, info.height, "cuda:0")
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    free_before, _ = torch.cuda.mem_get_info()
    ctx.render_noalloc(fb.film(), 4, 8192, 0, DEPTH, RR)
    torch.cuda.synchronize()
    free_after, _ = torch.cuda.mem_get_info()
    assert free_after == free_before
    assert int(fb.ColorSampleCount.min()) == 4
    ctx.close()


def test_noalloc_stats_count_as_render(scene_dir):
    """Ray, connection and non-finite counts of lt_render_noalloc equal
    lt_render's for the same samples (a sphere without normals shades with
    NaN, as the reference's integrator.cpp:179-183 does)."""
    sc = S.tiny_scene(width=32, height=32, name="noalloc_nan")
    sc.meshes[0].normals = np.zeros((0, 3), np.float32)
    ctx = Context(0)
    ctx.load_scene_json(sc.write(scene_dir))
    info = ctx.scene_info()
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    fa = FrameBuffer(info.width, info.height, "cuda:0")
    ctx.render(fa.film(), 3, 0, 8, RR)
    ra = ctx.stats()
    fb = FrameBuffer(info.width, info.height, "cuda:0")
    ctx.render_noalloc(fb.film(), 3, 2048, 0, 8, RR)
    rb = ctx.stats()
    assert ra.nonfinite_samples > 0 and rb.nonfinite_samples == ra.nonfinite_samples
    for k in ("main_rays", "light_rays", "bsdf_rays", "light_traversals", "samples"):
        assert getattr(rb, k) == getattr(ra, k), k
    ctx.close()
