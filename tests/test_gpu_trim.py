"""lt_trim: a context gives its work buffers back (wavefront arenas, the
differentiable forward's sample buffer, host-call staging) and keeps its
scene; the next calls allocate them again and render the same samples."""
import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.diff import DiffScene
from lantern_gb300.integrator import FrameBuffer, render_host

pytestmark = pytest.mark.gpu


def test_trim_frees_buffers_and_keeps_the_scene(scene_dir):
    path = S.nine_spheres(width=96, height=64, slices=16, stacks=8, name="trim_nine").write(scene_dir)
    ds = DiffScene(path)
    ctx = ds.ctx
    ctx.set_stream(torch.cuda.current_stream().cuda_stream)
    spp, depth = 64, 8
    films = []
    for k in range(2):
        fb = FrameBuffer(ds.width, ds.height, "cuda:0")
        ctx.render(fb.film(), spp, 0, depth, 3)
        d = ds.render(*ds.defaults(), spp=spp, max_depth=depth)
        h = render_host(ctx, ds.width, ds.height, 2, 5, depth, 3)
        torch.cuda.synchronize()
        films.append((fb, d, h))
        if k == 0:
            free_before, _ = torch.cuda.mem_get_info()
            ctx.trim()
            torch.cuda.synchronize()
            free_after, _ = torch.cuda.mem_get_info()
            # the buffers of 393,216 samples in flight (about 190 MB) went back
            assert free_after > free_before
    (a, da, ha), (b, db, hb) = films
    assert torch.equal(a.ColorSampleCount, b.ColorSampleCount) and torch.equal(a.Bounces, b.Bounces)
    assert torch.allclose(a.ColorData, b.ColorData, rtol=1e-5, atol=1e-6)
    for x, y in zip(da, db):  # the differentiable forward is deterministic
        assert torch.equal(x, y)
    assert np.array_equal(ha["counts"], hb["counts"]) and np.array_equal(ha["bounces"], hb["bounces"])
    assert np.allclose(ha["rgb"], hb["rgb"], rtol=1e-5, atol=1e-6)
