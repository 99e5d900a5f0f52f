"""Batched multi-scene rendering (lt_render_batch) against one lt_render per
scene: the same samples are traced either way, so per pixel the sample counts
and summed path lengths are equal and the colour sums agree up to the order of
the float additions into the film."""
import ctypes as C
import os

import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.integrator import FrameBuffer, Integrator, RenderBatch, Scene
from lantern_gb300.native import Film, LanternError

pytestmark = pytest.mark.gpu


def _load(scene_dir, sc):
    s = Scene(0)
    s.LoadSceneFromJSON(sc.write(scene_dir))
    return s


def _pair(s, depth, first_frame):
    fa = FrameBuffer(s.width, s.height, "cuda:0")
    fb = FrameBuffer(s.width, s.height, "cuda:0")
    return (Integrator(s, fa, max_depth=depth, rr_depth=3, first_frame=first_frame),
            Integrator(s, fb, max_depth=depth, rr_depth=3, first_frame=first_frame))


def _same(a: FrameBuffer, b: FrameBuffer):
    assert torch.equal(a.ColorSampleCount, b.ColorSampleCount)
    assert torch.equal(a.Bounces, b.Bounces)
    x, y = a.ColorData.double(), b.ColorData.double()
    scale = float(x.abs().max()) + 1e-30
    assert float((x - y).abs().max()) <= 1e-5 * scale, float((x - y).abs().max()) / scale


def _check_batch(scenes, spps, depths, frames):
    single, batched = [], []
    for s, d, f0 in zip(scenes, depths, frames):
        a, b = _pair(s, d, f0)
        single.append(a)
        batched.append(b)
    for it, spp in zip(single, spps):
        it.RenderFrame(spp)
    RenderBatch(batched, spps)
    torch.cuda.synchronize()
    for a, b, spp in zip(single, batched, spps):
        _same(a.frame_buffer, b.frame_buffer)
        assert int(b.frame_buffer.ColorSampleCount.min()) == spp
        assert b.frame_number == a.frame_number
    return batched


def test_batch_equals_individual_renders(scene_dir):
    scenes = [_load(scene_dir, S.tiny_scene(width=48, height=40, name="bt_tiny")),
              _load(scene_dir, S.nine_spheres(width=64, height=64, name="bt_c0", slices=16, stacks=8)),
              _load(scene_dir, S.medium_sphere_scene(width=40, height=56, name="bt_med")),
              _load(scene_dir, S.displaced_icosphere_scene(width=64, height=48, levels=4, name="bt_ico"))]
    # ragged spp, depths and first frames; one scene twice with different frames
    order = [0, 1, 2, 3, 0]
    _check_batch([scenes[i] for i in order], [4, 3, 16, 5, 2], [8, 10, 32, 6, 8], [0, 7, 1, 100, 4])


def test_batch_renders_wavefront_filling_scenes_alone(scene_dir):
    """A scene whose samples fill the owner's wavefront (here paths_in_flight
    8192: three of the five renders) is rendered with the single-scene kernels
    after the captured loop of the others; every film is still the
    single-scene render's, and the statistics count every sample."""
    scenes = [_load(scene_dir, S.tiny_scene(width=48, height=40, name="bt_tiny")),
              _load(scene_dir, S.nine_spheres(width=64, height=64, name="bt_c0", slices=16, stacks=8)),
              _load(scene_dir, S.medium_sphere_scene(width=40, height=56, name="bt_med")),
              _load(scene_dir, S.displaced_icosphere_scene(width=64, height=48, levels=4, name="bt_ico"))]
    scenes[0].ctx.set_tuning(paths_in_flight=8192)
    order, spps = [0, 1, 2, 3, 0], [4, 3, 16, 5, 2]
    _check_batch([scenes[i] for i in order], spps, [8, 10, 32, 6, 8], [0, 7, 1, 100, 4])
    st = scenes[0].ctx.stats()
    assert st.samples == sum(scenes[i].width * scenes[i].height * n for i, n in zip(order, spps))
    assert st.main_rays > 0 and st.kernel_launches > 0


def test_batch_edge_cases(scene_dir):
    s = _load(scene_dir, S.tiny_scene(width=24, height=24, name="bt_edge"))
    # spp 0 (no work) and max_depth 0 (counts only) next to a normal scene
    a, b = _pair(s, 0, 0)
    c, d = _pair(s, 8, 0)
    e, f = _pair(s, 8, 0)
    a.RenderFrame(3)
    c.RenderFrame(0)
    e.RenderFrame(2)
    RenderBatch([b, d, f], [3, 0, 2])
    torch.cuda.synchronize()
    for x, y in ((a, b), (c, d), (e, f)):
        _same(x.frame_buffer, y.frame_buffer)
    assert int(b.frame_buffer.ColorSampleCount.max()) == 3 and float(b.frame_buffer.ColorData.abs().max()) == 0.0
    assert int(d.frame_buffer.ColorSampleCount.max()) == 0
    # an empty batch is a no-op
    RenderBatch([], [])


def test_batch_rejects_bad_arguments(scene_dir):
    s = _load(scene_dir, S.tiny_scene(width=16, height=16, name="bt_bad"))
    host = {"rgb": np.zeros((16, 16, 3), np.float32), "b": np.zeros((16, 16), np.uint32),
            "n": np.zeros((16, 16), np.uint32)}
    film = Film(host["rgb"].ctypes.data, host["b"].ctypes.data, host["n"].ctypes.data, 16, 16, 0)
    with pytest.raises(LanternError, match="LT_ERR_INVALID"):
        s.ctx.render_batch([s.ctx], [(1, 0, 8, 3)], [film])
    fb = FrameBuffer(8, 8, "cuda:0")  # wrong size
    with pytest.raises(LanternError, match="LT_ERR_INVALID"):
        s.ctx.render_batch([s.ctx], [(1, 0, 8, 3)], [fb.film()])
    # one entry more than LT_MAX_BATCH is rejected before any work is queued
    from lantern_gb300.native import MAX_BATCH
    ok = FrameBuffer(16, 16, "cuda:0")
    with pytest.raises(LanternError, match="LT_ERR_INVALID"):
        s.ctx.render_batch([s.ctx] * (MAX_BATCH + 1), [(1, 0, 8, 3)] * (MAX_BATCH + 1), [ok.film()] * (MAX_BATCH + 1))
    with pytest.raises(LanternError, match="LT_ERR_INVALID"):
        s.ctx.set_tuning(trace_threads=96)
    with pytest.raises(LanternError, match="LT_ERR_UNSUPPORTED"):
        s.ctx.set_tuning(bvh_width=3)


def test_generated_batch_with_tuning(scene_dir):
    gen = S.batch_scenes(count=10, max_resolution=128, max_triangles=30_000, name="bt_gen")
    scenes = [_load(scene_dir, sc) for sc in gen]
    owner = scenes[0].ctx
    t = owner.autotune_batch([s.ctx for s in scenes],
                             [(1, 0, sc.render["max_depth"], 3) for sc in gen], spp_cap=1)
    assert t.trace_threads in (64, 128, 256) and t.loop_iterations in (2, 4, 8) and t.ms > 0
    assert owner.tuning().as_dict() == t.as_dict()
    # a tuning that differs from the default in every field still gives the same image
    owner.set_tuning(paths_in_flight=4096, trace_threads=64, shade_threads=256, loop_iterations=8, bvh_width=8)
    _check_batch(scenes, [sc.render["spp"] // 4 + 1 for sc in gen], [sc.render["max_depth"] for sc in gen],
                 list(range(len(gen))))
    st = owner.stats()
    assert st.iterations > 0 and st.kernel_launches > 2 * st.iterations


def test_diff_batch_equals_individual(scene_dir):
    from lantern_gb300.diff import DiffScene, adjoint_batch, render_batch
    s1 = DiffScene(S.tiny_scene(width=40, height=32, name="bd_tiny").write(scene_dir))
    s2 = DiffScene(S.differentiable_scene(width=48, height=40, slices=16, stacks=8, name="bd_diff").write(scene_dir))
    s3 = DiffScene(S.medium_sphere_scene(width=32, height=24, name="bd_med").write(scene_dir))
    scenes = [s1, s2, s3, s1]
    g = torch.Generator(device="cuda:0").manual_seed(7)
    params = []
    for sc in scenes:
        a, e, sa, ss = sc.defaults()
        a = (a * (0.7 + 0.3 * torch.rand(a.shape, generator=g, device=a.device))).contiguous()
        params.append((a, e, sa * 1.1, ss * 0.9))
    spp, ff = [3, 4, 2, 5], [0, 1, 2, 9]
    outs = render_batch(scenes, params, spp, ff, max_depth=8, rr_depth=3, keep_samples=True)
    dI = []
    for k, sc in enumerate(scenes):
        ref = sc.render(*params[k], spp[k], ff[k], 8, 3, keep_samples=True)
        for x, y in zip(outs[k], ref):
            assert torch.equal(x, y)  # same per-sample arithmetic, films summed in sample order
        dI.append(torch.rand((sc.height, sc.width, 3), generator=g, device="cuda:0") - 0.5)
    for samples in ([o[3] for o in outs], None):
        gb = adjoint_batch(scenes, params, dI, spp, ff, 8, 3, samples=samples)
        for k, sc in enumerate(scenes):
            gs = sc.adjoint(*params[k], dI[k], spp[k], ff[k], 8, 3, samples=None if samples is None else samples[k])
            for x, y in zip(gb[k], gs):
                scale = float(y.abs().max()) + 1e-30
                assert float((x - y).abs().max()) <= 1e-4 * scale, (k, float((x - y).abs().max()) / scale)


def test_batch_with_textures_and_procedural_primitives(scene_dir):
    """Image and uv albedo textures and grid / geosphere primitives in a batch,
    next to a plain scene, equal to one render per scene."""
    scenes = [_load(scene_dir, S.textured_scene(os.path.join(scene_dir, "textures"), width=40, height=32,
                                                name="bt_tex")),
              _load(scene_dir, S.procedural_scene(width=32, height=24, name="bt_proc")),
              _load(scene_dir, S.tiny_scene(width=24, height=20, name="bt_tiny2"))]
    _check_batch(scenes, [3, 4, 2], [8, 8, 6], [2, 9, 0])


def test_diff_batch_with_a_job_that_runs_alone(scene_dir):
    """A job of 2^24 samples or more (here 512x512 at 64 spp) fills the
    default wavefront by itself: lt_render_diff_batch renders it on the
    single-scene wavefront and lt_render_adjoint_batch replays it there, the
    other jobs together on one wavefront. Films and per-sample radiance equal
    the single-scene calls' bit for bit; every job's gradients equal its
    single-scene adjoint's (up to the order of the float sums)."""
    from lantern_gb300.diff import DiffScene, adjoint_batch, render_batch
    big = DiffScene(S.differentiable_scene(width=512, height=512, slices=16, stacks=8, name="ba_big").write(scene_dir))
    s1 = DiffScene(S.tiny_scene(width=40, height=32, name="ba_tiny").write(scene_dir))
    s2 = DiffScene(S.medium_sphere_scene(width=32, height=24, name="ba_med").write(scene_dir))
    scenes, spp = [s1, big, s2], [3, 64, 2]
    assert big.width * big.height * spp[1] >= 1 << 24
    params = [sc.defaults() for sc in scenes]
    outs = render_batch(scenes, params, spp, 0, max_depth=6, rr_depth=3, keep_samples=True)
    for k, sc in enumerate(scenes):
        ref = sc.render(*params[k], spp[k], 0, 6, 3, keep_samples=True)
        for x, y in zip(outs[k], ref):
            assert torch.equal(x, y), k
    g = torch.Generator(device="cuda:0").manual_seed(5)
    dI = [torch.rand((sc.height, sc.width, 3), generator=g, device="cuda:0") - 0.5 for sc in scenes]
    gb = adjoint_batch(scenes, params, dI, spp, 0, 6, 3, samples=[o[3] for o in outs])
    for k, sc in enumerate(scenes):
        gs = sc.adjoint(*params[k], dI[k], spp[k], 0, 6, 3, samples=outs[k][3])
        for x, y in zip(gb[k], gs):
            scale = float(y.abs().max()) + 1e-30
            assert float((x - y).abs().max()) <= 1e-4 * scale, (k, float((x - y).abs().max()) / scale)
        assert float(gb[k][0].abs().max()) > 0
