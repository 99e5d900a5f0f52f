"""Final resolve (lt_resolve): film sums -> tone-mapped image, as the
reference's visualizer computes it (visualizer.cpp:352-364,1308;
final_resolve_ps.glsl:24-43), checked against the oracle's restatement
(orc_resolve) bit for bit; and the PNG / EXR writers."""
import numpy as np
import pytest

from oracle import oracle as O


def _film(h=37, w=53, seed=0):
    rng = np.random.default_rng(seed)
    rgb = (rng.uniform(0, 1, (h, w, 3)) ** 4 * 60).astype(np.float32)
    counts = rng.integers(0, 9, (h, w)).astype(np.uint32)
    counts[0, :5] = 0
    rgb[0, :3] = 0.0  # 0 / 0: NaN, as the reference's division gives
    return rgb, counts


def _numpy_resolve(rgb, counts, tonemap, stops):
    e = np.float32(2.0) ** np.float32(stops)
    n = counts.astype(np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        c = np.concatenate([e * (rgb / n[..., None]), np.full(n.shape + (1,), e * np.float32(1), np.float32)], -1)
        if tonemap == 1:
            x = np.maximum(np.float32(0), c - np.float32(0.004))
            c = (x * (np.float32(6.2) * x + np.float32(0.5))) / (x * (np.float32(6.2) * x + np.float32(1.7))
                                                                + np.float32(0.06))
            c[..., 3] = 1.0
    c = np.fmin(np.fmax(c, np.float32(0)), np.float32(1)).astype(np.float32)
    return c, np.rint(c * np.float32(255)).astype(np.uint8)


@pytest.mark.parametrize("tonemap,stops", [(0, 0.0), (0, -1.5), (1, 0.0), (1, 2.0)])
def test_oracle_resolve_matches_shader_formula(tonemap, stops):
    rgb, counts = _film()
    a, a8, spp = O.resolve(rgb, counts, tonemap, stops)
    b, b8 = _numpy_resolve(rgb, counts, tonemap, stops)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(a8, b8)
    assert spp == (int(counts.min()), int(counts.max()), int(counts.sum()))


def test_png_and_exr_round_trip(tmp_path):
    from lantern_gb300 import image as I
    rgb, counts = _film()
    a, a8, _ = O.resolve(rgb, counts, 1, 0.0)
    I.write_png(str(tmp_path / "x.png"), a8)
    assert np.array_equal(I.read_png(str(tmp_path / "x.png")), a8)
    I.write_exr(str(tmp_path / "x.exr"), a)
    assert np.array_equal(I.read_exr(str(tmp_path / "x.exr")), a)
    I.write_exr(str(tmp_path / "y.exr"), a[..., :3])
    assert np.array_equal(I.read_exr(str(tmp_path / "y.exr")), a[..., :3])


@pytest.mark.gpu
@pytest.mark.parametrize("tonemap,stops", [(0, 0.0), (1, 0.0), (1, -2.0)])
def test_gpu_resolve_bit_exact(scene_dir, tonemap, stops):
    import torch
    import lantern_gb300.scenes as S
    from lantern_gb300 import image as I
    from lantern_gb300.integrator import FrameBuffer, Integrator, Scene
    sc = Scene(0)
    sc.LoadSceneFromJSON(S.tiny_scene(width=61, height=43, name="resolve_tiny").write(scene_dir))
    fb = FrameBuffer(sc.width, sc.height, "cuda:0")
    Integrator(sc, fb, max_depth=8).RenderFrame(3)
    fb.ColorSampleCount[0, :4] = 0  # pixels without samples
    fb.ColorData[0, :2] = 0.0
    rgba, rgba8, spp = I.resolve(sc.ctx, fb, tonemap, stops)
    torch.cuda.synchronize()
    rgb, counts = fb.ColorData.cpu().numpy(), fb.ColorSampleCount.cpu().numpy().astype(np.uint32)
    a, a8, ospp = O.resolve(rgb, counts, tonemap, stops)
    assert np.array_equal(rgba.cpu().numpy().view(np.uint32), a.view(np.uint32))
    assert np.array_equal(rgba8.cpu().numpy(), a8)
    assert (spp[0], spp[1]) == ospp[:2] and spp[2] == pytest.approx(ospp[2] / counts.size)
    # host film through the same entry point
    from lantern_gb300.native import Film
    host_rgb, host_n = np.ascontiguousarray(rgb), np.ascontiguousarray(counts)
    hb = np.zeros_like(host_n)
    f = Film(host_rgb.ctypes.data, hb.ctypes.data, host_n.ctypes.data, sc.width, sc.height, 0)
    out = np.empty((sc.height, sc.width, 4), np.float32)
    out8 = np.empty((sc.height, sc.width, 4), np.uint8)
    r = sc.ctx.resolve(f, tonemap, stops, out.ctypes.data, out8.ctypes.data)
    assert np.array_equal(out.view(np.uint32), a.view(np.uint32)) and np.array_equal(out8, a8)
    assert (r.min_spp, r.max_spp, r.sum_spp) == ospp
