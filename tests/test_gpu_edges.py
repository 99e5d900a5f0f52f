"""Edge cases of the render and intersection paths against the oracle, through
the C ABI (liblantern_gpu.so), with both BVH widths.

* A scene without geometry: every camera ray misses, the film holds
  spp x background (integrator.cpp:118-121), no bounces.
* A scene without lights: SampleOneLight returns black (integrator.cpp:255-261),
  only emission seen by the path and the background contribute.
* Two lights: the light choice's rejection loop and its x numLights weight
  (integrator.cpp:263-270) on paths that hit either light.
* Ragged film sizes (neither a multiple of the 8x8 tile nor of a warp) and a
  single pixel.
* Rays with zero direction components, empty extents (tfar < tnear), a zero
  direction, and an empty ray batch.
"""
import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.integrator import FrameBuffer, Integrator, Scene, intersect
from lantern_gb300.native import MISS
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CAMERA = {"phi": 1.1, "theta": 0.0, "radius": 6.0, "fov": 0.785398, "target": [0.0, 0.5, 0.0]}


def _empty(width=5, height=3, name="edge_empty"):
    return S.Scene(width, height, camera=dict(CAMERA), background=(0.2, 0.3, 0.4),
                   render={"spp": 2, "max_depth": 8, "rr_depth": 3}, name=name)


def _no_lights(name="edge_nolight"):
    return S.unlit_scene(name=name)


def _two_lights(name="edge_twolights"):
    return S.two_light_scene(name=name)


def _render_both(path, spp, depth, bvh_width):
    sc = Scene(0)
    sc.LoadSceneFromJSON(path)
    sc.ctx.set_tuning(bvh_width=bvh_width)
    fb = FrameBuffer(sc.width, sc.height, "cuda:0")
    Integrator(sc, fb, max_depth=depth, rr_depth=3).RenderFrame(spp)
    torch.cuda.synchronize()
    ref = O.OracleScene(path).render(spp, max_depth=depth, rr_depth=3, keying=O.KEY_PIXEL)
    got = {"rgb": fb.ColorData.cpu().numpy(), "counts": fb.ColorSampleCount.cpu().numpy(),
           "bounces": fb.Bounces.cpu().numpy()}
    sc.ctx.close()
    return got, ref


@pytest.mark.parametrize("bvh_width", [2, 4, 8])
def test_empty_scene_renders_the_background(scene_dir, bvh_width):
    path = _empty().write(scene_dir)
    got, ref = _render_both(path, 3, 8, bvh_width)
    assert np.array_equal(got["counts"], ref["counts"].astype(np.int32))
    assert np.all(got["counts"] == 3) and np.all(got["bounces"] == 0)
    assert np.array_equal(got["rgb"], ref["rgb"])
    assert np.allclose(got["rgb"], 3 * np.array([0.2, 0.3, 0.4], np.float32), rtol=1e-6)


@pytest.mark.parametrize("make,spp,depth", [
    (_no_lights, 4, 8),
    (_two_lights, 4, 8),
    (lambda: S.tiny_scene(width=37, height=23, name="edge_ragged"), 3, 10),
], ids=["no_lights", "two_lights", "ragged_37x23"])
@pytest.mark.parametrize("bvh_width", [2, 4, 8])
def test_edge_scene_matches_oracle_path_by_path(scene_dir, make, spp, depth, bvh_width):
    path = make().write(scene_dir)
    got, ref = _render_both(path, spp, depth, bvh_width)
    assert np.array_equal(got["counts"], ref["counts"].astype(np.int32))
    close = np.isclose(got["rgb"], ref["rgb"], rtol=2e-4, atol=1e-5).all(-1)
    assert close.mean() > 0.97, close.mean()
    assert (got["bounces"] == ref["bounces"].astype(np.int32)).mean() > 0.97
    m_g, m_o = got["rgb"].astype(np.float64).mean(), ref["rgb"].astype(np.float64).mean()
    assert abs(m_g - m_o) <= 0.01 * abs(m_o) + 1e-6


@pytest.mark.parametrize("bvh_width", [2, 4, 8])
def test_single_pixel_film(scene_dir, bvh_width):
    """One pixel, direct light only (depth 1: no roulette, no bounce sampled
    from a transcendental), so every path takes the oracle's decisions."""
    path = S.tiny_scene(width=1, height=1, name="edge_1x1").write(scene_dir)
    got, ref = _render_both(path, 16, 1, bvh_width)
    assert np.array_equal(got["counts"], ref["counts"].astype(np.int32))
    assert np.array_equal(got["bounces"], ref["bounces"].astype(np.int32))
    assert np.allclose(got["rgb"], ref["rgb"], rtol=2e-4, atol=1e-5)


@pytest.mark.parametrize("bvh_width", [2, 4, 8])
def test_intersect_degenerate_rays(scene_dir, bvh_width):
    path = S.nine_spheres(width=16, height=16, slices=16, stacks=8, name="edge_isect").write(scene_dir)
    sc = Scene(0)
    sc.LoadSceneFromJSON(path)
    ctx = sc.ctx
    ctx.set_tuning(bvh_width=bvh_width)
    orc = O.OracleScene(path)
    rng = np.random.default_rng(17)
    n = 3000
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform([-2.0, 0.05, -2.0], [2.0, 1.5, 2.0], size=(n, 3))
    axis = rng.integers(0, 3, n)
    sign = rng.choice([-1.0, 1.0], n)
    rays[np.arange(n), 4 + axis] = sign               # axis-aligned: two zero components
    two = rng.random(n) < 0.3                          # some in a coordinate plane: one zero component
    rays[two, 4 + (axis[two] + 1) % 3] = 0.5
    rays[:, 7] = np.inf
    rays[: n // 10, 3] = 5.0                           # tnear > tfar: empty extent
    rays[: n // 10, 7] = 1.0
    rays[n // 10: n // 5, 4:7] = 0.0                   # zero direction
    gh, oh = intersect(ctx, rays), orc.intersect(rays)
    gprim, oprim = gh[:, 3].view(np.uint32), oh[:, 3]
    assert np.all(gprim[: n // 5] == MISS) and np.all(oprim[: n // 5] == MISS)
    assert np.array_equal(gprim == MISS, oprim == MISS)
    hit = oprim != MISS
    assert hit.sum() > n // 4
    diff = hit & (gprim != oprim)
    ot = oh[:, 0].view(np.float32)
    assert np.all(gh[diff, 0] == ot[diff])  # exact ties only
    rel = np.abs(gh[hit, 0] - ot[hit]) / np.abs(ot[hit])
    assert rel.max() <= 1e-5
    assert intersect(ctx, np.zeros((0, 8), np.float32)).shape == (0, 4)
    sc.ctx.close()
