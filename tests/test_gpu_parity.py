"""GPU path against the oracle, through the C ABI (liblantern_gpu.so).

* Intersection (lt_intersect) against the oracle's Embree-semantics closest
  hit: primitive bit-exact except exact ties, t within 1e-5 relative.
* Rendering (lt_render) against the oracle with the same per-(pixel, frame)
  sampler keying: the same paths are traced, so sample counts are exact and
  colours agree pixel by pixel except where a transcendental function's last
  bit (CUDA vs glibc sinf/cosf/logf/expf) sends a path elsewhere.
"""
import os

import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.integrator import FrameBuffer, Integrator, Scene, intersect, render_host
from lantern_gb300.native import MISS, Context, LanternError
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = Context(0)
    yield c
    c.close()


def _positions(path, p):
    """World-space vertices of one scene-JSON primitive (as the oracle builds them)."""
    if p["type"] == "lmf":
        pos = O.read_lmf(os.path.join(os.path.dirname(path), p["file_path"]))["positions"]
    elif p["type"] == "grid":
        pos = O.grid_mesh(p["width"], p["depth"], int(p["m"]), int(p["n"]))[0]
    else:
        pos = O.geosphere_mesh(p["radius"], int(p["n"]))[0]
    return O.apply_transform(pos, p["transform"]) if "transform" in p else pos


def _scene_rays(path, n, seed):
    orc = O.OracleScene(path)
    allp = np.concatenate([_positions(path, p) for p in orc.json["primitives"]])
    lo, hi = allp.min(0), allp.max(0)
    c, e = (lo + hi) / 2, (hi - lo) / 2
    rays = S.random_rays(n, c - 0.6 * e, c + 0.6 * e, seed=seed)
    return orc, rays


def _compare_hits(gh, oh):
    gprim = gh[:, 3].view(np.uint32)
    oprim = oh[:, 3]
    ot = oh[:, 0].view(np.float32)
    gt = gh[:, 0]
    hit = oprim != MISS
    assert np.array_equal(gprim == MISS, oprim == MISS), "hit/miss differs"
    diff = hit & (gprim != oprim)
    # exact ties only: the oracle's t for the GPU's primitive equals the oracle's best t
    assert np.all(gt[diff] == ot[diff]), f"{diff.sum()} primitive mismatches that are not ties"
    rel = np.abs(gt[hit] - ot[hit]) / np.maximum(np.abs(ot[hit]), 1e-30)
    assert rel.max(initial=0) <= 1e-5
    return int(hit.sum()), int(diff.sum())


@pytest.fixture(params=[2, 4, 8], ids=["bvh2", "bvh4", "bvh8"])
def width(request, ctx):
    """BVH width of the traversal (lt_tuning.bvh_width); the shared context is
    set back to 2 afterwards."""
    ctx.set_tuning(bvh_width=request.param)
    yield request.param
    ctx.set_tuning(bvh_width=2)


@pytest.mark.parametrize("make", [
    lambda: S.nine_spheres(width=64, height=64, name="isect_nine"),
    lambda: S.displaced_icosphere_scene(width=64, height=64, levels=5, name="isect_ico5"),
    lambda: S.tiny_scene(name="isect_tiny"),
    lambda: S.procedural_scene(name="isect_procedural"),
])
def test_intersect_matches_oracle(ctx, width, scene_dir, make):
    path = make().write(scene_dir)
    ctx.load_scene_json(path)
    orc, rays = _scene_rays(path, 1 << 16, seed=7)
    oh = orc.intersect(rays)
    gh = intersect(ctx, torch.from_numpy(rays).cuda()).cpu().numpy()
    nhit, nties = _compare_hits(gh, oh)
    assert nhit > 1000
    # host-memory path gives the same answer
    gh2 = intersect(ctx, rays)
    assert np.array_equal(gh.view(np.uint32), gh2.view(np.uint32))


@pytest.fixture(scope="module")
def icosphere_workload(scene_dir):
    """The 1.3M-triangle workload's scene (8-level displaced icosphere on the
    ground, under the light), its oracle and 1,048,576 rays of the intersection
    micro-bench's distribution: origins uniform in the icosphere's bounding box,
    directions uniform on the sphere, seed 2, tnear 0, tfar inf."""
    import json
    path = S.ensure_written(S.displaced_icosphere_scene(name="icosphere"), scene_dir)
    with open(path) as fh:
        prims = json.load(fh)["primitives"]
    pos = np.concatenate([_positions(path, p) for p in prims if p["name"].startswith("ico_")])
    rays = S.random_rays(1 << 20, pos.min(0), pos.max(0), seed=2)
    orc = O.OracleScene(path)
    return path, orc, rays, orc.intersect(rays)


def test_intersect_matches_oracle_on_the_icosphere_workload(ctx, width, icosphere_workload):
    """lt_intersect on the 1,310,720-triangle mesh the micro-bench times, all
    three BVH widths, against the oracle's BVH2: primitive bit-exact except
    exact ties, t within 1e-5 relative."""
    path, orc, rays, oh = icosphere_workload
    ctx.load_scene_json(path)
    assert ctx.scene_info().num_triangles == 1310724
    gh = intersect(ctx, torch.from_numpy(rays).cuda()).cpu().numpy()
    nhit, nties = _compare_hits(gh, oh)
    assert nhit > (1 << 19)


def test_intersect_tnear_tfar_rule(ctx, width, scene_dir):
    """Rays clipped exactly at, and one float short of, each hit distance (and
    starting there) are accepted or rejected as the oracle's Embree rule says:
    |den|*tnear < T <= |den|*tfar, evaluated in float."""
    path = S.tiny_scene(name="isect_rule").write(scene_dir)
    ctx.load_scene_json(path)
    orc, rays = _scene_rays(path, 4096, seed=3)
    oh = orc.intersect(rays)
    hit = oh[:, 3] != MISS
    t = oh[hit, 0].view(np.float32)
    cases = []
    for tfar in (t, np.nextafter(t, np.float32(0)), np.nextafter(t, np.float32(np.inf))):
        r = rays[hit].copy()
        r[:, 7] = tfar
        cases.append(r)
    r = rays[hit].copy()
    r[:, 3] = t                      # tnear = hit distance: that hit is excluded
    cases.append(r)
    for r in cases:
        _compare_hits(intersect(ctx, r), orc.intersect(r))
    assert (intersect(ctx, cases[0])[:, 3].view(np.uint32) != MISS).mean() > 0.5


@pytest.mark.parametrize("make,spp,depth", [
    (lambda: S.tiny_scene(width=48, height=40, name="paths_tiny"), 6, 12),
    (lambda: S.nine_spheres(width=64, height=64, name="paths_nine"), 4, 8),
    (lambda: S.medium_sphere_scene(width=40, height=40, reference_expressible=True, name="paths_med_ref"), 4, 32),
    (lambda: S.medium_sphere_scene(width=40, height=40, name="paths_med_hg"), 4, 32),
    (lambda: S.medium_sphere_scene(width=40, height=40, non_scattering=True, name="paths_med_absorb"), 4, 32),
    (lambda: S.procedural_scene(width=48, height=40, name="paths_procedural"), 4, 8),
])
@pytest.mark.parametrize("bvh_width", [2, 4, 8])
def test_render_matches_oracle_path_by_path(scene_dir, make, spp, depth, bvh_width):
    path = make().write(scene_dir)
    sc = Scene(0)
    sc.LoadSceneFromJSON(path)
    sc.ctx.set_tuning(bvh_width=bvh_width)
    fb = FrameBuffer(sc.width, sc.height, "cuda:0")
    Integrator(sc, fb, max_depth=depth, rr_depth=3).RenderFrame(spp)
    torch.cuda.synchronize()
    rgb = fb.ColorData.cpu().numpy()
    ref = O.OracleScene(path).render(spp, max_depth=depth, rr_depth=3, keying=O.KEY_PIXEL)
    assert np.array_equal(fb.ColorSampleCount.cpu().numpy(), ref["counts"].astype(np.int32))
    close = np.isclose(rgb, ref["rgb"], rtol=2e-4, atol=1e-5).all(-1)
    assert close.mean() > 0.97, close.mean()
    same_b = fb.Bounces.cpu().numpy() == ref["bounces"].astype(np.int32)
    assert same_b.mean() > 0.97
    m_g, m_o = rgb.astype(np.float64).mean(), ref["rgb"].astype(np.float64).mean()
    assert abs(m_g - m_o) <= 0.01 * abs(m_o) + 1e-6


def test_render_is_additive_and_host_path_agrees(scene_dir):
    path = S.tiny_scene(width=32, height=24, name="additive").write(scene_dir)
    sc = Scene(0)
    sc.LoadSceneFromJSON(path)
    fb = FrameBuffer(sc.width, sc.height, "cuda:0")
    it = Integrator(sc, fb, max_depth=10)
    it.RenderFrame(2)
    it.RenderFrame(3)
    torch.cuda.synchronize()
    one = FrameBuffer(sc.width, sc.height, "cuda:0")
    Integrator(sc, one, max_depth=10).RenderFrame(5)
    torch.cuda.synchronize()
    assert torch.equal(fb.ColorSampleCount, one.ColorSampleCount)
    assert torch.equal(fb.Bounces, one.Bounces)
    assert torch.allclose(fb.ColorData, one.ColorData, rtol=1e-5, atol=1e-6)
    host = render_host(sc.ctx, sc.width, sc.height, 5, max_depth=10)
    assert np.array_equal(host["counts"].astype(np.int32), one.ColorSampleCount.cpu().numpy())
    assert np.allclose(host["rgb"], one.ColorData.cpu().numpy(), rtol=1e-5, atol=1e-6)


def test_max_depth_zero_counts_only(ctx, scene_dir):
    path = S.tiny_scene(width=8, height=8, name="depth0").write(scene_dir)
    ctx.load_scene_json(path)
    film = render_host(ctx, 8, 8, 3, max_depth=0)
    assert np.all(film["counts"] == 3) and np.all(film["rgb"] == 0) and np.all(film["bounces"] == 0)


def test_errors_are_reported(ctx, scene_dir, tmp_path):
    c = Context(0)
    with pytest.raises(LanternError) as e:
        render_host(c, 4, 4, 1)
    assert e.value.status == 8  # LT_ERR_STATE: no scene yet
    with pytest.raises(LanternError) as e:
        c.load_scene_json(str(tmp_path / "missing.json"))
    assert e.value.status == 5  # LT_ERR_IO
    bad = tmp_path / "bad.json"
    bad.write_text('{"camera": {"client_width": 4, ')
    with pytest.raises(LanternError) as e:
        c.load_scene_json(str(bad))
    assert e.value.status == 6  # LT_ERR_PARSE
    path = S.tiny_scene(width=8, height=8, name="err_size").write(scene_dir)
    c.load_scene_json(path)
    with pytest.raises(LanternError) as e:
        render_host(c, 9, 8, 1)
    assert e.value.status == 1  # LT_ERR_INVALID: film size
    c.close()


@pytest.mark.parametrize("make", [
    lambda: S.nine_spheres(width=64, height=64, name="isect_nine"),
    lambda: S.displaced_icosphere_scene(width=64, height=64, levels=6, name="isect_ico6"),
    lambda: S.procedural_scene(name="isect_procedural_build"),
])
def test_gpu_bvh_build_matches_host_build(scene_dir, make):
    """The device path (triangle setup and mesh transforms in lt_setup.cu, then
    the device builder) makes the host path's splits: same node count and
    depth, and closest hits identical to the oracle's."""
    from lantern_gb300.native import BVH_GPU, BVH_HOST
    path = make().write(scene_dir)
    orc, rays = _scene_rays(path, 1 << 15, seed=11)
    oh = orc.intersect(rays)
    infos = {}
    for builder in (BVH_HOST, BVH_GPU):
        c = Context(0)
        c.set_bvh_builder(builder)
        c.load_scene_json(path)
        infos[builder] = c.scene_info()
        _compare_hits(intersect(c, rays), oh)
        c.close()
    assert infos[BVH_GPU].num_bvh_nodes == infos[BVH_HOST].num_bvh_nodes
    assert infos[BVH_GPU].num_triangles == infos[BVH_HOST].num_triangles


def test_scene_destroy_keeps_the_context(scene_dir):
    """lt_scene_destroy frees the scene; rendering then reports LT_ERR_STATE,
    and the same context loads and renders a scene again."""
    path = S.tiny_scene(width=8, height=8, name="scene_destroy").write(scene_dir)
    c = Context(0)
    c.load_scene_json(path)
    first = render_host(c, 8, 8, 2)
    c.destroy_scene()
    with pytest.raises(LanternError) as e:
        render_host(c, 8, 8, 1)
    assert e.value.status == 8  # LT_ERR_STATE
    c.load_scene_json(path)
    again = render_host(c, 8, 8, 2)
    assert np.array_equal(first["counts"], again["counts"]) and np.array_equal(first["bounces"], again["bounces"])
    assert np.allclose(first["rgb"], again["rgb"], rtol=1e-5, atol=1e-6)
    c.close()
