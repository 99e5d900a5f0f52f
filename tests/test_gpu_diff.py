"""Differentiable rendering (extension): forward estimator and path-replay
adjoint, through the C ABI.

* At the scene's own parameter values the differentiable forward traces the
  same paths as lt_render (same counts, same colours up to summation order).
* Adjoint gradients agree with central finite differences of the same
  estimator (sampling copies held at the base values, h = 1e-3, loss in
  float64): within 2% per parameter for every parameter whose gradient is
  not negligible, on 64 randomly chosen parameters including the medium's.
* The GPU adjoint of a 32x32 crop agrees with the host restatement's gradient
  in double precision (oracle/lt_diff_ref.cpp), in both of its forms: on the
  wavefront (given the forward's per-sample radiance) and one thread per
  sample replaying each path twice (without it).
Both checks run on a small scene and on the differentiable workload itself
(nine spheres of 64x32 segments plus the fog sphere, 512x512, 32 spp, depth 8).
* The two forms add the same terms (only the order of the float sums
  differs): on scenes with every material, media and two lights, with and
  without a crop, with pixels whose loss gradient is zero.
"""
import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.diff import DiffScene, finite_difference_check, render_image
from lantern_gb300.integrator import FrameBuffer, Integrator, Scene

pytestmark = pytest.mark.gpu


def _small(scene_dir, w=48, h=48, name="diff_small"):
    return S.differentiable_scene(width=w, height=h, slices=16, stacks=8, name=name).write(scene_dir)


def test_diff_forward_matches_render(scene_dir):
    path = _small(scene_dir, 40, 32, "diff_fwd")
    ds = DiffScene(path)
    a, e, sa, ss = ds.defaults()
    rgb, b, n = ds.render(a, e, sa, ss, spp=6, max_depth=8)
    sc = Scene(0)
    sc.LoadSceneFromJSON(path)
    fb = FrameBuffer(sc.width, sc.height, "cuda:0")
    Integrator(sc, fb, max_depth=8, rr_depth=3).RenderFrame(6)
    torch.cuda.synchronize()
    assert torch.equal(n, fb.ColorSampleCount)
    assert torch.equal(b, fb.Bounces)
    assert torch.allclose(rgb, fb.ColorData, rtol=1e-4, atol=1e-6)


def _fd_check(path, spp, depth, min_checked):
    """diff.finite_difference_check at the initial parameters (albedo 0.5,
    sigma_s = sigma_a = 1) against the image of the true ones (seed 3): 64
    parameters (seed 4: the six medium coefficients, the light's emission
    entries, albedo entries), h = 1e-3, every compared gradient within 2%."""
    ds = DiffScene(path)
    a0, e0, sa0, ss0 = ds.defaults()
    true, init = S.differentiable_targets(ds.num_triangles)
    dev = ds.device
    with torch.no_grad():
        target = render_image(ds, torch.from_numpy(true["albedo"]).to(dev), e0,
                              torch.from_numpy(true["sigma_a"]).to(dev), torch.from_numpy(true["sigma_s"]).to(dev),
                              spp, 0, depth, 3)
    theta = (torch.from_numpy(init["albedo"]).to(dev), e0, torch.from_numpy(init["sigma_a"]).to(dev),
             torch.from_numpy(init["sigma_s"]).to(dev))
    r = finite_difference_check(ds, theta, target, spp, max_depth=depth, count=64, seed=4, h=1e-3)
    assert r["parameters"] == 64
    assert not r["failures"], r["failures"][:10]
    assert r["checked"] >= min_checked, r["checked"]
    return r


def test_adjoint_matches_finite_differences(scene_dir):
    _fd_check(_small(scene_dir), spp=8, depth=6, min_checked=60)


def test_adjoint_matches_finite_differences_on_the_differentiable_workload(scene_dir):
    """The acceptance check at the workload's own size: 512x512, 32 spp, depth 8."""
    path = S.ensure_written(S.differentiable_scene(name="diff_c3"), scene_dir)
    _fd_check(path, spp=32, depth=8, min_checked=60)


def _crop_check(path, spp, depth, crop):
    """GPU adjoint of the samples of `crop` against the same gradient from the
    host restatement in double precision (oracle/lt_diff_ref.cpp): relative
    L2 error of each gradient array below 2e-3."""
    from oracle import oracle as O
    ds = DiffScene(path)
    orc = O.OracleScene(path)
    a0, e0, sa0, ss0 = ds.defaults()
    true, init = S.differentiable_targets(ds.num_triangles)
    e_np = e0.cpu().numpy()
    tgt, _ = orc.diff_render(true["albedo"], e_np, true["sigma_a"], true["sigma_s"], spp, max_depth=depth, crop=crop)
    cur, _ = orc.diff_render(init["albedo"], e_np, init["sigma_a"], init["sigma_s"], spp, max_depth=depth, crop=crop)
    dI = (2.0 * (cur - tgt) / spp / spp).astype(np.float32)  # d/d(film sum) of sum((img - target)^2)
    _, g64 = orc.diff_render(init["albedo"], e_np, init["sigma_a"], init["sigma_s"], spp, max_depth=depth,
                             crop=crop, dI=dI, fp64=True)
    dev = ds.device
    theta = (torch.from_numpy(init["albedo"]).to(dev), e0, torch.from_numpy(init["sigma_a"]).to(dev),
             torch.from_numpy(init["sigma_s"]).to(dev))
    samples = ds.render(*theta, spp, 0, depth, 3, keep_samples=True)[3]
    worst = 0.0
    for smp in (samples, None):  # the wavefront form, then the replay-twice kernel
        g = ds.adjoint(*theta, torch.from_numpy(dI).to(dev), spp, 0, depth, 3, crop=crop, samples=smp)
        torch.cuda.synchronize()
        for name, gg in zip(("albedo", "emission", "sigma_a", "sigma_s"), g):
            ref = g64[name].reshape(-1)
            got = gg.detach().cpu().numpy().astype(np.float64).reshape(-1)
            assert np.linalg.norm(ref) > 0, name
            rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
            assert rel < 2e-3, (name, smp is None, rel)
            worst = max(worst, rel)
    return worst


def test_adjoint_crop_matches_fp64_host_reference(scene_dir):
    _crop_check(_small(scene_dir), spp=8, depth=6, crop=(16, 8, 48, 40))


def test_adjoint_crop_matches_fp64_host_reference_on_the_differentiable_workload(scene_dir):
    """A 32x32 crop of the 512x512, 32-spp, depth-8 workload (pixels 440-471 x
    250-281): part of the fog sphere, a Lambert sphere and the ground, so every
    gradient array (albedo, emission, sigma_a, sigma_s) is nonzero."""
    path = S.ensure_written(S.differentiable_scene(name="diff_c3"), scene_dir)
    _crop_check(path, spp=32, depth=8, crop=(440, 250, 472, 282))


def _assert_grads_close(got, ref, tol=1e-4):
    for name, x, y in zip(("albedo", "emission", "sigma_a", "sigma_s"), got, ref):
        scale = float(y.abs().max()) if y.numel() else 0.0
        err = float((x - y).abs().max()) if y.numel() else 0.0
        assert err <= tol * scale + 1e-30, (name, err, scale)


@pytest.mark.parametrize("kind", ["diff", "medium", "materials", "two_lights"])
def test_wavefront_adjoint_matches_replay_kernel(scene_dir, kind):
    """The adjoint on the wavefront (with the forward's per-sample radiance)
    against the kernel that replays every path twice (without it): the same
    gradient terms, summed in another order. The loss gradient is zero on a
    band of rows (those samples add nothing), albedo is perturbed per
    triangle, first frame 3; the whole film and a crop."""
    make = {"diff": lambda: S.differentiable_scene(width=44, height=36, slices=16, stacks=8, name="wa_diff"),
            "medium": lambda: S.medium_sphere_scene(width=40, height=32, name="wa_med"),
            "materials": lambda: S.tiny_scene(width=40, height=30, name="wa_mat"),
            "two_lights": lambda: S.two_light_scene(width=36, height=28, name="wa_two")}[kind]
    ds = DiffScene(make().write(scene_dir))
    g = torch.Generator(device="cuda:0").manual_seed(11)
    a, e, sa, ss = ds.defaults()
    a = (a * (0.6 + 0.4 * torch.rand(a.shape, generator=g, device=a.device))).contiguous()
    theta = (a, e, sa * 1.2, ss * 0.8)
    spp, ff = 6, 3
    samples = ds.render(*theta, spp, ff, 8, 3, keep_samples=True)[3]
    dI = torch.rand((ds.height, ds.width, 3), generator=g, device="cuda:0") - 0.5
    dI[ds.height // 3: ds.height // 2] = 0.0
    for crop in (None, (3, 2, ds.width - 5, ds.height - 3)):
        wave = ds.adjoint(*theta, dI, spp, ff, 8, 3, crop=crop, samples=samples)
        replay = ds.adjoint(*theta, dI, spp, ff, 8, 3, crop=crop)
        torch.cuda.synchronize()
        assert float(wave[0].abs().max()) > 0 and float(wave[1].abs().max()) > 0
        _assert_grads_close(wave, replay)


def test_wavefront_adjoint_of_an_empty_crop_and_depth_zero(scene_dir):
    ds = DiffScene(_small(scene_dir, 24, 20, "wa_edge"))
    a, e, sa, ss = ds.defaults()
    samples = ds.render(a, e, sa, ss, 2, 0, 8, 3, keep_samples=True)[3]
    dI = torch.ones((ds.height, ds.width, 3), device="cuda:0")
    for crop, depth in (((5, 5, 5, 9), 8), (None, 0)):
        gr = ds.adjoint(a, e, sa, ss, dI, 2, 0, depth, 3, crop=crop, samples=samples)
        torch.cuda.synchronize()
        assert all(float(x.abs().max()) == 0.0 for x in gr if x.numel())
