"""Differentiable rendering (extension): forward estimator and path-replay
adjoint, through the C ABI.

* At the scene's own parameter values the differentiable forward traces the
  same paths as lt_render (same counts, same colours up to summation order).
* Adjoint gradients agree with central finite differences of the same
  estimator (sampling copies held at the base values, h = 1e-3, loss in
  float64): within 2% per parameter for every parameter whose gradient is
  not negligible, on 64 randomly chosen parameters including the medium's.
"""
import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.diff import DiffScene, render_image
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


def test_adjoint_matches_finite_differences(scene_dir):
    path = _small(scene_dir)
    ds = DiffScene(path)
    a0, e0, sa0, ss0 = ds.defaults()
    true, init = S.differentiable_targets(ds.num_triangles)
    dev = ds.device
    spp, depth = 8, 6
    # target image with the true parameters
    with torch.no_grad():
        target = render_image(ds, torch.from_numpy(true["albedo"]).to(dev), e0,
                              torch.from_numpy(true["sigma_a"]).to(dev), torch.from_numpy(true["sigma_s"]).to(dev),
                              spp, 0, depth, 3).double()
    theta = [torch.from_numpy(init["albedo"]).to(dev).requires_grad_(), e0.clone().requires_grad_(),
             torch.from_numpy(init["sigma_a"]).to(dev).requires_grad_(),
             torch.from_numpy(init["sigma_s"]).to(dev).requires_grad_()]
    img = render_image(ds, *theta, spp, 0, depth, 3)
    loss = ((img.double() - target) ** 2).sum()
    loss.backward()
    grads = [t.grad.detach().cpu().numpy() for t in theta]
    base = [t.detach().clone() for t in theta]
    detached = (base[0], base[2], base[3])

    def loss_at(k, idx, delta):
        p = [t.clone() for t in base]
        p[k].view(-1)[idx] += delta
        rgb, _, _ = ds.render(*p, spp=spp, max_depth=depth, detached=detached)
        return float((((rgb / spp).double() - target) ** 2).sum())

    rng = np.random.default_rng(4)
    cands = [(2, i) for i in range(3)] + [(3, i) for i in range(3)]
    nz = np.flatnonzero(np.abs(grads[0]).reshape(-1) > 0)
    cands += [(0, int(i)) for i in rng.choice(nz, size=min(48, nz.size), replace=False)]
    nze = np.flatnonzero(np.abs(grads[1]).reshape(-1) > 0)
    cands += [(1, int(i)) for i in rng.choice(nze, size=min(10, nze.size), replace=False)]
    cands = cands[:64]
    h = 1e-3
    gmax = max(np.abs(g).max() for g in grads)
    bad = []
    for k, i in cands:
        fd = (loss_at(k, i, h) - loss_at(k, i, -h)) / (2 * h)
        ad = float(grads[k].reshape(-1)[i])
        if max(abs(fd), abs(ad)) < 1e-4 * gmax:
            continue
        if abs(ad - fd) > 0.02 * max(abs(fd), abs(ad)):
            bad.append((k, i, ad, fd))
    assert not bad, bad[:10]


def test_adjoint_crop_matches_fp64_host_reference(scene_dir):
    """GPU adjoint of the samples of a 32x32 crop against the same gradient from
    the host restatement in double precision (oracle/lt_diff_ref.cpp)."""
    from oracle import oracle as O
    path = _small(scene_dir)
    ds = DiffScene(path)
    orc = O.OracleScene(path)
    a0, e0, sa0, ss0 = ds.defaults()
    true, init = S.differentiable_targets(ds.num_triangles)
    spp, depth, crop = 8, 6, (16, 8, 48, 40)
    e_np = e0.cpu().numpy()
    tgt, _ = orc.diff_render(true["albedo"], e_np, true["sigma_a"], true["sigma_s"], spp, max_depth=depth)
    cur, _ = orc.diff_render(init["albedo"], e_np, init["sigma_a"], init["sigma_s"], spp, max_depth=depth)
    dI = (2.0 * (cur - tgt) / spp / spp).astype(np.float32)  # d/d(film sum) of sum((img - target)^2)
    _, g64 = orc.diff_render(init["albedo"], e_np, init["sigma_a"], init["sigma_s"], spp, max_depth=depth,
                             crop=crop, dI=dI, fp64=True)
    dev = ds.device
    g = ds.adjoint(torch.from_numpy(init["albedo"]).to(dev), e0, torch.from_numpy(init["sigma_a"]).to(dev),
                   torch.from_numpy(init["sigma_s"]).to(dev), torch.from_numpy(dI).to(dev), spp, 0, depth, 3,
                   crop=crop)
    torch.cuda.synchronize()
    for name, gg in zip(("albedo", "emission", "sigma_a", "sigma_s"), g):
        ref = g64[name].reshape(-1)
        got = gg.detach().cpu().numpy().astype(np.float64).reshape(-1)
        assert np.linalg.norm(ref) > 0, name
        rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert rel < 2e-3, (name, rel)
