"""Differentiable rendering: a torch.autograd.Function over lt_render_diff /
lt_render_adjoint (path-replay backpropagation in liblantern_gpu.so).

Parameters are CUDA tensors: per-triangle RGB albedo (T, 3), per-triangle RGB
emission (T, 3; only emissive meshes' triangles emit), per-medium RGB sigma_a
and sigma_s (M, 3). The forward pass renders the image (colour sum / spp); the
backward pass replays every sample from its (pixel, frame) seed and returns the
gradients of the loss with respect to all four tensors. Nothing per path is
stored between the two passes.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np
import torch

from . import native
from .native import Context, Film, RenderParams


class DiffParams(C.Structure):
    _fields_ = [("albedo", C.c_void_p), ("emission", C.c_void_p), ("sigma_a", C.c_void_p),
                ("sigma_s", C.c_void_p), ("albedo_detached", C.c_void_p), ("sigma_a_detached", C.c_void_p),
                ("sigma_s_detached", C.c_void_p)]


class DiffJob(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("params", RenderParams), ("dp", DiffParams), ("film", Film),
                ("sample_radiance", C.c_void_p), ("d_loss_d_film", C.c_void_p), ("grad_albedo", C.c_void_p),
                ("grad_emission", C.c_void_p), ("grad_sigma_a", C.c_void_p), ("grad_sigma_s", C.c_void_p)]


def _bind(L):
    if getattr(L, "_diff_bound", False):
        return
    p = C.c_void_p
    L.lt_render_diff_batch.argtypes = [p, C.POINTER(DiffJob), C.c_uint32]
    L.lt_render_adjoint_batch.argtypes = [p, C.POINTER(DiffJob), C.c_uint32]
    L.lt_diff_defaults.argtypes = [p, p, p, p, p]
    L.lt_render_diff.argtypes = [p, C.POINTER(RenderParams), C.POINTER(DiffParams), C.POINTER(Film), p]
    L.lt_render_adjoint.argtypes = [p, C.POINTER(RenderParams), C.POINTER(DiffParams), p, p, p, p, p,
                                    C.POINTER(C.c_uint32), p]
    L._diff_bound = True


def _ptr(t: Optional[torch.Tensor]):
    return None if t is None else t.data_ptr()


def _dev(t: torch.Tensor, device) -> torch.Tensor:
    return t.detach().to(device=device, dtype=torch.float32).contiguous()


class DiffScene:
    """A loaded scene plus the sizes of its differentiable parameters."""

    def __init__(self, path: Optional[str] = None, device: int = 0, ctx: Optional[Context] = None):
        """Loads the scene JSON at `path` into a new context, or uses `ctx`, a
        context that already holds the scene."""
        self.ctx = ctx or Context(device)
        device = self.ctx.device
        _bind(self.ctx.L)
        if ctx is None:
            self.ctx.load_scene_json(path)
        info = self.ctx.scene_info()
        self.width, self.height = info.width, info.height
        self.num_triangles, self.num_media = info.num_triangles, info.num_media
        self.device = torch.device(f"cuda:{device}")

    def defaults(self):
        """The scene's own values: (albedo, emission, sigma_a, sigma_s) CUDA tensors."""
        T, M = self.num_triangles, max(self.num_media, 1)
        a, e = np.zeros((T, 3), np.float32), np.zeros((T, 3), np.float32)
        sa, ss = np.zeros((M, 3), np.float32), np.zeros((M, 3), np.float32)
        native.check(self.ctx.L, self.ctx.h, self.ctx.L.lt_diff_defaults(
            self.ctx.h, a.ctypes.data, e.ctypes.data, sa.ctypes.data, ss.ctypes.data))
        return tuple(torch.from_numpy(x).to(self.device) for x in (a, e, sa, ss))

    def _params(self, albedo, emission, sigma_a, sigma_s, detached=None):
        keep = [_dev(albedo, self.device), _dev(emission, self.device), _dev(sigma_a, self.device),
                _dev(sigma_s, self.device)]
        det = [None, None, None]
        if detached is not None:
            det = [None if d is None else _dev(d, self.device) for d in detached]
        keep += det
        return keep, DiffParams(*[_ptr(k) for k in keep])

    def render(self, albedo, emission, sigma_a, sigma_s, spp: int, first_frame: int = 0, max_depth: int = 8,
               rr_depth: int = 3, detached=None, keep_samples: bool = False):
        """Film (rgb sum, bounces, counts) of the differentiable estimator, and
        with keep_samples every sample's radiance (for the adjoint).
        `detached` = (albedo, sigma_a, sigma_s) sampling copies, or None."""
        keep, dp = self._params(albedo, emission, sigma_a, sigma_s, detached)
        rgb = torch.zeros((self.height, self.width, 3), dtype=torch.float32, device=self.device)
        b = torch.zeros((self.height, self.width), dtype=torch.int32, device=self.device)
        n = torch.zeros_like(b)
        samples = (torch.empty((spp, self.height, self.width, 3), dtype=torch.float32, device=self.device)
                   if keep_samples else None)
        film = Film(rgb.data_ptr(), b.data_ptr(), n.data_ptr(), self.width, self.height, 1)
        self.ctx.set_stream(torch.cuda.current_stream(self.device).cuda_stream)
        prm = RenderParams(spp, first_frame, max_depth, rr_depth)
        native.check(self.ctx.L, self.ctx.h, self.ctx.L.lt_render_diff(self.ctx.h, C.byref(prm), C.byref(dp),
                                                                         C.byref(film), _ptr(samples)))
        del keep
        if keep_samples:
            return rgb, b, n, samples
        return rgb, b, n

    def adjoint(self, albedo, emission, sigma_a, sigma_s, d_loss_d_sum: torch.Tensor, spp: int,
                first_frame: int = 0, max_depth: int = 8, rr_depth: int = 3, detached=None, crop=None,
                samples: Optional[torch.Tensor] = None):
        keep, dp = self._params(albedo, emission, sigma_a, sigma_s, detached)
        grads = [torch.zeros_like(k) for k in keep[:4]]
        dI = _dev(d_loss_d_sum, self.device)
        crop_arr = None if crop is None else (C.c_uint32 * 4)(*crop)
        self.ctx.set_stream(torch.cuda.current_stream(self.device).cuda_stream)
        prm = RenderParams(spp, first_frame, max_depth, rr_depth)
        native.check(self.ctx.L, self.ctx.h, self.ctx.L.lt_render_adjoint(
            self.ctx.h, C.byref(prm), C.byref(dp), dI.data_ptr(), *[g.data_ptr() for g in grads], crop_arr,
            _ptr(samples)))
        del keep
        return grads


class RenderImage(torch.autograd.Function):
    """image = render(albedo, emission, sigma_a, sigma_s); backward by path replay."""

    @staticmethod
    def forward(ctx, albedo, emission, sigma_a, sigma_s, scene: DiffScene, spp: int, first_frame: int,
                max_depth: int, rr_depth: int):
        rgb, _, _, samples = scene.render(albedo, emission, sigma_a, sigma_s, spp, first_frame, max_depth, rr_depth,
                                          keep_samples=True)
        ctx.scene = scene
        ctx.cfg = (spp, first_frame, max_depth, rr_depth)
        ctx.save_for_backward(albedo, emission, sigma_a, sigma_s, samples)
        return rgb / spp

    @staticmethod
    def backward(ctx, grad_image):
        albedo, emission, sigma_a, sigma_s, samples = ctx.saved_tensors
        spp, first_frame, max_depth, rr_depth = ctx.cfg
        g = ctx.scene.adjoint(albedo, emission, sigma_a, sigma_s, grad_image.contiguous() / spp, spp,
                              first_frame, max_depth, rr_depth, samples=samples)
        return g[0], g[1], g[2], g[3], None, None, None, None, None


def render_image(scene: DiffScene, albedo, emission, sigma_a, sigma_s, spp: int, first_frame: int = 0,
                 max_depth: int = 8, rr_depth: int = 3) -> torch.Tensor:
    return RenderImage.apply(albedo, emission, sigma_a, sigma_s, scene, spp, first_frame, max_depth, rr_depth)


def _batch_call(fn, owner: DiffScene, jobs):
    arr = (DiffJob * len(jobs))(*jobs)
    owner.ctx.set_stream(torch.cuda.current_stream(owner.device).cuda_stream)
    native.check(owner.ctx.L, owner.ctx.h, fn(owner.ctx.h, arr, len(jobs)))


def render_batch(scenes, params, spp, first_frame=0, max_depth: int = 8, rr_depth: int = 3,
                 keep_samples: bool = False):
    """lt_render_diff_batch: the differentiable forward render of several
    scenes in one launch. scenes: DiffScenes (the first one's context runs the
    launch); params: per scene (albedo, emission, sigma_a, sigma_s); spp,
    first_frame, max_depth, rr_depth: one value or one per scene. Returns per
    scene (rgb, bounces, counts[, samples]) as DiffScene.render does."""
    n = len(scenes)
    per = lambda v: list(v) if isinstance(v, (list, tuple)) else [v] * n
    spp, first_frame, max_depth, rr_depth = per(spp), per(first_frame), per(max_depth), per(rr_depth)
    jobs, keep, out = [], [], []
    for k, sc in enumerate(scenes):
        kp, dp = sc._params(*params[k])
        rgb = torch.zeros((sc.height, sc.width, 3), dtype=torch.float32, device=sc.device)
        b = torch.zeros((sc.height, sc.width), dtype=torch.int32, device=sc.device)
        cnt = torch.zeros_like(b)
        smp = (torch.empty((spp[k], sc.height, sc.width, 3), dtype=torch.float32, device=sc.device)
               if keep_samples else None)
        film = Film(rgb.data_ptr(), b.data_ptr(), cnt.data_ptr(), sc.width, sc.height, 1)
        jobs.append(DiffJob(sc.ctx.h.value, RenderParams(spp[k], first_frame[k], max_depth[k], rr_depth[k]), dp,
                            film, _ptr(smp), None, None, None, None, None))
        keep.append(kp)
        out.append((rgb, b, cnt, smp) if keep_samples else (rgb, b, cnt))
    _batch_call(scenes[0].ctx.L.lt_render_diff_batch, scenes[0], jobs)
    del keep
    return out


def adjoint_batch(scenes, params, d_loss_d_sum, spp, first_frame=0, max_depth: int = 8, rr_depth: int = 3,
                  samples=None):
    """lt_render_adjoint_batch: per scene the gradients (albedo, emission,
    sigma_a, sigma_s) of the loss whose derivative with respect to the film
    colour sums is d_loss_d_sum[k], in one call. samples: per-scene
    per-sample radiance from render_batch(keep_samples=True) (the paths are
    then replayed on the wavefront), or None."""
    n = len(scenes)
    per = lambda v: list(v) if isinstance(v, (list, tuple)) else [v] * n
    spp, first_frame, max_depth, rr_depth = per(spp), per(first_frame), per(max_depth), per(rr_depth)
    samples = samples if samples is not None else [None] * n
    jobs, keep, grads = [], [], []
    for k, sc in enumerate(scenes):
        kp, dp = sc._params(*params[k])
        g = [torch.zeros_like(x) for x in kp[:4]]
        dI = _dev(d_loss_d_sum[k], sc.device)
        film = Film(None, None, None, sc.width, sc.height, 1)
        jobs.append(DiffJob(sc.ctx.h.value, RenderParams(spp[k], first_frame[k], max_depth[k], rr_depth[k]), dp,
                            film, _ptr(samples[k]), dI.data_ptr(), *[x.data_ptr() for x in g]))
        keep.append((kp, dI))
        grads.append(g)
    _batch_call(scenes[0].ctx.L.lt_render_adjoint_batch, scenes[0], jobs)
    torch.cuda.current_stream(scenes[0].device).synchronize()
    del keep
    return grads


def finite_difference_check(scene: DiffScene, theta, target: torch.Tensor, spp: int, first_frame: int = 0,
                            max_depth: int = 8, rr_depth: int = 3, count: int = 64, seed: int = 4,
                            h: float = 1e-3, rel_tol: float = 0.02):
    """Adjoint gradient of L = sum((image - target)^2), image = film / spp,
    against central finite differences of the same estimator.

    theta = (albedo, emission, sigma_a, sigma_s) CUDA tensors; target is the
    reference image (H, W, 3). The adjoint comes from RenderImage's backward;
    each difference renders twice with one parameter moved by +-h and the
    sampling copies (detached albedo, sigma_a, sigma_s) held at theta, so both
    sides differentiate the same function of the parameters (the forward is
    deterministic: every sample's radiance is gathered in the estimator's order
    and the film sums the samples per pixel in frame order).
    Parameters, drawn with `seed`: every sigma_a and sigma_s entry, up to 10
    emission entries whose adjoint gradient is nonzero, then albedo entries with
    a nonzero gradient up to `count` in all. A parameter is compared unless
    both gradients are below 1e-8 of
    the largest gradient of its array (float noise). Returns {"parameters", "checked",
    "max_rel_err", "failures": [(array, index, adjoint, fd), ...], "pairs"}:
    failures are the comparisons whose relative difference exceeds rel_tol,
    pairs every (array, index, adjoint, fd) drawn."""
    base = [t.detach().to(scene.device, torch.float32).contiguous() for t in theta]
    tgt = target.detach().to(scene.device).double()
    th = [t.clone().requires_grad_() for t in base]
    img = render_image(scene, *th, spp, first_frame, max_depth, rr_depth)
    loss = ((img.double() - tgt) ** 2).sum()
    loss.backward()
    grads = [t.grad.detach().cpu().numpy().reshape(-1) for t in th]
    detached = (base[0], base[2], base[3])

    def loss_at(k, idx, delta):
        p = [t.clone() for t in base]
        p[k].view(-1)[idx] += delta
        rgb, _, _ = scene.render(*p, spp=spp, first_frame=first_frame, max_depth=max_depth, rr_depth=rr_depth,
                                 detached=detached)
        return float((((rgb / spp).double() - tgt) ** 2).sum())

    rng = np.random.default_rng(seed)
    cands = ([(2, i) for i in range(3 * scene.num_media)] + [(3, i) for i in range(3 * scene.num_media)])
    nze = np.flatnonzero(np.abs(grads[1]) > 0)
    cands += [(1, int(i)) for i in rng.choice(nze, size=min(10, nze.size), replace=False)]
    nz = np.flatnonzero(np.abs(grads[0]) > 0)
    cands += [(0, int(i)) for i in rng.choice(nz, size=min(max(count - len(cands), 0), nz.size), replace=False)]
    cands = cands[:count]
    gmax = [float(np.abs(g).max()) if g.size else 0.0 for g in grads]
    names = ("albedo", "emission", "sigma_a", "sigma_s")
    failures, worst, checked, pairs = [], 0.0, 0, []
    for k, i in cands:
        fd = (loss_at(k, i, h) - loss_at(k, i, -h)) / (2 * h)
        ad = float(grads[k][i])
        pairs.append((names[k], i, ad, fd))
        if max(abs(fd), abs(ad)) <= 1e-8 * gmax[k]:
            continue
        checked += 1
        rel = abs(ad - fd) / max(abs(fd), abs(ad))
        worst = max(worst, rel)
        if rel > rel_tol:
            failures.append((names[k], i, ad, fd))
    return {"parameters": len(cands), "checked": checked, "max_rel_err": worst, "failures": failures,
            "pairs": pairs}

