"""Renders through liblantern_gpu_checked.so (the kernels built with their
device-side bound checks) for tests/test_gpu_checked_build.py, in a process of
its own: LANTERN_GPU_CHECKED=1 makes lantern_gb300.native load the checked
library instead of the plain one.

Every render goes through the public API and must finish without a failed
check (LT_ERR_CHECK). The parity scenes are compared with the oracle as in
test_gpu_parity.py (the checks leave the arithmetic alone, so the same paths
are traced); a batch and the fixed-scratch render with the single-scene
renders; the differentiable forward and adjoint only run. Last, the test-only
film pixel limit makes a normal render fail a check, and the same context then
renders cleanly again. Prints one JSON object.
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
os.environ["LANTERN_GPU_CHECKED"] = "1"

import numpy as np  # noqa: E402
import torch  # noqa: E402

import lantern_gb300.scenes as S  # noqa: E402
from lantern_gb300 import native  # noqa: E402
from lantern_gb300.diff import DiffScene  # noqa: E402
from lantern_gb300.integrator import FrameBuffer, Integrator, RenderBatch, Scene  # noqa: E402
from lantern_gb300.native import LanternError  # noqa: E402
from oracle import oracle as O  # noqa: E402

SCENES = os.path.join(ROOT, "_scenes")


def _scene(sc):
    s = Scene(0)
    s.LoadSceneFromJSON(sc.write(SCENES))
    return s


def _render(s, spp, depth, **tuning):
    if tuning:
        s.ctx.set_tuning(**tuning)
    fb = FrameBuffer(s.width, s.height, "cuda:0")
    Integrator(s, fb, max_depth=depth, rr_depth=3).RenderFrame(spp)
    torch.cuda.synchronize()
    return fb


def parity(out):
    cases = [(S.tiny_scene(width=48, height=40, name="chk_tiny"), 6, 12, (2, 4, 8)),
             (S.nine_spheres(width=64, height=64, name="chk_nine"), 4, 8, (2, 4, 8)),
             (S.medium_sphere_scene(width=40, height=40, name="chk_med_hg"), 4, 32, (2, 8)),
             (S.medium_sphere_scene(width=40, height=40, non_scattering=True, name="chk_med_abs"), 4, 32, (2,)),
             (S.procedural_scene(width=48, height=40, name="chk_proc"), 4, 8, (2,)),
             (S.textured_scene(os.path.join(SCENES, "textures"), width=48, height=40, name="chk_tex"), 4, 8, (2,))]
    res = []
    for sc, spp, depth, widths in cases:
        path = sc.write(SCENES)
        ref = O.OracleScene(path).render(spp, max_depth=depth, rr_depth=3, keying=O.KEY_PIXEL)
        s = Scene(0)
        s.LoadSceneFromJSON(path)
        for w in widths:
            fb = _render(s, spp, depth, bvh_width=w)
            counts = np.array_equal(fb.ColorSampleCount.cpu().numpy(), ref["counts"].astype(np.int32))
            same_b = float((fb.Bounces.cpu().numpy() == ref["bounces"].astype(np.int32)).mean())
            close = float(np.isclose(fb.ColorData.cpu().numpy(), ref["rgb"], rtol=2e-4, atol=1e-5).all(-1).mean())
            res.append({"scene": sc.name, "width": w, "counts": counts, "bounces": same_b, "colour": close})
    out["parity"] = res


def refills(out):
    """A wavefront smaller than the render: paths restart from work items at
    the top of the queue every iteration, and the last iterations go to the
    one-warp-per-ray kernel."""
    s = _scene(S.displaced_icosphere_scene(width=64, height=64, levels=5, name="chk_ico5"))
    fb = _render(s, 16, 10, paths_in_flight=1024)
    out["refills"] = {"min": int(fb.ColorSampleCount.min()), "max": int(fb.ColorSampleCount.max())}


def batch_and_noalloc(out):
    scenes = [_scene(S.tiny_scene(width=32, height=24, name="chkb_tiny")),
              _scene(S.nine_spheres(width=40, height=40, slices=16, stacks=8, name="chkb_nine")),
              _scene(S.medium_sphere_scene(width=24, height=32, name="chkb_med"))]
    spps = [3, 2, 4]
    single = [_render(s, n, 8) for s, n in zip(scenes, spps)]
    fbs = [FrameBuffer(s.width, s.height, "cuda:0") for s in scenes]
    RenderBatch([Integrator(s, f, max_depth=8, rr_depth=3) for s, f in zip(scenes, fbs)], spps)
    torch.cuda.synchronize()
    out["batch"] = all(torch.equal(a.ColorSampleCount, b.ColorSampleCount) and torch.equal(a.Bounces, b.Bounces)
                       for a, b in zip(single, fbs))
    s = scenes[1]
    fb = FrameBuffer(s.width, s.height, "cuda:0")
    s.ctx.render_noalloc(fb.film(), 2, 4096, max_depth=8)
    torch.cuda.synchronize()
    out["noalloc"] = bool(torch.equal(fb.ColorSampleCount, single[1].ColorSampleCount) and
                          torch.equal(fb.Bounces, single[1].Bounces))


def differentiable(out):
    path = S.differentiable_scene(width=32, height=32, slices=16, stacks=8, name="chk_diff").write(SCENES)
    ds = DiffScene(path)
    a, e, sa, ss = ds.defaults()
    rgb, b, n, smp = ds.render(a, e, sa, ss, spp=4, max_depth=8, keep_samples=True)
    g_wave = ds.adjoint(a, e, sa, ss, torch.ones_like(rgb), spp=4, max_depth=8, samples=smp)
    g_replay = ds.adjoint(a, e, sa, ss, torch.ones_like(rgb), spp=4, max_depth=8)
    torch.cuda.synchronize()
    out["diff"] = {"counts": int(n.min()), "grad_finite": bool(all(torch.isfinite(g).all() for g in g_wave + g_replay))}


def planted_limit(out):
    """A film pixel limit below the film's size: the render fails its pixel
    check (the accesses it skips were in bounds), and renders cleanly again
    once the limit is lifted."""
    s = _scene(S.tiny_scene(width=4, height=3, name="chk_limit"))
    L = native.load()
    L.lt_debug_set_check_pixel_limit(5)
    try:
        _render(s, 2, 6)
        out["planted"] = {"status": "LT_OK"}
    except LanternError as err:
        out["planted"] = {"status": native.STATUS.get(err.status, str(err.status)), "message": str(err)}
    finally:
        L.lt_debug_set_check_pixel_limit(0)
    fb = _render(s, 2, 6)
    out["after_planted"] = {"min": int(fb.ColorSampleCount.min()), "max": int(fb.ColorSampleCount.max())}


def main():
    out = {"library": os.path.basename(native.load()._name)}
    for step in (parity, refills, batch_and_noalloc, differentiable, planted_limit):
        try:
            step(out)
        except LanternError as err:  # a failed check (or any other status) ends the step
            out.setdefault("errors", []).append(f"{step.__name__}: {err}")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
