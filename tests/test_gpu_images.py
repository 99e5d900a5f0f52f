"""GPU renders against the reference's own renders, statistically.

The reference draws one PCG32 stream per 8x8 tile and frame; the GPU draws one
per (pixel, frame), so individual samples differ and the images are compared
as estimates of the same integral (the acceptance rule for the path): per
channel, the image mean is within 1% of the reference's (the mean of its two
renders), and the RMSE
between the GPU image and A is at most 1.1 times the RMSE between A and an
independently seeded reference render B, at equal samples per pixel. The
reference renders are fixtures made by tests/golden/make_golden.py.
"""
import os

import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.integrator import FrameBuffer, Integrator, Scene

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _render(path, spp, depth, first_frame=0):
    sc = Scene(0)
    sc.LoadSceneFromJSON(path)
    fb = FrameBuffer(sc.width, sc.height, "cuda:0")
    Integrator(sc, fb, max_depth=depth, rr_depth=3, first_frame=first_frame).RenderFrame(spp)
    torch.cuda.synchronize()
    assert int(fb.ColorSampleCount.min()) == spp and int(fb.ColorSampleCount.max()) == spp
    return fb.image().cpu().numpy().astype(np.float64)


def _rmse(x, y):
    return float(np.sqrt(np.mean((x - y) ** 2)))


@pytest.mark.parametrize("make,spp,depth,fixture", [
    (lambda: S.nine_spheres(name="golden_c0"), 16, 8, "reference_c0_images.npz"),
    (lambda: S.tiny_scene(width=96, height=96, name="golden_tiny96"), 64, 12, "reference_tiny_images.npz"),
    (lambda: S.medium_sphere_scene(width=128, height=128, reference_expressible=True, name="golden_c2r"),
     512, 32, "reference_c2r_images.npz"),
    (lambda: S.displaced_icosphere_scene(width=160, height=160, name="golden_ico"), 64, 10,
     "reference_ico_images.npz"),
    ("textured", 64, 8, "reference_textured_images.npz"),
])
def test_image_matches_reference_statistically(scene_dir, make, spp, depth, fixture):
    g = np.load(os.path.join(GOLDEN, fixture))
    a, b = g["a"].astype(np.float64), g["b"].astype(np.float64)
    if make == "textured":
        scene = S.textured_scene(os.path.join(scene_dir, "golden_textures"), width=96, height=96,
                                 name="golden_textured")
    else:
        scene = make()
    img = _render(scene.write(scene_dir), spp, depth)
    assert np.all(np.isfinite(img))
    ma = 0.5 * (a.mean((0, 1)) + b.mean((0, 1)))
    assert np.all(np.abs(img.mean((0, 1)) - ma) <= 0.01 * ma), (img.mean((0, 1)), ma)
    assert _rmse(img, a) <= 1.1 * _rmse(a, b), (_rmse(img, a), _rmse(a, b))
