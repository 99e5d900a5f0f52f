"""The oracle against golden vectors produced by the reference's own code
(tests/golden/make_golden.py): sampler streams, tent filter, camera rays and
the films of a small render must be reproduced bit for bit."""
import ctypes as C
import os

import numpy as np
import pytest

import lantern_gb300.scenes as S
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def test_sampler_streams():
    g = _load("reference_blocks.npz")
    L = O.lib()
    for (seed, seq), u, f in zip(g["pcg_seeds"], g["pcg_uint"], g["pcg_float"]):
        ou = np.zeros(64, np.uint32)
        of = np.zeros(64, np.float32)
        L.orc_pcg_stream(int(seed), int(seq), 64, O.uptr(ou), None)
        L.orc_pcg_stream(int(seed), int(seq), 64, None, O.fptr(of))
        assert np.array_equal(ou, u)
        assert np.array_equal(of.view(np.uint32), f.view(np.uint32))


def test_tent_filter():
    g = _load("reference_blocks.npz")
    L = O.lib()
    out = np.array([L.orc_filter_sample(C.c_float(float(x))) for x in g["filter_x"]], np.float32)
    assert np.array_equal(out.view(np.uint32), g["filter_u"].view(np.uint32))
    assert np.all(np.abs(out) <= 1.05)


def test_camera_rays(scene_dir):
    g = _load("reference_blocks.npz")
    path = S.nine_spheres(name="golden_nine").write(scene_dir)
    orc = O.OracleScene(path)
    L = O.lib()
    for (x, y), seed, i, ray in zip(g["camera_px"], g["camera_seed"], range(64), g["camera_rays"]):
        f = np.zeros(2, np.float32)
        L.orc_pcg_stream(int(seed), i, 2, None, O.fptr(f))
        u, v = L.orc_filter_sample(C.c_float(float(f[0]))), L.orc_filter_sample(C.c_float(float(f[1])))
        d, o = np.zeros(3, np.float32), np.zeros(3, np.float32)
        L.orc_camera_ray(orc.h, int(x), int(y), u, v, O.fptr(d), O.fptr(o))
        assert np.array_equal(np.concatenate([o, d]).view(np.uint32), ray.view(np.uint32))


def test_reference_film(scene_dir):
    g = _load("reference_film_tiny.npz")
    path = S.tiny_scene(width=24, height=16, name="golden_tiny").write(scene_dir)
    r = O.OracleScene(path).render(3, max_depth=8, rr_depth=3, keying=O.KEY_TILE, two_films=True, threads=2)
    for k in ("rgb", "bounces", "counts", "rgb_b", "bounces_b", "counts_b"):
        a, b = r[k], g[k]
        if a.dtype == np.float32:
            a, b = a.view(np.uint32), b.view(np.uint32)
        assert np.array_equal(a, b), k
    assert sum(r["rays"]) == int(g["rays"])


def test_c0_reference_images_are_consistent():
    """The two golden renders are independent estimates of one image."""
    g = _load("reference_c0_images.npz")
    a, b = g["a"].astype(np.float64), g["b"].astype(np.float64)
    assert a.shape == (256, 256, 3)
    assert np.all(np.isfinite(a)) and np.all(np.isfinite(b))
    ma, mb = a.mean((0, 1)), b.mean((0, 1))
    assert np.all(np.abs(ma - mb) <= 0.01 * ma)
    assert not np.array_equal(a, b)


@pytest.mark.parametrize("keying", [O.KEY_PIXEL, O.KEY_TILE])
def test_oracle_c0_statistics_match_reference(scene_dir, keying):
    """The oracle with the GPU's per-pixel keying renders the same image as the
    reference (statistically): per-channel means within 1%, RMSE to reference
    render A within 1.1x the A-to-B RMSE."""
    g = _load("reference_c0_images.npz")
    a, b = g["a"].astype(np.float64), g["b"].astype(np.float64)
    path = S.nine_spheres(name="golden_c0").write(scene_dir)
    r = O.OracleScene(path).render(16, first_frame=500_000, max_depth=8, rr_depth=3, keying=keying)
    img = r["rgb"].astype(np.float64) / r["counts"][..., None]
    assert np.all(np.abs(img.mean((0, 1)) - a.mean((0, 1))) <= 0.01 * a.mean((0, 1)))
    rmse = lambda x, y: float(np.sqrt(np.mean((x - y) ** 2)))  # noqa: E731
    assert rmse(img, a) <= 1.1 * rmse(a, b)
