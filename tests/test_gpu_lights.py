"""Area-light setup on the device (scene table row: the scene loader feeding the
device, with the transform, area and bounding sphere computed there).

With the GPU builder lt_scene_create transforms the vertices, sets up the
triangles and computes every area light's triangles, area (the sequential sum
of scene.cpp:527-534), bounding sphere (CalculateBoundingSphere's two Ritter
passes and tightening pass, scene.cpp:49-80) and radiance (area_light.h:16-21)
on the device, one thread per light in the reference's order. They must equal
the host builder's values and the oracle's (which is pinned to the compiled
reference) bit for bit, and both builds must render the same image.
"""
import json
import math

import numpy as np
import pytest
import torch

import lantern_gb300.scenes as S
from lantern_gb300.integrator import FrameBuffer
from lantern_gb300.native import BVH_GPU, BVH_HOST, Context
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rotated_scaled(angle, scale, t):
    c, s = math.cos(angle), math.sin(angle)
    return [scale * c, 0.0, scale * s, t[0], 0.0, scale, 0.0, t[1], -scale * s, 0.0, scale * c, t[2],
            0.0, 0.0, 0.0, 1.0]


def _emissive_sphere_scene(scene_dir):
    """The tiny scene plus a second light: an emissive 64x32 UV sphere (3,968
    triangles) placed by a rotation, scale and translation in the scene JSON."""
    sc = S.tiny_scene(width=40, height=32, name="lights_sphere")
    p, n, i = S.uv_sphere(0.35, 64, 32)
    sc.meshes.append(S.Mesh("glow", p, n, i, sc.meshes[-1].material,
                            emission={"color": [0.9, 0.6, 0.3], "radiant_power": 40.0}))
    path = sc.write(scene_dir)
    with open(path) as fh:
        j = json.load(fh)
    for prim in j["primitives"]:
        if prim["name"] == "glow":
            prim["transform"] = _rotated_scaled(0.7, 1.3, (0.8, 1.9, -0.4))
    with open(path, "w") as fh:
        json.dump(j, fh, indent=1)
    return path


SCENES = {
    "nine_spheres": lambda d: S.nine_spheres(width=32, height=32, slices=16, stacks=8, name="lights_nine").write(d),
    "two_lights": lambda d: S.two_light_scene(name="lights_two").write(d),
    "procedural": lambda d: S.procedural_scene(width=24, height=24, name="lights_proc").write(d),
    "emissive_sphere": _emissive_sphere_scene,
}


def _load(path, builder):
    c = Context(0)
    c.set_bvh_builder(builder)
    c.load_scene_json(path)
    return c


def _bits(x):
    return np.asarray(x, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", list(SCENES))
def test_device_light_setup_equals_host_and_oracle(scene_dir, name):
    path = SCENES[name](scene_dir)
    gpu, host = _load(path, BVH_GPU), _load(path, BVH_HOST)
    lg, lh = gpu.lights(), host.lights()
    ref = O.OracleScene(path).lights()
    assert len(lg) == len(lh) == len(ref) > 0
    for a, b, (area, sphere, rad) in zip(lg, lh, ref):
        assert (a.mesh, a.num_triangles) == (b.mesh, b.num_triangles)
        for x, y in ((a, b),):
            assert _bits(x.area) == _bits(y.area)
            assert np.array_equal(_bits(list(x.sphere)), _bits(list(y.sphere)))
            assert np.array_equal(_bits(list(x.radiance)), _bits(list(y.radiance)))
        assert _bits(a.area) == _bits(area)
        assert np.array_equal(_bits(list(a.sphere)), _bits(sphere))
        assert np.array_equal(_bits(list(a.radiance)), _bits(rad))
    # both builds render the same samples
    info = gpu.scene_info()
    films = []
    for c in (gpu, host):
        fb = FrameBuffer(info.width, info.height, "cuda:0")
        c.set_stream(torch.cuda.current_stream().cuda_stream)
        c.render(fb.film(), 3, 0, 8, 3)
        films.append(fb)
    torch.cuda.synchronize()
    assert torch.equal(films[0].ColorSampleCount, films[1].ColorSampleCount)
    assert torch.equal(films[0].Bounces, films[1].Bounces)
    assert torch.allclose(films[0].ColorData, films[1].ColorData, rtol=1e-5, atol=1e-6)
    gpu.close()
    host.close()
