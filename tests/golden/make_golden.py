"""Generate the golden fixtures in tests/golden from the reference itself.

Run where the reference tree is available (it builds oracle/_ref with
oracle/build_ref.sh): ``python tests/golden/make_golden.py``. Every array
comes out of the reference's own code (liblantern_ref.so):

* reference_blocks.npz -- UniformSampler streams (math/uniform_sampler.h),
  tent ReconstructionFilter::Sample (camera/reconstruction_filter.cpp) and
  PinholeCamera::CalculateRayFromPixel rays (camera/pinhole_camera.cpp) for the
  nine-sphere scene;
* reference_film_tiny.npz -- both swap films of 3 RenderFrame calls of the
  three-material scene at 24x16, max depth 8 (integrator.cpp);
* reference_ico_images.npz, reference_textured_images.npz -- the same pairs for the
  1.3M-triangle icosphere scene and the textured / procedural scene;
* reference_c0_images.npz -- the nine-sphere scene (config 0: 256x256, 16 spp,
  max depth 8, roulette after bounce 3) rendered twice with independent
  streams (frames 0-15 and 1000000-1000015), stored as float16 images
  (colour sum / sample count), for the statistical image test.
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import lantern_gb300.scenes as S  # noqa: E402
from oracle import oracle as O  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
SCENES = os.path.join(ROOT, "_scenes")


def blocks():
    import ctypes as C
    L = O.ref_lib()
    seeds = [(0, 0), (12345, 7), ((1 << 63) + 5, 1000000), (0xDEADBEEF, 3)]
    uints = np.zeros((len(seeds), 64), np.uint32)
    floats = np.zeros((len(seeds), 64), np.float32)
    for i, (s, q) in enumerate(seeds):
        L.lref_pcg_stream(s, q, 64, O.uptr(uints[i]), None)
        L.lref_pcg_stream(s, q, 64, None, O.fptr(floats[i]))
    rng = np.random.default_rng(11)
    fx = np.concatenate([np.linspace(0, 1, 257, dtype=np.float32)[:-1],
                         rng.random(256, dtype=np.float32),
                         np.array([0.0, 0.5, np.nextafter(np.float32(0.5), np.float32(0)),
                                   np.nextafter(np.float32(1), np.float32(0))], np.float32)])
    fs = np.zeros_like(fx)
    L.lref_filter_sample(O.fptr(fx), fx.size, O.fptr(fs))
    path = S.nine_spheres(name="golden_nine").write(SCENES)
    ref = O.ReferenceScene(path)
    px = rng.integers(0, 256, size=(64, 2))
    cseeds = rng.integers(0, 2**63, size=64, dtype=np.uint64)
    rays = np.zeros((64, 6), np.float32)
    for i in range(64):
        L.lref_camera_ray(ref.h, int(px[i, 0]), int(px[i, 1]), C.c_ulonglong(int(cseeds[i])), C.c_ulonglong(i),
                          O.fptr(rays[i]))
    np.savez(os.path.join(OUT, "reference_blocks.npz"), pcg_seeds=np.array(seeds, dtype=np.uint64),
             pcg_uint=uints, pcg_float=floats, filter_x=fx, filter_u=fs, camera_px=px.astype(np.uint32),
             camera_seed=cseeds, camera_rays=rays)


def film_tiny():
    path = S.tiny_scene(width=24, height=16, name="golden_tiny").write(SCENES)
    r = O.ReferenceScene(path).render(3, max_depth=8, rr_depth=3)
    np.savez_compressed(os.path.join(OUT, "reference_film_tiny.npz"),
                        **{k: r[k] for k in ("rgb", "bounces", "counts", "rgb_b", "bounces_b", "counts_b")},
                        rays=np.uint64(r["rays"]))


def image_pair(scene, spp, depth, out_name):
    """Two reference renders with independent streams (frames 0.. and 1000000..)."""
    path = scene.write(SCENES)
    ref = O.ReferenceScene(path)
    imgs = {}
    for tag, first in (("a", 0), ("b", 1_000_000)):
        t = time.time()
        r = ref.render(spp, first_frame=first, max_depth=depth, rr_depth=3)
        rgb = r["rgb"].astype(np.float64) + r["rgb_b"]
        cnt = (r["counts"] + r["counts_b"]).astype(np.float64)
        imgs[tag] = (rgb / cnt[..., None]).astype(np.float16)
        imgs[f"seconds_{tag}"] = np.float64(r["seconds"])
        imgs[f"rays_{tag}"] = np.uint64(r["rays"])
        print(f"{out_name} {tag}: {time.time() - t:.1f}s, {r['rays']} rays")
    np.savez_compressed(os.path.join(OUT, out_name), **imgs)


def c0_images():
    # config 0: 256x256, 16 spp, max depth 8
    image_pair(S.nine_spheres(name="golden_c0"), 16, 8, "reference_c0_images.npz")
    # Lambert + mirror + dielectric spheres: 96x96, 64 spp, max depth 12
    image_pair(S.tiny_scene(width=96, height=96, name="golden_tiny96"), 64, 12, "reference_tiny_images.npz")
    # config 2 in the reference's terms (isotropic phase, scalar sigma_s): 128x128, 512 spp, depth 32
    # (the medium's light paths are heavy-tailed: 512 spp keeps the standard error of
    # the image mean near 0.2%)
    image_pair(S.medium_sphere_scene(width=128, height=128, reference_expressible=True, name="golden_c2r"),
               512, 32, "reference_c2r_images.npz")


def more_images():
    # config 1's scene (1,310,724 triangles; Lambert, mirror, dielectric meshes) at
    # 160x160, 64 spp, max depth 10
    image_pair(S.displaced_icosphere_scene(width=160, height=160, name="golden_ico"), 64, 10,
               "reference_ico_images.npz")
    # uv and image albedo textures, grid and geosphere primitives: 96x96, 64 spp, depth 8
    image_pair(S.textured_scene(os.path.join(SCENES, "golden_textures"), width=96, height=96,
                                name="golden_textured"), 64, 8, "reference_textured_images.npz")


if __name__ == "__main__":
    import sys
    O.build_reference()
    if "--more" in sys.argv:  # only the fixtures added last
        more_images()
        sys.exit(0)
    blocks()
    film_tiny()
    c0_images()
    more_images()
    for f in sorted(os.listdir(OUT)):
        print(f, os.path.getsize(os.path.join(OUT, f)))
