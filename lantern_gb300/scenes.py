"""Seeded synthetic scenes in Lantern's own on-disk formats (scene JSON + LMF).

The benchmark configurations have no public assets, so every scene here is
generated from a numpy seed and written the way Lantern reads scenes:

* meshes go to ``.lmf`` files in the binary layout of
  ``source/core/io/lantern_model_file.cpp:67-102`` (``WriteLFM``): magic
  ``LMF\\0``, ``u8`` vertices per primitive, ``u32`` flags, ``u64`` vertex count
  + float32 positions, ``u64`` index count + ``u32`` indices, then optional
  ``u64`` float count + float32 normals;
* the scene goes to a JSON file with the keys parsed by
  ``source/core/scene/scene.cpp:215-446`` (camera, bsdfs, media, materials,
  primitives with ``emission``).

Two keys are extensions that the reference loader does not know and ignores:
a ``render`` block (spp, max_depth, rr_depth) and the ``henyey_greenstein``
medium type (RGB sigma_a / sigma_s and anisotropy ``g``).

Mesh topology follows the reference generators where one exists:
``uv_sphere`` is ``CreateSphere`` (``source/core/scene/geometry_generator.cpp:123-212``,
2*slices*(stacks-1) triangles). Every mesh carries per-vertex normals, because a
mesh without normals makes the reference shade with a NaN normal
(``integrator.cpp:179-183``).
"""
from __future__ import annotations

import json
import os
import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

F32 = np.float32


# --------------------------------------------------------------------------- meshes
@dataclass
class Mesh:
    name: str
    positions: np.ndarray  # (V, 3) float32, world space
    normals: np.ndarray    # (V, 3) float32
    indices: np.ndarray    # (T, 3) uint32
    material: str
    emission: Optional[dict] = None  # {"color": [r,g,b], "radiant_power": p}
    texcoords: Optional[np.ndarray] = None  # (V, 2) float32

    @property
    def num_triangles(self) -> int:
        return int(self.indices.shape[0])


def uv_sphere(radius: float, slices: int, stacks: int, center=(0.0, 0.0, 0.0)):
    """UV sphere with the vertex/index order of ``CreateSphere``
    (``geometry_generator.cpp:123-212``): top pole, (stacks-1) rings of
    (slices+1) vertices, bottom pole; fan at each pole, quads between rings."""
    r = F32(radius)
    pos = [np.array([[0.0, r, 0.0]], dtype=F32)]
    nrm = [np.array([[0.0, 1.0, 0.0]], dtype=F32)]
    phi_step = F32(np.pi) / F32(stacks)
    theta_step = F32(2.0) * F32(np.pi) / F32(slices)
    i = np.arange(1, stacks, dtype=F32)
    j = np.arange(0, slices + 1, dtype=F32)
    phi = (i * phi_step)[:, None]
    theta = (j * theta_step)[None, :]
    sp, cp = np.sin(phi).astype(F32), np.cos(phi).astype(F32)
    st, ct = np.sin(theta).astype(F32), np.cos(theta).astype(F32)
    x = (r * sp) * st
    y = np.broadcast_to(r * cp, x.shape)
    z = (r * sp) * ct
    ring = np.stack([x, y, z], axis=-1).reshape(-1, 3).astype(F32)
    ring_n = ring / np.linalg.norm(ring, axis=1, keepdims=True)
    pos.append(ring)
    nrm.append(ring_n.astype(F32))
    pos.append(np.array([[0.0, -r, 0.0]], dtype=F32))
    nrm.append(np.array([[0.0, -1.0, 0.0]], dtype=F32))
    positions = np.concatenate(pos).astype(F32)
    normals = np.concatenate(nrm).astype(F32)

    idx = []
    for k in range(1, slices + 1):
        idx.append((0, k + 1, k))
    base = 1
    rc = slices + 1
    for a in range(stacks - 2):
        for b in range(slices):
            idx.append((base + a * rc + b, base + a * rc + b + 1, base + (a + 1) * rc + b))
            idx.append((base + (a + 1) * rc + b, base + a * rc + b + 1, base + (a + 1) * rc + b + 1))
    south = positions.shape[0] - 1
    base = south - rc
    for k in range(slices):
        idx.append((south, base + k, base + k + 1))
    indices = np.asarray(idx, dtype=np.uint32)
    positions = positions + np.asarray(center, dtype=F32)[None, :]
    return positions.astype(F32), normals, indices


def quad(center, half_x: float, half_z: float, y_normal: float):
    """Axis-aligned quad in the xz plane as two triangles, normal (0, +-1, 0)."""
    cx, cy, cz = center
    p = np.array([[cx - half_x, cy, cz - half_z], [cx + half_x, cy, cz - half_z],
                  [cx + half_x, cy, cz + half_z], [cx - half_x, cy, cz + half_z]], dtype=F32)
    n = np.tile(np.array([[0.0, y_normal, 0.0]], dtype=F32), (4, 1))
    if y_normal > 0:
        idx = np.array([[0, 2, 1], [0, 3, 2]], dtype=np.uint32)
    else:
        idx = np.array([[0, 1, 2], [0, 2, 3]], dtype=np.uint32)
    return p, n, idx


def icosphere(levels: int):
    """Unit icosahedron subdivided ``levels`` times with shared vertices
    (20 * 4**levels triangles, 10 * 4**levels + 2 vertices)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
                  [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                  [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                  [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                  [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    for _ in range(levels):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        e.sort(axis=1)
        key = e[:, 0] * (1 << 32) + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a = (uniq >> 32).astype(np.int64)
        b = (uniq & 0xFFFFFFFF).astype(np.int64)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid], axis=0)
        m = inv.reshape(3, -1) + nv  # midpoints of edges (0,1), (1,2), (2,0)
        m01, m12, m20 = m[0], m[1], m[2]
        f = np.concatenate([
            np.stack([f[:, 0], m01, m20], 1),
            np.stack([f[:, 1], m12, m01], 1),
            np.stack([f[:, 2], m20, m12], 1),
            np.stack([m01, m12, m20], 1)], axis=0)
    return v, f


def _value_noise3(p: np.ndarray, seed: int) -> np.ndarray:
    """Seeded value noise on the integer lattice with quintic interpolation."""
    rng = np.random.default_rng(seed)
    perm = rng.permutation(256).astype(np.int64)
    perm = np.concatenate([perm, perm])
    vals = rng.uniform(-1.0, 1.0, 256)
    pi = np.floor(p).astype(np.int64)
    pf = p - pi
    w = pf * pf * pf * (pf * (pf * 6.0 - 15.0) + 10.0)
    xi, yi, zi = pi[:, 0] & 255, pi[:, 1] & 255, pi[:, 2] & 255

    def h(dx, dy, dz):
        return vals[perm[perm[perm[(xi + dx) & 255] + ((yi + dy) & 255)] + ((zi + dz) & 255)]]

    x0 = h(0, 0, 0) + w[:, 0] * (h(1, 0, 0) - h(0, 0, 0))
    x1 = h(0, 1, 0) + w[:, 0] * (h(1, 1, 0) - h(0, 1, 0))
    x2 = h(0, 0, 1) + w[:, 0] * (h(1, 0, 1) - h(0, 0, 1))
    x3 = h(0, 1, 1) + w[:, 0] * (h(1, 1, 1) - h(0, 1, 1))
    y0 = x0 + w[:, 1] * (x1 - x0)
    y1 = x2 + w[:, 1] * (x3 - x2)
    return y0 + w[:, 2] * (y1 - y0)


def fbm(p: np.ndarray, octaves: int, seed: int) -> np.ndarray:
    out = np.zeros(p.shape[0])
    amp, freq, norm = 1.0, 2.0, 0.0
    for o in range(octaves):
        out += amp * _value_noise3(p * freq, seed + o)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    return out / norm


def vertex_normals(pos: np.ndarray, idx: np.ndarray) -> np.ndarray:
    p = pos.astype(np.float64)
    fn = np.cross(p[idx[:, 1]] - p[idx[:, 0]], p[idx[:, 2]] - p[idx[:, 0]])
    n = np.zeros_like(p)
    for c in range(3):
        for k in range(3):
            n[:, c] += np.bincount(idx[:, k], weights=fn[:, c], minlength=p.shape[0])
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    return n.astype(F32)


def displaced_icosphere(levels: int, radius: float, amplitude: float, octaves: int,
                        seed: int, center=(0.0, 0.0, 0.0)):
    v, f = icosphere(levels)
    d = fbm(v * 2.0, octaves, seed)
    r = radius * (1.0 + amplitude * d)
    pos = (v * r[:, None] + np.asarray(center)[None, :]).astype(F32)
    # outward winding: the base icosahedron faces are counter-clockwise seen from outside
    idx = f.astype(np.uint32)
    nrm = vertex_normals(pos, idx)
    return pos, nrm, idx, f


# --------------------------------------------------------------------------- scenes
@dataclass
class Scene:
    width: int
    height: int
    camera: dict
    meshes: List[Mesh] = field(default_factory=list)
    bsdfs: List[dict] = field(default_factory=list)
    media: List[dict] = field(default_factory=list)
    materials: List[dict] = field(default_factory=list)
    background: tuple = (0.0, 0.0, 0.0)
    render: dict = field(default_factory=dict)
    name: str = "scene"
    procedural: List[dict] = field(default_factory=list)  # "grid" / "geosphere" primitive entries

    @property
    def num_triangles(self) -> int:
        return sum(m.num_triangles for m in self.meshes)

    def to_json_dict(self, lmf_names: Dict[str, str]) -> dict:
        cam = dict(self.camera)
        cam["client_width"] = self.width
        cam["client_height"] = self.height
        prims = []
        for m in self.meshes:
            p = {"name": m.name, "type": "lmf", "file_path": lmf_names[m.name],
                 "material": m.material}
            if m.emission is not None:
                p["emission"] = m.emission
            prims.append(p)
        prims += [dict(p) for p in self.procedural]
        d = {"background_color": list(self.background), "camera": cam,
             "bsdfs": self.bsdfs, "materials": self.materials, "primitives": prims}
        if self.media:
            d["media"] = self.media
        if self.render:
            d["render"] = self.render
        return d

    def write(self, directory: str) -> str:
        """Write ``<name>.json`` and one ``.lmf`` per mesh into ``directory``;
        returns the JSON path."""
        os.makedirs(directory, exist_ok=True)
        names = {}
        for m in self.meshes:
            fn = f"{self.name}_{m.name}.lmf"
            write_lmf(os.path.join(directory, fn), m.positions, m.indices, m.normals, m.texcoords)
            names[m.name] = fn
        path = os.path.join(directory, f"{self.name}.json")
        with open(path, "w") as fh:
            json.dump(self.to_json_dict(names), fh, indent=1)
        return path


def write_lmf(path: str, positions: np.ndarray, indices: np.ndarray,
              normals: Optional[np.ndarray] = None, texcoords: Optional[np.ndarray] = None,
              verts_per_prim: int = 3) -> None:
    """Binary LMF exactly as ``WriteLFM`` (``lantern_model_file.cpp:67-102``)
    lays it out. The format document says float counts/indices; the code writes
    a vertex count and uint32 indices, and the code is what readers follow."""
    pos = np.ascontiguousarray(positions, dtype="<f4").reshape(-1)
    idx = np.ascontiguousarray(indices, dtype="<u4").reshape(-1)
    flags = 0
    if normals is not None and normals.size:
        flags |= 1
    if texcoords is not None and texcoords.size:
        flags |= 2
    with open(path, "wb") as fh:
        fh.write(b"LMF\x00")
        fh.write(struct.pack("<B", verts_per_prim))
        fh.write(struct.pack("<I", flags))
        fh.write(struct.pack("<Q", pos.size // 3))
        fh.write(pos.tobytes())
        fh.write(struct.pack("<Q", idx.size))
        fh.write(idx.tobytes())
        if flags & 1:
            n = np.ascontiguousarray(normals, dtype="<f4").reshape(-1)
            fh.write(struct.pack("<Q", n.size))
            fh.write(n.tobytes())
        if flags & 2:
            t = np.ascontiguousarray(texcoords, dtype="<f4").reshape(-1)
            fh.write(struct.pack("<Q", t.size))
            fh.write(t.tobytes())


def _lambert(name, albedo):
    return {"name": name, "type": "lambert",
            "albedo": {"type": "constant", "value": [float(a) for a in albedo]}}


def _ground_and_light(scene: Scene) -> None:
    p, n, i = quad((0.0, 0.0, 0.0), 10.0, 10.0, 1.0)
    scene.bsdfs.append(_lambert("ground", (0.5, 0.5, 0.5)))
    scene.materials.append({"name": "ground", "bsdf": "ground"})
    scene.meshes.append(Mesh("ground", p, n, i, "ground"))
    p, n, i = quad((0.0, 5.0, 0.0), 1.0, 1.0, -1.0)
    scene.bsdfs.append(_lambert("light", (0.0, 0.0, 0.0)))
    scene.materials.append({"name": "light", "bsdf": "light"})
    # radiance L = color * P / (pi * A) (area_light.h:16-21): L = 15 for A = 4
    scene.meshes.append(Mesh("light", p, n, i, "light",
                             emission={"color": [1.0, 1.0, 1.0],
                                       "radiant_power": float(15.0 * np.pi * 4.0)}))


def nine_spheres(width=256, height=256, spp=16, max_depth=8, rr_depth=3, seed=0,
                 slices=64, stacks=32, name="nine_spheres") -> Scene:
    """Nine UV spheres (r 0.5) on a 3x3 grid with 1.2 spacing, a 20x20 ground
    quad and a 2x2 area light at y=5 (emission 15); Lambert albedo per channel
    U(0.2, 0.9) from ``seed``; 45 degree pinhole camera."""
    rng = np.random.default_rng(seed)
    sc = Scene(width, height,
               camera={"phi": 1.1, "theta": 0.0, "radius": 6.0, "fov": 0.785398,
                       "target": [0.0, 0.5, 0.0]},
               render={"spp": spp, "max_depth": max_depth, "rr_depth": rr_depth},
               name=name)
    k = 0
    for gx in (-1.2, 0.0, 1.2):
        for gz in (-1.2, 0.0, 1.2):
            alb = rng.uniform(0.2, 0.9, 3)
            bn = f"sphere{k}"
            sc.bsdfs.append(_lambert(bn, alb))
            sc.materials.append({"name": bn, "bsdf": bn})
            p, n, i = uv_sphere(0.5, slices, stacks, center=(gx, 0.5, gz))
            sc.meshes.append(Mesh(bn, p, n, i, bn))
            k += 1
    _ground_and_light(sc)
    return sc


def displaced_icosphere_scene(width=1024, height=1024, spp=64, max_depth=10, rr_depth=3,
                              levels=8, seed=1, name="icosphere") -> Scene:
    """Icosahedron subdivided ``levels`` times (1,310,720 triangles at 8) with
    seeded fBm radial displacement (amplitude 0.05, 6 octaves) on the ground,
    under the area light. The mesh is split into three meshes by base
    icosahedron face so that Lambert, mirror and dielectric (IOR 1.5) are each
    assigned per mesh."""
    sc = Scene(width, height,
               camera={"phi": 1.15, "theta": 0.4, "radius": 4.5, "fov": 0.785398,
                       "target": [0.0, 0.9, 0.0]},
               render={"spp": spp, "max_depth": max_depth, "rr_depth": rr_depth},
               name=name)
    pos, nrm, idx, _ = displaced_icosphere(levels, 1.0, 0.05, 6, seed, center=(0.0, 1.05, 0.0))
    # faces of each level are ordered [corner0 | corner1 | corner2 | center] blocks of the
    # previous level, so the base face of face k is k mod 20
    base_face = np.arange(idx.shape[0]) % 20
    groups = [("diffuse", base_face < 10), ("mirror", (base_face >= 10) & (base_face < 15)),
              ("glass", base_face >= 15)]
    sc.bsdfs.append(_lambert("diffuse", (0.8, 0.45, 0.3)))
    sc.bsdfs.append({"name": "mirror", "type": "mirror",
                     "albedo": {"type": "constant", "value": [0.95, 0.95, 0.95]}})
    sc.bsdfs.append({"name": "glass", "type": "ideal_specular_dielectric",
                     "albedo": {"type": "constant", "value": [0.98, 0.98, 0.98]}, "ior": 1.5})
    for nm, mask in groups:
        sc.materials.append({"name": nm, "bsdf": nm})
        sub = idx[mask]
        used, remap = np.unique(sub.reshape(-1), return_inverse=True)
        sc.meshes.append(Mesh(f"ico_{nm}", pos[used], nrm[used],
                              remap.reshape(-1, 3).astype(np.uint32), nm))
    _ground_and_light(sc)
    return sc


def medium_sphere_scene(width=512, height=512, spp=256, max_depth=32, rr_depth=3,
                        reference_expressible=False, name="medium_sphere", non_scattering=False) -> Scene:
    """Dielectric sphere (IOR 1.33, 128x64) holding a homogeneous medium, on the
    nine-sphere ground under the same light. The full form has RGB
    sigma_s=(2.0,1.5,1.0), sigma_a=(0.05,0.1,0.2) and Henyey-Greenstein g=0.3
    (an extension). ``reference_expressible`` gives the form the reference JSON
    can state: isotropic phase, scalar sigma_s=1.5 as ``scattering_distance``
    1/1.5, and sigma_a as ``absorption_color`` exp(-sigma_a) at distance 1.
    ``non_scattering`` gives the reference's absorbing-only medium
    (non_scattering_medium.h) with the same sigma_a."""
    sc = Scene(width, height,
               camera={"phi": 1.1, "theta": 0.0, "radius": 6.0, "fov": 0.785398,
                       "target": [0.0, 0.8, 0.0]},
               render={"spp": spp, "max_depth": max_depth, "rr_depth": rr_depth},
               name=name)
    sigma_a = np.array([0.05, 0.1, 0.2])
    if non_scattering:
        sc.media.append({"name": "fog", "type": "non_scattering",
                         "absorption_color": [float(x) for x in np.exp(-sigma_a)],
                         "absorption_at_distance": 1.0})
    elif reference_expressible:
        sc.media.append({"name": "fog", "type": "isotropic_scattering",
                         "absorption_color": [float(x) for x in np.exp(-sigma_a)],
                         "absorption_at_distance": 1.0,
                         "scattering_distance": float(1.0 / 1.5)})
    else:
        sc.media.append({"name": "fog", "type": "henyey_greenstein",
                         "sigma_a": [float(x) for x in sigma_a],
                         "sigma_s": [2.0, 1.5, 1.0], "g": 0.3})
    sc.bsdfs.append({"name": "water", "type": "ideal_specular_dielectric",
                     "albedo": {"type": "constant", "value": [1.0, 1.0, 1.0]}, "ior": 1.33})
    sc.materials.append({"name": "water", "bsdf": "water", "medium": "fog"})
    p, n, i = uv_sphere(1.0, 128, 64, center=(0.0, 1.0, 0.0))
    sc.meshes.append(Mesh("ball", p, n, i, "water"))
    _ground_and_light(sc)
    return sc


def differentiable_scene(width=512, height=512, spp=32, max_depth=8, rr_depth=3, slices=64, stacks=32,
                         name="diff_scene") -> Scene:
    """Differentiable workload: the nine-sphere scene plus a dielectric sphere
    (IOR 1.33, radius 0.6, to the right of the grid) holding the RGB
    Henyey-Greenstein fog of the medium workload (sigma_s, sigma_a, g = 0.3)."""
    sc = nine_spheres(width=width, height=height, spp=spp, max_depth=max_depth, rr_depth=rr_depth, seed=0,
                      slices=slices, stacks=stacks, name=name)
    sc.media.append({"name": "fog", "type": "henyey_greenstein", "sigma_a": [0.05, 0.1, 0.2],
                     "sigma_s": [2.0, 1.5, 1.0], "g": 0.3})
    sc.bsdfs.append({"name": "water", "type": "ideal_specular_dielectric",
                     "albedo": {"type": "constant", "value": [1.0, 1.0, 1.0]}, "ior": 1.33})
    sc.materials.append({"name": "water", "bsdf": "water", "medium": "fog"})
    p, n, i = uv_sphere(0.6, slices, stacks, center=(2.4, 0.6, 0.0))
    sc.meshes.append(Mesh("fog_ball", p, n, i, "water"))
    return sc


def differentiable_targets(num_triangles: int, seed: int = 3):
    """Differentiable workload parameters: true per-triangle albedo U(0.2, 0.9)
    (seed 3) and the fog's own coefficients; initial guess albedo 0.5 and sigma_s = sigma_a = 1."""
    rng = np.random.default_rng(seed)
    true = {"albedo": rng.uniform(0.2, 0.9, size=(num_triangles, 3)).astype(F32),
            "sigma_a": np.array([[0.05, 0.1, 0.2]], F32), "sigma_s": np.array([[2.0, 1.5, 1.0]], F32)}
    init = {"albedo": np.full((num_triangles, 3), 0.5, F32),
            "sigma_a": np.ones((1, 3), F32), "sigma_s": np.ones((1, 3), F32)}
    return true, init


def batch_scenes(count: int = 64, seed: int = 5, max_depth: int = 10, rr_depth: int = 3, max_resolution: int = 1024,
                 max_triangles: int = 500_000, name: str = "batch"):
    """The batched workload: `count` scenes with sizes drawn per scene from one
    generator seeded `seed`:

    * resolution from {128, 256, 512, 1024}^2 (capped at max_resolution);
    * triangle target log-uniform in [1,000, max_triangles], met as closely as
      1-4 displaced icospheres of one subdivision level (20 * 4^L triangles
      each, at most max_triangles in all) allow, on the ground quad under the
      area light;
    * spp from {4, 16, 64};
    * 30% of the scenes also hold the dielectric fog ball of the medium
      workload (RGB sigma_s, sigma_a, Henyey-Greenstein g = 0.3);
    * every second scene is marked for the adjoint (``render["adjoint"]``).

    Sphere materials: Lambert (60%), mirror (20%), dielectric IOR 1.5 (20%)."""
    rng = np.random.default_rng(seed)
    bases = {}
    scenes = []
    for s in range(count):
        res = int(min(rng.choice([128, 256, 512, 1024]), max_resolution))
        target = float(np.exp(rng.uniform(np.log(1000.0), np.log(max_triangles))))
        spp = int(rng.choice([4, 16, 64]))
        medium = bool(rng.uniform() < 0.3)
        level, k = min(((lv, kk) for lv in range(1, 9) for kk in range(1, 5) if kk * 20 * 4 ** lv <= max_triangles),
                       key=lambda c: abs(np.log(c[1] * 20 * 4 ** c[0] / target)))
        theta = float(rng.uniform(-0.6, 0.6))
        sc = Scene(res, res,
                   camera={"phi": 1.1, "theta": theta, "radius": 6.0, "fov": 0.785398,
                           "target": [0.0, 0.6, 0.0]},
                   render={"spp": spp, "max_depth": max_depth, "rr_depth": rr_depth,
                           "adjoint": s % 2 == 1, "target_triangles": int(target)},
                   name=f"{name}{s:03d}")
        if level not in bases:
            bases[level] = icosphere(level)
        v, f = bases[level]
        for j in range(k):
            cx = (j - (k - 1) / 2.0) * 1.3
            radius = float(rng.uniform(0.45, 0.6))
            d = fbm(v * 2.0, 4, seed * 1000 + s * 8 + j)
            r = radius * (1.0 + 0.08 * d)
            pos = (v * r[:, None] + np.array([cx, radius + 0.05, 0.0])[None, :]).astype(F32)
            idx = f.astype(np.uint32)
            u = rng.uniform()
            bn = f"s{j}"
            if u < 0.6:
                sc.bsdfs.append(_lambert(bn, rng.uniform(0.2, 0.9, 3)))
            elif u < 0.8:
                sc.bsdfs.append({"name": bn, "type": "mirror",
                                 "albedo": {"type": "constant", "value": [0.95, 0.95, 0.95]}})
            else:
                sc.bsdfs.append({"name": bn, "type": "ideal_specular_dielectric",
                                 "albedo": {"type": "constant", "value": [0.98, 0.98, 0.98]}, "ior": 1.5})
            sc.materials.append({"name": bn, "bsdf": bn})
            sc.meshes.append(Mesh(bn, pos, vertex_normals(pos, idx), idx, bn))
        if medium:
            sc.media.append({"name": "fog", "type": "henyey_greenstein", "sigma_a": [0.05, 0.1, 0.2],
                             "sigma_s": [2.0, 1.5, 1.0], "g": 0.3})
            sc.bsdfs.append({"name": "water", "type": "ideal_specular_dielectric",
                             "albedo": {"type": "constant", "value": [1.0, 1.0, 1.0]}, "ior": 1.33})
            sc.materials.append({"name": "water", "bsdf": "water", "medium": "fog"})
            p, n, i = uv_sphere(0.6, 64, 32, center=(0.0, 0.6, 1.4))
            sc.meshes.append(Mesh("fog_ball", p, n, i, "water"))
        _ground_and_light(sc)
        scenes.append(sc)
    return scenes


def _translate(x, y, z):
    return [1.0, 0.0, 0.0, x, 0.0, 1.0, 0.0, y, 0.0, 0.0, 1.0, z, 0.0, 0.0, 0.0, 1.0]


def procedural_scene(width=64, height=64, spp=4, max_depth=8, rr_depth=3, name="procedural") -> Scene:
    """The reference's generated primitives (scene.cpp:408-426): a ``grid``
    floor (20 x 20, 11 x 11 vertices), a Lambert ``geosphere`` (radius 0.8,
    3 subdivisions) and a glass one (radius 0.6, 2 subdivisions) placed by
    transforms, under the LMF area light of the other scenes."""
    sc = Scene(width, height,
               camera={"phi": 1.1, "theta": 0.3, "radius": 6.0, "fov": 0.785398, "target": [0.0, 0.5, 0.0]},
               render={"spp": spp, "max_depth": max_depth, "rr_depth": rr_depth}, name=name)
    sc.bsdfs += [_lambert("floor", (0.6, 0.6, 0.55)), _lambert("red", (0.8, 0.25, 0.2)),
                 {"name": "glass", "type": "ideal_specular_dielectric",
                  "albedo": {"type": "constant", "value": [1.0, 1.0, 1.0]}, "ior": 1.5},
                 _lambert("light", (0.0, 0.0, 0.0))]
    for m in ("floor", "red", "glass", "light"):
        sc.materials.append({"name": m, "bsdf": m})
    sc.procedural += [
        {"name": "floor", "type": "grid", "width": 20.0, "depth": 20.0, "n": 11, "m": 11, "material": "floor"},
        {"name": "ball", "type": "geosphere", "radius": 0.8, "n": 3, "material": "red",
         "transform": _translate(-1.0, 0.8, 0.0)},
        {"name": "gem", "type": "geosphere", "radius": 0.6, "n": 2, "material": "glass",
         "transform": _translate(1.2, 0.6, 0.5)}]
    p, n, i = quad((0.0, 5.0, 0.0), 1.0, 1.0, -1.0)
    sc.meshes.append(Mesh("light", p, n, i, "light",
                          emission={"color": [1.0, 1.0, 1.0], "radiant_power": float(15.0 * np.pi * 4.0)}))
    return sc


def texture_images(directory: str):
    """Two seeded test images written as PNG into `directory`: a 37x23 RGB
    pattern and a 16x9 grey ramp. Returns their absolute paths."""
    from .image import write_png
    os.makedirs(directory, exist_ok=True)
    rng = np.random.default_rng(11)
    y, x = np.mgrid[0:23, 0:37]
    rgb = np.stack([(x * 7) % 256, (y * 11) % 256, rng.integers(0, 256, (23, 37))], axis=-1).astype(np.uint8)
    grey = np.tile((np.arange(16) * 16)[None, :], (9, 1)).astype(np.uint8)[:, :, None]
    paths = [os.path.abspath(os.path.join(directory, "tex_rgb.png")),
             os.path.abspath(os.path.join(directory, "tex_grey.png"))]
    write_png(paths[0], rgb)
    write_png(paths[1], grey)
    return paths


def textured_scene(image_dir: str, width=64, height=48, spp=4, max_depth=8, rr_depth=3,
                   name="textured") -> Scene:
    """Albedo textures (scene.cpp:266-318): a grid floor with the ``uv``
    texture (albedo = (u, v, 0)), two upright LMF quads with ``image``
    textures (an RGB and a grey PNG; texture coordinates inside [0.1, 0.9], the
    range where the reference's nearest lookup stays inside the image), and a
    constant-albedo geosphere, under the LMF area light."""
    rgb_png, grey_png = texture_images(image_dir)
    sc = Scene(width, height,
               camera={"phi": 1.2, "theta": 0.2, "radius": 6.5, "fov": 0.785398, "target": [0.0, 0.8, 0.0]},
               render={"spp": spp, "max_depth": max_depth, "rr_depth": rr_depth}, name=name)
    sc.bsdfs += [{"name": "uvfloor", "type": "lambert", "albedo": {"type": "uv"}},
                 {"name": "picture", "type": "lambert", "albedo": {"type": "image", "file_path": rgb_png}},
                 {"name": "ramp", "type": "mirror", "albedo": {"type": "image", "file_path": grey_png}},
                 _lambert("ball", (0.7, 0.7, 0.7)), _lambert("light", (0.0, 0.0, 0.0))]
    for m in ("uvfloor", "picture", "ramp", "ball", "light"):
        sc.materials.append({"name": m, "bsdf": m})
    sc.procedural += [
        {"name": "floor", "type": "grid", "width": 12.0, "depth": 12.0, "n": 5, "m": 4, "material": "uvfloor"},
        {"name": "ball", "type": "geosphere", "radius": 0.5, "n": 2, "material": "ball",
         "transform": _translate(0.0, 0.5, 1.0)}]
    for nm, mat, x0 in (("picture", "picture", -2.2), ("ramp", "ramp", 0.3)):
        p = np.array([[x0, 0.0, -1.0], [x0 + 1.9, 0.0, -1.0], [x0 + 1.9, 2.2, -1.0], [x0, 2.2, -1.0]], F32)
        n = np.tile(np.array([[0.0, 0.0, 1.0]], F32), (4, 1))
        t = np.array([[0.1, 0.1], [0.9, 0.1], [0.9, 0.9], [0.1, 0.9]], F32)
        i = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
        sc.meshes.append(Mesh(nm, p, n, i, mat, texcoords=t))
    p, n, i = quad((0.0, 5.0, 0.0), 1.0, 1.0, -1.0)
    sc.meshes.append(Mesh("light", p, n, i, "light",
                          emission={"color": [1.0, 1.0, 1.0], "radiant_power": float(15.0 * np.pi * 4.0)}))
    return sc


def tiny_scene(width=32, height=32, spp=4, max_depth=8, rr_depth=3, name="tiny") -> Scene:
    """Smallest scene with every reference material: three low-poly spheres
    (Lambert, mirror, dielectric) over the ground, under the light."""
    sc = Scene(width, height,
               camera={"phi": 1.1, "theta": 0.0, "radius": 6.0, "fov": 0.785398,
                       "target": [0.0, 0.5, 0.0]},
               render={"spp": spp, "max_depth": max_depth, "rr_depth": rr_depth},
               name=name)
    specs = [("red", _lambert("red", (0.8, 0.2, 0.2)), (-1.2, 0.5, 0.0)),
             ("mirror", {"name": "mirror", "type": "mirror",
                         "albedo": {"type": "constant", "value": [0.9, 0.9, 0.9]}}, (0.0, 0.5, 0.0)),
             ("glass", {"name": "glass", "type": "ideal_specular_dielectric",
                        "albedo": {"type": "constant", "value": [1.0, 1.0, 1.0]}, "ior": 1.5},
              (1.2, 0.5, 0.0))]
    for nm, b, c in specs:
        sc.bsdfs.append(b)
        sc.materials.append({"name": nm, "bsdf": nm})
        p, n, i = uv_sphere(0.5, 16, 8, center=c)
        sc.meshes.append(Mesh(nm, p, n, i, nm))
    _ground_and_light(sc)
    return sc


def unlit_scene(width=13, height=7, name="unlit") -> Scene:
    """tiny_scene without its emitter, under a (0.5, 0.6, 0.7) background:
    SampleOneLight returns black (integrator.cpp:255-261), so only the
    background reaches the film."""
    sc = tiny_scene(width=width, height=height, name=name)
    sc.meshes = [m for m in sc.meshes if m.emission is None]
    sc.background = (0.5, 0.6, 0.7)
    return sc


def two_light_scene(width=24, height=20, name="two_lights") -> Scene:
    """tiny_scene plus a second, smaller emitter (a 0.5 x 0.5 quad at
    (2.5, 3, 0), colour (1, 0.5, 0.25), radiant power 8 pi): the light choice's
    rejection loop and its x numLights weight (integrator.cpp:263-270) apply on
    paths that hit either light."""
    sc = tiny_scene(width=width, height=height, name=name)
    p, n, i = quad((2.5, 3.0, 0.0), 0.5, 0.5, -1.0)
    sc.bsdfs.append({"name": "light2", "type": "lambert", "albedo": {"type": "constant", "value": [0.0, 0.0, 0.0]}})
    sc.materials.append({"name": "light2", "bsdf": "light2"})
    sc.meshes.append(Mesh("light2", p, n, i, "light2",
                          emission={"color": [1.0, 0.5, 0.25], "radiant_power": float(8.0 * np.pi)}))
    return sc


def random_rays(n: int, lo: np.ndarray, hi: np.ndarray, seed: int = 2) -> np.ndarray:
    """(n, 8) float32 ray records (org.xyz, tnear, dir.xyz, tfar): origins uniform
    in the box [lo, hi], directions uniform on the sphere, tnear 0, tfar inf."""
    rng = np.random.default_rng(seed)
    r = np.empty((n, 8), dtype=F32)
    r[:, 0:3] = rng.uniform(lo, hi, size=(n, 3)).astype(F32)
    r[:, 3] = 0.0
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r[:, 4:7] = d.astype(F32)
    r[:, 7] = np.inf
    return r


def ensure_written(scene: Scene, directory: str) -> str:
    """Write the scene unless an identical JSON is already on disk."""
    path = os.path.join(directory, f"{scene.name}.json")
    if os.path.exists(path):
        names = {m.name: f"{scene.name}_{m.name}.lmf" for m in scene.meshes}
        try:
            with open(path) as fh:
                if json.load(fh) == json.loads(json.dumps(scene.to_json_dict(names))) and all(
                        os.path.exists(os.path.join(directory, v)) for v in names.values()):
                    return path
        except (OSError, ValueError):
            pass
    return scene.write(directory)
