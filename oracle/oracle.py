"""ctypes front end for the CPU oracle and for the compiled reference integrator.

TEST INFRASTRUCTURE ONLY. Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline / reference legs import this module; the product
(lantern_gb300) never does.

* ``liboracle.so`` -- oracle/lt_oracle.c, the project's C restatement of the
  reference's per-pixel loop (built by :func:`build_oracle`).
* ``liblantern_ref.so`` -- the reference's own integrator built by
  oracle/build_ref.sh (present where the reference tree was staged).

:func:`load_scene` reads a Lantern scene JSON and its LMF files the way
``Scene::ParseJSON`` / ``AddLMF`` do (source/core/scene/scene.cpp:215-446,
502-582; io/lantern_model_file.cpp:33-65) and hands it to the oracle.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import struct
import subprocess
import threading
from contextlib import contextmanager
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD, "liboracle.so")
REF_SO = os.path.join(REF_DIR, "liblantern_ref.so")
# The reference tree: LANTERN_REFERENCE, else a checkout named "reference" next
# to this repository.
REF_TREE = os.environ.get("LANTERN_REFERENCE") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))

BSDF = {"lambert": 0, "mirror": 1, "ideal_specular_dielectric": 2}
MED_NON_SCATTERING, MED_ISOTROPIC, MED_HG = 1, 2, 3
KEY_TILE, KEY_PIXEL = 0, 1

_lock = threading.Lock()
_lib = None
_ref = None


def build_oracle(force: bool = False) -> str:
    """Compile oracle/lt_oracle.c (C) and oracle/lt_diff_ref.cpp (C++) into
    oracle/_build/liboracle.so."""
    src = os.path.join(HERE, "lt_oracle.c")
    cpp = os.path.join(HERE, "lt_diff_ref.cpp")
    hdr = os.path.join(HERE, "lt_oracle.h")
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(ORACLE_SO)
            and os.path.getmtime(ORACLE_SO) >= max(os.path.getmtime(f) for f in (src, cpp, hdr))):
        return ORACLE_SO
    pid = os.getpid()
    obj_c, obj_cpp = os.path.join(BUILD, f"lt_oracle.{pid}.o"), os.path.join(BUILD, f"lt_diff_ref.{pid}.o")
    flags = ["-O2", "-ffp-contract=off", "-fPIC"]
    subprocess.check_call(["gcc", "-std=c11"] + flags + ["-c", src, "-o", obj_c])
    subprocess.check_call(["g++", "-std=c++17"] + flags + ["-c", cpp, "-o", obj_cpp])
    tmp = ORACLE_SO + f".{pid}.tmp"
    subprocess.check_call(["g++", "-shared", "-o", tmp, obj_c, obj_cpp, "-lm", "-lpthread"])
    os.replace(tmp, ORACLE_SO)
    for o in (obj_c, obj_cpp):
        os.remove(o)
    return ORACLE_SO


def build_reference() -> Optional[str]:
    """Run oracle/build_ref.sh (stages from the reference tree when present,
    else compiles already-staged sources). Returns the library path or None."""
    if not (os.path.isdir(os.path.join(REF_TREE, "source")) or os.path.isdir(os.path.join(REF_DIR, "src"))):
        return None
    r = subprocess.run(["bash", os.path.join(HERE, "build_ref.sh")], capture_output=True, text=True,
                       env=dict(os.environ, LANTERN_REFERENCE=REF_TREE))
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout[-2000:] + r.stderr[-4000:])
    return REF_SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            L = C.CDLL(build_oracle())
            p, u32, u64, f32, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_int
            fp = C.POINTER(C.c_float)
            up = C.POINTER(C.c_uint32)
            L.orc_scene_new.restype = p
            L.orc_scene_free.argtypes = [p]
            L.orc_set_camera.argtypes = [p, f32, f32, f32, u32, u32, fp, f32]
            L.orc_set_background.argtypes = [p, fp]
            L.orc_add_medium.argtypes = [p, i32, fp, fp, f32]
            L.orc_add_medium.restype = i32
            L.orc_add_medium_ref.argtypes = [p, i32, fp, f32, f32]
            L.orc_add_medium_ref.restype = i32
            L.orc_add_material.argtypes = [p, i32, fp, f32, i32]
            L.orc_add_material.restype = i32
            L.orc_add_mesh.argtypes = [p, fp, u32, fp, up, u32, i32, fp, f32]
            L.orc_add_mesh.restype = i32
            L.orc_scene_commit.argtypes = [p]
            L.orc_light_info.argtypes = [p, i32, fp, fp, fp]
            L.orc_num_triangles.argtypes = [p]
            L.orc_num_triangles.restype = u32
            L.orc_num_lights.argtypes = [p]
            L.orc_num_lights.restype = i32
            L.orc_intersect.argtypes = [p, fp, up, u64, i32, up, i32]
            L.orc_render.argtypes = [p, p, u32, u32, fp, up, up, fp, up, up, C.POINTER(C.c_uint64)]
            L.orc_render_path.argtypes = [p, p, u32, u32, u32, fp, up]
            L.orc_pcg_stream.argtypes = [u64, u64, u32, up, fp]
            L.orc_tile_seed.argtypes = [u32, u32]
            L.orc_tile_seed.restype = u32
            L.orc_filter_sample.argtypes = [f32]
            L.orc_filter_sample.restype = f32
            L.orc_camera_ray.argtypes = [p, u32, u32, f32, f32, fp, fp]
            dp = C.POINTER(C.c_double)
            L.orc_diff_render.argtypes = [p, C.c_int, fp, fp, fp, fp, u32, u32, u32, u32, up, fp, dp, dp, dp, dp, dp,
                                          C.c_int]
            L.orc_resolve.argtypes = [fp, up, u64, C.c_int, f32, fp, C.POINTER(C.c_uint8), up,
                                      C.POINTER(C.c_uint64)]
            L.orc_add_image.argtypes = [p, C.POINTER(C.c_uint8), u32, u32, u32]
            L.orc_add_image.restype = i32
            L.orc_set_material_texture.argtypes = [p, i32, i32]
            L.orc_set_mesh_texcoords.argtypes = [p, i32, fp]
            _lib = L
    return _lib


def ref_lib():
    """The compiled reference integrator, or None when it is not built."""
    global _ref
    with _lock:
        if _ref is None and os.path.exists(REF_SO):
            L = C.CDLL(REF_SO)
            p, u32 = C.c_void_p, C.c_uint32
            fp = C.POINTER(C.c_float)
            up = C.POINTER(C.c_uint32)
            L.lref_scene_load.argtypes = [C.c_char_p]
            L.lref_scene_load.restype = p
            L.lref_scene_free.argtypes = [p]
            L.lref_scene_size.argtypes = [p, up, up]
            L.lref_render.argtypes = [p, u32, u32, u32, u32, fp, up, up, fp, up, up,
                                      C.POINTER(C.c_ulonglong)]
            L.lref_render.restype = C.c_double
            L.lref_pcg_stream.argtypes = [C.c_ulonglong, C.c_ulonglong, u32, up, fp]
            L.lref_filter_sample.argtypes = [fp, u32, fp]
            L.lref_camera_ray.argtypes = [p, u32, u32, C.c_ulonglong, C.c_ulonglong, fp]
            L.lref_image_load.argtypes = [C.c_char_p, C.POINTER(C.c_uint8), C.c_size_t, C.POINTER(C.c_int),
                                          C.POINTER(C.c_int), C.POINTER(C.c_int)]
            _ref = L
    return _ref


def fptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_float)) if a is not None else None


def uptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_uint32)) if a is not None else None


# ------------------------------------------------------------------ scene files
def read_lmf(path: str) -> dict:
    """ReadLMF (io/lantern_model_file.cpp:33-65)."""
    with open(path, "rb") as fh:
        data = fh.read()
    if data[:4] != b"LMF\x00":
        raise ValueError(f"{path}: bad LMF magic")
    vpp = data[4]
    flags = struct.unpack_from("<I", data, 5)[0]
    off = 9
    nv = struct.unpack_from("<Q", data, off)[0]
    off += 8
    pos = np.frombuffer(data, "<f4", nv * 3, off).reshape(-1, 3)
    off += nv * 12
    ni = struct.unpack_from("<Q", data, off)[0]
    off += 8
    idx = np.frombuffer(data, "<u4", ni, off)
    off += ni * 4
    nrm = tex = None
    if flags & 1:
        nn = struct.unpack_from("<Q", data, off)[0]
        off += 8
        nrm = np.frombuffer(data, "<f4", nn, off).reshape(-1, 3)
        off += nn * 4
    if flags & 2:
        nt = struct.unpack_from("<Q", data, off)[0]
        off += 8
        tex = np.frombuffer(data, "<f4", nt, off).reshape(-1, 2)
    return {"vpp": vpp, "positions": pos, "indices": idx, "normals": nrm, "texcoords": tex}


def apply_transform(pos: np.ndarray, t: list) -> np.ndarray:
    """``transform * float3a(p, 1)`` (scene.cpp:517-522, linearspace4.h:43-47,165):
    row r = ((x*m[r][0] + y*m[r][1]) + z*m[r][2]) + 1*m[r][3] in float32."""
    m = np.asarray(t, dtype=np.float32).reshape(4, 4)
    x, y, z = pos[:, 0], pos[:, 1], pos[:, 2]
    one = np.float32(1.0)
    out = np.empty_like(pos, dtype=np.float32)
    for r in range(3):
        out[:, r] = ((x * m[r, 0] + y * m[r, 1]) + z * m[r, 2]) + one * m[r, 3]
    return out


def grid_mesh(width: float, depth: float, m: int, n: int):
    """CreateGrid (geometry_generator.cpp:515-566) in float32: m rows of n
    vertices, row i at z = -(depth/2 - i*dz), normals +y, two triangles per cell."""
    f32 = np.float32
    half_w, half_d = f32(0.5) * f32(width), f32(0.5) * f32(depth)
    dx, dz = f32(width) / f32(n - 1), f32(depth) / f32(m - 1)
    z = half_d - np.arange(m, dtype=f32) * dz
    x = -half_w + np.arange(n, dtype=f32) * dx
    pos = np.zeros((m, n, 3), f32)
    pos[:, :, 0] = x[None, :]
    pos[:, :, 2] = -z[:, None]
    nrm = np.zeros((m * n, 3), f32)
    nrm[:, 1] = 1.0
    i, j = np.meshgrid(np.arange(m - 1, dtype=np.uint32), np.arange(n - 1, dtype=np.uint32), indexing="ij")
    a = (i * n + j).reshape(-1)
    b = ((i + 1) * n + j).reshape(-1)
    idx = np.stack([a, a + 1, b, b, a + 1, b + 1], axis=1).reshape(-1).astype(np.uint32)
    du, dv = f32(1) / f32(n - 1), f32(1) / f32(m - 1)
    tex = np.zeros((m, n, 2), f32)
    tex[:, :, 0] = (np.arange(n, dtype=f32) * du)[None, :]
    tex[:, :, 1] = (np.arange(m, dtype=f32) * dv)[:, None]
    return pos.reshape(-1, 3), nrm, idx, tex.reshape(-1, 2)


def geosphere_mesh(radius: float, subdivisions: int):
    """CreateGeosphere with Subdivide (geometry_generator.cpp:214-356) in
    float32: icosahedron, each subdivision four triangles per triangle with six
    fresh vertices, then n = v * (1 / sqrt(dot(v, v))), position = radius * n."""
    f32 = np.float32
    X, Z = f32(0.525731), f32(0.850651)
    pos = np.array([[-X, 0, -Z], [X, 0, -Z], [-X, 0, Z], [X, 0, Z], [0, Z, -X], [0, Z, X], [0, -Z, -X],
                    [0, -Z, X], [Z, X, 0], [-Z, X, 0], [Z, -X, 0], [-Z, -X, 0]], dtype=f32)
    tri = np.array([1, 4, 0, 4, 9, 0, 4, 5, 9, 8, 5, 4, 1, 8, 4, 1, 10, 8, 10, 3, 8, 8, 3, 5, 3, 2, 5, 3, 7, 2,
                    3, 10, 7, 10, 6, 7, 6, 11, 7, 6, 0, 11, 6, 1, 0, 10, 1, 6, 11, 0, 9, 2, 11, 9, 5, 2, 9, 11,
                    2, 7], dtype=np.uint32).reshape(-1, 3)
    half = f32(0.5)
    for _ in range(subdivisions):
        v0, v1, v2 = pos[tri[:, 0]], pos[tri[:, 1]], pos[tri[:, 2]]
        m0, m1, m2 = half * (v0 + v1), half * (v1 + v2), half * (v0 + v2)
        pos = np.stack([v0, v1, v2, m0, m1, m2], axis=1).reshape(-1, 3)
        b = (6 * np.arange(tri.shape[0], dtype=np.uint32))[:, None]
        tri = (b + np.array([0, 3, 5, 3, 4, 5, 5, 4, 2, 3, 1, 4], dtype=np.uint32)[None, :]).reshape(-1, 3)
    d = (pos[:, 0] * pos[:, 0] + pos[:, 1] * pos[:, 1]) + pos[:, 2] * pos[:, 2]
    inv = f32(1) / np.sqrt(d)
    nrm = (pos * inv[:, None]).astype(f32)
    return (f32(radius) * nrm).astype(f32), nrm, tri.reshape(-1).astype(np.uint32), None


class OracleScene:
    """A scene loaded into the oracle."""

    def __init__(self, json_path: str):
        L = lib()
        self.path = os.path.abspath(json_path)
        with open(self.path) as fh:
            j = json.load(fh)
        self.json = j
        self.h = L.orc_scene_new()
        f32 = np.float32
        cam = j["camera"]
        self.width = int(cam["client_width"])
        self.height = int(cam["client_height"])
        tgt = np.array(cam.get("target", [0, 0, 0]), dtype=f32)
        L.orc_set_camera(self.h, f32(cam.get("phi", np.pi / 4)), f32(cam.get("theta", 0.0)),
                         f32(cam.get("radius", 10.0)), self.width, self.height, fptr(tgt),
                         f32(cam.get("fov", np.pi / 4)))
        bg = np.array(j.get("background_color", [0, 0, 0]), dtype=f32)
        L.orc_set_background(self.h, fptr(bg))
        media = {}
        for m in j.get("media", []):
            t = m["type"]
            if t == "henyey_greenstein":
                sa = np.array(m["sigma_a"], dtype=f32)
                ss = np.array(m["sigma_s"], dtype=f32)
                media[m["name"]] = L.orc_add_medium(self.h, MED_HG, fptr(sa), fptr(ss), f32(m.get("g", 0.0)))
            else:
                col = np.array(m["absorption_color"], dtype=f32)
                typ = MED_ISOTROPIC if t == "isotropic_scattering" else MED_NON_SCATTERING
                media[m["name"]] = L.orc_add_medium_ref(
                    self.h, typ, fptr(col), f32(m["absorption_at_distance"]),
                    f32(m.get("scattering_distance", 1.0)))
        bsdfs = {b["name"]: b for b in j.get("bsdfs", [])}
        mats, images = {}, {}
        base = os.path.dirname(self.path)
        for m in j.get("materials", []):
            b = bsdfs[m["bsdf"]]
            alb = np.array(b["albedo"].get("value", [0, 0, 0]), dtype=f32)
            mi = L.orc_add_material(self.h, BSDF[b["type"]], fptr(alb), f32(b.get("ior", 1.0)),
                                    media.get(m.get("medium"), -1))
            kind = b["albedo"]["type"]
            if kind == "uv":
                L.orc_set_material_texture(self.h, mi, -2)
            elif kind == "image":
                ip = b["albedo"]["file_path"]
                if not os.path.isabs(ip) and not os.path.exists(ip):
                    ip = os.path.join(base, ip)
                if ip not in images:
                    tex = read_png(ip)
                    images[ip] = L.orc_add_image(self.h, tex.ctypes.data_as(C.POINTER(C.c_uint8)), tex.shape[1],
                                                 tex.shape[0], tex.shape[2])
                L.orc_set_material_texture(self.h, mi, images[ip])
            mats[m["name"]] = mi
        self._keep = []
        for p in j.get("primitives", []):
            if p["type"] == "lmf":
                lmf = read_lmf(os.path.join(base, p["file_path"]))
                if lmf["vpp"] != 3:
                    raise NotImplementedError("triangle LMF only")
                pos, nrm, idx, tc = lmf["positions"], lmf["normals"], lmf["indices"], lmf["texcoords"]
            elif p["type"] == "grid":
                pos, nrm, idx, tc = grid_mesh(p["width"], p["depth"], int(p["m"]), int(p["n"]))
            elif p["type"] == "geosphere":
                pos, nrm, idx, tc = geosphere_mesh(p["radius"], int(p["n"]))
            else:
                raise NotImplementedError(f"primitive type {p['type']}")
            pos = np.ascontiguousarray(pos, dtype=f32)
            if "transform" in p:
                pos = apply_transform(pos, p["transform"])  # normals stay as generated (scene.cpp:481-482)
            nrm = None if nrm is None else np.ascontiguousarray(nrm, dtype=f32)
            idx = np.ascontiguousarray(idx, dtype=np.uint32)
            em = None
            power = f32(0)
            if "emission" in p:
                em = np.array(p["emission"]["color"], dtype=f32)
                power = f32(p["emission"]["radiant_power"])
            self._keep += [pos, nrm, idx, em]
            gid = L.orc_add_mesh(self.h, fptr(pos), pos.shape[0], fptr(nrm), uptr(idx), idx.size // 3,
                                 mats[p["material"]], fptr(em), power)
            if tc is not None and np.asarray(tc).size == 2 * pos.shape[0]:
                tc = np.ascontiguousarray(tc, dtype=f32).reshape(-1)
                L.orc_set_mesh_texcoords(self.h, gid, fptr(tc))
        L.orc_scene_commit(self.h)
        self._keep = []

    def __del__(self):
        try:
            lib().orc_scene_free(self.h)
        except Exception:
            pass

    @property
    def num_triangles(self) -> int:
        return int(lib().orc_num_triangles(self.h))

    def intersect(self, rays: np.ndarray, use_bvh: bool = True, counters: bool = False,
                  threads: int = 0):
        rays = np.ascontiguousarray(rays, dtype=np.float32)
        n = rays.shape[0]
        hits = np.zeros((n, 4), dtype=np.uint32)
        cnt = np.zeros((n, 2), dtype=np.uint32) if counters else None
        lib().orc_intersect(self.h, fptr(rays), uptr(hits), n, int(use_bvh), uptr(cnt),
                            threads or os.cpu_count())
        return (hits, cnt) if counters else hits

    def diff_defaults(self):
        """The scene's own (albedo, emission, sigma_a, sigma_s) as parameter arrays."""
        L = lib()
        L.orc_tri_geom.restype = C.c_uint32
        L.orc_tri_geom.argtypes = [C.c_void_p, C.c_uint32]
        L.orc_geom_info.argtypes = [C.c_void_p, C.c_uint32] + [C.POINTER(C.c_int)] * 3
        L.orc_material_info.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), C.POINTER(C.c_int)]
        L.orc_medium_info.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_float),
                                      C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.orc_num_media.argtypes = [C.c_void_p]
        T = self.num_triangles
        albedo, emission = np.zeros((T, 3), np.float32), np.zeros((T, 3), np.float32)
        geoms = {}
        for t in range(T):
            g = L.orc_tri_geom(self.h, t)
            if g not in geoms:
                mat, light, hn = C.c_int(), C.c_int(), C.c_int()
                L.orc_geom_info(self.h, g, C.byref(mat), C.byref(light), C.byref(hn))
                b, ior, med = C.c_int(), C.c_float(), C.c_int()
                alb = (C.c_float * 3)()
                L.orc_material_info(self.h, mat.value, C.byref(b), alb, C.byref(ior), C.byref(med))
                rad = np.zeros(3, np.float32)
                if light.value >= 0:
                    area, sph = C.c_float(), (C.c_float * 4)()
                    r3 = (C.c_float * 3)()
                    L.orc_light_info(self.h, light.value, C.byref(area), sph, r3)
                    rad = np.array(list(r3), np.float32)
                geoms[g] = (np.array(list(alb), np.float32), rad)
            albedo[t], emission[t] = geoms[g]
        M = max(L.orc_num_media(self.h), 1)
        sa, ss = np.zeros((M, 3), np.float32), np.zeros((M, 3), np.float32)
        for m in range(L.orc_num_media(self.h)):
            ty, g = C.c_int(), C.c_float()
            a3, s3 = (C.c_float * 3)(), (C.c_float * 3)()
            L.orc_medium_info(self.h, m, C.byref(ty), a3, s3, C.byref(g))
            sa[m], ss[m] = list(a3), list(s3)
        return albedo, emission, sa, ss

    def lights(self):
        """Per area light, in mesh order: (area, bounding sphere (4), radiance (3))
        as float32 arrays, computed the way AddLMF and AreaLight's constructor
        do (scene.cpp:49-80, 527-534; area_light.h:16-21)."""
        L = lib()
        out = []
        for i in range(L.orc_num_lights(self.h)):
            area, sph, r3 = C.c_float(), (C.c_float * 4)(), (C.c_float * 3)()
            L.orc_light_info(self.h, i, C.byref(area), sph, r3)
            out.append((np.float32(area.value), np.array(list(sph), np.float32), np.array(list(r3), np.float32)))
        return out

    def diff_render(self, albedo, emission, sigma_a, sigma_s, spp: int, max_depth: int = 8, rr_depth: int = 3,
                    first_frame: int = 0, crop=None, dI=None, fp64: bool = True, threads: int = 0):
        """Differentiable estimator and its gradient on the host (lt_diff_ref.cpp):
        returns (film colour sums float64 (H, W, 3), dict of float64 gradients)."""
        f = lambda a: np.ascontiguousarray(a, dtype=np.float32)  # noqa: E731
        albedo, emission, sigma_a, sigma_s = f(albedo), f(emission), f(sigma_a), f(sigma_s)
        if crop is None:
            crop = (0, 0, self.width, self.height)
        crop_a = np.asarray(crop, dtype=np.uint32)
        rgb = np.zeros((self.height, self.width, 3), np.float64)
        g = {k: np.zeros(v.shape, np.float64) for k, v in
             (("albedo", albedo), ("emission", emission), ("sigma_a", sigma_a), ("sigma_s", sigma_s))}
        dptr = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
        dI_a = None if dI is None else f(dI)
        lib().orc_diff_render(self.h, int(fp64), fptr(albedo), fptr(emission), fptr(sigma_a), fptr(sigma_s), spp,
                              first_frame, max_depth, rr_depth, uptr(crop_a), fptr(dI_a), dptr(rgb),
                              dptr(g["albedo"]), dptr(g["emission"]), dptr(g["sigma_a"]), dptr(g["sigma_s"]),
                              threads or os.cpu_count())
        return rgb, g

    def render(self, frames: int, first_frame: int = 0, max_depth: int = 1500, rr_depth: int = 3,
               keying: int = KEY_PIXEL, threads: int = 0, two_films: bool = False):
        class Opts(C.Structure):
            _fields_ = [("max_depth", C.c_uint32), ("rr_depth", C.c_uint32),
                        ("keying", C.c_uint32), ("threads", C.c_uint32)]
        o = Opts(max_depth, rr_depth, keying, threads or os.cpu_count())
        n = self.width * self.height
        rgb_a = np.zeros((self.height, self.width, 3), np.float32)
        b_a = np.zeros((self.height, self.width), np.uint32)
        c_a = np.zeros_like(b_a)
        rgb_b = b_b = c_b = None
        if two_films:
            rgb_b, b_b, c_b = np.zeros_like(rgb_a), np.zeros_like(b_a), np.zeros_like(c_a)
        rc = (C.c_uint64 * 3)()
        lib().orc_render(self.h, C.byref(o), first_frame, frames, fptr(rgb_a), uptr(b_a), uptr(c_a),
                         fptr(rgb_b), uptr(b_b), uptr(c_b), rc)
        del n
        out = {"rgb": rgb_a, "bounces": b_a, "counts": c_a, "rays": [int(x) for x in rc]}
        if two_films:
            out.update({"rgb_b": rgb_b, "bounces_b": b_b, "counts_b": c_b})
        return out


@contextmanager
def _cwd(path):
    old = os.getcwd()
    os.chdir(path)
    try:
        yield
    finally:
        os.chdir(old)


class ReferenceScene:
    """A scene loaded by the reference's own Scene::LoadSceneFromJSON."""

    def __init__(self, json_path: str):
        L = ref_lib()
        if L is None:
            raise RuntimeError("reference library not built (oracle/build_ref.sh)")
        path = os.path.abspath(json_path)
        # the reference looks for scene.schema.json in the working directory
        with _cwd(REF_DIR):
            self.h = L.lref_scene_load(path.encode())
        if not self.h:
            raise RuntimeError(f"reference failed to load {json_path}")
        w, h = C.c_uint32(), C.c_uint32()
        L.lref_scene_size(self.h, C.byref(w), C.byref(h))
        self.width, self.height = w.value, h.value

    def __del__(self):
        try:
            ref_lib().lref_scene_free(self.h)
        except Exception:
            pass

    def render(self, frames: int, first_frame: int = 0, max_depth: int = 1500, rr_depth: int = 3):
        """Returns films A and B and wall seconds; frame 0 lands in B."""
        shp = (self.height, self.width)
        rgb_a, rgb_b = np.zeros(shp + (3,), np.float32), np.zeros(shp + (3,), np.float32)
        b_a, b_b = np.zeros(shp, np.uint32), np.zeros(shp, np.uint32)
        c_a, c_b = np.zeros(shp, np.uint32), np.zeros(shp, np.uint32)
        rays = C.c_ulonglong()
        secs = ref_lib().lref_render(self.h, first_frame, frames, max_depth, rr_depth, fptr(rgb_a),
                                     uptr(b_a), uptr(c_a), fptr(rgb_b), uptr(b_b), uptr(c_b),
                                     C.byref(rays))
        return {"rgb": rgb_a, "bounces": b_a, "counts": c_a, "rgb_b": rgb_b, "bounces_b": b_b,
                "counts_b": c_b, "seconds": secs, "rays": rays.value}


def resolve(rgb, counts, tonemap: int, exposure_stops: float):
    """orc_resolve on (H, W, 3) float32 colour sums and (H, W) counts:
    returns (rgba float32 (H, W, 4), rgba8 uint8 (H, W, 4), (min, max, sum) spp)."""
    rgb = np.ascontiguousarray(rgb, dtype=np.float32)
    counts = np.ascontiguousarray(counts, dtype=np.uint32)
    h, w = counts.shape
    out = np.empty((h, w, 4), np.float32)
    out8 = np.empty((h, w, 4), np.uint8)
    mm = np.zeros(2, np.uint32)
    sm = C.c_uint64(0)
    L = lib()
    L.orc_resolve(fptr(rgb), uptr(counts), h * w, tonemap, C.c_float(exposure_stops), fptr(out),
                  out8.ctypes.data_as(C.POINTER(C.c_uint8)), uptr(mm), C.byref(sm))
    return out, out8, (int(mm[0]), int(mm[1]), int(sm.value))


def read_png(path: str) -> np.ndarray:
    """A PNG file as stbi_load(path, &w, &h, &n, 0) returns it (the reference's
    image cache, image_cache.cpp:23-31): (h, w, n) uint8; grey 1, grey+alpha 2,
    RGB 3, RGBA 4 channels; palette -> RGB (RGBA with tRNS); a tRNS key on
    grey/RGB adds alpha; 1/2/4-bit grey scaled to 0..255; 16-bit keeps the high
    byte. Not interlaced."""
    import zlib
    data = open(path, "rb").read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError(f"{path}: not a PNG file")
    pos, idat, plte, trns = 8, b"", b"", b""
    w = h = depth = ctype = interlace = 0
    while pos + 12 <= len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body[:13])
        elif tag == b"PLTE":
            plte = body
        elif tag == b"tRNS":
            trns = body
        elif tag == b"IDAT":
            idat += body
        elif tag == b"IEND":
            break
        pos += 12 + n
    if interlace:
        raise ValueError("interlaced PNG files are not supported")
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    stride = (w * chans * depth + 7) // 8
    bpp = max(1, (chans * depth + 7) // 8)
    raw = np.frombuffer(zlib.decompress(idat), np.uint8)[:h * (stride + 1)].reshape(h, stride + 1)
    img = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f, src = raw[y, 0], raw[y, 1:].astype(np.int32)
        row = np.zeros(stride, np.int32)
        for i in range(stride):
            a = row[i - bpp] if i >= bpp else 0
            b = prev[i]
            c = prev[i - bpp] if i >= bpp else 0
            if f == 0:
                pr = 0
            elif f == 1:
                pr = a
            elif f == 2:
                pr = b
            elif f == 3:
                pr = (a + b) >> 1
            else:
                p_ = a + b - c
                pa, pb, pc = abs(p_ - a), abs(p_ - b), abs(p_ - c)
                pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            row[i] = (src[i] + pr) & 255
        img[y] = row
        prev = row
    img = img.astype(np.uint32)
    if depth == 16:
        samples = (img[:, 0::2] << 8) | img[:, 1::2]
    elif depth == 8:
        samples = img
    else:
        per = 8 // depth
        bits = np.zeros((h, stride * per), np.uint32)
        for k in range(per):
            bits[:, k::per] = (img >> (8 - depth * (k + 1))) & ((1 << depth) - 1)
        samples = bits
    samples = samples[:, :w * chans].reshape(h, w, chans)
    if ctype == 3:
        pal = np.frombuffer(plte, np.uint8).reshape(-1, 3)
        idx = samples[:, :, 0]
        out = pal[np.minimum(idx, len(pal) - 1)]
        if trns:
            t = np.frombuffer(trns, np.uint8)
            alpha = np.where(idx < len(t), t[np.minimum(idx, len(t) - 1)], 255).astype(np.uint8)
            out = np.concatenate([out, alpha[:, :, None]], axis=2)
        return np.ascontiguousarray(out)
    if depth == 16:
        out = (samples >> 8).astype(np.uint8)
    elif depth == 8:
        out = samples.astype(np.uint8)
    else:
        out = (samples * (255 // ((1 << depth) - 1))).astype(np.uint8)
    if trns and ctype in (0, 2):
        key = [(trns[2 * c] << 8) | trns[2 * c + 1] for c in range(chans)]
        if depth <= 8:
            key = [k & 255 for k in key]
        keyed = np.all(samples == np.array(key, np.uint32)[None, None, :], axis=2)
        out = np.concatenate([out, np.where(keyed, 0, 255).astype(np.uint8)[:, :, None]], axis=2)
    return np.ascontiguousarray(out)


def reference_image_load(path: str):
    """The reference's stb_image decode of `path` ((h, w, n) uint8), or None
    when the reference build is absent."""
    L = ref_lib()
    if L is None:
        return None
    w, h, n = C.c_int(), C.c_int(), C.c_int()
    if L.lref_image_load(path.encode(), None, 0, C.byref(w), C.byref(h), C.byref(n)) != 0:
        raise ValueError(f"stb_image could not load {path}")
    out = np.empty((h.value, w.value, n.value), np.uint8)
    L.lref_image_load(path.encode(), out.ctypes.data_as(C.POINTER(C.c_uint8)), out.nbytes, C.byref(w), C.byref(h),
                      C.byref(n))
    return out
