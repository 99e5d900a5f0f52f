"""ctypes binding of liblantern_gpu.so (include/lantern_gpu.h).

The library is built in-tree by :mod:`lantern_gb300.build`. There is no CPU
fallback: :func:`load` raises when the library cannot be built or loaded, and
every C-ABI error is raised as :class:`LanternError` with the library's message.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

LT_OK = 0
STATUS = {0: "LT_OK", 1: "LT_ERR_INVALID", 2: "LT_ERR_CUDA", 3: "LT_ERR_OOM", 4: "LT_ERR_TIMEOUT",
          5: "LT_ERR_IO", 6: "LT_ERR_PARSE", 7: "LT_ERR_UNSUPPORTED", 8: "LT_ERR_STATE",
          9: "LT_ERR_CHECK"}
BSDF_LAMBERT, BSDF_MIRROR, BSDF_DIELECTRIC = 0, 1, 2
MEDIUM_NON_SCATTERING, MEDIUM_ISOTROPIC, MEDIUM_HG = 1, 2, 3
MISS = 0xFFFFFFFF

# exported symbols (include/lantern_gpu.h)
SYMBOLS = ["lt_abi_version", "lt_ctx_create", "lt_ctx_destroy", "lt_last_error", "lt_set_stream", "lt_get_stream",
           "lt_sync", "lt_trim",
           "lt_scene_create", "lt_scene_destroy", "lt_scene_load_json", "lt_scene_info_get", "lt_scene_mesh_offsets", "lt_scene_lights_get", "lt_render",
           "lt_render_stats_get", "lt_intersect", "lt_render_noalloc", "lt_set_bvh_builder", "lt_get_tuning",
           "lt_set_tuning", "lt_set_stage_timing", "lt_render_batch", "lt_autotune_batch", "lt_resolve",
           "lt_render_diff_batch", "lt_render_adjoint_batch", "lt_image_load",
           "lt_debug_fail_allocations", "lt_debug_set_iteration_limit", "lt_debug_set_check_pixel_limit", "lt_set_queue_trace", "lt_queue_trace_get"]
BVH_GPU, BVH_HOST = 0, 1
NOALLOC_MAX_PATHS = 65536  # LT_NOALLOC_MAX_PATHS
MAX_BATCH = 2048  # LT_MAX_BATCH
ABI_VERSION = 3  # LT_ABI_VERSION
TONEMAP_CLAMP, TONEMAP_FILMIC = 0, 1


class LanternError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


ALBEDO_CONSTANT, ALBEDO_UV, ALBEDO_IMAGE = 0, 1, 2


class MaterialDesc(C.Structure):
    _fields_ = [("bsdf", C.c_int32), ("albedo", C.c_float * 3), ("ior", C.c_float), ("medium", C.c_int32),
                ("albedo_kind", C.c_int32), ("image", C.c_uint32)]


class ImageDesc(C.Structure):
    _fields_ = [("texels", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("channels", C.c_uint32)]


class MediumDesc(C.Structure):
    _fields_ = [("type", C.c_int32), ("sigma_a", C.c_float * 3), ("sigma_s", C.c_float * 3), ("g", C.c_float)]


class MeshDesc(C.Structure):
    _fields_ = [("positions", C.POINTER(C.c_float)), ("normals", C.POINTER(C.c_float)),
                ("indices", C.POINTER(C.c_uint32)), ("num_vertices", C.c_uint32),
                ("num_triangles", C.c_uint32), ("material", C.c_int32), ("emissive", C.c_int32),
                ("emission_color", C.c_float * 3), ("radiant_power", C.c_float),
                ("texcoords", C.POINTER(C.c_float)), ("transform", C.POINTER(C.c_float))]


class CameraDesc(C.Structure):
    _fields_ = [("phi", C.c_float), ("theta", C.c_float), ("radius", C.c_float), ("fov", C.c_float),
                ("target", C.c_float * 3), ("width", C.c_uint32), ("height", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("camera", CameraDesc), ("background", C.c_float * 3),
                ("materials", C.POINTER(MaterialDesc)), ("num_materials", C.c_uint32),
                ("media", C.POINTER(MediumDesc)), ("num_media", C.c_uint32),
                ("meshes", C.POINTER(MeshDesc)), ("num_meshes", C.c_uint32),
                ("images", C.POINTER(ImageDesc)), ("num_images", C.c_uint32)]


class LightInfo(C.Structure):
    _fields_ = [("mesh", C.c_uint32), ("num_triangles", C.c_uint32), ("area", C.c_float),
                ("sphere", C.c_float * 4), ("radiance", C.c_float * 3)]


class SceneInfo(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("num_triangles", C.c_uint32),
                ("num_meshes", C.c_uint32), ("num_lights", C.c_uint32), ("num_bvh_nodes", C.c_uint32),
                ("device_bytes", C.c_uint64), ("build_ms", C.c_float), ("num_media", C.c_uint32)]


class Film(C.Structure):
    _fields_ = [("rgb", C.c_void_p), ("bounces", C.c_void_p), ("counts", C.c_void_p),
                ("width", C.c_uint32), ("height", C.c_uint32), ("on_device", C.c_int32)]


class RenderParams(C.Structure):
    _fields_ = [("spp", C.c_uint32), ("first_frame", C.c_uint32), ("max_depth", C.c_uint32),
                ("rr_depth", C.c_uint32)]


class RenderStats(C.Structure):
    _fields_ = [("main_rays", C.c_uint64), ("light_rays", C.c_uint64), ("bsdf_rays", C.c_uint64),
                ("samples", C.c_uint64), ("iterations", C.c_uint32), ("kernel_launches", C.c_uint32),
                ("gpu_ms", C.c_float), ("trace_ms", C.c_float), ("shade_ms", C.c_float),
                ("light_traversals", C.c_uint64), ("nonfinite_samples", C.c_uint64),
                ("init_ms", C.c_float), ("idle_ms", C.c_float)]


class Tuning(C.Structure):
    _fields_ = [("paths_in_flight", C.c_uint32), ("trace_threads", C.c_uint32), ("shade_threads", C.c_uint32),
                ("loop_iterations", C.c_uint32), ("bvh_width", C.c_uint32), ("ms", C.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class QueueLengths(C.Structure):
    _fields_ = [("path_rays", C.c_uint32), ("camera_rays", C.c_uint32), ("connection_records", C.c_uint32)]


class SppRange(C.Structure):
    _fields_ = [("min_spp", C.c_uint32), ("max_spp", C.c_uint32), ("sum_spp", C.c_uint64)]


_lock = threading.Lock()
_lib = None


def load(build_if_needed: bool = True) -> C.CDLL:
    """Load liblantern_gpu.so, building it first if it is missing or stale.

    With LANTERN_GPU_CHECKED=1 in the environment the process loads
    liblantern_gpu_checked.so instead: the same library with its kernels'
    bound checks compiled in (renders fail with LT_ERR_CHECK where an index
    would leave its array), for test runs."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.CHECKED_LIB if os.environ.get("LANTERN_GPU_CHECKED") == "1" else _build.LIB
        if build_if_needed and not _build.up_to_date():
            _build.build()
        if not os.path.exists(path):
            raise LanternError(2, f"{path} is not built")
        L = C.CDLL(path)
        p = C.c_void_p
        L.lt_abi_version.restype = C.c_int
        if L.lt_abi_version() != ABI_VERSION:
            raise RuntimeError(f"liblantern_gpu.so has ABI {L.lt_abi_version()}, this binding expects {ABI_VERSION}")
        L.lt_ctx_create.argtypes = [C.c_int, C.POINTER(p)]
        L.lt_ctx_destroy.argtypes = [p]
        L.lt_ctx_destroy.restype = None
        L.lt_last_error.argtypes = [p]
        L.lt_last_error.restype = C.c_char_p
        L.lt_set_stream.argtypes = [p, p]
        L.lt_get_stream.argtypes = [p]
        L.lt_get_stream.restype = p
        L.lt_sync.argtypes = [p]
        L.lt_trim.argtypes = [p]
        L.lt_scene_create.argtypes = [p, C.POINTER(SceneDesc)]
        L.lt_scene_load_json.argtypes = [p, C.c_char_p]
        L.lt_scene_destroy.argtypes = [p]
        L.lt_scene_info_get.argtypes = [p, C.POINTER(SceneInfo)]
        L.lt_scene_mesh_offsets.argtypes = [p, C.POINTER(C.c_uint32), C.c_uint32]
        L.lt_scene_lights_get.argtypes = [p, C.POINTER(LightInfo), C.c_uint32]
        L.lt_render.argtypes = [p, C.POINTER(RenderParams), C.POINTER(Film)]
        L.lt_render_stats_get.argtypes = [p, C.POINTER(RenderStats)]
        L.lt_intersect.argtypes = [p, p, p, C.c_uint64, C.c_int32]
        L.lt_render_noalloc.argtypes = [p, C.POINTER(RenderParams), C.POINTER(Film), C.c_uint32]
        L.lt_set_bvh_builder.argtypes = [p, C.c_int32]
        L.lt_get_tuning.argtypes = [p, C.POINTER(Tuning)]
        L.lt_set_tuning.argtypes = [p, C.POINTER(Tuning)]
        L.lt_set_stage_timing.argtypes = [p, C.c_int32]
        L.lt_render_batch.argtypes = [p, C.POINTER(p), C.POINTER(RenderParams), C.POINTER(Film), C.c_uint32]
        L.lt_autotune_batch.argtypes = [p, C.POINTER(p), C.POINTER(RenderParams), C.c_uint32, C.c_uint32,
                                        C.POINTER(Tuning)]
        L.lt_resolve.argtypes = [p, C.POINTER(Film), C.c_int32, C.c_float, p, p, C.POINTER(SppRange)]
        L.lt_image_load.argtypes = [C.c_char_p, p, C.c_size_t, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                    C.POINTER(C.c_uint32)]
        L.lt_debug_fail_allocations.argtypes = [C.c_uint32]
        L.lt_debug_fail_allocations.restype = None
        L.lt_debug_set_iteration_limit.argtypes = [C.c_uint64]
        L.lt_debug_set_iteration_limit.restype = None
        L.lt_set_queue_trace.argtypes = [p, C.c_uint32]
        L.lt_queue_trace_get.argtypes = [p, C.POINTER(QueueLengths), C.c_uint32, C.POINTER(C.c_uint32)]
        L.lt_debug_set_check_pixel_limit.argtypes = [C.c_uint32]
        L.lt_debug_set_check_pixel_limit.restype = None
        _lib = L
        return L


def check(L, ctx, status: int) -> None:
    if status != LT_OK:
        raise LanternError(status, L.lt_last_error(ctx).decode(errors="replace"))


def load_image(path: str):
    """lt_image_load: a PNG file as the scene loader decodes image textures,
    (height, width, channels) uint8 (stbi_load with 0 requested channels)."""
    import numpy as np
    L = load()
    w, h, n = C.c_uint32(), C.c_uint32(), C.c_uint32()
    b = os.path.abspath(path).encode()
    st = L.lt_image_load(b, None, 0, C.byref(w), C.byref(h), C.byref(n))
    if st != LT_OK:
        raise LanternError(st, L.lt_last_error(None).decode(errors="replace"))
    out = np.empty((h.value, w.value, n.value), np.uint8)
    st = L.lt_image_load(b, out.ctypes.data, out.nbytes, C.byref(w), C.byref(h), C.byref(n))
    if st != LT_OK:
        raise LanternError(st, L.lt_last_error(None).decode(errors="replace"))
    return out


class Context:
    """One lt_ctx: a CUDA device, its stream, one scene and the wavefront buffers."""

    def __init__(self, device: int = 0):
        self.L = load()
        h = C.c_void_p()
        st = self.L.lt_ctx_create(device, C.byref(h))
        if st != LT_OK:
            raise LanternError(st, self.L.lt_last_error(None).decode(errors="replace"))
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            self.L.lt_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        check(self.L, self.h, st)

    def set_stream(self, stream_ptr: int | None):
        """Issue work on this cudaStream_t (0 = CUDA's legacy default stream)."""
        self._check(self.L.lt_set_stream(self.h, C.c_void_p(stream_ptr or 0)))

    def get_stream(self) -> int:
        return self.L.lt_get_stream(self.h) or 0

    def sync(self):
        self._check(self.L.lt_sync(self.h))

    def trim(self):
        """lt_trim: free the work buffers (wavefronts, sample buffer, staging);
        the scene stays."""
        self._check(self.L.lt_trim(self.h))

    def set_bvh_builder(self, builder: int):
        """BVH_GPU (default) or BVH_HOST for the next scene load."""
        self._check(self.L.lt_set_bvh_builder(self.h, builder))

    def load_scene_json(self, path: str):
        self._check(self.L.lt_scene_load_json(self.h, os.path.abspath(path).encode()))

    def create_scene(self, desc: SceneDesc):
        self._check(self.L.lt_scene_create(self.h, C.byref(desc)))

    def destroy_scene(self):
        """lt_scene_destroy: frees the scene, keeps the context."""
        self._check(self.L.lt_scene_destroy(self.h))

    def scene_info(self) -> SceneInfo:
        info = SceneInfo()
        self._check(self.L.lt_scene_info_get(self.h, C.byref(info)))
        return info

    def lights(self):
        """lt_scene_lights_get: per area light (mesh, num_triangles, area,
        sphere[4], radiance[3])."""
        n = self.scene_info().num_lights
        arr = (LightInfo * max(1, n))()
        self._check(self.L.lt_scene_lights_get(self.h, arr, len(arr)))
        return list(arr)[:n]

    def mesh_offsets(self):
        info = self.scene_info()
        arr = (C.c_uint32 * max(1, info.num_meshes))()
        self._check(self.L.lt_scene_mesh_offsets(self.h, arr, len(arr)))
        return list(arr)[:info.num_meshes]

    def render(self, film: Film, spp: int, first_frame: int = 0, max_depth: int = 1500, rr_depth: int = 3):
        prm = RenderParams(spp, first_frame, max_depth, rr_depth)
        self._check(self.L.lt_render(self.h, C.byref(prm), C.byref(film)))

    def render_noalloc(self, film: Film, spp: int, paths_in_flight: int, first_frame: int = 0,
                       max_depth: int = 1500, rr_depth: int = 3):
        """lt_render_noalloc: the same render with the library's fixed device
        scratch, for callers that must not have the library allocate memory."""
        prm = RenderParams(spp, first_frame, max_depth, rr_depth)
        self._check(self.L.lt_render_noalloc(self.h, C.byref(prm), C.byref(film), paths_in_flight))

    def stats(self) -> RenderStats:
        s = RenderStats()
        self._check(self.L.lt_render_stats_get(self.h, C.byref(s)))
        return s

    def intersect(self, rays_ptr: int, hits_ptr: int, n: int, on_device: bool):
        self._check(self.L.lt_intersect(self.h, C.c_void_p(rays_ptr), C.c_void_p(hits_ptr), n, int(on_device)))

    def tuning(self) -> Tuning:
        t = Tuning()
        self._check(self.L.lt_get_tuning(self.h, C.byref(t)))
        return t

    def set_stage_timing(self, on: bool):
        """lt_set_stage_timing: per-stage kernel times in stats() (events around every launch)."""
        self._check(self.L.lt_set_stage_timing(self.h, 1 if on else 0))

    def set_queue_trace(self, rows: int):
        """lt_set_queue_trace: record the queue lengths of up to `rows`
        iterations of every later wavefront loop (0: off)."""
        self._check(self.L.lt_set_queue_trace(self.h, rows))

    def queue_trace(self):
        """lt_queue_trace_get: the last loop's rows as a (rows, 3) uint32 array
        of (path rays, camera rays, connection records)."""
        import numpy as np
        n = C.c_uint32()
        self._check(self.L.lt_queue_trace_get(self.h, None, 0, C.byref(n)))
        arr = (QueueLengths * max(n.value, 1))()
        self._check(self.L.lt_queue_trace_get(self.h, arr, n.value, C.byref(n)))
        return np.array([(r.path_rays, r.camera_rays, r.connection_records) for r in arr[:n.value]],
                        dtype=np.uint32).reshape(-1, 3)

    def set_tuning(self, **fields):
        """lt_set_tuning with the given fields changed from the current tuning."""
        t = self.tuning()
        for k, v in fields.items():
            setattr(t, k, v)
        self._check(self.L.lt_set_tuning(self.h, C.byref(t)))

    @staticmethod
    def _batch_args(scenes, params):
        n = len(scenes)
        hs = (C.c_void_p * n)(*[s.h.value for s in scenes])
        ps = (RenderParams * n)(*[RenderParams(*p) for p in params])
        return n, hs, ps

    def render_batch(self, scenes, params, films):
        """lt_render_batch: scenes = Contexts holding a scene, params = (spp,
        first_frame, max_depth, rr_depth) per scene, films = device Films."""
        n, hs, ps = self._batch_args(scenes, params)
        fs = (Film * n)(*films)
        self._check(self.L.lt_render_batch(self.h, hs, ps, fs, n))

    def resolve(self, film: Film, tonemap: int, exposure_stops: float, rgba_ptr: int | None,
                rgba8_ptr: int | None) -> SppRange:
        r = SppRange()
        self._check(self.L.lt_resolve(self.h, C.byref(film), tonemap, exposure_stops, C.c_void_p(rgba_ptr or 0),
                                      C.c_void_p(rgba8_ptr or 0), C.byref(r)))
        return r

    def autotune_batch(self, scenes, params, spp_cap: int = 1) -> Tuning:
        n, hs, ps = self._batch_args(scenes, params)
        t = Tuning()
        self._check(self.L.lt_autotune_batch(self.h, hs, ps, n, spp_cap, C.byref(t)))
        return t
