"""Host-side mirror of the reference's Scene / FrameBuffer / Integrator interface.

The reference drives rendering as (source/lantern/main.cpp:52-77)::

    Scene scene; scene.LoadSceneFromJSON(path);
    FrameBuffer a(w, h), b(w, h); std::atomic<FrameBuffer*> swap(&b);
    Integrator integ(&scene, &a, &swap);
    for (;;) integ.RenderFrame();     // one sample per pixel per call

The same names work here, with the film in GPU memory (torch tensors) and the
rendering done by liblantern_gpu.so. ``RenderFrame(n)`` renders n frames in
one call (n RenderFrame calls of the reference), all accumulated additively.
"""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from .native import Context, Film


class FrameBuffer:
    """FrameBuffer (source/core/camera/frame_buffer.h:16-30): per-pixel colour sum
    (float3), summed path length and sample count, here as CUDA tensors."""

    def __init__(self, width: int, height: int, device: int | str | torch.device = "cuda"):
        self.Width = width
        self.Height = height
        dev = torch.device(device if not isinstance(device, int) else f"cuda:{device}")
        self.ColorData = torch.zeros((height, width, 3), dtype=torch.float32, device=dev)
        self.Bounces = torch.zeros((height, width), dtype=torch.int32, device=dev)
        self.ColorSampleCount = torch.zeros((height, width), dtype=torch.int32, device=dev)

    def Reset(self):
        self.ColorData.zero_()
        self.Bounces.zero_()
        self.ColorSampleCount.zero_()

    def film(self) -> Film:
        return Film(self.ColorData.data_ptr(), self.Bounces.data_ptr(), self.ColorSampleCount.data_ptr(),
                    self.Width, self.Height, 1)

    def image(self) -> torch.Tensor:
        """ColorData / ColorSampleCount, the division the reference's display does
        (visualizer.cpp:361-364)."""
        return self.ColorData / self.ColorSampleCount.clamp(min=1).unsqueeze(-1).to(torch.float32)

    def save(self, path: str, frame_number: int) -> None:
        """Checkpoint: colour sums, bounce sums, sample counts and the next frame
        number (an .npz file). The reference keeps exactly this state between
        RenderFrame calls (integrator.h:38-41)."""
        np.savez(path, rgb=self.ColorData.cpu().numpy(), bounces=self.Bounces.cpu().numpy(),
                 counts=self.ColorSampleCount.cpu().numpy(), frame_number=np.int64(frame_number))

    @staticmethod
    def load(path: str, device: int | str | torch.device = "cuda"):
        """(FrameBuffer, next frame number) from a checkpoint written by save()."""
        z = np.load(path)
        h, w = z["counts"].shape
        fb = FrameBuffer(w, h, device)
        fb.ColorData.copy_(torch.from_numpy(z["rgb"]))
        fb.Bounces.copy_(torch.from_numpy(z["bounces"]))
        fb.ColorSampleCount.copy_(torch.from_numpy(z["counts"]))
        return fb, int(z["frame_number"])


class Scene:
    """Scene (source/core/scene/scene.h:33-98) for the GPU integrator."""

    def __init__(self, device: int = 0):
        self.ctx = Context(device)
        self.device = device
        self.width = self.height = 0

    def LoadSceneFromJSON(self, path: str) -> bool:
        self.ctx.load_scene_json(path)
        info = self.ctx.scene_info()
        self.width, self.height = info.width, info.height
        return True

    def info(self):
        return self.ctx.scene_info()


class Integrator:
    """Integrator (source/core/integrator/integrator.h:24-51): RenderFrame adds one
    sample per pixel (per frame) to the current film; the frame number is the
    sample index that keys each pixel's sampler."""

    def __init__(self, scene: Scene, frame_buffer: FrameBuffer, max_depth: int = 1500, rr_depth: int = 3,
                 first_frame: int = 0):
        if (frame_buffer.Width, frame_buffer.Height) != (scene.width, scene.height):
            raise ValueError("frame buffer size differs from the scene camera")
        self.scene = scene
        self.frame_buffer = frame_buffer
        self.max_depth = max_depth
        self.rr_depth = rr_depth
        self.frame_number = first_frame

    def RenderFrame(self, frames: int = 1):
        stream = torch.cuda.current_stream(self.frame_buffer.ColorData.device)
        self.scene.ctx.set_stream(stream.cuda_stream)
        self.scene.ctx.render(self.frame_buffer.film(), frames, self.frame_number, self.max_depth, self.rr_depth)
        self.frame_number += frames

    def stats(self):
        return self.scene.ctx.stats()

    def checkpoint(self, path: str) -> None:
        """Saves the film and the frame number. Because every sample's sampler is
        keyed by (pixel, frame), resume() + RenderFrame(n) continues with exactly
        the samples an uninterrupted render would have taken."""
        self.frame_buffer.save(path, self.frame_number)

    @staticmethod
    def resume(scene: "Scene", path: str, max_depth: int = 1500, rr_depth: int = 3) -> "Integrator":
        fb, frame = FrameBuffer.load(path, torch.device(f"cuda:{scene.device}"))
        return Integrator(scene, fb, max_depth=max_depth, rr_depth=rr_depth, first_frame=frame)


def render_host(ctx: Context, width: int, height: int, spp: int, first_frame: int = 0, max_depth: int = 1500,
                rr_depth: int = 3, film: Optional[dict] = None) -> dict:
    """Render into host (numpy) buffers through the C ABI's host-memory path."""
    if film is None:
        film = {"rgb": np.zeros((height, width, 3), np.float32),
                "bounces": np.zeros((height, width), np.uint32),
                "counts": np.zeros((height, width), np.uint32)}
    f = Film(film["rgb"].ctypes.data, film["bounces"].ctypes.data, film["counts"].ctypes.data, width, height, 0)
    ctx.render(f, spp, first_frame, max_depth, rr_depth)
    return film


def intersect(ctx: Context, rays, on_device: Optional[bool] = None):
    """Closest hits for (n, 8) float32 rays (org, tnear, dir, tfar); returns
    (n, 4) hits (t, u, v, prim bits) of the same kind (torch CUDA or numpy)."""
    if isinstance(rays, torch.Tensor):
        rays = rays.contiguous()
        hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device=rays.device)
        ctx.set_stream(torch.cuda.current_stream(rays.device).cuda_stream)
        ctx.intersect(rays.data_ptr(), hits.data_ptr(), rays.shape[0], True)
        return hits
    rays = np.ascontiguousarray(rays, dtype=np.float32)
    hits = np.empty((rays.shape[0], 4), dtype=np.float32)
    ctx.intersect(rays.ctypes.data, hits.ctypes.data, rays.shape[0], False)
    return hits



def RenderBatch(integrators, frames=1, owner: Optional[Context] = None):
    """RenderFrame(frames[i]) of every integrator, done together by
    lt_render_batch: the scenes' samples share one wavefront and one captured
    loop (a scene that fills the wavefront by itself is rendered alone after
    it). `owner` holds that wavefront (default: the first integrator's scene
    context). Each integrator's frame number advances as RenderFrame's would."""
    if isinstance(frames, int):
        frames = [frames] * len(integrators)
    if not integrators:
        return
    owner = owner or integrators[0].scene.ctx
    owner.set_stream(torch.cuda.current_stream(integrators[0].frame_buffer.ColorData.device).cuda_stream)
    owner.render_batch([it.scene.ctx for it in integrators],
                       [(f, it.frame_number, it.max_depth, it.rr_depth) for it, f in zip(integrators, frames)],
                       [it.frame_buffer.film() for it in integrators])
    for it, f in zip(integrators, frames):
        it.frame_number += f
