"""Headless display output: the visualizer's final resolve (lt_resolve) and
image files.

The reference shows the film in a window: it divides each pixel's colour sum
by its sample count (visualizer.cpp:352-364), scales by 2^exposure
(visualizer.cpp:1308) and tone maps with clamp or a filmic curve
(final_resolve_ps.glsl:24-43) into a UNORM swapchain. Here the same pass
writes device buffers (lt_resolve in liblantern_gpu.so), and ``write_png`` /
``write_exr`` store the 8-bit or float result. Both writers are plain
encoders of the file formats (PNG: zlib stream of filter-0 scanlines;
OpenEXR: single-part scanline file, uncompressed FLOAT channels).
"""
from __future__ import annotations

import struct
import zlib

import numpy as np
import torch

from .integrator import FrameBuffer
from .native import TONEMAP_CLAMP, TONEMAP_FILMIC, Context

__all__ = ["resolve", "write_png", "write_exr", "TONEMAP_CLAMP", "TONEMAP_FILMIC"]


def resolve(ctx: Context, fb: FrameBuffer, tonemap: int = TONEMAP_CLAMP, exposure_stops: float = 0.0):
    """Tone-mapped image of a device FrameBuffer: (rgba float32 (H, W, 4),
    rgba8 uint8 (H, W, 4)) CUDA tensors, and (min, max, mean) samples per pixel."""
    dev = fb.ColorData.device
    rgba = torch.empty((fb.Height, fb.Width, 4), dtype=torch.float32, device=dev)
    rgba8 = torch.empty((fb.Height, fb.Width, 4), dtype=torch.uint8, device=dev)
    ctx.set_stream(torch.cuda.current_stream(dev).cuda_stream)
    r = ctx.resolve(fb.film(), tonemap, exposure_stops, rgba.data_ptr(), rgba8.data_ptr())
    npix = max(1, fb.Width * fb.Height)
    return rgba, rgba8, (r.min_spp, r.max_spp, r.sum_spp / npix)


def _chunk(tag: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def write_png(path: str, img8) -> None:
    """8-bit (H, W, C) array or tensor, C = 1 (grey), 2 (grey + alpha), 3 (RGB)
    or 4 (RGBA), to a PNG file."""
    a = img8.cpu().numpy() if isinstance(img8, torch.Tensor) else np.asarray(img8)
    a = np.ascontiguousarray(a, dtype=np.uint8)
    h, w, c = a.shape
    if c not in (1, 2, 3, 4):
        raise ValueError("write_png wants 1 to 4 channels")
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[c]
    raw = np.concatenate([np.zeros((h, 1), np.uint8), a.reshape(h, w * c)], axis=1).tobytes()
    with open(path, "wb") as fh:
        fh.write(b"\x89PNG\r\n\x1a\n")
        fh.write(_chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)))
        fh.write(_chunk(b"IDAT", zlib.compress(raw, 6)))
        fh.write(_chunk(b"IEND", b""))


def read_png(path: str) -> np.ndarray:
    """Reader for the RGBA files write_png makes (8-bit, filter 0 rows)."""
    data = open(path, "rb").read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, tag = struct.unpack(">I4s", data[pos:pos + 8])
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            if depth != 8 or ctype != 6:
                raise ValueError("only 8-bit RGBA")
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    rows = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, 1 + 4 * w)
    if np.any(rows[:, 0] != 0):
        raise ValueError("only filter type 0")
    return rows[:, 1:].reshape(h, w, 4).copy()


def write_exr(path: str, rgba) -> None:
    """Float (H, W, 3 or 4) array or tensor to an uncompressed scanline
    OpenEXR file with 32-bit FLOAT channels (A, B, G, R stored in name order)."""
    a = rgba.cpu().numpy() if isinstance(rgba, torch.Tensor) else np.asarray(rgba)
    a = np.ascontiguousarray(a, dtype="<f4")
    h, w, c = a.shape
    names = ["R", "G", "B", "A"][:c]
    order = sorted(range(c), key=lambda k: names[k])  # channels are stored sorted by name

    def attr(name, typ, value):
        return name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<i", len(value)) + value

    chlist = b"".join(names[k].encode() + b"\0" + struct.pack("<iB3xii", 2, 0, 1, 1) for k in order) + b"\0"
    header = (struct.pack("<ii", 20000630, 2)
              + attr("channels", "chlist", chlist)
              + attr("compression", "compression", b"\0")
              + attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1))
              + attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1))
              + attr("lineOrder", "lineOrder", b"\0")
              + attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
              + attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0))
              + attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
              + b"\0")
    line_bytes = w * c * 4
    table_end = len(header) + 8 * h
    offsets = [table_end + y * (8 + line_bytes) for y in range(h)]
    with open(path, "wb") as fh:
        fh.write(header)
        fh.write(struct.pack(f"<{h}Q", *offsets))
        for y in range(h):
            fh.write(struct.pack("<ii", y, line_bytes))
            fh.write(np.ascontiguousarray(a[y][:, order].T).tobytes())


def read_exr(path: str) -> np.ndarray:
    """Reader for the files write_exr makes; returns (H, W, C) float32 in R, G, B, A order."""
    data = open(path, "rb").read()
    if struct.unpack("<i", data[:4])[0] != 20000630:
        raise ValueError("not an OpenEXR file")
    pos, attrs = 8, {}
    while data[pos] != 0:
        e = data.index(b"\0", pos)
        name = data[pos:e].decode()
        e2 = data.index(b"\0", e + 1)
        size = struct.unpack("<i", data[e2 + 1:e2 + 5])[0]
        attrs[name] = data[e2 + 5:e2 + 5 + size]
        pos = e2 + 5 + size
    pos += 1
    chans, p = [], 0
    cl = attrs["channels"]
    while cl[p] != 0:
        e = cl.index(b"\0", p)
        chans.append(cl[p:e].decode())
        p = e + 1 + 16
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    offsets = struct.unpack(f"<{h}Q", data[pos:pos + 8 * h])
    out = np.empty((h, w, len(chans)), np.float32)
    for y, off in enumerate(offsets):
        n = struct.unpack("<i", data[off + 4:off + 8])[0]
        out[y] = np.frombuffer(data[off + 8:off + 8 + n], "<f4").reshape(len(chans), w).T
    want = [k for k in ["R", "G", "B", "A"] if k in chans]
    return out[:, :, [chans.index(k) for k in want]]
