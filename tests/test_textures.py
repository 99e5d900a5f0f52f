"""Albedo textures: PNG decoding and the uv / image textures of the scene JSON.

* The PNG decoder of the scene loader (lt_image_load, lantern_gb300/csrc/lt_image.cpp)
  and the oracle's (oracle.read_png) against the reference's own stb_image
  (stbi_load with 0 requested channels) on encoded variants: colour types 0, 2,
  3, 4, 6; bit depths 1, 2, 4, 8, 16; tRNS keys and palette alpha; every
  scanline filter; stored, fixed and dynamic deflate blocks.
* A scene with uv and image albedo rendered by the tile-keyed oracle is
  bit-identical to the compiled reference's render.
* On the GPU, the same scene rendered path by path agrees with the oracle.
"""
import os
import struct
import zlib

import numpy as np
import pytest

import lantern_gb300.scenes as S
from lantern_gb300 import native
from oracle import oracle as O


def _chunk(tag, body):
    return struct.pack(">I", len(body)) + tag + body + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)


def _filter_row(kind, row, prev, bpp):
    out = bytearray(len(row))
    for i, x in enumerate(row):
        a = row[i - bpp] if i >= bpp else 0
        b = prev[i]
        c = prev[i - bpp] if i >= bpp else 0
        if kind == 0:
            p = 0
        elif kind == 1:
            p = a
        elif kind == 2:
            p = b
        elif kind == 3:
            p = (a + b) >> 1
        else:
            q = a + b - c
            pa, pb, pc = abs(q - a), abs(q - b), abs(q - c)
            p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
        out[i] = (x - p) & 255
    return bytes(out)


def encode_png(samples, depth, ctype, palette=None, trns=None, level=6, seed=0):
    """samples: (h, w, chans) integers < 2**depth (palette indices for type 3)."""
    h, w, ch = samples.shape
    rows = []
    for y in range(h):
        vals = samples[y].reshape(-1).astype(np.int64)
        if depth == 16:
            row = b"".join(struct.pack(">H", int(v)) for v in vals)
        elif depth == 8:
            row = bytes(int(v) for v in vals)
        else:
            bits = "".join(format(int(v), f"0{depth}b") for v in vals)
            bits += "0" * (-len(bits) % 8)
            row = bytes(int(bits[i:i + 8], 2) for i in range(0, len(bits), 8))
        rows.append(row)
    bpp = max(1, (ch * depth + 7) // 8)
    rng = np.random.default_rng(seed)
    raw, prev = b"", bytes(len(rows[0]))
    for row in rows:
        kind = int(rng.integers(0, 5))
        raw += bytes([kind]) + _filter_row(kind, row, prev, bpp)
        prev = row
    png = b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0))
    if palette is not None:
        png += _chunk(b"PLTE", bytes(np.asarray(palette, np.uint8).reshape(-1)))
    if trns is not None:
        png += _chunk(b"tRNS", trns)
    z = zlib.compress(raw, level)
    png += _chunk(b"IDAT", z[: len(z) // 2]) + _chunk(b"IDAT", z[len(z) // 2:])  # split IDAT
    return png + _chunk(b"IEND", b"")


def _variants():
    rng = np.random.default_rng(5)
    out = []
    for depth in (1, 2, 4, 8, 16):
        g = rng.integers(0, 2 ** depth, (7, 13, 1))
        out.append((f"grey{depth}", g, depth, 0, None, None))
    g8 = rng.integers(0, 256, (9, 11, 1))
    g8[0, :3] = 77
    out.append(("grey8_trns", g8, 8, 0, None, struct.pack(">H", 77)))
    for depth in (8, 16):
        out.append((f"rgb{depth}", rng.integers(0, 2 ** depth, (6, 10, 3)), depth, 2, None, None))
        out.append((f"greyalpha{depth}", rng.integers(0, 2 ** depth, (5, 9, 2)), depth, 4, None, None))
        out.append((f"rgba{depth}", rng.integers(0, 2 ** depth, (8, 5, 4)), depth, 6, None, None))
    rgb = rng.integers(0, 256, (6, 7, 3))
    rgb[1, 2] = (10, 20, 30)
    out.append(("rgb8_trns", rgb, 8, 2, None, struct.pack(">HHH", 10, 20, 30)))
    pal = rng.integers(0, 256, (16, 3))
    for depth in (1, 2, 4, 8):
        idx = rng.integers(0, min(16, 2 ** depth), (7, 9, 1))
        out.append((f"palette{depth}", idx, depth, 3, pal[: min(16, 2 ** depth)], None))
    idx = rng.integers(0, 16, (5, 6, 1))
    out.append(("palette8_alpha", idx, 8, 3, pal, bytes(rng.integers(0, 256, 10).astype(np.uint8))))
    return out


@pytest.mark.parametrize("level", [0, 1, 9])
def test_png_decoders_agree(tmp_path, level):
    for name, samples, depth, ctype, pal, trns in _variants():
        path = str(tmp_path / f"{name}_{level}.png")
        with open(path, "wb") as fh:
            fh.write(encode_png(samples, depth, ctype, pal, trns, level, seed=len(name)))
        ours = native.load_image(path)
        orc = O.read_png(path)
        assert ours.shape == orc.shape and np.array_equal(ours, orc), name
        ref = O.reference_image_load(path)
        if ref is not None:
            assert ref.shape == ours.shape and np.array_equal(ref, ours), name


def test_image_load_errors(tmp_path):
    bad = tmp_path / "bad.png"
    bad.write_bytes(b"\x89PNG\r\n\x1a\n" + b"\x00" * 20)
    with pytest.raises(native.LanternError, match="LT_ERR_PARSE"):
        native.load_image(str(bad))
    with pytest.raises(native.LanternError, match="LT_ERR_IO"):
        native.load_image(str(tmp_path / "missing.png"))
    # a 65536 x 65536 16-bit RGBA header over a few bytes of image data: rejected
    # as malformed before a 34 GB buffer is reserved for it
    huge = tmp_path / "huge.png"
    huge.write_bytes(b"\x89PNG\r\n\x1a\n" + _chunk(b"IHDR", struct.pack(">IIBBBBB", 65536, 65536, 16, 6, 0, 0, 0))
                     + _chunk(b"IDAT", zlib.compress(b"\x00" * 64)) + _chunk(b"IEND", b""))
    with pytest.raises(native.LanternError, match="LT_ERR_PARSE"):
        native.load_image(str(huge))


def test_textured_oracle_matches_reference(reference_available, scene_dir):
    if not reference_available:
        pytest.skip("reference build not available here")
    path = S.textured_scene(os.path.join(scene_dir, "textures"), width=48, height=40, name="textured_48").write(
        scene_dir)
    orc = O.OracleScene(path)
    ref = O.ReferenceScene(path)
    a = orc.render(3, max_depth=8, rr_depth=3, keying=O.KEY_TILE, two_films=True, threads=4)
    b = ref.render(3, max_depth=8, rr_depth=3)
    for k in ("rgb", "bounces", "counts", "rgb_b", "bounces_b", "counts_b"):
        x, y = a[k], b[k]
        if x.dtype == np.float32:
            x, y = x.view(np.uint32), y.view(np.uint32)
        assert np.array_equal(x, y), k
    assert float(a["rgb"].mean()) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("bvh_width", [2, 4, 8])
def test_gpu_textured_render_matches_oracle(scene_dir, bvh_width):
    import torch
    from lantern_gb300.integrator import FrameBuffer, Integrator, Scene
    path = S.textured_scene(os.path.join(scene_dir, "textures"), width=48, height=40, name="textured_gpu").write(
        scene_dir)
    sc = Scene(0)
    sc.LoadSceneFromJSON(path)
    sc.ctx.set_tuning(bvh_width=bvh_width)
    fb = FrameBuffer(sc.width, sc.height, "cuda:0")
    Integrator(sc, fb, max_depth=8, rr_depth=3).RenderFrame(4)
    torch.cuda.synchronize()
    ref = O.OracleScene(path).render(4, max_depth=8, rr_depth=3, keying=O.KEY_PIXEL)
    rgb = fb.ColorData.cpu().numpy()
    assert np.array_equal(fb.ColorSampleCount.cpu().numpy(), ref["counts"].astype(np.int32))
    close = np.isclose(rgb, ref["rgb"], rtol=2e-4, atol=1e-5).all(-1)
    assert close.mean() > 0.97, close.mean()
    assert (fb.Bounces.cpu().numpy() == ref["bounces"].astype(np.int32)).mean() > 0.97
