"""Facet-data maps as images: the reference's ray-cast renderer
(src/cpp/illum_renderer_cli.cpp:160-316) with the ray casting on the GPU
(ilg_render) and the colouring and PNG file written here without external
dependencies.

    rgb = render(ctx, data, mode="ortho", az=30, el=60, width=800, height=800)
    write_png("map.png", rgb)
"""
from __future__ import annotations

import ctypes as C
import struct
import zlib

import numpy as np

from . import _check, lib

MODES = {"ortho": 0, "orthographic": 0, "equal-area-cylindrical": 1, "eac": 1}


def facet_image(ctx, mode="ortho", az=0.0, el=0.0, width=512, height=512) -> np.ndarray:
    """height x width facet indices (-1: background) seen by each pixel."""
    out = np.zeros((height, width), np.int32)
    _check(lib().ilg_render(ctx._h, MODES[mode], float(az), float(el), int(width), int(height),
                            out.ctypes.data_as(C.c_void_p)))
    return out


def jet(x: np.ndarray) -> np.ndarray:
    """The reference's jet map (illum_renderer_cli.cpp:283-292)."""
    r = np.clip(np.where(x < 0.7, 4 * x - 1.5, -4 * x + 4.5), 0.0, 1.0)
    g = np.clip(np.where(x < 0.5, 4 * x - 0.5, -4 * x + 3.5), 0.0, 1.0)
    b = np.clip(np.where(x < 0.3, 4 * x + 0.5, -4 * x + 2.5), 0.0, 1.0)
    return np.floor(255 * np.stack([r, g, b], -1)).astype(np.uint8)


def grayscale(x: np.ndarray) -> np.ndarray:
    v = (255 * np.clip(x, 0.0, 1.0)).astype(np.uint8)
    return np.stack([v, v, v], -1)


def render(ctx, data, mode="ortho", az=0.0, el=0.0, width=512, height=512, minval=None, maxval=None,
           cmap="jet") -> np.ndarray:
    """RGB image (height x width x 3 uint8) of per-facet `data`: values
    clamped to [minval, maxval], scaled by the data range (or the given
    bounds) and coloured; pixels that see no facet stay black, as in the
    reference."""
    data = np.asarray(data, np.float64).ravel()
    if data.size != ctx.num_faces:
        raise ValueError("input data and mesh have incompatible sizes")
    if minval is not None:
        data = np.maximum(data, minval)
    if maxval is not None:
        data = np.minimum(data, maxval)
    lo = data.min() if minval is None else minval
    hi = data.max() if maxval is None else maxval
    idx = facet_image(ctx, mode, az, el, width, height)
    img = np.zeros((height, width, 3), np.uint8)
    hit = idx >= 0
    x = (data[idx[hit]] - lo) / (hi - lo) if hi > lo else np.zeros(hit.sum())
    img[hit] = (grayscale if cmap == "grayscale" else jet)(x)
    return img


def write_png(path: str, rgb: np.ndarray) -> None:
    """8-bit RGB PNG (no filtering, zlib-compressed scanlines)."""
    rgb = np.ascontiguousarray(rgb, np.uint8)
    h, w, _ = rgb.shape
    raw = b"".join(b"\x00" + rgb[i].tobytes() for i in range(h))

    def chunk(tag: bytes, body: bytes) -> bytes:
        return struct.pack(">I", len(body)) + tag + body + struct.pack(">I", zlib.crc32(tag + body) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0)))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))


def read_png(path: str) -> np.ndarray:
    """Reads back what write_png writes (8-bit RGB, filter 0)."""
    with open(path, "rb") as f:
        data = f.read()
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG file")
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag = data[pos + 4:pos + 8]
        body = data[pos + 8:pos + 8 + n]
        if tag == b"IHDR":
            w, h = struct.unpack(">II", body[:8])
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = zlib.decompress(idat)
    rows = [raw[i * (3 * w + 1) + 1:(i + 1) * (3 * w + 1)] for i in range(h)]
    return np.frombuffer(b"".join(rows), np.uint8).reshape(h, w, 3)
