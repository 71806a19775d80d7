"""Image files of the headless loop: 8-bit PNG frames and half-float EXR images.

The reference writes every frame of its headless loop as an RGBA8 PNG (enqueueSaveImage
"%03u.png", renderer/renderer_main.cpp:1646-1655, encoded by fpng in common/common_host.cpp:
422-441) and HDR images as EXR through tinyexr (saveImageHDR, common/common_host.cpp:443-515:
channels stored A, B, G, R as HALF, no compression, optional brightness scale and row flip).
Neither encoder ships with the reference (ext/fpng and ext/tinyexr are empty submodules); these
writers follow the PNG (ISO/IEC 15948) and OpenEXR 2 scan-line file layouts directly. The
pixels come from the device: ``Renderer.image_rgba8`` runs the tone-map + sRGB kernel.
"""
from __future__ import annotations

import struct
import zlib
from pathlib import Path

import numpy as np


def _png_chunk(tag: bytes, data: bytes) -> bytes:
    return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)


def rgba8_array(image) -> np.ndarray:
    """(h, w, 4) uint8 view of an image given as (h, w, 4) bytes or (h, w) RGBA words (R low)."""
    a = np.asarray(image)
    if a.dtype == np.uint32 and a.ndim == 2:
        return a.astype("<u4").view(np.uint8).reshape(a.shape[0], a.shape[1], 4)
    if a.dtype == np.uint8 and a.ndim == 3 and a.shape[2] == 4:
        return a
    raise ValueError("expected (h, w, 4) uint8 or (h, w) uint32 RGBA")


def encode_png(image, level: int = 6) -> bytes:
    """PNG bytes of an RGBA8 image (colour type 6, 8 bits, filter 0 on every row)."""
    a = np.ascontiguousarray(rgba8_array(image))
    h, w = a.shape[:2]
    raw = np.zeros((h, 1 + 4 * w), dtype=np.uint8)
    raw[:, 1:] = a.reshape(h, 4 * w)
    ihdr = struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)
    return (b"\x89PNG\r\n\x1a\n" + _png_chunk(b"IHDR", ihdr) +
            _png_chunk(b"IDAT", zlib.compress(raw.tobytes(), level)) + _png_chunk(b"IEND", b""))


def write_png(path, image, level: int = 6) -> Path:
    p = Path(path)
    p.write_bytes(encode_png(image, level))
    return p


def _attr(name: str, kind: str, data: bytes) -> bytes:
    return name.encode() + b"\0" + kind.encode() + b"\0" + struct.pack("<i", len(data)) + data


def encode_exr(rgb, brightness: float = 1.0, flip_y: bool = False) -> bytes:
    """OpenEXR bytes of an (h, w, c) float image, c in 1..4, as saveImageHDR stores it: four HALF
    channels A, B, G, R (missing channels 0), values scaled by `brightness`, one scan line per
    block, no compression."""
    a = np.asarray(rgb, dtype=np.float32)
    if a.ndim != 3 or not 1 <= a.shape[2] <= 4:
        raise ValueError("expected an (h, w, c) float image with 1 to 4 channels")
    h, w, c = a.shape
    planes = np.zeros((4, h, w), dtype=np.float32)  # R, G, B, A
    for k in range(c):
        planes[k] = brightness * a[:, :, k]
    if flip_y:
        planes = planes[:, ::-1]
    half = planes.astype(np.float16)
    chlist = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", 1, 0, 1, 1) for n in "ABGR") + b"\0"
    header = (struct.pack("<ii", 20000630, 2) +
              _attr("channels", "chlist", chlist) +
              _attr("compression", "compression", b"\0") +
              _attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)) +
              _attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)) +
              _attr("lineOrder", "lineOrder", b"\0") +
              _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)) +
              _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0)) +
              _attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\0")
    line_bytes = 4 * 2 * w
    first = len(header) + 8 * h
    offsets = np.arange(h, dtype=np.uint64) * np.uint64(8 + line_bytes) + np.uint64(first)
    order = [3, 2, 1, 0]  # A, B, G, R planes
    lines = []
    for y in range(h):
        data = b"".join(half[k, y].astype("<f2").tobytes() for k in order)
        lines.append(struct.pack("<ii", y, line_bytes) + data)
    return header + offsets.astype("<u8").tobytes() + b"".join(lines)


def write_exr(path, rgb, brightness: float = 1.0, flip_y: bool = False) -> Path:
    p = Path(path)
    p.write_bytes(encode_exr(rgb, brightness, flip_y))
    return p
