"""Image files: the headless loop's 8-bit PNG frames and half-float EXR images, and the reading of
EXR environment maps.

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


# OpenEXR scan-line layout (OpenEXR 2 file format): compression codes and scan lines per chunk.
EXR_NONE, EXR_RLE, EXR_ZIPS, EXR_ZIP = 0, 1, 2, 3
_EXR_LINES = {EXR_NONE: 1, EXR_RLE: 1, EXR_ZIPS: 1, EXR_ZIP: 16}
_EXR_TYPES = {0: np.dtype("<u4"), 1: np.dtype("<f2"), 2: np.dtype("<f4")}  # UINT, HALF, FLOAT


def _exr_predict_interleave(raw: bytes) -> bytes:
    """ZIP/RLE pre-pass of the writer: bytes split into even and odd halves, then deltas + 128."""
    a = np.frombuffer(raw, dtype=np.uint8)
    t = np.concatenate([a[0::2], a[1::2]]).astype(np.int16)
    d = t.copy()
    d[1:] = (t[1:] - t[:-1] + 128) % 256
    return d.astype(np.uint8).tobytes()


def _exr_unpredict_deinterleave(data: bytes) -> bytes:
    d = np.frombuffer(data, dtype=np.uint8).astype(np.int64)
    t = (np.cumsum(d - 128) + 128) % 256  # t[i] = t[i-1] + d[i] - 128, t[0] = d[0]
    t = t.astype(np.uint8)
    half = (len(t) + 1) // 2
    out = np.empty(len(t), dtype=np.uint8)
    out[0::2] = t[:half]
    out[1::2] = t[half:]
    return out.tobytes()


def _rle_encode(data: bytes) -> bytes:
    out, i, n = bytearray(), 0, len(data)
    while i < n:
        j = i + 1
        while j < n and j - i < 128 and data[j] == data[i]:
            j += 1
        if j - i >= 3:
            out += struct.pack("b", j - i - 1) + data[i:i + 1]
            i = j
            continue
        j = i
        while j < n and j - i < 127 and not (j + 2 < n and data[j] == data[j + 1] == data[j + 2]):
            j += 1
        j = max(j, i + 1)
        out += struct.pack("b", -(j - i)) + data[i:j]
        i = j
    return bytes(out)


def _rle_decode(data: bytes, expect: int) -> bytes:
    out, i = bytearray(), 0
    while i < len(data) and len(out) < expect:
        c = struct.unpack_from("b", data, i)[0]
        i += 1
        if c < 0:
            out += data[i:i - c]
            i -= c
        else:
            out += data[i:i + 1] * (c + 1)
            i += 1
    if len(out) != expect:
        raise ValueError("EXR: RLE chunk decodes to the wrong size")
    return bytes(out)


def encode_exr(rgb, brightness: float = 1.0, flip_y: bool = False, compression: int = EXR_NONE,
               pixel_type: int = 1) -> bytes:
    """OpenEXR bytes of an (h, w, c) float image, c in 1..4. The defaults are what saveImageHDR
    stores: four HALF channels A, B, G, R (missing channels 0), values scaled by `brightness`,
    one scan line per chunk, no compression. `compression` (EXR_NONE, EXR_RLE, EXR_ZIPS, EXR_ZIP)
    and `pixel_type` (1 HALF, 2 FLOAT) select the other scan-line encodings."""
    a = np.asarray(rgb, dtype=np.float32)
    if a.ndim != 3 or not 1 <= a.shape[2] <= 4:
        raise ValueError("expected an (h, w, c) float image with 1 to 4 channels")
    if compression not in _EXR_LINES or pixel_type not in (1, 2):
        raise ValueError("unsupported EXR compression or pixel type")
    h, w, c = a.shape
    planes = np.zeros((4, h, w), dtype=np.float32)  # R, G, B, A
    for k in range(c):
        planes[k] = brightness * a[:, :, k]
    if flip_y:
        planes = planes[:, ::-1]
    dt = _EXR_TYPES[pixel_type]
    vals = planes.astype(dt)
    chlist = b"".join(n.encode() + b"\0" + struct.pack("<iB3xii", pixel_type, 0, 1, 1) for n in "ABGR") + b"\0"
    header = (struct.pack("<ii", 20000630, 2) +
              _attr("channels", "chlist", chlist) +
              _attr("compression", "compression", bytes([compression])) +
              _attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)) +
              _attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)) +
              _attr("lineOrder", "lineOrder", b"\0") +
              _attr("pixelAspectRatio", "float", struct.pack("<f", 1.0)) +
              _attr("screenWindowCenter", "v2f", struct.pack("<ff", 0.0, 0.0)) +
              _attr("screenWindowWidth", "float", struct.pack("<f", 1.0)) + b"\0")
    lines = _EXR_LINES[compression]
    order = [3, 2, 1, 0]  # A, B, G, R planes
    chunks = []
    for y0 in range(0, h, lines):
        raw = b"".join(vals[k, y].tobytes() for y in range(y0, min(y0 + lines, h)) for k in order)
        data = raw
        if compression in (EXR_ZIPS, EXR_ZIP):
            data = zlib.compress(_exr_predict_interleave(raw))
        elif compression == EXR_RLE:
            data = _rle_encode(_exr_predict_interleave(raw))
        if len(data) >= len(raw):
            data = raw  # stored as is when the codec does not shrink the chunk
        chunks.append(struct.pack("<ii", y0, len(data)) + data)
    first = len(header) + 8 * len(chunks)
    offsets, pos = [], first
    for ch in chunks:
        offsets.append(pos)
        pos += len(ch)
    return header + np.array(offsets, dtype="<u8").tobytes() + b"".join(chunks)


def decode_exr(data: bytes) -> np.ndarray:
    """(h, w, 4) float32 RGBA of a single-part scan-line OpenEXR image with UINT, HALF or FLOAT
    channels and NONE, RLE, ZIPS or ZIP compression: what LoadEXR (tinyexr) returns for the
    reference's environment maps (renderer/renderer_scene.cpp:1140-1165). R, G, B and A are looked
    up by name (a lone Y channel is grey; missing colour channels are 0, missing alpha 1). Tiled,
    deep, multi-part files and the other codecs (PIZ, PXR24, B44, DWA) are refused."""
    if len(data) < 8 or struct.unpack_from("<i", data, 0)[0] != 20000630:
        raise ValueError("not an OpenEXR file (bad magic number)")
    version = struct.unpack_from("<i", data, 4)[0]
    if version & 0xFF != 2 or version & 0x1A00:
        raise ValueError("only single-part scan-line OpenEXR images are supported")
    pos, attrs = 8, {}
    while data[pos] != 0:
        end = data.index(b"\0", pos)
        name = data[pos:end].decode()
        tend = data.index(b"\0", end + 1)
        size = struct.unpack_from("<i", data, tend + 1)[0]
        attrs[name] = (data[end + 1:tend].decode(), data[tend + 5:tend + 5 + size])
        pos = tend + 5 + size
    pos += 1
    ch = attrs["channels"][1]
    channels, q = [], 0
    while ch[q] != 0:
        end = ch.index(b"\0", q)
        ptype, _, xs, ys = struct.unpack_from("<iB3xii", ch, end + 1)
        if ptype not in _EXR_TYPES or xs != 1 or ys != 1:
            raise ValueError("unsupported EXR channel type or subsampling")
        channels.append((ch[q:end].decode(), _EXR_TYPES[ptype]))
        q = end + 17
    comp = attrs["compression"][1][0]
    if comp not in _EXR_LINES:
        raise ValueError(f"unsupported EXR compression {comp} (NONE, RLE, ZIPS and ZIP are read)")
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    lines = _EXR_LINES[comp]
    nchunks = (h + lines - 1) // lines
    offsets = np.frombuffer(data, dtype="<u8", count=nchunks, offset=pos)
    line_bytes = sum(w * dt.itemsize for _, dt in channels)
    planes = {name: np.zeros((h, w), dtype=np.float32) for name, _ in channels}
    for off in offsets:
        off = int(off)
        y, size = struct.unpack_from("<ii", data, off)
        nl = min(lines, y1 + 1 - y)
        expect = nl * line_bytes
        chunk = data[off + 8:off + 8 + size]
        if size < expect:
            if comp in (EXR_ZIPS, EXR_ZIP):
                chunk = _exr_unpredict_deinterleave(zlib.decompress(chunk))
            elif comp == EXR_RLE:
                chunk = _exr_unpredict_deinterleave(_rle_decode(chunk, expect))
            else:
                raise ValueError("EXR: truncated uncompressed chunk")
        if len(chunk) != expect:
            raise ValueError("EXR: chunk size mismatch")
        p = 0
        for li in range(nl):
            row = y - y0 + li
            for name, dt in channels:
                planes[name][row] = np.frombuffer(chunk, dtype=dt, count=w, offset=p).astype(np.float32)
                p += w * dt.itemsize
    out = np.zeros((h, w, 4), dtype=np.float32)
    out[..., 3] = 1.0
    if "Y" in planes and not {"R", "G", "B"} & planes.keys():
        for k in range(3):
            out[..., k] = planes["Y"]
    for k, name in enumerate("RGBA"):
        if name in planes:
            out[..., k] = planes[name]
    return out


def read_exr(path) -> np.ndarray:
    return decode_exr(Path(path).read_bytes())


def write_exr(path, rgb, brightness: float = 1.0, flip_y: bool = False, compression: int = EXR_NONE,
              pixel_type: int = 1) -> Path:
    p = Path(path)
    p.write_bytes(encode_exr(rgb, brightness, flip_y, compression, pixel_type))
    return p
