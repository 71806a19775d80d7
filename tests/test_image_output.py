"""Image output of the headless loop on the CPU: the oracle's tone map + sRGB conversion against
the reference's own functions (sRGB_gamma_s and RGBSpectrum from common/basic_types.h, the
tone-map formula of post_process_kernels.cu:10-41 and the byte conversion of
common_host.cpp:517-568, evaluated by oracle/ref_kat_basic.cu), and the PNG / EXR writers
decoded back."""
import json
import struct
import zlib
from pathlib import Path

import numpy as np
import pytest

from oracle import orc
from rtc8_gb300 import image

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def basic():
    return json.loads((GOLDEN / "ref_basic_types.json").read_text())


def test_srgb_gamma_matches_reference(basic):
    out = orc.srgb_gamma(np.float32(basic["srgb_gamma_in"]))
    np.testing.assert_array_equal(out, np.float32(basic["srgb_gamma_out"]))


def test_tonemap_matches_reference(basic):
    mean = np.float32(basic["tonemap_mean_rgb"]).reshape(-1, 3)
    rgb, rgba = orc.tonemap(mean)
    np.testing.assert_array_equal(rgb.ravel(), np.float32(basic["tonemap_out_rgb"]))
    np.testing.assert_array_equal(rgba[:, :3].ravel(), np.uint8(basic["tonemap_srgb_bytes"]))
    assert np.all(rgba[:, 3] == 255)
    # without the gamma the bytes are the linear values
    _, lin = orc.tonemap(mean, srgb=False)
    assert np.all(lin[:, :3] <= rgba[:, :3])


def decode_png(data: bytes) -> np.ndarray:
    """Minimal decoder for the writer's output (8-bit RGBA, any of the five row filters)."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w = 8, b"", 0
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag, body = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        assert struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])[0] == zlib.crc32(tag + body) & 0xFFFFFFFF
        if tag == b"IHDR":
            w, h, depth, ctype = struct.unpack(">IIBB", body[:10])
            assert (depth, ctype) == (8, 6)
        elif tag == b"IDAT":
            idat += body
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, 1 + 4 * w)
    assert np.all(raw[:, 0] == 0)
    return raw[:, 1:].reshape(h, w, 4)


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    img = rng.integers(0, 256, size=(37, 53, 4), dtype=np.uint8)
    p = image.write_png(tmp_path / "000.png", img)
    np.testing.assert_array_equal(decode_png(p.read_bytes()), img)
    words = img.view("<u4").reshape(37, 53)
    np.testing.assert_array_equal(decode_png(image.encode_png(words)), img)


def test_exr_layout_and_values():
    rng = np.random.default_rng(2)
    rgb = rng.random((5, 7, 3)).astype(np.float32) * 4
    data = image.encode_exr(rgb, brightness=2.0, flip_y=True)
    assert struct.unpack("<ii", data[:8]) == (20000630, 2)
    pos, attrs = 8, {}
    while data[pos] != 0:
        end = data.index(b"\0", pos)
        name = data[pos:end].decode()
        tend = data.index(b"\0", end + 1)
        size = struct.unpack("<i", data[tend + 1:tend + 5])[0]
        attrs[name] = data[tend + 5:tend + 5 + size]
        pos = tend + 5 + size
    pos += 1
    assert attrs["compression"] == b"\0" and struct.unpack("<iiii", attrs["dataWindow"]) == (0, 0, 6, 4)
    ch, names, types = attrs["channels"], [], []
    q = 0
    while ch[q] != 0:  # name, then int32 pixel type, uint8 pLinear, 3 reserved, int32 x/y sampling
        end = ch.index(b"\0", q)
        names.append(ch[q:end].decode())
        types.append(struct.unpack("<iB3xii", ch[end + 1:end + 17]))
        q = end + 17
    assert names == ["A", "B", "G", "R"] and all(t == (1, 0, 1, 1) for t in types)  # HALF, 1x1
    offsets = np.frombuffer(data[pos:pos + 8 * 5], dtype="<u8")
    planes = {}
    for y, off in enumerate(offsets):
        yy, size = struct.unpack("<ii", data[off:off + 8])
        assert yy == y and size == 4 * 2 * 7
        line = np.frombuffer(data[off + 8:off + 8 + size], dtype="<f2").reshape(4, 7)
        for k, ch in enumerate("ABGR"):
            planes.setdefault(ch, []).append(line[k])
    got = np.stack([np.array(planes[c]) for c in "RGB"], axis=-1).astype(np.float32)
    expect = (2.0 * rgb)[::-1].astype(np.float16).astype(np.float32)
    np.testing.assert_array_equal(got, expect)
    assert np.all(np.array(planes["A"]) == 0)


@pytest.mark.parametrize("compression", [image.EXR_NONE, image.EXR_RLE, image.EXR_ZIPS, image.EXR_ZIP])
@pytest.mark.parametrize("pixel_type", [1, 2])
def test_exr_reader_round_trip(compression, pixel_type):
    rng = np.random.default_rng(4)
    rgb = (rng.random((37, 29, 3)) * 8).astype(np.float32)
    rgb[:5, :5] = 0.25  # runs for the RLE codec
    out = image.decode_exr(image.encode_exr(rgb, compression=compression, pixel_type=pixel_type))
    expect = rgb.astype(np.float16 if pixel_type == 1 else np.float32).astype(np.float32)
    np.testing.assert_array_equal(out[..., :3], expect)
    assert np.all(out[..., 3] == 0)  # the writer stores A = 0 where the image has no alpha


def _y_only_exr(y: np.ndarray) -> bytes:
    """A one-channel (Y, FLOAT) uncompressed scan-line file, built field by field."""
    h, w = y.shape
    chlist = b"Y\0" + struct.pack("<iB3xii", 2, 0, 1, 1) + b"\0"
    header = (struct.pack("<ii", 20000630, 2) + image._attr("channels", "chlist", chlist) +
              image._attr("compression", "compression", b"\0") +
              image._attr("dataWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)) +
              image._attr("displayWindow", "box2i", struct.pack("<iiii", 0, 0, w - 1, h - 1)) +
              image._attr("lineOrder", "lineOrder", b"\0") + b"\0")
    first = len(header) + 8 * h
    offs = np.arange(h, dtype="<u8") * np.uint64(8 + 4 * w) + np.uint64(first)
    body = b"".join(struct.pack("<ii", r, 4 * w) + y[r].astype("<f4").tobytes() for r in range(h))
    return header + offs.tobytes() + body


def test_exr_reader_gray_and_refusals():
    y = np.linspace(0, 2, 6 * 4, dtype=np.float32).reshape(6, 4)
    rgba = image.decode_exr(_y_only_exr(y))
    for k in range(3):
        np.testing.assert_array_equal(rgba[..., k], y)
    assert np.all(rgba[..., 3] == 1.0)  # no alpha channel: opaque
    data = bytearray(image.encode_exr(y[..., None], pixel_type=2))
    with pytest.raises(ValueError, match="magic"):
        image.decode_exr(b"\x00" * 16)
    tiled = bytearray(data)
    tiled[4:8] = struct.pack("<i", 2 | 0x200)
    with pytest.raises(ValueError, match="scan-line"):
        image.decode_exr(bytes(tiled))
    piz = bytearray(data)
    i = piz.index(b"compression\0compression\0") + len(b"compression\0compression\0") + 4
    piz[i] = 4  # PIZ
    with pytest.raises(ValueError, match="compression 4"):
        image.decode_exr(bytes(piz))
