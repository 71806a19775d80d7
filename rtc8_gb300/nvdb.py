"""NanoVDB grids (.nvdb files) as density volumes, over the C ABI.

The reference loads its volume with ``nanovdb::io::readGrid`` (grid 0 of the scene's ``volume``
file, renderer/renderer_scene.cpp:2158-2172, 2468) and hands the grid to
``Scene::allocateVolumeGrid`` (renderer/renderer_scene.cpp:491-537). Here the file's segment
headers and the grid's tree are read by the library's host code (csrc/vpt_nvdb.cu);
``Renderer.load_nvdb`` uploads the grid as the tracer's sparse leaves. Grids stored with the ZIP
codec are inflated here with zlib (the same ``compress`` stream that ext/nanovdb/nanovdb/util/
IO.h:257-276 writes) and passed to the library as an in-memory grid.
"""
from __future__ import annotations

import ctypes as C
import zlib
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import VptNanoVdbInfo, check

CODEC_NONE, CODEC_ZIP, CODEC_BLOSC = 0, 1, 2
GRID_TYPE_FLOAT = 1


def _info_dict(info: VptNanoVdbInfo) -> dict:
    d = {}
    for name, _ in VptNanoVdbInfo._fields_:
        v = getattr(info, name)
        if name == "name":
            v = v.decode()
        elif hasattr(v, "__len__"):
            v = list(v)
        d[name] = v
    return d


def file_info(path: str | Path, grid: int = 0) -> dict:
    """Metadata record of grid number `grid` of an .nvdb file (all segments counted)."""
    lib = _lib.load()
    info = VptNanoVdbInfo()
    check(lib.vpt_nvdb_file_info(str(path).encode(), grid, C.byref(info)), "vpt_nvdb_file_info")
    return _info_dict(info)


def list_grids(path: str | Path) -> list[dict]:
    """Metadata of every grid in the file, in file order."""
    first = file_info(path, 0)
    return [first] + [file_info(path, i) for i in range(1, first["grid_count"])]


def grid_index(path: str | Path, grid: int | str = 0) -> int:
    """Index of the grid named `grid` (the first one with that name, as io::readGrid by name,
    IO.h:632-660), or `grid` itself when it is an index."""
    if isinstance(grid, int):
        return grid
    for i, g in enumerate(list_grids(path)):
        if g["name"] == grid:
            return i
    raise KeyError(f"{path} holds no grid named {grid!r}")


def read_grid(path: str | Path, grid: int | str = 0) -> bytes:
    """The in-memory NanoVDB buffer of one grid of the file (inflated when ZIP-coded)."""
    idx = grid_index(path, grid)
    info = file_info(path, idx)
    with open(path, "rb") as f:
        f.seek(info["payload_offset"])
        if info["codec"] == CODEC_NONE:
            buf = f.read(info["grid_bytes"])
        elif info["codec"] == CODEC_ZIP:
            size = int(np.frombuffer(f.read(8), dtype="<u8")[0])
            buf = zlib.decompress(f.read(size))
        else:
            raise ValueError(f"{path}: grid {info['name']!r} uses codec {info['codec']} (BLOSC), which is not supported")
    if len(buf) != info["grid_bytes"]:
        raise ValueError(f"{path}: grid {info['name']!r} payload has {len(buf)} bytes, expected {info['grid_bytes']}")
    return buf


def grid_info(buf: bytes) -> dict:
    """Metadata of an in-memory grid, with the leaf-aligned extent a volume built from it holds."""
    lib = _lib.load()
    info = VptNanoVdbInfo()
    check(lib.vpt_nanovdb_grid_info(buf, len(buf), C.byref(info)), "vpt_nanovdb_grid_info")
    return _info_dict(info)


def decode_leaves(buf: bytes) -> tuple[np.ndarray, np.ndarray]:
    """The 8^3 leaves a volume built from this float grid holds: origins (n, 3) int32 index
    coordinates and values (n, 8, 8, 8) float32 indexed [x, y, z]."""
    lib = _lib.load()
    n = C.c_int64()
    check(lib.vpt_nanovdb_decode_leaves(buf, len(buf), 0, None, None, C.byref(n)), "vpt_nanovdb_decode_leaves")
    origins = np.zeros((n.value, 3), dtype=np.int32)
    values = np.zeros((n.value, 8, 8, 8), dtype=np.float32)
    check(lib.vpt_nanovdb_decode_leaves(buf, len(buf), n.value, _lib.ptr(origins, C.c_int32),
                                        _lib.ptr(values, C.c_float), C.byref(n)), "vpt_nanovdb_decode_leaves")
    return origins, values
