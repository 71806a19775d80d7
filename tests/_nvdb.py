"""Helpers of the NanoVDB tests: the committed .nvdb fixtures and the reference's reading of them
(tests/golden/nvdb, written by tests/golden/make_golden.py with NanoVDB 32.3)."""
from __future__ import annotations

import gzip
import json
import shutil
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden" / "nvdb"


def reference() -> dict:
    return json.loads((GOLDEN / "ref_nvdb_files.json").read_text())


def fixture_path(name: str, tmp_dir: Path) -> Path:
    """Path of fixture `name` (.nvdb), unpacked into tmp_dir when it is stored gzip-compressed."""
    plain = GOLDEN / name
    if plain.exists():
        return plain
    out = Path(tmp_dir) / name
    if not out.exists():
        with gzip.open(GOLDEN / (name + ".gz"), "rb") as src, open(out, "wb") as dst:
            shutil.copyfileobj(src, dst)
    return out


def voxel_hash(x: np.ndarray, y: np.ndarray, z: np.ndarray, v: np.ndarray) -> np.ndarray:
    """The generator's order-independent checksum term of each voxel (uint64, wrapping)."""
    u = lambda a: np.asarray(a, dtype=np.int64).astype(np.uint32).astype(np.uint64)  # noqa: E731
    key = (u(x) * np.uint64(73856093)) ^ (u(y) * np.uint64(19349663)) ^ (u(z) * np.uint64(83492791))
    bits = np.asarray(v, dtype=np.float32).view(np.uint32).astype(np.uint64)
    with np.errstate(over="ignore"):
        return (key | np.uint64(1)) * (bits + np.uint64(0x9E3779B97F4A7C15))


def dense_extent(origins: np.ndarray, values: np.ndarray, lo, hi) -> np.ndarray:
    """Dense voxels of the leaf-aligned extent [lo, hi) (x-major), 0 where no leaf is stored."""
    lo = np.asarray(lo)
    shape = tuple(int(h - l) for l, h in zip(lo, hi))
    out = np.zeros(shape, dtype=np.float32)
    for o, v in zip(origins, values):
        x, y, z = (int(c) for c in (o - lo))
        out[x:x + 8, y:y + 8, z:z + 8] = v
    return out


def lookup(dense: np.ndarray, lo, coords: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """Values of the dense extent at index coordinates (n, 3) and a mask of those inside it."""
    rel = np.asarray(coords) - np.asarray(lo)
    inside = np.all((rel >= 0) & (rel < np.array(dense.shape)), axis=1)
    vals = np.zeros(len(rel), dtype=np.float32)
    r = rel[inside]
    vals[inside] = dense[r[:, 0], r[:, 1], r[:, 2]]
    return vals, inside
