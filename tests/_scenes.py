"""Small seeded scenes shared by the oracle and GPU tests."""
from __future__ import annotations

import numpy as np

from rtc8_gb300.configs import C1, C1_REFERENCE_MODE, SceneConfig, VolumeSpec


def fbm_numpy(n: int, seed: int, octaves: int, lacunarity: float, gain: float, base_frequency: float,
              threshold: float = 0.0) -> np.ndarray:
    """Numpy restatement of the device fBm generator (integer lattice hash + quintic value noise),
    used to check the generator and to give the CPU tests a volume."""
    M = np.uint32(0xFFFFFFFF)

    def lattice(ix, iy, iz, s):
        with np.errstate(over="ignore"):
            h = np.uint32(s) * np.uint32(0x9E3779B1)
            for c in (ix, iy, iz):
                h = h ^ (c.astype(np.uint32) * np.uint32(0x85EBCA77))
                h = ((h << np.uint32(13)) | (h >> np.uint32(19))) * np.uint32(0xC2B2AE3D)
            h = h ^ (h >> np.uint32(16))
            h = h * np.uint32(0x7FEB352D)
            h = h ^ (h >> np.uint32(15))
            h = h * np.uint32(0x846CA68B)
            h = h ^ (h >> np.uint32(16))
        return (h >> np.uint32(8)).astype(np.float32) * np.float32(1.0 / 16777216.0)

    def fade(t):
        return t * t * t * (t * (t * np.float32(6) - np.float32(15)) + np.float32(10))

    def noise(x, y, z, s):
        fx, fy, fz = np.floor(x), np.floor(y), np.floor(z)
        ix, iy, iz = fx.astype(np.int32), fy.astype(np.int32), fz.astype(np.int32)
        wx, wy, wz = fade(x - fx), fade(y - fy), fade(z - fz)
        c = {(a, b, d): lattice(ix + a, iy + b, iz + d, s) for a in (0, 1) for b in (0, 1) for d in (0, 1)}
        lerp = lambda a, b, w: a + w * (b - a)
        x00 = lerp(c[0, 0, 0], c[1, 0, 0], wx)
        x10 = lerp(c[0, 1, 0], c[1, 1, 0], wx)
        x01 = lerp(c[0, 0, 1], c[1, 0, 1], wx)
        x11 = lerp(c[0, 1, 1], c[1, 1, 1], wx)
        return lerp(lerp(x00, x10, wy), lerp(x01, x11, wy), wz)

    idx = (np.arange(n, dtype=np.float32) + np.float32(0.5)) / np.float32(n)
    px, py, pz = np.meshgrid(idx, idx, idx, indexing="ij")
    freq, amp = np.float32(base_frequency), np.float32(1.0)
    total = np.zeros((n, n, n), dtype=np.float32)
    norm = np.float32(0.0)
    for o in range(octaves):
        total += amp * noise(px * freq, py * freq, pz * freq, (seed + 1013 * o) & 0xFFFFFFFF)
        norm += amp
        amp *= np.float32(gain)
        freq *= np.float32(lacunarity)
    v = total / norm
    lo, hi = v.min(), v.max()
    r = (v - lo) * (np.float32(1.0) / (hi - lo))
    if threshold > 0:
        r = np.where(r > threshold, (r - np.float32(threshold)) / np.float32(1 - threshold), np.float32(0))
    return r.astype(np.float32)


def small_reference_mode(size: int = 32, n: int = 32, schlick_k: float = 0.0, sigma: float = 20.0,
                         albedo: float = 0.99) -> SceneConfig:
    return C1_REFERENCE_MODE.replace(width=size, height=size, spp=2,
                                     volume=VolumeSpec(n=n, seed=3, octaves=4, sigma_t_max=sigma),
                                     phase_param=schlick_k, albedo=albedo)


def small_config_mode(size: int = 32, n: int = 32, g: float = 0.8, majorant_mode: int = 1) -> SceneConfig:
    return C1.replace(width=size, height=size, spp=2, volume=VolumeSpec(n=n, seed=3, octaves=4, sigma_t_max=20.0),
                      phase_param=g, majorant_mode=majorant_mode)


def volume_for(cfg: SceneConfig) -> np.ndarray:
    v = cfg.volume
    a = fbm_numpy(v.n, v.seed, v.octaves, v.lacunarity, v.gain, v.base_frequency, v.threshold)
    if v.union_seed is None:
        return a
    return np.maximum(a, fbm_numpy(v.n, v.union_seed, v.octaves, v.lacunarity, v.gain, v.base_frequency, v.threshold))
