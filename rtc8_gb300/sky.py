"""Hosek-Wilkie sky-model states for the sky environments.

The reference computes, every frame and for each of its 16 spectral bands, the model state of the
Hosek-Wilkie 2013 spectral sky (ext/hosek_wilkie_2013, arhosekskymodelstate_alloc_init) from the
sun direction, the turbidity and a per-band ground albedo, and uploads it with the model's solar
coefficient tables (renderer/renderer_scene.cpp:86-125, 555-592). This module does the same on
the host for any solar elevation, turbidity in [1, 10] and albedo:

* the configuration and radiance of each 40 nm channel are the model's published cooking: a
  quintic Bezier in (elevation / (pi / 2))^(1/3) over the dataset's six control points, blended
  linearly between the two neighbouring integer turbidities and between ground albedo 0 and 1;
* the solar disc is evaluated on the device per texel from the model's piecewise-cubic solar
  tables (45 pieces per turbidity) and its limb-darkening polynomials, so the states carry the
  coefficient tables of the two turbidities around the requested one.

The model's coefficient tables come from data/hosek_tables.bin, which rtc8_gb300/build.py
generates from the model's source in the reference checkout. Without that file only the
(elevation, turbidity, albedo) combinations stored in data/hosek_sky.json (states computed by the
same library) are available, and any other request raises.
"""
from __future__ import annotations

import functools
import json
import math
from pathlib import Path

import numpy as np

DATA = Path(__file__).resolve().parent / "data" / "hosek_sky.json"
TABLES = Path(__file__).resolve().parent / "data" / "hosek_tables.bin"

BANDS = 16
CHANNELS = 11                  # 320, 360, ..., 720 nm
STATE_FLOATS = 122             # configs[11][9], radiances[11], sky emission correction[11], solar radius
SOLAR_PIECES, SOLAR_ORDER = 45, 4
SOLAR_TABLE = SOLAR_PIECES * SOLAR_ORDER               # coefficients per channel and turbidity
# Device solar layout: turbidity weight, then per channel the tables of the two turbidities around
# the requested one, then the 6 limb-darkening coefficients per channel.
SOLAR_FLOATS = 1 + CHANNELS * 2 * SOLAR_TABLE + CHANNELS * 6
SOLAR_RADIUS = math.radians(0.51) / 2.0                # TERRESTRIAL_SOLAR_RADIUS of the model


@functools.lru_cache(maxsize=1)
def _table() -> dict:
    if not DATA.exists():
        raise RuntimeError(f"{DATA} is missing")
    return json.loads(DATA.read_text())


@functools.lru_cache(maxsize=1)
def _coefficients() -> dict | None:
    """The model's tables from data/hosek_tables.bin, or None when the file was not generated."""
    if not TABLES.exists():
        return None
    raw = TABLES.read_bytes()
    if raw[:6] != b"HOSEK1":
        raise RuntimeError(f"{TABLES} is not a sky-model table file")
    v = np.frombuffer(raw, dtype="<f8", offset=8)
    sizes = [("config", 1080), ("radiance", 120), ("solar", 1800), ("limb", 6)]
    if len(v) != CHANNELS * sum(n for _, n in sizes):
        raise RuntimeError(f"{TABLES} has an unexpected size")
    out, off = {}, 0
    for name, n in sizes:
        out[name] = v[off: off + CHANNELS * n].reshape(CHANNELS, n)
        off += CHANNELS * n
    return out


def tables_available() -> bool:
    return _coefficients() is not None


def cmf() -> np.ndarray:
    """The renderer's 16-band CIE 1931 CMF integrals: xs, ys, zs, centre wavelengths, integral."""
    return np.asarray(_table()["cmf"], dtype=np.float32)


def _bezier(points: np.ndarray, t: float) -> np.ndarray:
    """Quintic Bezier over six control points (last axis = point index)."""
    s = 1.0 - t
    return (math.pow(s, 5.0) * points[..., 0] + 5.0 * math.pow(s, 4.0) * t * points[..., 1] +
            10.0 * math.pow(s, 3.0) * math.pow(t, 2.0) * points[..., 2] +
            10.0 * math.pow(s, 2.0) * math.pow(t, 3.0) * points[..., 3] +
            5.0 * s * math.pow(t, 4.0) * points[..., 4] + math.pow(t, 5.0) * points[..., 5])


def model_state(solar_elevation: float, turbidity: float, albedo: float) -> tuple[np.ndarray, np.ndarray]:
    """Per-channel configurations (11 x 9) and radiances (11) in float64: the model's cooking
    (ArHosekSkyModel_CookConfiguration / _CookRadianceConfiguration) for an elevation in radians."""
    c = _coefficients()
    if c is None:
        raise RuntimeError(f"{TABLES} is missing: generate it with rtc8_gb300/build.py where the reference is")
    if not 1.0 <= turbidity <= 10.0 or not 0.0 <= albedo <= 1.0:
        raise ValueError("turbidity must lie in [1, 10] and albedo in [0, 1]")
    it = int(turbidity)
    rem = turbidity - it
    t = math.pow(solar_elevation / (math.pi / 2.0), 1.0 / 3.0)
    cfg = c["config"].reshape(CHANNELS, 2, 10, 6, 9)
    rad = c["radiance"].reshape(CHANNELS, 2, 10, 6)

    def cook(a0_lo, a1_lo, a0_hi, a1_hi):
        v = (1.0 - albedo) * (1.0 - rem) * _bezier(a0_lo, t)
        v = v + albedo * (1.0 - rem) * _bezier(a1_lo, t)
        if it == 10:
            return v
        v = v + (1.0 - albedo) * rem * _bezier(a0_hi, t)
        return v + albedo * rem * _bezier(a1_hi, t)

    hi = min(it, 9)
    configs = cook(np.moveaxis(cfg[:, 0, it - 1], 1, 2), np.moveaxis(cfg[:, 1, it - 1], 1, 2),
                   np.moveaxis(cfg[:, 0, hi], 1, 2), np.moveaxis(cfg[:, 1, hi], 1, 2))
    radiances = cook(rad[:, 0, it - 1], rad[:, 1, it - 1], rad[:, 0, hi], rad[:, 1, hi])
    return configs, radiances


def band_albedo(ground_albedo: float, band: int) -> float:
    """A negative ground albedo selects the renderer's per-band ramp (renderer_scene.cpp:576)."""
    return ground_albedo if ground_albedo >= 0 else 0.5 * (1.0 - (band + 0.5) / BANDS)


def solar_elevation_of(sun_dir) -> float:
    """renderer_scene.cpp:570: 0.5 pi - acos(clamp(dir.y)), in float as the renderer computes it."""
    y = np.float32(min(max(float(np.float32(sun_dir[1])), -1.0), 1.0))
    return float(np.float32(0.5 * np.pi) - np.arccos(y, dtype=np.float32))


def solar_table(turbidity: float) -> np.ndarray:
    """Device solar layout (SOLAR_FLOATS floats) for a turbidity: the weight of the upper turbidity,
    the piecewise-cubic tables of the lower and upper turbidity per channel, the limb-darkening
    coefficients per channel (analytic_sky_kernels.cu:69-191 reads the same tables)."""
    c = _coefficients()
    lo = int(turbidity) - 1
    frac = turbidity - (lo + 1)
    if lo == 9:
        lo, frac = 8, 1.0
    sol = c["solar"].reshape(CHANNELS, 10, SOLAR_TABLE)
    out = np.empty(SOLAR_FLOATS, dtype=np.float32)
    out[0] = frac
    out[1: 1 + CHANNELS * 2 * SOLAR_TABLE] = sol[:, lo: lo + 2].reshape(-1)
    out[1 + CHANNELS * 2 * SOLAR_TABLE:] = c["limb"].reshape(-1)
    return out


def states_for(solar_elevation: float, turbidity: float, ground_albedo: float) -> np.ndarray:
    """Model states of the 16 bands (16 x STATE_FLOATS float32), as the renderer uploads them."""
    out = np.empty((BANDS, STATE_FLOATS), dtype=np.float32)
    for b in range(BANDS):
        configs, radiances = model_state(solar_elevation, turbidity, band_albedo(ground_albedo, b))
        out[b, :99] = configs.reshape(-1)
        out[b, 99:110] = radiances
        out[b, 110:121] = 1.0
        out[b, 121] = SOLAR_RADIUS
    return out


def available() -> list[tuple[float, float, float]]:
    return [(e["elevation_deg"], e["turbidity"], e["albedo"]) for e in _table()["entries"]]


def _stored(spec, elevation_deg: float):
    for e in _table()["entries"]:
        if (abs(e["elevation_deg"] - elevation_deg) < 1e-6 and abs(e["turbidity"] - spec.turbidity) < 1e-6
                and abs(e["albedo"] - spec.ground_albedo) < 1e-6):
            return np.asarray(e["states"], dtype=np.float32)
    return None


def load_sky_state(spec, elevation_deg: float, sun_dir=None) -> dict:
    """States (16 x 122), solar layout (SOLAR_FLOATS) and CMF set (65 floats) of a SkySpec at a
    solar elevation in degrees (the sun direction, when given, sets the elevation exactly as the
    renderer derives it)."""
    if tables_available():
        elev = solar_elevation_of(sun_dir) if sun_dir is not None else math.radians(elevation_deg)
        return {"states": states_for(elev, spec.turbidity, spec.ground_albedo), "solar": solar_table(spec.turbidity),
                "cmf": cmf()}
    stored = _stored(spec, elevation_deg)
    if stored is None:
        raise KeyError(f"no sky state for elevation {elevation_deg}, turbidity {spec.turbidity}, albedo "
                       f"{spec.ground_albedo}: {TABLES} was not generated and the stored states cover only "
                       f"{available()}")
    if getattr(spec, "include_solar_disc", False):
        raise RuntimeError(f"{TABLES} is missing: the solar disc needs the model's solar tables (generate them "
                           "with rtc8_gb300/build.py where the reference is)")
    return {"states": stored, "solar": np.zeros(SOLAR_FLOATS, dtype=np.float32), "cmf": cmf()}
