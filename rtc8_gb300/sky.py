"""Hosek-Wilkie sky-model states for the sky configurations.

The per-band model states (renderer_scene.cpp:555-592 computes them on the host with
arhosekskymodelstate_alloc_init) are precomputed for the (solar elevation, turbidity, ground
albedo) combinations the configurations use and stored in data/hosek_sky.json together with
the renderer's 16-band CIE CMF integrals (basic_types.cpp:195-249).
"""
from __future__ import annotations

import functools
import json
from pathlib import Path

import numpy as np

DATA = Path(__file__).resolve().parent / "data" / "hosek_sky.json"


@functools.lru_cache(maxsize=1)
def _table() -> dict:
    if not DATA.exists():
        raise RuntimeError(f"{DATA} is missing (generate it with tests/golden/make_golden.py)")
    return json.loads(DATA.read_text())


def available() -> list[tuple[float, float, float]]:
    return [(e["elevation_deg"], e["turbidity"], e["albedo"]) for e in _table()["entries"]]


def load_sky_state(spec, elevation_deg: float) -> dict:
    """States (16 x 122 floats), solar terms (16 x 7) and CMF set (65 floats) of a SkySpec."""
    for e in _table()["entries"]:
        if (abs(e["elevation_deg"] - elevation_deg) < 1e-6 and abs(e["turbidity"] - spec.turbidity) < 1e-6
                and abs(e["albedo"] - spec.ground_albedo) < 1e-6):
            return {"states": np.asarray(e["states"], dtype=np.float32),
                    "solar": np.asarray(e["solar"], dtype=np.float32),
                    "cmf": np.asarray(_table()["cmf"], dtype=np.float32)}
    raise KeyError(f"no precomputed sky state for elevation {elevation_deg}, turbidity {spec.turbidity}, "
                   f"albedo {spec.ground_albedo}; available: {available()}")
