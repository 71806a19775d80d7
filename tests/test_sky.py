"""The Hosek-Wilkie sky model: the committed per-band model states and the radiance formula the
GPU sky kernel restates (oracle/sky.py), against the reference library's own
arhosekskymodel_radiance at fixed view and sun angles (tests/golden/ref_hosek_kat.json, written
by the library built from the reference's sources)."""
import json
from pathlib import Path

import numpy as np

from oracle import sky as osky
from rtc8_gb300 import sky
from rtc8_gb300.configs import C2

GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_hosek_kat.json"


def test_hosek_radiance_matches_reference_library():
    kat = json.loads(GOLDEN.read_text())
    assert (kat["elevation_deg"], kat["turbidity"], kat["albedo"]) == (20, 3, 0.3)
    st = sky.load_sky_state(C2.sky, 20.0)
    cmf = np.asarray(st["cmf"], dtype=np.float64)
    rows = np.asarray(kat["band_theta_gamma_radiance"], dtype=np.float64)
    assert rows.shape == (216, 4)
    for b, theta, gamma, ref in rows:
        band = osky.unpack_state(st["states"][int(b)])
        wl = min(max(float(cmf[48 + int(b)]), 320.0), 720.0)
        got = float(osky.sky_radiance(band, theta, gamma, wl))
        assert abs(got - ref) <= 2e-5 * abs(ref) + 1e-9, (b, theta, gamma, got, ref)
