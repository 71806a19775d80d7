"""The Hosek-Wilkie sky model: the committed per-band model states and the radiance formula the
GPU sky kernel restates (oracle/sky.py), against the reference library's own
arhosekskymodel_radiance at fixed view and sun angles (tests/golden/ref_hosek_kat.json, written
by the library built from the reference's sources)."""
import json
from pathlib import Path

import numpy as np
import pytest

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


STATES = Path(__file__).resolve().parent / "golden" / "ref_hosek_states.json"


def _needs_tables():
    if not sky.tables_available():
        pytest.skip("the sky-model tables were not generated (no reference checkout at build time)")


def test_cooked_states_match_reference_library():
    """States the product cooks from the model's tables equal the library's own
    arhosekskymodelstate_alloc_init at six further (elevation, turbidity, albedo) combinations,
    including turbidity 1 and 10, a grazing and a near-zenith sun, and the per-band albedo ramp."""
    _needs_tables()
    import math
    for e in json.loads(STATES.read_text())["entries"]:
        got = sky.states_for(math.radians(e["elevation_deg"]), e["turbidity"], e["albedo"])
        np.testing.assert_array_equal(got, np.asarray(e["states"], np.float32))
    for e in json.loads(sky.DATA.read_text())["entries"]:   # and the three stored ones
        got = sky.states_for(math.radians(e["elevation_deg"]), e["turbidity"], e["albedo"])
        np.testing.assert_array_equal(got, np.asarray(e["states"], np.float32))


def test_solar_disc_radiance_matches_reference_library():
    """The oracle's restatement of the direct solar radiance (piecewise cubic in elevation,
    turbidity and channel interpolation, limb darkening) against the library at texel elevations
    around the sun and angles inside the disc."""
    _needs_tables()
    tables = sky._coefficients()
    cmf = sky.cmf()
    for e in json.loads(STATES.read_text())["entries"]:
        for b, elev, gamma, ref in e["solar_kat"]:
            wl = min(max(float(cmf[48 + int(b)]), 320.0), 720.0)
            got = float(osky.solar_direct(tables, e["turbidity"], wl, elev, gamma, sky.SOLAR_RADIUS))
            assert got == pytest.approx(ref, rel=1e-7, abs=1e-12), (e["elevation_deg"], b, elev, gamma)


def test_sky_state_requests():
    """Any elevation works with the tables; turbidity outside [1, 10] is refused."""
    _needs_tables()
    from rtc8_gb300.configs import SkySpec
    st = sky.load_sky_state(SkySpec(turbidity=2.5, ground_albedo=-1.0), 37.0)
    assert st["states"].shape == (16, 122) and st["solar"].shape == (sky.SOLAR_FLOATS,)
    assert st["solar"][0] == pytest.approx(0.5)
    with pytest.raises(ValueError):
        sky.load_sky_state(SkySpec(turbidity=12.0), 20.0)
