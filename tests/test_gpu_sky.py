"""The GPU sky texture (vpt_generate_sky) against the oracle's float64 restatement of the
reference's sky kernel (oracle/sky.py): the model radiance of 16 bands, CIE XYZ, linear sRGB, the
saturation push, the sea blend of the lower hemisphere and, optionally, the solar disc with the
direct solar radiance at each disc texel's elevation. The model states come from the product's
cooking of the model tables (compared with the reference library on the CPU, tests/test_sky.py).
FP32 on the device against FP64: texels agree to 2e-3 relative, every texel to 1e-2."""
import math

import numpy as np
import pytest

from oracle import sky as osky
from rtc8_gb300 import sky
from rtc8_gb300.configs import C2, SkySpec, sun_direction
from rtc8_gb300.renderer import Renderer

pytestmark = pytest.mark.gpu


def _device_sky(w, h, spec, elevation, azimuth, disc):
    d = sun_direction(elevation, azimuth)
    st = sky.load_sky_state(spec, elevation, d)
    r = Renderer(8, 8)
    r.generate_sky(w, h, st["states"], st["solar"], st["cmf"], d, disc)
    got = r.download_environment(w, h).astype(np.float64)
    r.close()
    return got, st, d


@pytest.mark.parametrize("elevation,turbidity,albedo", [(20.0, 3.0, 0.3), (5.0, 2.0, 0.1), (45.0, 6.5, -1.0),
                                                        (70.0, 9.3, 0.8)])
def test_sky_texture_matches_oracle(cuda_device, elevation, turbidity, albedo):
    if (elevation, turbidity, albedo) != (20.0, 3.0, 0.3) and not sky.tables_available():
        pytest.skip("the sky-model tables were not generated")
    w, h = 96, 48
    spec = SkySpec(turbidity=turbidity, ground_albedo=albedo)
    got, st, d = _device_sky(w, h, spec, elevation, C2.sun_azimuth_deg, False)
    ref = osky.sky_texture(w, h, st["states"], st["cmf"], d.astype(np.float32))
    assert np.all(np.isfinite(got)) and got.max() > 0
    close = np.isclose(got, ref, rtol=2e-3, atol=1e-6).all(axis=-1)
    assert close.mean() >= 0.995, f"texels within 2e-3: {close.mean():.4f}"
    # every texel within 1e-2, so an error confined to a band of rows cannot hide
    np.testing.assert_allclose(got, ref, rtol=1e-2, atol=1e-6)
    # both hemispheres (the sky and the mirrored, sea-blended lower half) on their own
    for half in (slice(0, h // 2), slice(h // 2, h)):
        np.testing.assert_allclose(got[half].mean(axis=(0, 1)), ref[half].mean(axis=(0, 1)), rtol=1e-3)


@pytest.mark.parametrize("elevation,turbidity", [(20.0, 3.0), (8.0, 5.5), (55.0, 2.0)])
def test_solar_disc_matches_oracle(cuda_device, elevation, turbidity):
    """The disc texels (within 0.255 degrees of the sun) of the reference's full 3200 x 1600 sky
    texture carry the limb-darkened direct solar radiance evaluated at their own elevation."""
    if not sky.tables_available():
        pytest.skip("the sky-model tables were not generated")
    w, h = 3200, 1600
    spec = SkySpec(turbidity=turbidity, ground_albedo=-1.0, include_solar_disc=True)
    got, st, d = _device_sky(w, h, spec, elevation, 120.0, True)
    # a window of texels around the sun
    theta = math.acos(float(np.float32(d[1])))
    phi = math.atan2(-float(d[0]), float(d[2])) % (2 * math.pi)
    cy, cx = int(theta / math.pi * h), int(phi / (2 * math.pi) * w)
    win = (cy - 12, cy + 12, cx - 12, cx + 12)
    disc = {"tables": sky._coefficients(), "turbidity": turbidity}
    ref = osky.sky_texture(w, h, st["states"], st["cmf"], d.astype(np.float32), disc=disc, window=win)
    sub = got[win[0]:win[1], win[2]:win[3]]
    lum = sub @ np.array([0.2126729, 0.7151522, 0.0721750])
    assert (lum > 50 * np.median(lum)).sum() >= 8          # the disc is there and bright
    # The renderer takes the view-sun angle as acos of a float32 dot product; inside the disc that
    # cosine takes only a few dozen float32 values, and one step of it moves the limb-darkened
    # radiance by percents. Every texel lies within 2e-3 of the oracle evaluated at the float32
    # cosine or at most 2 float32 steps away from it, and most texels match the rounded cosine.
    near32 = osky.sky_texture(w, h, st["states"], st["cmf"], d.astype(np.float32), disc=disc, window=win,
                              cos_gamma_ulps=0)
    shifted = [osky.sky_texture(w, h, st["states"], st["cmf"], d.astype(np.float32), disc=disc, window=win,
                                cos_gamma_ulps=k) for k in (-2, -1, 1, 2)]
    lo = np.minimum.reduce([ref, near32] + shifted)
    hi = np.maximum.reduce([ref, near32] + shifted)
    assert np.all(sub >= lo * (1 - 2e-3) - 1e-6) and np.all(sub <= hi * (1 + 2e-3) + 1e-6)
    near = np.isclose(sub, near32, rtol=2e-3, atol=1e-6).all(axis=-1)
    assert near.mean() >= 0.97, f"texels within 2e-3 of the float32-cosine oracle: {near.mean():.4f}"
