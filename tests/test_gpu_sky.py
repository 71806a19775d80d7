"""The GPU sky texture (vpt_generate_sky, without the solar disc) against the oracle's float64
restatement of the reference's sky kernel (oracle/sky.py): the model radiance of 16 bands, CIE
XYZ, linear sRGB, the saturation push and the sea blend of the lower hemisphere. FP32 on the
device against FP64: texels agree to 2e-3 relative."""
import numpy as np
import pytest

from oracle import sky as osky
from rtc8_gb300 import sky
from rtc8_gb300.configs import C2, sun_direction
from rtc8_gb300.renderer import Renderer

pytestmark = pytest.mark.gpu


def test_sky_texture_matches_oracle(cuda_device):
    w, h = 96, 48
    st = sky.load_sky_state(C2.sky, 20.0)
    d = sun_direction(20.0, C2.sun_azimuth_deg)
    r = Renderer(8, 8)
    r.generate_sky(w, h, st["states"], st["solar"], st["cmf"], d, False)
    got = r.download_environment(w, h).astype(np.float64)
    ref = osky.sky_texture(w, h, st["states"], st["cmf"], d.astype(np.float32))
    assert np.all(np.isfinite(got)) and got.max() > 0
    close = np.isclose(got, ref, rtol=2e-3, atol=1e-6).all(axis=-1)
    assert close.mean() >= 0.995, f"texels within 2e-3: {close.mean():.4f}"
    # every texel within 1e-2, so an error confined to a band of rows cannot hide
    np.testing.assert_allclose(got, ref, rtol=1e-2, atol=1e-6)
    # both hemispheres (the sky and the mirrored, sea-blended lower half) on their own
    for half in (slice(0, h // 2), slice(h // 2, h)):
        np.testing.assert_allclose(got[half].mean(axis=(0, 1)), ref[half].mean(axis=(0, 1)), rtol=1e-3)
    r.close()
