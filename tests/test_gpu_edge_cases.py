"""Edge cases of the plain tracer against the oracle, through the C ABI, in reference mode and
configuration mode:

* an empty volume (all densities zero): every path escapes at its first segment without a
  lookup, and the image is the environment seen through the camera weight;
* a ragged image (19 x 7 = 133 pixels, not a multiple of the warp or of the launch shape);
* a grid two voxels thick whose extents (19 x 2 x 11) are not multiples of the 8^3 leaf, so
  partial leaves, the inclusive upper plane and out-of-grid stencil corners are exercised;
* a saturated volume (density 1 everywhere, so every interior lookup meets the majorant);
* one sample per pixel with both RNG stream layouts.

Decisions (vertex count, primary and shadow lookups, end code) must agree sample by sample as in
the main parity tests, and the image wherever they agree."""
import numpy as np
import pytest

from rtc8_gb300._lib import VptError
from rtc8_gb300.configs import VolumeSpec
from rtc8_gb300.renderer import Renderer, constant_environment

from ._scenes import small_config_mode, small_reference_mode
from .test_gpu_plain import DECISION_PARITY, _gpu_logged, _oracle

pytestmark = pytest.mark.gpu

END_ESCAPE = 1


def _volume(kind):
    if kind == "empty":
        return np.zeros((24, 24, 24), dtype=np.float32)
    if kind == "thin":
        return np.random.default_rng(11).random((19, 2, 11)).astype(np.float32)
    if kind == "saturated":
        return np.ones((16, 16, 16), dtype=np.float32)
    return np.random.default_rng(12).random((16, 16, 16)).astype(np.float32)  # ragged image


def _config(kind, mode):
    vox = _volume(kind)
    base = small_reference_mode(size=24) if mode == "reference" else small_config_mode(size=24)
    cfg = base.replace(volume=VolumeSpec(n=vox.shape[0], seed=1, octaves=1, sigma_t_max=20.0))
    if kind == "ragged":
        cfg = cfg.replace(width=19, height=7)
    return cfg, vox


def _run(cfg, vox, spp):
    env = constant_environment(cfg.env_constant if cfg.env_constant is not None else 0.5)
    g = _gpu_logged(cfg, vox, env, spp)
    o = _oracle(cfg, vox, env, spp)
    same = np.all(g["log"] == o["log"], axis=2)
    return g, o, same


@pytest.mark.parametrize("mode", ["reference", "config"])
@pytest.mark.parametrize("kind", ["empty", "ragged", "thin", "saturated"])
def test_edge_case_matches_oracle(cuda_device, kind, mode):
    cfg, vox = _config(kind, mode)
    g, o, same = _run(cfg, vox, spp=3)
    assert same.mean() >= DECISION_PARITY, f"identical decisions {same.mean():.5f}"
    pix_same = same.reshape(cfg.height, cfg.width, -1).all(axis=2)
    np.testing.assert_allclose(g["sum"][pix_same], o["sum"][pix_same], rtol=2e-3, atol=1e-6)
    assert g["errors"] == 0
    assert g["counters"]["samples"] == cfg.width * cfg.height * 3
    assert g["counters"]["lookups"] == int(g["log"][..., 1:3].astype(np.int64).sum())
    if kind == "empty":
        assert np.all(g["log"][..., 0] == 1) and np.all(g["log"][..., 1:3] == 0)
        assert np.all(g["log"][..., 3] == END_ESCAPE)
        assert g["sum"].min() > 0
    else:
        assert g["counters"]["lookups"] > 0


@pytest.mark.parametrize("streams", [0, 1])
def test_one_sample_per_pixel(cuda_device, streams):
    cfg, vox = _config("ragged", "config")
    cfg = cfg.replace(rng_stream_mode=streams)
    g, o, same = _run(cfg, vox, spp=1)
    assert same.mean() >= DECISION_PARITY
    if streams == 0:  # reference streams: the per-pixel states advance as in the oracle
        np.testing.assert_array_equal(g["rng"], o["rng"])
    pix_same = same.reshape(cfg.height, cfg.width, -1).all(axis=2)
    # the FP64 sums (the oracle keeps the running mean only for reference streams)
    np.testing.assert_allclose(g["sum"][pix_same], o["sum"][pix_same], rtol=2e-3, atol=1e-6)
    if streams == 0:
        np.testing.assert_allclose(g["mean"][pix_same], o["mean"][pix_same], rtol=2e-3, atol=1e-6)


def test_degenerate_volume_is_refused(cuda_device):
    r = Renderer(8, 8)
    with pytest.raises(VptError, match="bad arguments"):
        r.set_volume_dense(np.zeros((16, 1, 16), dtype=np.float32), 1.0 / 16, np.zeros(3, dtype=np.float32))
    with pytest.raises(VptError, match="bad arguments"):
        r.set_volume_dense(np.zeros((16, 16, 16), dtype=np.float32), 0.0, np.zeros(3, dtype=np.float32))
    r.close()
