"""GPU decision parity of the plain tracer at the parameters of the benchmarked workloads.

The small scenes of test_gpu_plain.py check every mode on 16^3-40^3 grids with a constant
environment. Here the tracer runs with the parameter sets that are timed:

* the 1024^2 sparse workload's scene at a reduced image: the 512^3 sparse fBm cloud generated on
  the device (checked bit for bit against the oracle's host generator), sigma_t max 200, albedo
  0.999, HG g 0.85, 32-voxel majorant cells, <= 256 bounces, sample-parallel streams, shadow-ray
  roulette 0.1, sun at 20 degrees plus the Hosek-Wilkie sky (turbidity 3, ground albedo 0.3) at
  its full 3200x1600 resolution;
* the stress workload's medium (two unioned clouds, threshold 0.78, sigma_t max 400, albedo
  0.9995, g 0.9, <= 1024 bounces, 64-voxel cells) on a 256^3 grid;
* the dense 64^3 workload at its full size (256^2 x 16 spp), in configuration mode and in the
  reference's own path rules;
* a strongly non-uniform environment (the sky plus a bright disc around the sun direction), so
  that the hierarchical importance walk, the environment pdf and the MIS weights run on a
  non-constant map (common_renderer_types.h:479-548, 2419-2458; renderer_kernel_common.h:297-403).

The environment texels come from the oracle's float64 sky restatement (oracle/sky.py) and are
given to both sides; the device sky kernel itself is compared with that restatement in
test_gpu_sky.py. Bar: >= 99.9% of samples with identical decisions (vertex count, primary and
shadow lookups, end code); where all of a pixel's samples agree, >= 99.9% of the pixels have FP64
sums within 2e-3, and their totals agree to 2e-4. The decision record does not hold two events
that can flip on the last bit of a float: a shadow ray's roulette at its last lookup (kill and
survival leave the same lookup count) and the environment texel an importance sample lands in
(a neighbouring texel gives the same lookups); on these long paths (hundreds of vertices, a
non-uniform sky) about 1e-4 of decision-identical pixels carry such a flip.
"""
import math

import numpy as np
import pytest

from oracle import orc
from oracle import sky as osky
from rtc8_gb300 import sky as psky
from rtc8_gb300.configs import C1, C1_REFERENCE_MODE, C2, C5, VolumeSpec, sun_direction
from rtc8_gb300.renderer import Renderer, setup_scene

pytestmark = pytest.mark.gpu

DECISION_PARITY = 0.999


def oracle_sky(cfg, width: int, height: int) -> np.ndarray:
    d = sun_direction(cfg.sun_elevation_deg, cfg.sun_azimuth_deg)
    st = psky.load_sky_state(cfg.sky, cfg.sun_elevation_deg, d)
    return osky.sky_texture(width, height, st["states"], st["cmf"], d.astype(np.float32)).astype(np.float32)


def add_sun_disc(env: np.ndarray, sun_dir, radius_deg: float, radiance: float) -> np.ndarray:
    """Adds `radiance` to every texel whose centre lies within `radius_deg` of `sun_dir`
    (texel rows are the polar angle from +y, columns phi as in from_polar_yup)."""
    h, w, _ = env.shape
    theta = math.pi * (np.arange(h) + 0.5) / h
    phi = 2 * math.pi * (np.arange(w) + 0.5) / w
    t, p = np.meshgrid(theta, phi, indexing="ij")
    dirs = np.stack([-np.sin(p) * np.sin(t), np.cos(t), np.cos(p) * np.sin(t)], axis=-1)
    cosang = dirs @ np.asarray(sun_dir, dtype=np.float64)
    out = env.copy()
    out[cosang >= math.cos(math.radians(radius_deg))] += np.float32(radiance)
    return out


def run_pair(cfg, vox, env, spp: int, device_volume: bool = False, stage: int = 0) -> dict:
    """Logged GPU launch (with per-warp leaf staging when `stage` > 0) and the oracle on the same
    scene; returns both results and the per-sample decision agreement."""
    import torch

    r = Renderer(cfg.width, cfg.height)
    r.set_leaf_staging(stage)
    if device_volume:
        setup_scene(r, cfg)                       # the product's own fBm generator
        got_vox = r.download_volume()
        assert np.array_equal(got_vox, vox), "device fBm differs from the oracle's generator"
        del got_vox
    else:
        setup_scene(r, cfg, volume=vox)
    r.set_environment_rgb(env)                    # the oracle's texels on both sides
    log = torch.zeros(cfg.width * cfg.height * spp * 4, dtype=torch.int32, device="cuda")
    r.launch_plain_logged(spp, log.data_ptr())
    r.synchronize()
    g = {"log": log.cpu().numpy().view(np.uint32).reshape(-1, spp, 4), "sum": r.download_sum()[0],
         "counters": r.counters(), "errors": r.device_errors(), "rng": r.rng_states()}
    r.close()
    sc = orc.scene_from_config(cfg, vox, env)
    rng = orc.seed_states(cfg.width, cfg.height, cfg.rng_seed)
    o = orc.render_plain(sc, rng, spp, log=True)
    o["rng"] = rng
    same = np.all(g["log"] == o["log"], axis=2)
    return {"gpu": g, "oracle": o, "same": same}


def check_parity(cfg, res, spp: int, min_vertices: int = 5) -> None:
    g, o, same = res["gpu"], res["oracle"], res["same"]
    frac = same.mean()
    assert frac >= DECISION_PARITY, f"identical decisions {frac:.5f} ({(~same).sum()} of {same.size} differ)"
    assert g["errors"] == 0
    assert o["log"][..., 0].max() >= min_vertices
    assert g["counters"]["samples"] == cfg.width * cfg.height * spp
    assert g["counters"]["lookups"] == int(g["log"][..., 1:3].astype(np.int64).sum())
    pix_same = same.reshape(cfg.height, cfg.width, -1).all(axis=2)
    close = np.isclose(g["sum"], o["sum"], rtol=2e-3, atol=1e-6).all(axis=-1)
    frac_close = close[pix_same].mean()
    assert frac_close >= 0.999, f"decision-identical pixels within 2e-3: {frac_close:.5f}"
    np.testing.assert_allclose(g["sum"][pix_same].sum(axis=0), o["sum"][pix_same].sum(axis=0), rtol=2e-4)
    if cfg.rng_stream_mode == 0:
        # per-pixel streams end where the oracle's end when every sample agreed
        assert np.mean(g["rng"][pix_same.reshape(-1)] == o["rng"][pix_same.reshape(-1)]) >= DECISION_PARITY


@pytest.fixture(scope="module")
def c2_volume():
    return orc.fbm_volume(C2.volume)


@pytest.fixture(scope="module")
def c2_sky():
    return oracle_sky(C2, C2.sky.width, C2.sky.height)


def test_sparse512_workload_parameters(cuda_device, c2_volume, c2_sky):
    """The 1024^2 sparse workload's scene, device-generated volume, at 256x256 x 4 spp."""
    cfg = C2.replace(width=256, height=256)
    spp = 4
    res = run_pair(cfg, c2_volume, c2_sky, spp, device_volume=True)
    check_parity(cfg, res, spp, min_vertices=20)
    o = res["oracle"]["log"]
    # the workload's features are exercised: long paths, shadow rays, the bounce cap is reachable
    assert o[..., 2].sum() > 0 and np.mean(o[..., 0] >= 10) > 0.05


def test_sparse512_workload_leaf_staging(cuda_device, c2_volume, c2_sky):
    """The same scene traced with per-warp leaf staging."""
    cfg = C2.replace(width=128, height=128)
    spp = 4
    res = run_pair(cfg, c2_volume, c2_sky, spp, stage=6)
    check_parity(cfg, res, spp, min_vertices=20)


def test_sparse512_workload_reference_streams(cuda_device, c2_volume, c2_sky):
    """The same scene with the reference's per-pixel streams (sequential samples per pixel)."""
    cfg = C2.replace(width=96, height=96, rng_stream_mode=0)
    spp = 2
    res = run_pair(cfg, c2_volume, c2_sky, spp)
    check_parity(cfg, res, spp, min_vertices=20)


def test_stress_workload_parameters(cuda_device):
    """The stress workload's medium (two unioned clouds, sigma_t max 400, albedo 0.9995, g 0.9,
    <= 1024 bounces, 64-voxel cells) on a 256^3 grid, at 256x256 x 4 spp."""
    vol = VolumeSpec(n=256, seed=C5.volume.seed, octaves=C5.volume.octaves, threshold=C5.volume.threshold,
                     sigma_t_max=C5.volume.sigma_t_max, union_seed=C5.volume.union_seed)
    cfg = C5.replace(width=256, height=256, volume=vol)
    vox = orc.fbm_volume(vol)
    env = oracle_sky(cfg, 1600, 800)
    spp = 4
    res = run_pair(cfg, vox, env, spp, device_volume=True)
    check_parity(cfg, res, spp, min_vertices=50)


@pytest.mark.parametrize("cfg", [C1, C1_REFERENCE_MODE], ids=["config_mode", "reference_mode"])
def test_dense64_workload_full_size(cuda_device, cfg):
    """The dense 64^3 workload at its full size: 256x256 x 16 spp."""
    vox = orc.fbm_volume(cfg.volume)
    env = np.full((32, 64, 3), cfg.env_constant, dtype=np.float32)
    res = run_pair(cfg, vox, env, cfg.spp, device_volume=True)
    check_parity(cfg, res, cfg.spp, min_vertices=10)


@pytest.mark.parametrize("mode", ["reference", "config"])
def test_nonuniform_environment_importance_walk(cuda_device, mode):
    """Environment = the Hosek-Wilkie sky plus a disc 1e3 brighter around the sun direction:
    NEE samples the disc through the hierarchical walk and escaping paths weigh it by MIS."""
    base = C1_REFERENCE_MODE if mode == "reference" else C1
    cfg = base.replace(width=128, height=128, volume=VolumeSpec(n=48, seed=7, octaves=4, sigma_t_max=12.0))
    sky_cfg = C2.replace(sun_elevation_deg=20.0)
    env = add_sun_disc(oracle_sky(sky_cfg, 1024, 512), sun_direction(20.0, sky_cfg.sun_azimuth_deg), 3.0, 500.0)
    assert env.max() / np.median(env) > 1e3
    vox = orc.fbm_volume(cfg.volume)
    spp = 8
    res = run_pair(cfg, vox, env, spp, device_volume=True)
    check_parity(cfg, res, spp)
    # the disc carries most of the environment's importance (luminance x sin(theta)), so the
    # walk picks it for most NEE samples
    lum = env @ np.array([0.2126729, 0.7151522, 0.0721750], np.float32)
    sin_t = np.sin(math.pi * (np.arange(env.shape[0]) + 0.5) / env.shape[0])[:, None]
    disc = lum > 100.0
    assert (lum * sin_t)[disc].sum() / (lum * sin_t).sum() > 0.5
