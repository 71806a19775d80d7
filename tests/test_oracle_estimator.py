"""Analytic checks of the oracle's end-to-end estimator (the reference has no golden images)."""
import math

import numpy as np
import pytest

from oracle import orc

# Camera looking down -z from z = 3 at a box [-0.5, 0.5]^3 (identity orientation).
CAM = dict(cam_aspect=1.0, cam_fovy=math.radians(30.0), cam_pos=[0.0, 0.0, 3.0], cam_quat=[0.0, 0.0, 0.0, 1.0])


def _sensor_weight(w, h, fovy, aspect=1.0):
    """Per-pixel E[|z|^3 * sensor area] of the reference camera (optix_pathtracing_kernels.cu:43-55, 77)."""
    vh = 2 * math.tan(fovy * 0.5)
    vw = aspect * vh
    ss = 64
    out = np.zeros((h, w))
    for py in range(h):
        for px in range(w):
            fx = (px + (np.arange(ss) + 0.5) / ss) / w
            fy = (py + (np.arange(ss) + 0.5) / ss) / h
            X, Y = np.meshgrid(vw * (-0.5 + fx), vh * (0.5 - fy))
            z = 1.0 / np.sqrt(X ** 2 + Y ** 2 + 1.0)
            out[py, px] = np.mean(z ** 3) * vw * vh
    return out


def test_furnace_constant_environment():
    """Albedo 1 medium under a constant environment: every pixel sees exactly the environment."""
    n = 8
    vox = np.full((n, n, n), 1.0, np.float32)
    env = np.full((16, 32, 3), 0.5, np.float32)
    W = H = 4
    sc = orc.make_scene(voxels=vox, voxel_size=1.0 / n, origin=[-0.5, -0.5, -0.5], density_coeff=3.0, albedo=1.0,
                        phase_kind=1, phase_param=0.5, env_rgb=env, width=W, height=H, rr_start=1, majorant_mode=0,
                        **CAM)
    rng = orc.seed_states(W, H, 11)
    spp = 4096
    res = orc.render_plain(sc, rng, spp)
    img = res["sum"][..., 1] / spp
    expect = 0.5 * _sensor_weight(W, H, CAM["cam_fovy"])
    np.testing.assert_allclose(img, expect, rtol=0.03)


@pytest.mark.parametrize("mode", [0, 1])
def test_pure_absorber_transmittance(mode):
    """Albedo 0: a pixel sees the environment times exp(-optical depth) along its primary ray."""
    n = 16
    vox = np.full((n, n, n), 1.0, np.float32)
    vox[:, :, : n // 2] = 0.25  # two slabs so the majorant grid has different cells
    env = np.full((16, 32, 3), 1.0, np.float32)
    sigma = 2.0
    W = H = 1
    cam = dict(CAM, cam_fovy=math.radians(2.0))
    cells, g = orc.majorants(vox)
    sc = orc.make_scene(voxels=vox, voxel_size=1.0 / n, origin=[-0.5, -0.5, -0.5], density_coeff=sigma, albedo=0.0,
                        phase_kind=0, phase_param=0.0, env_rgb=env, width=W, height=H, rr_start=1,
                        majorant_mode=mode, **cam)
    rng = orc.seed_states(W, H, 5)
    spp = 40000
    res = orc.render_plain(sc, rng, spp)
    est = res["sum"][0, 0, 1] / spp
    # optical depth along the axis ray z = 3 -> -3 through the trilinear field (background 0)
    t = np.linspace(-0.5, 0.5, 200001)
    idx = (0.5 - t) * n  # index coordinate along z for the ray travelling towards -z
    i0 = np.floor(idx).astype(int)
    w = idx - i0
    zline = vox[n // 2, n // 2, :]  # x = y = 0 maps to index 8 exactly: no x/y interpolation
    def v(i):
        return np.where((i >= 0) & (i < n), zline[np.clip(i, 0, n - 1)], 0.0)
    rho = v(i0) + w * (v(i0 + 1) - v(i0))
    tau = sigma * np.trapezoid(rho, t)
    sensor = _sensor_weight(1, 1, cam["cam_fovy"])[0, 0]
    expect = sensor * math.exp(-tau)
    se = math.sqrt(expect * (sensor - expect) / spp)
    assert abs(est - expect) < 4 * se + 1e-4 * expect


@pytest.mark.parametrize("mode", [0, 1])
def test_shadow_roulette_is_unbiased(mode):
    """Russian roulette on shadow-ray visibility (configuration mode) leaves the expectation of
    the image unchanged: the same scene with and without it, from independent streams, agrees
    within 4 standard errors of the difference of the two means (batch means estimate them)."""
    n = 8
    rng0 = np.random.default_rng(3)
    vox = (0.3 + rng0.random((n, n, n))).astype(np.float32)
    env = np.full((16, 32, 3), 0.3, np.float32)
    W = H = 4
    def render(thr, seed):
        sc = orc.make_scene(voxels=vox, voxel_size=1.0 / n, origin=[-0.5, -0.5, -0.5], density_coeff=6.0,
                            albedo=0.9, phase_kind=1, phase_param=0.6, env_rgb=env, width=W, height=H,
                            sun_dir=np.float32([0.3, 0.8, 0.52]) / np.linalg.norm([0.3, 0.8, 0.52]),
                            sun_irradiance=3.0, sun_prob=0.5, max_bounces=32, rr_start=4, majorant_mode=mode,
                            stream_mode=1, shadow_rr=thr, **CAM)
        rng = orc.seed_states(W, H, seed)
        means = []
        for b in range(24):
            res = orc.render_plain(sc, rng, 64, accum_base=64 * b)
            means.append(res["sum"].mean() / 64)
        return np.array(means), res
    a, _ = render(0.0, 21)
    b, _ = render(0.3, 22)
    se = math.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    assert abs(a.mean() - b.mean()) < 4 * se, (a.mean(), b.mean(), se)
    assert se < 0.05 * a.mean()
