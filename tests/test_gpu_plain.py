"""GPU parity of the plain volumetric tracer against the oracle, through the C ABI.

Path decisions (vertex count, primary and shadow lookups, end code) are compared sample by
sample; the bar is >= 99.9% identical decisions (the same RNG streams drive both), and the
accumulated images must agree where the decisions agree.
"""
import math

import numpy as np
import pytest

from oracle import orc
from rtc8_gb300.configs import C1, VolumeSpec
from rtc8_gb300.renderer import Renderer, constant_environment, frame_params, setup_scene

from ._scenes import fbm_numpy, small_config_mode, small_reference_mode, volume_for

pytestmark = pytest.mark.gpu

DECISION_PARITY = 0.999


def _gpu_logged(cfg, vox, env, spp, tracker=0, stage=0, **tracker_kw):
    import torch

    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg, volume=vox)
    r.set_tracker(tracker, **tracker_kw)
    r.set_leaf_staging(stage)
    if env is not None and cfg.sky is None:
        r.set_environment_rgb(env)
    log = torch.zeros(cfg.width * cfg.height * spp * 4, dtype=torch.int32, device="cuda")
    r.launch_plain_logged(spp, log.data_ptr())
    r.synchronize()
    s, n = r.download_sum()
    out = {"log": log.cpu().numpy().view(np.uint32).reshape(-1, spp, 4), "sum": s, "mean": r.download_mean(),
           "rng": r.rng_states(), "counters": r.counters(), "errors": r.device_errors()}
    r.close()
    return out


def _oracle(cfg, vox, env, spp):
    sc = orc.scene_from_config(cfg, vox, env)
    rng = orc.seed_states(cfg.width, cfg.height, cfg.rng_seed)
    res = orc.render_plain(sc, rng, spp, log=True)
    res["rng"] = rng
    return res


def _compare(cfg, spp, env=None):
    vox = volume_for(cfg)
    if env is None:
        env = constant_environment(cfg.env_constant if cfg.env_constant is not None else 0.5)
    g = _gpu_logged(cfg, vox, env, spp)
    o = _oracle(cfg, vox, env, spp)
    same = np.all(g["log"] == o["log"], axis=2)
    return g, o, same


@pytest.mark.parametrize("k", [0.0, 0.5])
def test_decision_parity_reference_mode(cuda_device, k):
    cfg = small_reference_mode(size=48, n=32, schlick_k=k)
    g, o, same = _compare(cfg, spp=4)
    frac = same.mean()
    assert frac >= DECISION_PARITY, f"identical decisions {frac:.5f}"
    assert o["log"][..., 0].max() > 5  # some paths scatter many times
    # images agree where every sample of a pixel made the same decisions
    pix_same = same.reshape(cfg.height, cfg.width, -1).all(axis=2)
    np.testing.assert_allclose(g["sum"][pix_same], o["sum"][pix_same], rtol=2e-3, atol=1e-6)
    np.testing.assert_allclose(g["mean"][pix_same], o["mean"][pix_same], rtol=2e-3, atol=1e-6)
    # lookups and vertices counted on the device equal the logged totals
    assert g["counters"]["lookups"] == int(g["log"][..., 1:3].astype(np.int64).sum())
    assert g["counters"]["samples"] == cfg.width * cfg.height * 4


@pytest.mark.parametrize("g_param,mode,streams,cell_log2",
                         [(0.8, 1, 1, 3), (0.8, 0, 1, 3), (-0.3, 1, 1, 3), (0.8, 1, 0, 3), (0.8, 1, 1, 4)])
def test_decision_parity_config_mode(cuda_device, g_param, mode, streams, cell_log2):
    """Both majorant modes, both RNG stream layouts and two majorant-cell sizes against the oracle."""
    cfg = small_config_mode(size=48, n=40, g=g_param, majorant_mode=mode).replace(rng_stream_mode=streams,
                                                                                   majorant_cell_log2=cell_log2)
    g, o, same = _compare(cfg, spp=4)
    frac = same.mean()
    assert frac >= DECISION_PARITY, f"identical decisions {frac:.5f}"
    pix_same = same.reshape(cfg.height, cfg.width, -1).all(axis=2)
    np.testing.assert_allclose(g["sum"][pix_same], o["sum"][pix_same], rtol=2e-3, atol=1e-6)


@pytest.mark.parametrize("streams", [0, 1])
def test_rng_streams_continue_across_launches(cuda_device, streams):
    cfg = small_config_mode(size=24, n=16).replace(rng_stream_mode=streams)
    vox = volume_for(cfg)
    a = Renderer(cfg.width, cfg.height)
    setup_scene(a, cfg, volume=vox)
    a.launch_plain(2)
    a.synchronize()
    b = Renderer(cfg.width, cfg.height)
    setup_scene(b, cfg, volume=vox)
    b.launch_plain(1)
    b.launch_plain(1)
    b.synchronize()
    np.testing.assert_array_equal(a.rng_states(), b.rng_states())
    np.testing.assert_allclose(a.download_sum()[0], b.download_sum()[0], rtol=1e-12)
    np.testing.assert_allclose(a.download_mean(), b.download_mean(), rtol=1e-6)
    a.close()
    b.close()


def test_global_and_grid_majorants_agree_statistically(cuda_device):
    """Delta tracking with one global majorant and with the 8^3 majorant grid estimate the same image."""
    base = C1.replace(width=32, height=32, volume=VolumeSpec(n=64, seed=1, octaves=4, sigma_t_max=20.0))
    spp = 256
    imgs = []
    for mode in (0, 1):
        cfg = base.replace(majorant_mode=mode, rng_seed=1000 + mode)
        r = Renderer(cfg.width, cfg.height)
        setup_scene(r, cfg)
        sq = np.zeros((cfg.height, cfg.width, 3))
        s = np.zeros((cfg.height, cfg.width, 3))
        prev = np.zeros((cfg.height, cfg.width, 3))
        for _ in range(8):
            r.launch_plain(spp // 8)
            cum = r.download_sum()[0]
            x = (cum - prev) / (spp // 8)  # mean of this batch of samples
            prev = cum
            s += x
            sq += x * x
        m = s / 8
        var_of_mean = (sq / 8 - m * m) / 7  # unbiased batch variance / 8 batches
        imgs.append((m, var_of_mean))
        r.close()
    (m0, v0), (m1, v1) = imgs
    z = np.abs(m0 - m1) / np.sqrt(v0 + v1 + 1e-12)
    assert np.mean(z[..., 1] < 3.0) > 0.97


def test_importance_map_matches_oracle(cuda_device):
    rng = np.random.default_rng(0)
    img = rng.gamma(0.7, 1.0, size=(40, 80, 3)).astype(np.float32)
    r = Renderer(4, 4)
    r.set_environment_rgb(img)
    mips, info = r.importance_map()
    omips, offs, oinfo = orc.importance_map(img)
    assert (info["map_w"], info["map_h"], info["num_mips"]) == (oinfo["map_w"], oinfo["map_h"], oinfo["num_mips"])
    np.testing.assert_allclose(mips, omips, rtol=2e-6, atol=1e-7)
    assert info["integral"] == pytest.approx(oinfo["integral"], rel=1e-5)
    r.close()


def test_fbm_generator_matches_numpy_restatement(cuda_device):
    spec = VolumeSpec(n=32, seed=9, octaves=5, threshold=0.4)
    r = Renderer(4, 4)
    r.generate_fbm_volume(spec, 1.0 / 32, np.array([-0.5, -0.5, -0.5], np.float32))
    r._dims = (32, 32, 32)
    got = r.download_volume()
    ref = fbm_numpy(32, 9, 5, 2.0, 0.5, 4.0, 0.4)
    np.testing.assert_allclose(got, ref, atol=2e-5)
    info = r.volume_info()
    assert 0 < info["active_leaves"] <= info["total_leaves"] == 64
    r.close()


def test_fbm_union_matches_numpy_restatement(cuda_device):
    spec = VolumeSpec(n=32, seed=9, octaves=5, threshold=0.5, union_seed=11)
    r = Renderer(4, 4)
    r.generate_fbm_volume(spec, 1.0 / 32, np.array([-0.5, -0.5, -0.5], np.float32))
    r._dims = (32, 32, 32)
    got = r.download_volume()
    a = fbm_numpy(32, 9, 5, 2.0, 0.5, 4.0, 0.5)
    b = fbm_numpy(32, 11, 5, 2.0, 0.5, 4.0, 0.5)
    np.testing.assert_allclose(got, np.maximum(a, b), atol=2e-5)
    assert (got > a).any() and (got > b).any()
    r.close()


def test_sparse_grid_majorants_match_oracle(cuda_device):
    vox = fbm_numpy(40, 4, 4, 2.0, 0.5, 4.0, 0.5)
    r = Renderer(4, 4)
    r.set_volume_dense(vox, 1.0 / 40, [-0.5, -0.5, -0.5])
    r._dims = vox.shape
    cells, g = orc.majorants(vox)
    np.testing.assert_array_equal(r.cell_majorants(), cells.reshape(-1))
    info = r.volume_info()
    assert info["global_majorant"] == np.float32(g)
    leaf_any = np.pad(vox, ((0, 0), (0, 0), (0, 0))).reshape(5, 8, 5, 8, 5, 8).max(axis=(1, 3, 5)) > 0
    assert info["active_leaves"] == int(leaf_any.sum())
    r.close()


def test_step_cap_sets_error_flag_and_matches_oracle(cuda_device):
    cfg = small_reference_mode(size=16, n=16, sigma=60.0).replace(max_steps_per_segment=3)
    g, o, same = _compare(cfg, spp=2)
    assert same.mean() >= DECISION_PARITY
    assert (g["log"][..., 3] == 5).any()
    assert g["errors"] & 0x1


@pytest.mark.parametrize("kind", ["reference", "config", "config_global"])
def test_wavefront_tracker_matches_megakernel(cuda_device, kind):
    """The wavefront tracker (event and tracking kernels alternating over per-slot state) draws
    every path's random numbers in the megakernel's order: identical decision logs, RNG states
    and sums, also when segments are suspended after a few lookups per pass."""
    if kind == "reference":
        cfg = small_reference_mode(size=40, n=32)
    else:
        cfg = small_config_mode(size=40, n=40, g=0.8, majorant_mode=1 if kind == "config" else 0)
    vox = volume_for(cfg)
    env = constant_environment(cfg.env_constant if cfg.env_constant is not None else 0.5)
    a = _gpu_logged(cfg, vox, env, 3, tracker=0)
    b = _gpu_logged(cfg, vox, env, 3, tracker=1, slots_per_sm=4, pass_steps=3)
    np.testing.assert_array_equal(a["log"], b["log"])
    np.testing.assert_array_equal(a["rng"], b["rng"])
    np.testing.assert_array_equal(a["sum"], b["sum"])
    np.testing.assert_array_equal(a["mean"], b["mean"])
    assert a["counters"] == b["counters"] and a["errors"] == b["errors"] == 0


@pytest.mark.parametrize("min_lanes", [1, 6])
def test_leaf_staging_keeps_every_decision(cuda_device, min_lanes):
    """Per-warp leaf staging (cp.async.bulk copies of shared leaves into shared memory) reads the
    same values as the unstaged tracker: identical decision logs, lookups and images."""
    cfg = small_config_mode(size=48, n=40, g=0.8, majorant_mode=1)
    vox = volume_for(cfg)
    env = constant_environment(cfg.env_constant)
    a = _gpu_logged(cfg, vox, env, 4)
    b = _gpu_logged(cfg, vox, env, 4, stage=min_lanes)
    np.testing.assert_array_equal(a["log"], b["log"])
    np.testing.assert_allclose(a["sum"], b["sum"], rtol=1e-12, atol=1e-15)   # FP64 atomics in launch order
    assert a["counters"] == b["counters"] and a["errors"] == b["errors"] == 0


@pytest.mark.parametrize("stage", [0, 4])
def test_production_launch_shapes_agree(cuda_device, stage):
    """The production launch (no decision log, sample-parallel streams: one 896-thread CTA per SM,
    a pixel's samples consecutive; CTAs of 128 with leaf staging) against the same launch forced to
    CTAs of 128 threads: each sample's path is the same, so the FP64 sums agree up to the order of
    the atomic additions, and the RNG seeds are untouched in both."""
    cfg = small_config_mode(size=48, n=32, g=0.6, majorant_mode=1).replace(rng_stream_mode=1)
    vox = volume_for(cfg)
    sums = []
    for threads in (0, 128):
        r = Renderer(cfg.width, cfg.height)
        setup_scene(r, cfg, volume=vox)
        r.set_leaf_staging(stage)
        r.set_launch_shape(0, threads, 0)
        r.launch_plain(8)
        r.launch_plain(8)
        r.synchronize()
        s, n = r.download_sum()
        assert n == 16 and r.device_errors() == 0
        sums.append(s)
        r.close()
    assert sums[0].sum() > 0
    np.testing.assert_allclose(sums[0], sums[1], rtol=1e-12, atol=1e-15)
