"""GPU radiance-cache passes against the oracle, through the C ABI.

The render and training passes of the tracer use the same per-pixel PCG32 streams as the
oracle's restatement, so path decisions are compared pixel by pixel: the bar is >= 99.9% of
pixels with the same final RNG state and the same terminal record. Records of agreeing pixels
must match (queries and throughputs within 1e-4 relative: FP32 on both sides, no FMA
contraction on either). Training vertices are numbered by a device atomic, so suffixes are
compared as chains (first vertex to last). The set-up kernels run on buffers downloaded from
the device and are compared with their restatement on the same inputs: exact for integer and
copy work, 1e-5 relative for arithmetic, the batch average within 1e-4 (summation order).
"""
import numpy as np
import pytest

from oracle import orc
from rtc8_gb300 import nrc
from rtc8_gb300.renderer import Renderer, constant_environment, setup_scene

from ._scenes import small_config_mode, small_reference_mode, volume_for

pytestmark = pytest.mark.gpu

DECISION_PARITY = 0.999


def _setup(cfg, vox, env):
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg, volume=vox)
    r.set_environment_rgb(env)
    return r


def _np(t):
    return t.cpu().numpy()


def _scene(cfg):
    vox = volume_for(cfg)
    env = constant_environment(cfg.env_constant if cfg.env_constant is not None else 0.5)
    return vox, env


@pytest.mark.parametrize("density_query,termination", [(False, 0.0), (True, 0.0), (False, 0.05)])
def test_render_pass_matches_oracle(cuda_device, density_query, termination):
    import torch

    cfg = small_reference_mode(size=48, n=32, sigma=60.0)
    vox, env = _scene(cfg)
    r = _setup(cfg, vox, env)
    r.nrc_set_query_density(density_query)
    r.nrc_set_termination_factor(termination)
    rng0 = r.rng_states().copy()
    r.launch_render_nrc()
    torch.cuda.synchronize()
    v = r.nrc_views()
    n = cfg.width * cfg.height
    g_rng = r.rng_states()
    g_term = _np(v["infer_terminal"])
    g_bits = g_term[:, 3].copy().view(np.uint32)
    g_query = _np(v["infer_query"])[:n]
    g_fc = _np(v["frame_contribution"])
    assert r.device_errors() == 0

    sc = orc.scene_from_config(cfg, vox, env)
    o_rng = rng0.copy()
    o = orc.nrc_pass(sc, o_rng, 1, cfg.width, cfg.height, density_query=density_query, termination=termination)
    same = (g_rng == o_rng) & (g_bits == o["terminal_bits"])
    assert same.mean() >= DECISION_PARITY, f"identical pixels {same.mean():.5f}"
    has_q = same & ((o["terminal_bits"] & 1) == 1)
    assert has_q.sum() > n // 20  # a good share of paths ends with a cache query
    assert (o["terminal_bits"] >> 1).max() > 2
    np.testing.assert_allclose(g_term[same, :3], o["terminal_tp"][same], rtol=1e-4, atol=1e-7)
    np.testing.assert_allclose(g_query[has_q], o["infer_query"][has_q], rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(g_fc[same], o["frame_contribution"][same], rtol=1e-4, atol=1e-7)
    if density_query:
        assert g_query[has_q, 7].max() > 0.05
    r.close()


def _train_pass(cfg, vox, env, offset, density_query=False, termination=0.0, train_termination=0.0):
    import torch

    r = _setup(cfg, vox, env)
    r.nrc_set_query_density(density_query)
    r.nrc_set_termination_factor(termination, train_termination)
    rng0 = r.rng_states().copy()
    r.prepare_nrc(0, offset, True)
    r.launch_generate_training(0)
    torch.cuda.synchronize()
    return r, rng0


@pytest.mark.parametrize("cfg_kind,train_termination", [("reference", 0.0), ("config", 0.0), ("config", 0.05)])
def test_training_pass_matches_oracle(cuda_device, cfg_kind, train_termination):
    if cfg_kind == "reference":
        cfg = small_reference_mode(size=64, n=32, sigma=60.0)
    else:
        cfg = small_config_mode(size=64, n=32, g=0.6, majorant_mode=1).replace(rng_stream_mode=0)
    vox, env = _scene(cfg)
    offset = 2654435761
    r, rng0 = _train_pass(cfg, vox, env, offset, termination=0.02, train_termination=train_termination)
    v = r.nrc_views()
    cnt = _np(v["counters"]).view(np.uint32)
    tw, th = int(cnt[2]), int(cnt[3])
    assert (tw, th) == (cfg.width // 4, cfg.height // 4)
    assert cnt[6] == offset and cnt[7] == tw * th
    ni = tw * th
    g_suffix = _np(v["train_suffix"]).view(np.uint32)[:ni]
    g_vert = _np(v["train_vertex"])
    g_vbits = g_vert[:, 3].copy().view(np.uint32)
    g_query = _np(v["train_query0"])
    g_target = _np(v["train_target0"])
    g_iq = _np(v["train_end_query"])[:ni]
    g_rng = r.rng_states()
    assert r.device_errors() == 0

    sc = orc.scene_from_config(cfg, vox, env)
    o_rng = rng0.copy()
    o = orc.nrc_pass(sc, o_rng, 2, tw, th, unbiased_offset=offset, termination=0.02,
                     train_termination=train_termination)
    g_chains = orc.suffix_chains(g_suffix, g_vbits, ni)
    o_chains = orc.suffix_chains(o["train_suffix"], o["train_bits"], ni)
    # pixel (px, py) of the training image uses the full image's stream py * width + px
    pix = np.array([(i // tw) * cfg.width + i % tw for i in range(ni)])
    same = (g_rng[pix] == o_rng[pix]) & ((g_suffix >> 22) == (o["train_suffix"] >> 22))
    same &= np.array([len(a) == len(b) for a, b in zip(g_chains, o_chains)])
    assert same.mean() >= DECISION_PARITY, f"identical suffixes {same.mean():.5f}"
    if same.all():
        assert int(cnt[0]) == int(o["num_train"][0])
    assert sum(len(c) for c in o_chains) > ni // 4 and max(len(c) for c in o_chains) > 2
    unb = (o["train_suffix"] >> 31) & 1
    assert 0 < unb.sum() <= ni // 16 + tw + th
    for i in np.nonzero(same)[0]:
        for gi, oi in zip(g_chains[i], o_chains[i]):
            assert (g_vbits[gi] >> 22) == (o["train_bits"][oi] >> 22)
            np.testing.assert_allclose(g_vert[gi, :3], o["train_local_tp"][oi], rtol=1e-4, atol=1e-7)
            np.testing.assert_allclose(g_query[gi], o["train_query"][oi], rtol=1e-4, atol=1e-5)
            np.testing.assert_allclose(g_target[gi], o["train_target"][oi], rtol=1e-4, atol=1e-6)
        if (o["train_suffix"][i] >> 22) & 1:
            np.testing.assert_allclose(g_iq[i], o["infer_query"][i], rtol=1e-4, atol=1e-5)
    r.close()


def test_propagate_shuffle_accumulate_match_oracle(cuda_device):
    """The three set-up kernels on the buffers of a real training pass and render pass, with
    random cache predictions, against their restatement on the same inputs."""
    import torch

    cfg = small_reference_mode(size=64, n=32, sigma=60.0)
    vox, env = _scene(cfg)
    r, _ = _train_pass(cfg, vox, env, 7)
    v = r.nrc_views()
    cnt = _np(v["counters"]).view(np.uint32).copy()
    ni = int(cnt[7])
    gen = torch.Generator(device="cuda").manual_seed(1)
    v["train_end_inferred"].copy_(torch.rand(v["train_end_inferred"].shape, device="cuda", generator=gen) * 2 - 0.5)
    torch.cuda.synchronize()
    before = {k: _np(v[k]).copy() for k in ("train_suffix", "train_end_inferred", "train_end_query", "train_vertex",
                                            "train_query0", "train_target0", "shufflers", "stats")}
    # propagate
    r.propagate()
    torch.cuda.synchronize()
    tgt = before["train_target0"].copy()
    orc.nrc_propagate(ni, before["train_suffix"].view(np.uint32), before["train_end_inferred"],
                      before["train_end_query"],
                      before["train_vertex"], before["train_query0"], tgt, 0.0)
    np.testing.assert_allclose(_np(v["train_target0"]), tgt, rtol=1e-5, atol=1e-7)
    assert np.abs(tgt - before["train_target0"]).max() > 0  # propagation changed targets
    # shuffle
    prop_q, prop_t = _np(v["train_query0"]).copy(), _np(v["train_target0"]).copy()
    r.shuffle(0)
    torch.cuda.synchronize()
    sh = before["shufflers"].view(np.uint32).copy()
    stats = before["stats"].copy()
    q1 = np.zeros((orc.TRAIN_BUFFER_SIZE, 14), np.float32)
    t1 = np.zeros((orc.TRAIN_BUFFER_SIZE, 3), np.float32)
    writers = orc.nrc_shuffle(int(cnt[0]), stats[0:9], sh, prop_q, prop_t, q1, t1, 0.0)
    assert np.array_equal(_np(v["shufflers"]).view(np.uint32), sh)
    one = writers == 1
    assert one.mean() > 0.3
    np.testing.assert_array_equal(_np(v["train_query1"])[:orc.TRAIN_PER_FRAME][one], q1[:orc.TRAIN_PER_FRAME][one])
    np.testing.assert_array_equal(_np(v["train_target1"])[:orc.TRAIN_PER_FRAME][one], t1[:orc.TRAIN_PER_FRAME][one])
    g_stats = _np(v["stats"])
    np.testing.assert_array_equal(g_stats[0:6], stats[0:6])
    np.testing.assert_allclose(g_stats[6:9], stats[6:9], rtol=1e-4)
    # render pass, random predictions, accumulate (as sample 0 and sample 1)
    r.launch_render_nrc()
    v["inferred"].copy_(torch.rand(v["inferred"].shape, device="cuda", generator=gen))
    torch.cuda.synchronize()
    n = cfg.width * cfg.height
    term, fc = _np(v["infer_terminal"]).copy(), _np(v["frame_contribution"]).copy()
    inf, iq = _np(v["inferred"]).copy(), _np(v["infer_query"]).copy()
    r.reset_accumulation()
    r.accumulate_inferred(0)
    r.accumulate_inferred(1)
    s_g, _ = r.download_sum()
    m_g = r.download_mean()
    s_o = np.zeros((n, 3), np.float64)
    m_o = np.zeros((n, 3), np.float32)
    orc.nrc_accumulate(n, term, fc, inf, iq, 0.0, 0, s_o, m_o)
    orc.nrc_accumulate(n, term, fc, inf, iq, 0.0, 1, s_o, m_o)
    np.testing.assert_allclose(s_g.reshape(n, 3), s_o, rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(m_g.reshape(n, 3), m_o, rtol=1e-6, atol=1e-9)
    assert r.device_errors() == 0
    r.close()


def test_prepare_adapts_training_image(cuda_device):
    """prepareNRC's adaptive size: from numTrainingData of the previous buffer."""
    import torch

    cfg = small_reference_mode(size=64, n=32)
    vox, env = _scene(cfg)
    r = _setup(cfg, vox, env)
    r.prepare_nrc(0, 1, True)
    torch.cuda.synchronize()
    v = r.nrc_views()
    for prev_count in (0, 16384, 65536, 200000):
        cnt = _np(v["counters"]).view(np.uint32).copy()
        cnt[0] = prev_count
        cnt[2], cnt[3] = 16, 12
        v["counters"].copy_(torch.from_numpy(cnt.view(np.int32)).cuda())
        r.prepare_nrc(1, 99, False)
        torch.cuda.synchronize()
        g = _np(v["counters"]).view(np.uint32)
        o = cnt.copy()
        stats = np.zeros(18, np.float32)
        suffix = np.zeros(cfg.width * cfg.height, np.uint32)
        orc.nrc_prepare(o, stats, suffix, cfg.width, cfg.height, 1, 99, False)
        assert np.array_equal(g[:8], o[:8]), (prev_count, g[:8], o[:8])
    assert np.all(_np(v["train_suffix"]).view(np.uint32) == orc.INVALID_VERTEX)
    r.close()


def _blocks(img, k=16):
    h, w, _ = img.shape
    return img.reshape(h // k, k, w // k, k, 3).mean(axis=(1, 3))


def _rel(a, b):
    return float(np.mean((a - b) ** 2) / np.mean(b ** 2))


def test_nrc_frame_loop_gain_over_truncated_paths(cuda_device):
    """The composite frame call runs the reference's loop with the tcgen05 cache. With the
    trained cache the image agrees with the plain estimate of the same scene (block averages of
    16 x 16 pixels, so that noise does not dominate); the same short render paths without the
    network (predictions forced to 0) are far darker: what the network adds is the radiance of
    the truncated path tails."""
    import torch

    cfg = small_config_mode(size=128, n=32, g=0.6, majorant_mode=1).replace(rng_stream_mode=0)
    vox, env = _scene(cfg)
    r = _setup(cfg, vox, env)
    net_cfg = nrc.default_config(nrc.NRC_ENCODING_VOLUME)
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=net_cfg)
    r.nrc_set_query_density(True)
    r.nrc_frame(cache, 8, 1, True)
    for _ in range(40):
        r.nrc_frame(cache, 1, 1, False)
    torch.cuda.synchronize()
    assert r.device_errors() == 0 and cache.device_errors() == 0
    assert cache.lib.nrc_step_count(cache.h) == 4 * 48
    r.reset_accumulation()
    for _ in range(64):
        r.nrc_frame(cache, 1, 1, False)
    img_nrc = r.image()
    assert np.all(np.isfinite(img_nrc))
    # the same render passes with the cache's predictions replaced by 0
    v = r.nrc_views()
    r.reset_accumulation()
    for i in range(64):
        r.launch_render_nrc()
        v["inferred"].zero_()
        r.accumulate_inferred(i)
    img_trunc = r.image()
    p = Renderer(cfg.width, cfg.height)
    setup_scene(p, cfg, volume=vox)
    p.set_environment_rgb(env)
    p.launch_plain(256)
    img_plain = p.image()
    rel_nrc = _rel(_blocks(img_nrc), _blocks(img_plain))
    rel_trunc = _rel(_blocks(img_trunc), _blocks(img_plain))
    assert rel_nrc < 0.02 and rel_nrc < 0.25 * rel_trunc, (rel_nrc, rel_trunc)
    assert r.device_errors() == 0
    cache.finalize()
    r.close()
    p.close()


def test_frame_with_training_sets_in_one_launch(cuda_device):
    """On sample-parallel streams the frame call traces all of its training iterations in the
    launch of its render samples (one training set per iteration; the first frame's eight in two
    launches of four). The cache trained that way gives the plain estimate's image, like the
    sequential frame loop above; every iteration still runs its four training steps."""
    import torch

    cfg = small_config_mode(size=128, n=32, g=0.6, majorant_mode=1).replace(rng_stream_mode=1)
    vox, env = _scene(cfg)
    r = _setup(cfg, vox, env)
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=nrc.default_config(nrc.NRC_ENCODING_VOLUME))
    r.nrc_set_query_density(True)
    r.nrc_frame(cache, 8, 4, True)
    for _ in range(10):
        r.nrc_frame(cache, 4, 4, False)
    torch.cuda.synchronize()
    assert r.device_errors() == 0 and cache.device_errors() == 0
    assert cache.lib.nrc_step_count(cache.h) == 4 * (8 + 40)
    r.reset_accumulation()
    for _ in range(16):
        r.nrc_frame(cache, 4, 4, False)
    img_nrc = r.image()
    assert np.all(np.isfinite(img_nrc))
    p = Renderer(cfg.width, cfg.height)
    setup_scene(p, cfg, volume=vox)
    p.set_environment_rgb(env)
    p.launch_plain(256)
    rel = _rel(_blocks(img_nrc), _blocks(p.image()))
    assert rel < 0.02, rel
    assert r.device_errors() == 0
    cache.finalize()
    r.close()
    p.close()


def _pcg_jump(states: np.ndarray, delta: int) -> np.ndarray:
    """PCG32 state advanced by `delta` draws (LCG jump-ahead by squaring, Brown 1994)."""
    mult, plus = 6364136223846793005, 1
    acc_mult, acc_plus = 1, 0
    m64 = (1 << 64) - 1
    while delta:
        if delta & 1:
            acc_mult = (acc_mult * mult) & m64
            acc_plus = (acc_plus * mult + plus) & m64
        plus = ((mult + 1) * plus) & m64
        mult = (mult * mult) & m64
        delta >>= 1
    return np.array([(acc_mult * int(s) + acc_plus) & m64 for s in states], dtype=np.uint64)


def test_batched_render_pass_matches_oracle(cuda_device):
    """spp samples per pixel in one launch on sample-parallel streams: sample s of pixel p starts
    2^40 * (base + s) draws into the pixel's stream; each slot matches the oracle's render pass
    started from that state, and the batched accumulation equals the restated one."""
    import torch

    cfg = small_config_mode(size=40, n=32, g=0.6, majorant_mode=1).replace(rng_stream_mode=1)
    vox, env = _scene(cfg)
    r = _setup(cfg, vox, env)
    seeds = r.rng_states().copy()
    spp = 3
    r.launch_plain(2)  # sample-parallel streams continue after the plain launch's two samples
    r.reset_accumulation()
    r.launch_render_nrc_batch(spp)
    torch.cuda.synchronize()
    v = r.nrc_views()
    n = cfg.width * cfg.height
    assert r.nrc_buffers().render_spp >= spp
    g_term = _np(v["infer_terminal"])[: n * spp]
    g_bits = g_term[:, 3].copy().view(np.uint32)
    g_fc = _np(v["frame_contribution"])[: n * spp]
    g_q = _np(v["infer_query"])[: n * spp]
    assert np.array_equal(r.rng_states(), seeds)  # seeds are not modified
    sc = orc.scene_from_config(cfg, vox, env)
    same_all = []
    for s in range(spp):
        st = _pcg_jump(seeds, (2 + s) << 40)
        o = orc.nrc_pass(sc, st, 1, cfg.width, cfg.height)
        sl = slice(s * n, (s + 1) * n)
        same = g_bits[sl] == o["terminal_bits"]
        same_all.append(same)
        np.testing.assert_allclose(g_fc[sl][same], o["frame_contribution"][same], rtol=1e-4, atol=1e-7)
        hq = same & ((o["terminal_bits"] & 1) == 1)
        np.testing.assert_allclose(g_q[sl][hq], o["infer_query"][hq], rtol=1e-4, atol=1e-5)
    assert np.concatenate(same_all).mean() >= DECISION_PARITY
    # batched accumulation with random predictions
    gen = torch.Generator(device="cuda").manual_seed(3)
    v["inferred"].copy_(torch.rand(v["inferred"].shape, device="cuda", generator=gen))
    torch.cuda.synchronize()
    inf, iq = _np(v["inferred"]).copy(), _np(v["infer_query"]).copy()
    r.accumulate_inferred_batch(0, spp)
    s_g, cnt = r.download_sum()
    assert cnt == spp
    s_o = np.zeros((n, 3), np.float64)
    m_o = np.zeros((n, 3), np.float32)
    for s in range(spp):
        sl = slice(s * n, (s + 1) * n)
        orc.nrc_accumulate(n, g_term[sl].copy(), g_fc[sl].copy(), inf[sl].copy(), iq[sl].copy(), 0.0, s, s_o, m_o)
    np.testing.assert_allclose(s_g.reshape(n, 3), s_o, rtol=1e-6, atol=1e-9)  # FMA in the kernel
    np.testing.assert_allclose(r.download_mean().reshape(n, 3), s_o / spp, rtol=1e-6, atol=1e-9)
    assert r.device_errors() == 0
    r.close()


def test_training_pass_uses_its_own_states_with_sample_parallel_streams(cuda_device):
    """With sample-parallel render streams the training pass draws from per-pixel states 2^62
    draws ahead of the context's seeds and leaves the seeds alone; its suffixes match the
    oracle's training pass started from those states."""
    import torch

    cfg = small_config_mode(size=64, n=32, g=0.6, majorant_mode=1).replace(rng_stream_mode=1)
    vox, env = _scene(cfg)
    r = _setup(cfg, vox, env)
    seeds = r.rng_states().copy()
    v = r.nrc_views()
    trng0 = _np(v["train_rng"]).view(np.uint64).copy()
    assert np.array_equal(trng0, _pcg_jump(seeds, 1 << 62))
    r.prepare_nrc(0, 5, True)
    r.launch_generate_training(0)
    torch.cuda.synchronize()
    assert np.array_equal(r.rng_states(), seeds)
    cnt = _np(v["counters"]).view(np.uint32)
    tw, th = int(cnt[2]), int(cnt[3])
    ni = tw * th
    sc = orc.scene_from_config(cfg, vox, env)
    o_rng = trng0.copy()
    o = orc.nrc_pass(sc, o_rng, 2, tw, th, unbiased_offset=5)
    pix = np.array([(i // tw) * cfg.width + i % tw for i in range(ni)])
    g_trng = _np(v["train_rng"]).view(np.uint64)
    same = (g_trng[pix] == o_rng[pix]) & ((_np(v["train_suffix"]).view(np.uint32)[:ni] >> 22) == (o["train_suffix"] >> 22))
    assert same.mean() >= DECISION_PARITY
    assert r.device_errors() == 0
    r.close()


def test_combined_training_and_render_launch_matches_separate_passes(cuda_device):
    """The frame call's combined launch (training pixels, then render samples) gives the same
    records as the separate training pass and batched render pass from the same states."""
    import torch

    cfg = small_config_mode(size=48, n=32, g=0.6, majorant_mode=1).replace(rng_stream_mode=1)
    vox, env = _scene(cfg)
    spp = 2
    a = _setup(cfg, vox, env)
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=nrc.default_config(nrc.NRC_ENCODING_VOLUME))
    trng0 = _np(a.nrc_views()["train_rng"]).view(np.uint64).copy()
    a.nrc_frame(cache, 1, spp, True)
    torch.cuda.synchronize()
    va = a.nrc_views()
    cnt = _np(va["counters"]).view(np.uint32).copy()
    offset, tw, th = int(cnt[6]), int(cnt[2]), int(cnt[3])
    ni = tw * th

    b = _setup(cfg, vox, env)
    vb = b.nrc_views()
    assert np.array_equal(_np(vb["train_rng"]).view(np.uint64), trng0)
    b.prepare_nrc(0, offset, True)
    b.launch_generate_training(0)
    b.launch_render_nrc_batch(spp)
    torch.cuda.synchronize()
    vb = b.nrc_views()
    n = cfg.width * cfg.height * spp
    for k in ("infer_terminal", "frame_contribution"):
        np.testing.assert_array_equal(_np(va[k])[:n], _np(vb[k])[:n])
    ta, tb = _np(va["infer_terminal"])[:n, 3].copy().view(np.uint32), _np(vb["infer_terminal"])[:n, 3].copy().view(np.uint32)
    hq = (ta & 1) == 1
    np.testing.assert_array_equal(_np(va["infer_query"])[:n][hq], _np(vb["infer_query"])[:n][hq])
    assert np.array_equal(_np(va["train_rng"]).view(np.uint64), _np(vb["train_rng"]).view(np.uint64))
    assert int(_np(vb["counters"]).view(np.uint32)[0]) == int(cnt[0])
    sa = _np(va["train_suffix"]).view(np.uint32)[:ni]
    sb = _np(vb["train_suffix"]).view(np.uint32)[:ni]
    assert np.array_equal(sa >> 22, sb >> 22)
    qa, qb = _np(va["train_query0"]), _np(vb["train_query0"])
    ba = _np(va["train_vertex"])[:, 3].copy().view(np.uint32)
    bb = _np(vb["train_vertex"])[:, 3].copy().view(np.uint32)
    for ca, cb in zip(orc.suffix_chains(sa, ba, ni), orc.suffix_chains(sb, bb, ni)):
        assert len(ca) == len(cb)
        for ia, ib in zip(ca, cb):
            np.testing.assert_array_equal(qa[ia], qb[ib])
    assert a.device_errors() == 0 and b.device_errors() == 0 and cache.device_errors() == 0
    cache.finalize()
    a.close()
    b.close()


def test_batched_frame_infers_only_the_query_slots(cuda_device):
    """A batched render frame lists the slots whose paths ended with a cache query and infers
    only those: the count equals the number of query slots, every query slot holds the network's
    prediction for its query (bit for bit, as a full inference gives it), and the other slots are
    not written."""
    import torch

    spp = 4
    cfg = small_config_mode(size=48, n=32, g=0.6, majorant_mode=1).replace(rng_stream_mode=1)
    vox, env = _scene(cfg)
    r = _setup(cfg, vox, env)
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=nrc.default_config(nrc.NRC_ENCODING_VOLUME))
    r.nrc_set_termination_factor(0.32, 0.08)
    r.nrc_frame(cache, 2, spp, True)  # allocates the render slots, trains a little
    torch.cuda.synchronize()
    v = r.nrc_views()
    v["inferred"].fill_(-1.0e30)
    r.nrc_frame(cache, 0, spp, False)  # render pass + indexed inference + accumulation
    torch.cuda.synchronize()
    n = cfg.width * cfg.height * spp
    bits = _np(v["infer_terminal"])[:n, 3].copy().view(np.uint32)
    has_query = (bits & 1) == 1
    assert 0 < has_query.sum() < n
    assert int(_np(v["counters"]).view(np.uint32)[8]) == int(has_query.sum())
    got = _np(v["inferred"])[:n]
    queries = v["infer_query"][:n][torch.from_numpy(has_query).cuda()].contiguous()
    ref = torch.zeros((queries.shape[0], 3), dtype=torch.float32, device="cuda")
    cache.infer(None, queries, queries.shape[0], ref)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(got[has_query], ref.cpu().numpy())
    assert np.all(got[~has_query] == -1.0e30)
    assert r.device_errors() == 0 and cache.device_errors() == 0
    cache.finalize()
    r.close()
