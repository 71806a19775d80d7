"""Oracle restatement of the radiance-cache passes and set-up kernels, checked on the CPU
against hand computations of the reference's formulas (nrc_set_up_kernels.cu,
renderer_main.cpp:218-229) and against the oracle's own plain tracer."""
import numpy as np
import pytest

from oracle import orc
from rtc8_gb300.renderer import constant_environment

from ._scenes import small_reference_mode, volume_for


def _lcg(s):
    return ((s * 1103515245 + 12345) & 0xFFFFFFFF) % (1 << 31)


def test_shufflers_follow_the_lcg():
    sh = orc.nrc_shufflers()
    s = 471313181
    for i in range(2000):
        s = _lcg(s)
        assert sh[i] == s
    assert len(np.unique(sh)) == len(sh)


@pytest.mark.parametrize("prev,cur,expect", [(0, (16, 12), (64, 48)), (16384, (16, 12), (32, 24)),
                                              (65536, (16, 12), (16, 12)), (262144, (16, 12), (8, 6))])
def test_prepare_adaptive_size(prev, cur, expect):
    cnt = np.zeros(16, np.uint32)
    cnt[0], cnt[2], cnt[3] = prev, cur[0], cur[1]
    stats = np.zeros(18, np.float32)
    suf = np.zeros(64 * 48, np.uint32)
    orc.nrc_prepare(cnt, stats, suf, 64, 48, 1, 5, False)
    assert (cnt[4], cnt[5]) == expect
    assert cnt[1] == 0 and cnt[6] == 5 and cnt[7] == expect[0] * expect[1]
    assert np.all(stats[9:12] == np.inf) and np.all(stats[12:15] == -np.inf) and np.all(stats[15:18] == 0)
    assert np.all(suf == orc.INVALID_VERTEX)
    orc.nrc_prepare(cnt, stats, suf, 64, 48, 0, 5, True)
    assert (cnt[2], cnt[3]) == (16, 12)


def _vertex(tp, prev, length=1, unbiased=0):
    bits = np.uint32((prev & 0x3FFFFF) | (length << 22) | (unbiased << 30))
    return np.array([tp[0], tp[1], tp[2], bits.view(np.float32)], np.float32)


def test_propagate_walks_the_suffix():
    # one suffix: vertices 0 -> 1 -> 2, terminal query with prediction; one suffix without query
    q0 = np.zeros((8, 14), np.float32)
    q0[:, 8:11] = 0.5   # diffuse
    q0[:, 11:14] = 0.25  # specular
    t0 = np.array([[1, 2, 3], [0.5, 0.5, 0.5], [0.1, 0.2, 0.3], [2, 2, 2]] + [[0, 0, 0]] * 4, np.float32)
    vert = np.stack([_vertex((1, 1, 1), orc.INVALID_VERTEX), _vertex((0.5, 0.5, 0.5), 0, 2),
                     _vertex((2, 2, 2), 1, 3), _vertex((1, 1, 1), orc.INVALID_VERTEX)] + [_vertex((0, 0, 0), 0)] * 4)
    suffix = np.array([2 | (1 << 22), 3, orc.INVALID_VERTEX], np.uint32)
    inferred = np.array([[1.0, -1.0, 4.0], [9, 9, 9], [9, 9, 9]], np.float32)
    iq = np.zeros((3, 14), np.float32)
    iq[0, 8:11] = 1.0
    iq[0, 11:14] = 1.0
    tgt = t0.copy()
    orc.nrc_propagate(3, suffix, inferred, iq, vert, q0, tgt, 0.0)
    refl = 0.75
    c = np.maximum(inferred[0], 0) * 2.0
    expect = t0.copy()
    for idx in (2, 1, 0):
        c = t0[idx] + vert[idx, :3] * c
        expect[idx] = c / refl
    expect[3] = t0[3] / refl  # suffix without query: NEE / implicit only
    np.testing.assert_allclose(tgt, expect, rtol=1e-6)
    # radianceScale divides the prediction
    tgt2 = t0.copy()
    orc.nrc_propagate(1, suffix, inferred, iq, vert, q0, tgt2, 4.0)
    assert tgt2[2, 2] < tgt[2, 2]


def test_shuffle_matches_python_restatement():
    rng = np.random.default_rng(0)
    num = 5000
    q0 = rng.random((orc.TRAIN_BUFFER_SIZE, 14)).astype(np.float32)
    t0 = rng.random((orc.TRAIN_BUFFER_SIZE, 3)).astype(np.float32) * 3
    t0[7] = [np.nan, 1, 1]
    q0[9, 3] = np.inf
    sh = orc.nrc_shufflers()
    stats = np.array([np.inf] * 3 + [-np.inf] * 3 + [0] * 3, np.float32)
    q1 = np.zeros_like(q0)
    t1 = np.zeros_like(t0)
    sh_py = sh.copy()
    writers = orc.nrc_shuffle(num, stats, sh, q0, t0, q1, t1, 2.0)
    exp_q = np.zeros_like(q0)
    exp_t = np.zeros_like(t0)
    tgts = []
    for i in range(orc.TRAIN_PER_FRAME):
        sh_py[i] = _lcg(int(sh_py[i]))
        dst = int(sh_py[i]) % orc.TRAIN_PER_FRAME
        src = i % num
        q = q0[src].copy()
        t = t0[src].copy()
        if not np.all(np.isfinite(q)):
            q[:] = 0
        if not (np.all(np.isfinite(t)) and np.all(t >= 0)):
            t[:] = 0
        tgts.append(t.copy())
        exp_q[dst] = q
        exp_t[dst] = np.minimum(t * np.float32(2.0), np.float32(1e6))
    assert np.array_equal(sh, sh_py)
    np.testing.assert_array_equal(q1, exp_q)
    np.testing.assert_array_equal(t1, exp_t)
    tg = np.array(tgts)
    np.testing.assert_array_equal(stats[0:3], tg.min(0))
    np.testing.assert_array_equal(stats[3:6], tg.max(0))
    np.testing.assert_allclose(stats[6:9], tg.astype(np.float64).mean(0), rtol=1e-6)
    assert writers.sum() == orc.TRAIN_PER_FRAME
    # no training data: zero records in place, shufflers untouched
    sh2 = orc.nrc_shufflers()
    q1[:] = 1
    orc.nrc_shuffle(0, stats, sh2, q0, t0, q1, t1, 0.0)
    assert np.all(q1[:orc.TRAIN_PER_FRAME] == 0) and np.array_equal(sh2, orc.nrc_shufflers())


def test_accumulate_formula():
    n = 4
    term = np.zeros((n, 4), np.float32)
    term[:, :3] = [[1, 1, 1], [0.5, 0.5, 0.5], [2, 2, 2], [1, 1, 1]]
    bits = np.array([1, 0, 1 | (3 << 1), 1], np.uint32)
    term[:, 3] = bits.view(np.float32)
    fc = np.array([[0.1, 0.2, 0.3], [1, 1, 1], [0, 0, 0], [np.inf, 0, 0]], np.float32)
    inf = np.array([[1, 2, 3], [5, 5, 5], [-1, 1, 0.5], [1, 1, 1]], np.float32)
    iq = np.zeros((n, 14), np.float32)
    iq[:, 8:11] = 0.5
    s = np.zeros((n, 3))
    m = np.zeros((n, 3), np.float32)
    orc.nrc_accumulate(n, term, fc, inf, iq, 0.0, 0, s, m)
    orc.nrc_accumulate(n, term, fc, inf, iq, 0.0, 1, s, m)
    c0 = fc[0] + term[0, :3] * inf[0] * 0.5
    c1 = fc[1]
    c2 = fc[2] + term[2, :3] * np.maximum(inf[2], 0) * 0.5
    np.testing.assert_allclose(s[:3], 2 * np.array([c0, c1, c2]), rtol=1e-6)
    np.testing.assert_allclose(m[:3], np.array([c0, c1, c2]), rtol=1e-6)
    assert np.all(s[3] == 0)  # non-finite result counts as 0


def _small_scene():
    cfg = small_reference_mode(size=32, n=32, sigma=60.0)
    env = constant_environment(0.5)
    return cfg, orc.scene_from_config(cfg, volume_for(cfg), env)


def test_render_pass_agrees_with_plain_paths_that_escape():
    """Until a radiance-cache path stops at a cache query it draws the same random numbers and
    adds the same terms as the plain path: paths that escape agree with plain 1-spp paths."""
    cfg, sc = _small_scene()
    rng = orc.seed_states(cfg.width, cfg.height, cfg.rng_seed)
    r_nrc = rng.copy()
    o = orc.nrc_pass(sc, r_nrc, 1, cfg.width, cfg.height, log=True)
    r_plain = rng.copy()
    pl = orc.render_plain(sc, r_plain, 1, log=True)
    esc = o["log"][:, 3] == 1
    assert esc.sum() > 100 and (o["log"][:, 3] == 6).sum() > 100
    assert np.all(pl["log"][esc, 0, 3] == 1)
    assert np.array_equal(r_nrc[esc], r_plain[esc])
    np.testing.assert_array_equal(o["frame_contribution"][esc], pl["sum"].reshape(-1, 3)[esc].astype(np.float32))
    cache = o["log"][:, 3] == 6
    assert np.all(o["terminal_bits"][cache] & 1 == 1) and np.all(o["terminal_bits"][esc] & 1 == 0)
    # every cache query lies in the world box with the medium's reflectance
    q = o["infer_query"][cache]
    assert np.all((q[:, :3] >= 0) & (q[:, :3] <= 1)) and np.all(q[:, 8:11] == np.float32(cfg.albedo))


def test_training_pass_chains_are_consistent():
    cfg, sc = _small_scene()
    rng = orc.seed_states(cfg.width, cfg.height, cfg.rng_seed)
    tw, th = cfg.width // 4, cfg.height // 4
    o = orc.nrc_pass(sc, rng, 2, tw, th, unbiased_offset=3)
    chains = orc.suffix_chains(o["train_suffix"], o["train_bits"], tw * th)
    assert sum(len(c) for c in chains) == int(o["num_train"][0]) > tw * th // 4
    for i, ch in enumerate(chains):
        unb = (int(o["train_suffix"][i]) >> 31) & 1
        px, py = i % tw, i // tw
        assert unb == int(((py % 4) * 4 + px % 4 + 3) % 16 == 0)
        for k, idx in enumerate(ch):
            b = int(o["train_bits"][idx])
            assert (b >> 22) & 0xFF == k + 1 and (b >> 30) & 1 == unb
            if k:
                assert idx > ch[k - 1]
        if ch:
            assert (int(o["train_suffix"][i]) >> 23) & 0xFF >= len(ch)
    assert np.all(np.isfinite(o["train_target"][: int(o["num_train"][0])]))
