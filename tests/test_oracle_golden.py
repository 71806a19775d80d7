"""The oracle against golden vectors from the reference's own sources and published algorithms.

Fixtures in tests/golden/ were produced by tests/golden/make_golden.py from programs that link
the reference's NanoVDB headers, common/basic_types.{h,cpp} and the Hosek-Wilkie model.
"""
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import orc

GOLDEN = Path(__file__).resolve().parent / "golden"


def _load(name):
    return json.loads((GOLDEN / name).read_text())


def _f32(a):
    return np.asarray(a, dtype=np.float32)


# ------------------------------------------------------------------ RNG
def test_pcg32_matches_published_demo_vector():
    """O'Neill's pcg32 demo (pcg32_srandom_r(42, 54)) is the same XSH-RR generator the reference
    uses with increment 1 (common_renderer_types.h:101-125). The Python restatement below is pinned
    to the published outputs, then checked against the oracle for increment 1."""
    M = (1 << 64) - 1

    def out(old):
        x = (((old >> 18) ^ old) >> 27) & 0xFFFFFFFF
        r = old >> 59
        return ((x >> r) | (x << ((-r) & 31))) & 0xFFFFFFFF

    inc = (54 << 1) | 1
    s = (0 * 6364136223846793005 + inc) & M
    s = (s + 42) & M
    s = (s * 6364136223846793005 + inc) & M
    got = []
    for _ in range(6):
        got.append(out(s))
        s = (s * 6364136223846793005 + inc) & M
    assert got == [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E]

    state = 0x853C49E6748FEA9B
    floats, _ = orc.pcg_floats(state, 64)
    s = state
    for i in range(64):
        u = out(s)
        s = (s * 6364136223846793005 + 1) & M
        bits = (u >> 9) | 0x3F800000
        expect = np.frombuffer(np.uint32(bits).tobytes(), dtype=np.float32)[0] - np.float32(1.0)
        assert floats[i] == expect
    assert (floats >= 0).all() and (floats < 1).all()


def test_mt19937_64_seed_stream():
    """std::mt19937_64 (renderer_main.cpp:86-93): the C++ standard fixes the 10000th output of the
    default-seeded engine to 9981545732273789042."""
    seeds = orc.seed_states(10000, 1, 5489)
    assert int(seeds[9999]) == 9981545732273789042


# ------------------------------------------------------------------ NanoVDB
@pytest.fixture(scope="module")
def nvdb():
    return _load("ref_nanovdb.json")


def _nvdb_scene(d):
    n = d["n"]
    vox = _f32(d["voxels"]).reshape(n, n, n)
    return orc.make_scene(voxels=vox, voxel_size=d["voxel_size"], origin=_f32(d["origin"]), density_coeff=1.0,
                          albedo=1.0, phase_kind=0, phase_param=0.0, env_rgb=None, width=1, height=1,
                          cam_aspect=1.0, cam_fovy=0.7, cam_pos=[0, 0, 3], cam_quat=[0, 0, 0, 1])


def test_trilinear_sampler_bit_exact(nvdb):
    sc = _nvdb_scene(nvdb)
    pts = _f32(nvdb["sample_points"])
    out = np.zeros(len(pts) // 3, dtype=np.float32)
    orc.lib().orc_sample_density(sc.ref, orc.p(pts, orc.C.c_float), len(out), orc.p(out, orc.C.c_float))
    np.testing.assert_array_equal(out, _f32(nvdb["sample_values"]))


def test_world_box_and_majorant(nvdb):
    sc = _nvdb_scene(nvdb).scene
    wb = nvdb["world_bbox"]
    assert list(sc.bbox_min) == pytest.approx(wb[:3], abs=0) and list(sc.bbox_max) == pytest.approx(wb[3:], abs=0)
    assert np.float32(sc.global_majorant) == np.float32(nvdb["global_majorant"])


def test_world_to_index_bit_exact(nvdb):
    sc = _nvdb_scene(nvdb).scene
    w = _f32(nvdb["world_points"]).reshape(-1, 3)
    inv = np.float32(sc.inv_voxel_size)
    idx = (w - _f32(nvdb["origin"])) * inv
    np.testing.assert_array_equal(idx.reshape(-1), _f32(nvdb["world_to_index"]))


def test_ray_clip_bit_exact(nvdb):
    sc = _nvdb_scene(nvdb)
    org, dirs = _f32(nvdb["ray_origins"]), _f32(nvdb["ray_dirs"])
    n = len(org) // 3
    t0, t1 = np.zeros(n, np.float32), np.zeros(n, np.float32)
    hit = np.zeros(n, np.int32)
    orc.lib().orc_clip_rays(sc.ref, orc.p(org, orc.C.c_float), orc.p(dirs, orc.C.c_float), n,
                            orc.p(t0, orc.C.c_float), orc.p(t1, orc.C.c_float), orc.p(hit, orc.C.c_int32))
    ref = _f32(nvdb["ray_hit_t0_t1"]).reshape(-1, 3)
    np.testing.assert_array_equal(hit, ref[:, 0].astype(np.int32))
    m = hit == 1
    assert m.sum() > 20
    np.testing.assert_array_equal(t0[m], ref[m, 1])
    np.testing.assert_array_equal(t1[m], ref[m, 2])


# ------------------------------------------------------------------ basic_types.h math
@pytest.fixture(scope="module")
def basic():
    return _load("ref_basic_types.json")


def test_polar_yup_matches_reference(basic):
    dirs = _f32(basic["dirs"])
    out = np.zeros(2 * (len(dirs) // 3), np.float32)
    orc.lib().orc_polar_yup(orc.p(dirs, orc.C.c_float), len(dirs) // 3, orc.p(out, orc.C.c_float))
    np.testing.assert_allclose(out, _f32(basic["polar_yup_theta_phi"]), rtol=0, atol=2e-7)


def test_coordinate_system_matches_reference(basic):
    dirs = _f32(basic["dirs"])
    out = np.zeros(6 * (len(dirs) // 3), np.float32)
    orc.lib().orc_coordinate_system(orc.p(dirs, orc.C.c_float), len(dirs) // 3, orc.p(out, orc.C.c_float))
    np.testing.assert_array_equal(out, _f32(basic["coordinate_system_tb"]))


def test_quaternion_matrix_matches_reference(basic):
    q = _f32(basic["quats"]).reshape(-1, 4)
    ref = _f32(basic["quat_matrices_colmajor"]).reshape(-1, 9)
    for i in range(len(q)):
        m = np.zeros(9, np.float32)
        qi = np.ascontiguousarray(q[i])
        orc.lib().orc_quat_to_matrix(orc.p(qi, orc.C.c_float), orc.p(m, orc.C.c_float))
        np.testing.assert_allclose(m, ref[i], rtol=0, atol=1e-7)


def test_cmf_bands_are_the_renderer_table(basic):
    from rtc8_gb300 import sky

    cmf = _f32(basic["cmf_xs_ys_zs_centers_integral"])
    assert cmf.shape == (65,)
    assert cmf[48] == pytest.approx(374.6875) and cmf[63] == pytest.approx(815.3125)
    assert cmf[64] == pytest.approx(float(cmf[16:32].sum()), rel=1e-6)
    np.testing.assert_array_equal(sky.load_sky_state(__import__("rtc8_gb300.configs").configs.C2.sky, 20.0)["cmf"],
                                  cmf)


# ------------------------------------------------------------------ importance map and env sampling
def _env_scene(img):
    return orc.make_scene(voxels=np.zeros((2, 2, 2), np.float32), voxel_size=1.0, origin=[0, 0, 0],
                          density_coeff=1.0, albedo=1.0, phase_kind=0, phase_param=0.0, env_rgb=img, width=1,
                          height=1, cam_aspect=1.0, cam_fovy=0.7, cam_pos=[0, 0, 3], cam_quat=[0, 0, 0, 1])


def _test_env(w=48, h=24, seed=0):
    rng = np.random.default_rng(seed)
    img = rng.gamma(0.7, 1.0, size=(h, w, 3)).astype(np.float32)
    img[h // 3, w // 4] = 200.0
    return img


def test_importance_map_integral_is_sum_of_first_mip():
    img = _test_env()
    mips, offs, info = orc.importance_map(img)
    mw, mh = info["map_w"], info["map_h"]
    assert (mw, mh) == (64, 32)
    assert info["integral"] == pytest.approx(float(mips[: mw * mh].astype(np.float64).sum()), rel=1e-5)


def test_env_sample_pdf_matches_evaluate():
    """The reference's own intent (compute_light_probs.cu:213-229: sampled vs evaluated pdf)."""
    img = _test_env()
    sc = _env_scene(img)
    rng = np.random.default_rng(1)
    u = rng.random((4096, 2), dtype=np.float32)
    n = len(u)
    d, pdf, c = np.zeros(3 * n, np.float32), np.zeros(n, np.float32), np.zeros(3 * n, np.float32)
    orc.lib().orc_env_sample(sc.ref, orc.p(u, orc.C.c_float), n, orc.p(d, orc.C.c_float), orc.p(pdf, orc.C.c_float),
                             orc.p(c, orc.C.c_float))
    pe, ce = np.zeros(n, np.float32), np.zeros(3 * n, np.float32)
    orc.lib().orc_env_evaluate(sc.ref, orc.p(d, orc.C.c_float), n, orc.p(pe, orc.C.c_float), orc.p(ce, orc.C.c_float))
    ok = pdf > 0
    assert ok.mean() > 0.99
    close = np.isclose(pdf[ok], pe[ok], rtol=2e-3)
    assert close.mean() > 0.995
    np.testing.assert_allclose(np.linalg.norm(d.reshape(-1, 3), axis=1), 1.0, atol=1e-5)


def test_env_sampling_is_unbiased_for_radiance_integral():
    """E[L(w) / p(w)] over importance samples equals the direct quadrature of the image."""
    img = _test_env(32, 16, 3)
    sc = _env_scene(img)
    rng = np.random.default_rng(2)
    u = rng.random((200000, 2), dtype=np.float32)
    n = len(u)
    d, pdf, c = np.zeros(3 * n, np.float32), np.zeros(n, np.float32), np.zeros(3 * n, np.float32)
    orc.lib().orc_env_sample(sc.ref, orc.p(u, orc.C.c_float), n, orc.p(d, orc.C.c_float), orc.p(pdf, orc.C.c_float),
                             orc.p(c, orc.C.c_float))
    lum = c.reshape(-1, 3) @ np.array([0.2126729, 0.7151522, 0.0721750])
    est = np.mean(np.where(pdf > 0, lum / np.maximum(pdf, 1e-30), 0))
    h, w = img.shape[:2]
    theta = np.pi * (np.arange(h) + 0.5) / h
    solid = (2 * np.pi / w) * (np.pi / h) * np.sin(theta)
    quad = float(((img @ np.array([0.2126729, 0.7151522, 0.0721750])) * solid[:, None]).sum())
    assert est == pytest.approx(quad, rel=0.02)


# ------------------------------------------------------------------ phase functions
@pytest.mark.parametrize("kind,param", [(0, 0.0), (0, 0.5), (0, -0.3), (1, 0.0), (1, 0.8), (1, 0.9), (1, -0.4)])
def test_phase_function_normalised_and_consistent(kind, param):
    rng = np.random.default_rng(7)
    u = rng.random((100000, 2), dtype=np.float32)
    n = len(u)
    dl, pdf = np.zeros(3 * n, np.float32), np.zeros(n, np.float32)
    orc.lib().orc_phase_sample(kind, param, orc.p(u, orc.C.c_float), n, orc.p(dl, orc.C.c_float),
                               orc.p(pdf, orc.C.c_float))
    pe = np.zeros(n, np.float32)
    orc.lib().orc_phase_eval(kind, param, orc.p(dl, orc.C.c_float), n, orc.p(pe, orc.C.c_float))
    np.testing.assert_allclose(pdf, pe, rtol=2e-3)
    # integral of p over the sphere by stratified quadrature in cos(theta)
    cz = np.linspace(-1, 1, 200001, dtype=np.float64)
    loc = np.stack([np.sqrt(1 - cz ** 2), np.zeros_like(cz), cz], 1).astype(np.float32)
    pv = np.zeros(len(cz), np.float32)
    orc.lib().orc_phase_eval(kind, param, orc.p(np.ascontiguousarray(loc), orc.C.c_float), len(cz),
                             orc.p(pv, orc.C.c_float))
    integral = 2 * np.pi * np.trapezoid(pv.astype(np.float64), cz)
    assert integral == pytest.approx(1.0, rel=2e-3)
    # mean cosine along the propagation direction (local z = -cos)
    mean_cos = float(np.mean(-dl.reshape(-1, 3)[:, 2]))
    if kind == 1:
        assert mean_cos == pytest.approx(param, abs=0.01)
