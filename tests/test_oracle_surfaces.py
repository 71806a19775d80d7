"""Known answers for the oracle's surface path (CPU): hits, emission seen directly, the world box,
and an energy check of area-light sampling against BSDF sampling."""
from __future__ import annotations

import math

import numpy as np

from oracle import orc
from rtc8_gb300 import surfaces as S
from rtc8_gb300.configs import C1
from rtc8_gb300.renderer import constant_environment


def _emitter_scene(e: float = 5.0):
    mats = [S.Material(S.SIMPLE_PBR, (0.9, 0.9, 0.9), 0.5, 0.0, (e, e, e))]
    sc = S.SurfaceScene(mats, [], [])
    # the reference's rectangle faces -y; rotated about x so that it faces +z, towards the camera
    t = np.zeros((3, 4), np.float32)
    t[0, 0] = 1.0
    t[1, 2] = 1.0
    t[2, 1] = -1.0
    t[:, 3] = (0.0, 0.0, -1.0)
    sc.add(S.rectangle(4.0, 4.0, 0), t)
    return sc


def _scene(cfg, surf, volume_enabled=False, env=None):
    vox = np.zeros((8, 8, 8), np.float32)
    sc = orc.scene_from_config(cfg, vox, env)
    orc.attach_surfaces(sc, surf, volume_enabled)
    return sc


def test_closest_hit_and_ties():
    sc = _emitter_scene()
    prep = orc.OracleSurfaces(sc)
    org = np.array([[0, 0, 3], [0.3, -0.2, 3], [5, 5, 3], [0, 0, -3]], np.float32)
    d = np.array([[0, 0, -1]] * 4, np.float32)
    tri, tb = prep.closest(org, d)
    assert tri[0] >= 0 and abs(tb[0, 0] - 4.0) < 1e-6
    assert tri[1] >= 0 and abs(tb[1, 0] - 4.0) < 1e-6
    assert tri[2] == -1 and tri[3] == -1            # outside the rectangle / behind the ray
    # two coincident copies of a triangle: the lower index wins
    sc.add(S.rectangle(4.0, 4.0, 0), sc.instances[0].transform)
    tri2, _ = orc.OracleSurfaces(sc).closest(org[:1], d[:1])
    assert tri2[0] == tri[0]


def test_emitter_seen_directly_is_emittance_over_pi():
    e = 5.0
    cfg = C1.replace(width=16, height=16, sun_elevation_deg=None, env_constant=None, cam_direction=(0, 0, 1),
                     cam_distance_diagonals=1.0, fov_deg=20.0, rng_stream_mode=1, rr_start_vertex=1, max_bounces=1)
    sc = _scene(cfg, _emitter_scene(e))
    out = orc.render_plain(sc, orc.seed_states(16, 16, cfg.rng_seed), 4, log=True)
    # every camera ray hits the emitter first; with one bounce allowed nothing else adds light, so
    # the image equals that of the same camera looking into a constant environment of E / pi
    # (pixel values are radiance over the camera's direction density)
    empty = orc.scene_from_config(cfg.replace(env_constant=e / math.pi), np.zeros((8, 8, 8), np.float32),
                                  constant_environment(e / math.pi))
    ref = orc.render_plain(empty, orc.seed_states(16, 16, cfg.rng_seed), 4)
    np.testing.assert_allclose(out["sum"], ref["sum"], rtol=1e-6)
    assert out["sum"].min() > 0
    assert (out["log"][..., 3] == 4).all()          # ended by the bounce cap


def test_world_box_is_the_union_of_volume_and_instances():
    cfg = C1.replace(width=4, height=4)
    sc = _scene(cfg, S.room_scene(), volume_enabled=True)
    s = sc.scene
    assert list(s.world_min) == [np.float32(-0.9), np.float32(-0.6), np.float32(-0.9)]
    assert list(s.world_max) == [np.float32(0.9), np.float32(0.9), np.float32(0.9)]
    lo, hi = np.array(s.world_min, np.float32), np.array(s.world_max, np.float32)
    c = (lo + hi) * np.float32(0.5)
    assert math.isclose(s.world_radius, float(np.linalg.norm(hi - c)), rel_tol=1e-6)


def test_emitting_closed_room_furnace():
    """A closed room whose walls are all Lambert with reflectance rho and emittance E holds the
    radiance E / (pi (1 - rho)) everywhere. The estimate combines emission hits weighted against
    area-light sampling with NEE of every wall triangle, so the area-sampling density and the
    density computeSurfacePoint assigns to a hit must agree, or the sum is biased."""
    e = 1.0
    mat = S.Material(S.LAMBERT, (0.8, 0.8, 0.8), emittance=(e, e, e))
    rho = ((204 / 255 + 0.055) / 1.055) ** 2.4         # the 8-bit sRGB decode of 0.8
    sc = S.SurfaceScene([mat], [], [])
    sc.add(S.box((1.0, 1.0, 1.0), 0, inward=True))
    sc.add(S.box((0.3, 0.3, 0.3), 0), S.rotation_y(25.0, 0.2, -0.5, -0.1))
    cfg = C1.replace(width=8, height=8, sun_elevation_deg=None, env_constant=None, cam_direction=(0.2, 0.1, 1.0),
                     cam_distance_diagonals=0.45, fov_deg=60.0, rng_stream_mode=1, rr_start_vertex=1, max_bounces=0)
    out = orc.render_plain(_scene(cfg, sc), orc.seed_states(8, 8, cfg.rng_seed), 512)["sum"]
    radiance = e / math.pi / (1 - rho)
    env = orc.scene_from_config(cfg.replace(env_constant=radiance), np.zeros((8, 8, 8), np.float32),
                                constant_environment(radiance))
    ref = orc.render_plain(env, orc.seed_states(8, 8, cfg.rng_seed), 512)["sum"]
    np.testing.assert_allclose(out.sum(axis=(0, 1)), ref.sum(axis=(0, 1)), rtol=0.02)


def test_sphere_mesh_is_closed_and_outward():
    m = S.sphere(0.5, 0, 12, 6)
    p = m.vertices[:, 0:3]
    assert len(m.triangles) == 2 * 12 * (6 - 1)
    np.testing.assert_allclose(np.linalg.norm(m.vertices[:, 3:6], axis=1), 1.0, rtol=1e-6)
    np.testing.assert_allclose(np.linalg.norm(p, axis=1), 0.5, rtol=1e-6)
    t = m.triangles
    gn = np.cross(p[t[:, 1]] - p[t[:, 0]], p[t[:, 2]] - p[t[:, 0]])
    assert (np.einsum("ij,ij->i", gn, p[t].mean(axis=1)) > 0).all()
    # closed: the triangles' area approaches the sphere's
    area = 0.5 * np.linalg.norm(gn, axis=1).sum()
    assert 0.85 * 4 * math.pi * 0.25 < area < 4 * math.pi * 0.25


def test_radiance_cache_queries_at_surfaces():
    """The oracle's render pass over the room writes surface queries with the shading normal,
    roughness and the materials' reflectances (Lambert: roughness 1, no specular; SimplePBR:
    specular F0 > 0), and its training pass records surface vertices."""
    from rtc8_gb300.configs import C_ROOM_REFERENCE_MODE

    cfg = C_ROOM_REFERENCE_MODE.replace(width=24, height=24)
    vox = orc.fbm_volume(cfg.volume)
    sc = orc.scene_from_config(cfg, vox, constant_environment(cfg.env_constant))
    orc.attach_surfaces(sc, S.room_scene(), True)
    rng = orc.seed_states(cfg.width, cfg.height, cfg.rng_seed)
    o = orc.nrc_pass(sc, rng.copy(), 1, cfg.width, cfg.height, termination=0.02)
    q = o["infer_query"][(o["terminal_bits"] & 1) == 1]
    assert len(q) > 0.25 * cfg.width * cfg.height
    assert (q[:, 0:3] >= -1e-5).all() and (q[:, 0:3] <= 1 + 1e-5).all()   # in the world box (walls on its faces)
    assert ((q[:, 7] == 1.0) & (q[:, 11:14].max(axis=1) == 0)).any()   # Lambert walls
    assert (q[:, 11:14].max(axis=1) > 0).any()
    t = orc.nrc_pass(sc, rng.copy(), 2, cfg.width // 4, cfg.height // 4, unbiased_offset=7, termination=0.02)
    n = int(t["num_train"][0])
    tq = t["train_query"][:n]
    assert n > 0 and ((tq[:, 7] == 1.0) | (tq[:, 11:14].max(axis=1) > 0)).any()
