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
