"""Surface path (triangle meshes around and inside the volume) against the oracle.

The GPU traces the BVH of the product's host builder, the oracle an exhaustive search over
the same world triangles; both restate the reference's surface loop (optix_pathtracing_kernels.cu
:84-356, renderer_kernel_common.h:72-403, common_renderer_types.h:1483-1985). Decision records
(vertices, primary and shadow lookups, end code) must agree for >= 99.9% of the samples.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import orc
from rtc8_gb300 import surfaces as S
from rtc8_gb300.configs import C_ROOM, C_ROOM_REFERENCE_MODE
from rtc8_gb300.renderer import Renderer, constant_environment, setup_scene

pytestmark = pytest.mark.gpu

DECISION_PARITY = 0.999
# Device and oracle differ in the last bits of fast-math transcendentals (the reference's own
# build flags on the device, libm in the oracle), and each path vertex is a fresh chance for such
# a difference to flip a decision. Surface paths here are three times longer than the volume
# workloads' (7.6 vertices), so the bar is set per vertex at the volume tests' level: their 0.1%
# of samples at 2.5 vertices per path is 4e-4 diverging samples per vertex. At least 99.5% of the
# samples stay identical.
PER_VERTEX = 4e-4
SURFACE_PARITY = 0.995


def run_pair(cfg, scene, spp: int, volume_enabled: bool = True) -> dict:
    import torch

    vox = orc.fbm_volume(cfg.volume)
    env = constant_environment(cfg.env_constant)
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg.replace(surfaces=None), volume=vox)
    r.set_surfaces(scene)
    if not volume_enabled:
        r.clear_volume()
    info = r.surface_info()
    log = torch.zeros(cfg.width * cfg.height * spp * 4, dtype=torch.int32, device="cuda")
    r.launch_plain_logged(spp, log.data_ptr())
    r.synchronize()
    g = {"log": log.cpu().numpy().view(np.uint32).reshape(-1, spp, 4), "sum": r.download_sum()[0],
         "counters": r.counters(), "errors": r.device_errors(), "rng": r.rng_states(), "info": info}
    r.close()
    sc = orc.scene_from_config(cfg, vox, env)
    orc.attach_surfaces(sc, scene, volume_enabled)
    rng = orc.seed_states(cfg.width, cfg.height, cfg.rng_seed)
    o = orc.render_plain(sc, rng, spp, log=True)
    o["rng"] = rng
    o["world"] = (list(sc.scene.world_min), list(sc.scene.world_max))
    return {"gpu": g, "oracle": o, "same": np.all(g["log"] == o["log"], axis=2)}


def check(cfg, res, spp: int) -> None:
    g, o, same = res["gpu"], res["oracle"], res["same"]
    frac = same.mean()
    per_vertex = (~same).sum() / max(int(o["log"][..., 0].astype(np.int64).sum()), 1)
    assert frac >= SURFACE_PARITY and per_vertex <= PER_VERTEX, \
        f"identical decisions {frac:.5f} ({(~same).sum()} of {same.size} differ, {per_vertex:.2e} per vertex)"
    assert g["errors"] == 0
    assert g["counters"]["samples"] == cfg.width * cfg.height * spp
    pix_same = same.reshape(cfg.height, cfg.width, -1).all(axis=2)
    close = np.isclose(g["sum"], o["sum"], rtol=2e-3, atol=1e-6).all(axis=-1)
    assert close[pix_same].mean() >= 0.999, f"decision-identical pixels within 2e-3: {close[pix_same].mean():.5f}"
    np.testing.assert_allclose(g["sum"][pix_same].sum(axis=0), o["sum"][pix_same].sum(axis=0), rtol=2e-4)
    # the world box (and with it the environment shadow rays) is the oracle's
    box = g["info"]["world_box"]
    assert np.allclose(box[:3], o["world"][0], rtol=0, atol=0) and np.allclose(box[3:], o["world"][1], rtol=0, atol=0)


def test_room_configuration_mode(cuda_device):
    cfg = C_ROOM.replace(width=64, height=64)
    res = run_pair(cfg, S.room_scene(), 16)
    check(cfg, res, 16)
    log = res["oracle"]["log"]
    assert log[..., 0].max() >= 8 and (log[..., 2] > 0).any()   # long paths with shadow tracking


def test_room_reference_mode(cuda_device):
    cfg = C_ROOM_REFERENCE_MODE.replace(width=48, height=48)
    res = run_pair(cfg, S.room_scene(), 8)
    check(cfg, res, 8)
    pix_same = res["same"].reshape(-1, 8).all(axis=1)
    assert np.mean(res["gpu"]["rng"][pix_same] == res["oracle"]["rng"][pix_same]) >= DECISION_PARITY


def test_surfaces_without_volume(cuda_device):
    cfg = C_ROOM.replace(width=64, height=64)
    res = run_pair(cfg, S.room_scene(), 8, volume_enabled=False)
    check(cfg, res, 8)
    assert res["gpu"]["counters"]["lookups"] == 0 and res["oracle"]["log"][..., 1:3].sum() == 0


def test_tessellated_mesh_through_the_bvh(cuda_device):
    """Scenes above the flat-list size (64 triangles) are traversed through the BVH: the room
    with a 224-triangle sphere (smooth shading normals) and two copies of the room's blocks inside
    the cloud, against the oracle's exhaustive search; both reference and configuration mode."""
    sc = S.room_scene()
    sc.add(S.sphere(0.22, 5, 16, 8), S.translation(0.05, 0.05, 0.4))
    sc.add(S.sphere(0.12, 4, 12, 6), S.translation(-0.35, 0.3, -0.2))
    assert sc.num_triangles > 64
    for cfg in (C_ROOM.replace(width=48, height=48), C_ROOM_REFERENCE_MODE.replace(width=40, height=40)):
        res = run_pair(cfg, sc, 8)
        check(cfg, res, 8)
        info = res["gpu"]["info"]
        assert info["triangles"] == sc.num_triangles and info["bvh_nodes"] > 31


def test_instanced_groups_and_transforms(cuda_device):
    """A geometry group (two meshes) placed twice with rotation, scale and translation, and an
    instance whose uniform scale differs from its transform's (the reference's two scales)."""
    sc = S.room_scene()
    blocks = len(sc.meshes)
    sc.meshes += [S.box((0.1, 0.1, 0.1), 4), S.rectangle(0.2, 0.2, 3)]
    t1 = S.rotation_y(35.0, 0.2, 0.2, 0.45)
    t1[:, :3] *= 0.8
    sc.instances.append(S.Instance(blocks, 2, t1, 0.8))
    sc.instances.append(S.Instance(blocks, 2, S.translation(-0.3, 0.45, 0.5, 1.2), 1.0))
    cfg = C_ROOM.replace(width=56, height=56)
    res = run_pair(cfg, sc, 12)
    check(cfg, res, 12)
    assert res["gpu"]["info"]["emitters"] == 2 + 2 * 2


def test_surface_info_and_rejected_input(cuda_device):
    from rtc8_gb300._lib import VptError

    r = Renderer(8, 8)
    sc = S.room_scene()
    r.set_surfaces(sc)
    info = r.surface_info()
    assert info["triangles"] == sc.num_triangles
    assert info["emitters"] == 2 and info["bvh_nodes"] >= 1
    bad = S.room_scene()
    bad.meshes[0].triangles = bad.meshes[0].triangles.copy()
    bad.meshes[0].triangles[0, 0] = 999
    with pytest.raises(VptError, match="out of range"):
        r.set_surfaces(bad)
    bad = S.room_scene()
    bad.instances[0].first_geometry = 50
    with pytest.raises(VptError, match="out of bounds"):
        r.set_surfaces(bad)
    r.set_surfaces(None)
    assert r.surface_info()["triangles"] == 0
    r.close()
