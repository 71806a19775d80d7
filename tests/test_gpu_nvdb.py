"""Volumes loaded from .nvdb files on the GPU, through the C ABI: the majorants of the sparse
upload against the reference's scan (renderer_scene.cpp:498-509) and against the dense upload
of the same voxels, the file entry point, and path-decision parity of renders through the
loaded volume against the oracle given the same voxels, map and clip box."""
import dataclasses
import math

import numpy as np
import pytest

from oracle import orc
from rtc8_gb300 import nvdb
from rtc8_gb300._lib import VptError
from rtc8_gb300.configs import look_at
from rtc8_gb300.renderer import Renderer, constant_environment, frame_params

from ._nvdb import dense_extent, fixture_path, reference
from ._scenes import small_config_mode, small_reference_mode

pytestmark = pytest.mark.gpu

DECISION_PARITY = 0.999
FLOAT_GRIDS = [("multi.nvdb", 0), ("multi.nvdb", 1), ("sphere_fog.nvdb", 0)]


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    d = tmp_path_factory.mktemp("nvdb")
    return {name: fixture_path(name, d) for name in ("multi.nvdb", "sphere_fog.nvdb", "sphere_zip.nvdb")}


def _decoded(buf):
    g = nvdb.grid_info(buf)
    o, v = nvdb.decode_leaves(buf)
    return g, dense_extent(o, v, g["extent_min"], g["extent_max"])


@pytest.mark.parametrize("name,index", FLOAT_GRIDS)
def test_sparse_upload_majorants(cuda_device, files, name, index):
    ref = reference()[name][index]
    buf = nvdb.read_grid(files[name], index)
    g, dense = _decoded(buf)
    r = Renderer(16, 16)
    r.set_volume_nanovdb(buf)
    info = r.volume_info()
    assert np.float32(info["global_majorant"]) == np.float32(ref["global_majorant"])
    assert info["active_leaves"] == g["flat_leaves"]
    assert info["total_leaves"] == np.prod(np.array(dense.shape) // 8)
    cells = r.cell_majorants()
    # the dense upload of the same voxels derives its cells with the same apron
    d = Renderer(16, 16)
    d.set_volume_dense(dense, 1.0, np.zeros(3, np.float32))
    np.testing.assert_array_equal(cells, d.cell_majorants())
    assert cells.max() >= info["global_majorant"] > 0
    assert r.device_errors() == 0
    r.close()
    d.close()


def test_file_entry_point(cuda_device, files):
    r = Renderer(16, 16)
    lib = r.lib
    rc = lib.vpt_set_volume_nvdb_file(r.ctx, str(files["multi.nvdb"]).encode(), 1)
    assert rc == 0, lib.vpt_last_error()
    a = r.cell_majorants()
    b_r = Renderer(16, 16)
    b_r.load_nvdb(files["multi.nvdb"], "block")
    np.testing.assert_array_equal(a, b_r.cell_majorants())
    assert r.volume_info()["global_majorant"] == b_r.volume_info()["global_majorant"] == np.float32(0.5)
    # a ZIP-coded grid is refused by the file entry point and accepted after host inflation
    rc = lib.vpt_set_volume_nvdb_file(r.ctx, str(files["sphere_zip.nvdb"]).encode(), 0)
    assert rc != 0 and b"codec 1" in lib.vpt_last_error()
    b_r.load_nvdb(files["sphere_zip.nvdb"])
    assert b_r.volume_info()["global_majorant"] == np.float32(1.0)
    with pytest.raises(VptError, match="grid type 2"):
        b_r.load_nvdb(files["multi.nvdb"], "temperature")
    r.close()
    b_r.close()


def _camera(cfg, g):
    lo, hi = np.array(g["world_min"]), np.array(g["world_max"])
    center = (lo + hi) / 2
    d = np.array([0.3, 0.4, 1.0])
    pos = center + d / np.linalg.norm(d) * 1.2 * np.linalg.norm(hi - lo)
    return pos, look_at(pos, center)


def _render_pair(cfg, buf, spp):
    import torch

    g, dense = _decoded(buf)
    env = constant_environment(0.5)
    pos, quat = _camera(cfg, g)
    p = frame_params(cfg)
    p.cam_position[:] = [float(x) for x in pos]
    p.cam_orientation[:] = [float(x) for x in quat]
    r = Renderer(cfg.width, cfg.height)
    r.set_volume_nanovdb(buf)
    r.set_environment_rgb(env)
    r.set_frame(p)
    r.seed_rng(cfg.rng_seed)
    log = torch.zeros(cfg.width * cfg.height * spp * 4, dtype=torch.int32, device="cuda")
    r.launch_plain_logged(spp, log.data_ptr())
    r.synchronize()
    s, _ = r.download_sum()
    gpu = {"log": log.cpu().numpy().view(np.uint32).reshape(-1, spp, 4), "sum": s, "rng": r.rng_states(),
           "errors": r.device_errors(), "majorant": r.volume_info()["global_majorant"]}
    r.close()
    # the oracle on the decoded voxels, with the upload's map, clip box and majorant
    sc = orc.scene_from_config(cfg, dense, env, cam_pos=np.float32(pos), cam_quat=np.float32(quat))
    s_ = sc.scene
    inv = np.float32(g["map_inv_mat_f"][0])
    s_.inv_voxel_size = float(inv)
    bmin = np.float32(g["world_min"])
    bmax = np.float32(g["world_max"])
    for a in range(3):
        s_.origin[a] = float(np.float32(g["map_vec_d"][a] + g["extent_min"][a] * g["map_mat_d"][4 * a]))
        s_.bbox_min[a] = s_.world_min[a] = float(bmin[a])
        s_.bbox_max[a] = s_.world_max[a] = float(bmax[a])
    center = (bmin + bmax) * np.float32(0.5)
    dd = (bmax - center).astype(np.float32)
    s_.world_radius = float(np.sqrt(np.float32(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2])))
    s_.global_majorant = float(gpu["majorant"])
    rng = orc.seed_states(cfg.width, cfg.height, cfg.rng_seed)
    o = orc.render_plain(sc, rng, spp, log=True)
    o["rng"] = rng
    return gpu, o


@pytest.mark.parametrize("mode", ["reference", "config"])
def test_render_through_nvdb_volume_matches_oracle(cuda_device, files, mode):
    """Reference mode (one global majorant, the reference's tracking): >= 99.9% identical path
    decisions. Configuration mode (majorant-grid DDA, no counterpart in the reference, compared
    statistically): the fog sphere's lower y face lies on a majorant-cell boundary, so the cell
    a ray entering through it starts in is decided by the last bit of the entry point, where
    the GPU's and the host's sin/cos differ by an ulp for some scattered directions; the bar
    there is 95% identical decisions and agreeing image means."""
    if mode == "reference":
        cfg = small_reference_mode(size=40, sigma=3.0)
    else:
        cfg = small_config_mode(size=40, g=0.7, majorant_mode=1)
        cfg = cfg.replace(volume=dataclasses.replace(cfg.volume, sigma_t_max=3.0))
    buf = nvdb.read_grid(files["sphere_fog.nvdb"])
    g, o = _render_pair(cfg, buf, spp=2)
    assert g["errors"] == 0
    same = np.all(g["log"] == o["log"], axis=2)
    bar = DECISION_PARITY if mode == "reference" else 0.95
    assert same.mean() >= bar, f"identical decisions {same.mean():.5f}"
    assert o["log"][..., 0].max() > 5 and (o["log"][..., 1] > 0).mean() > 0.3  # paths enter the sphere
    pix_same = same.reshape(cfg.height, cfg.width, -1).all(axis=2)
    close = np.isclose(g["sum"][pix_same], o["sum"][pix_same], rtol=2e-3, atol=1e-6).all(axis=-1)
    if mode == "reference":
        assert close.all()
    else:
        # A shadow ray's roulette at its last lookup ends it (no light) or lets it reach the light
        # with the same lookup count, so that outcome is not in the decision record; an ulp in
        # its visibility can flip it for a rare sample.
        assert close.mean() >= 0.995, f"pixels with identical decisions and equal sums {close.mean():.4f}"
    a, b = g["sum"].reshape(-1), o["sum"].reshape(-1)
    sigma = math.sqrt((a.var() + b.var()) / a.size)
    assert abs(a.mean() - b.mean()) <= 3 * sigma
    assert math.isfinite(float(a.sum()))
