"""The NanoVDB reader of the library (csrc/vpt_nvdb.cu, host code) against the reference's own
reading of .nvdb files written by NanoVDB 32.3 (tests/golden/nvdb): file metadata, the decoded
voxels bit-exact against the reference's accessor (renderer_scene.cpp:498-509 reads the grid
the same way), tiles and negative index coordinates, ZIP-coded grids, and the refusals.

Only host entry points of the library are called: no GPU is needed."""
import numpy as np
import pytest

from oracle import orc
from rtc8_gb300 import nvdb
from rtc8_gb300._lib import VptError

from ._nvdb import dense_extent, fixture_path, lookup, reference, voxel_hash

FILES = ["multi.nvdb", "sphere_fog.nvdb", "sphere_zip.nvdb"]
FLOAT_GRIDS = [("multi.nvdb", 0), ("multi.nvdb", 1), ("sphere_fog.nvdb", 0), ("sphere_zip.nvdb", 0)]


@pytest.fixture(scope="module")
def ref():
    return reference()


@pytest.fixture(scope="module")
def files(tmp_path_factory):
    d = tmp_path_factory.mktemp("nvdb")
    return {name: fixture_path(name, d) for name in FILES}


@pytest.mark.parametrize("name", FILES)
def test_file_metadata_matches_reference(ref, files, name):
    grids = nvdb.list_grids(files[name])
    assert len(grids) == len(ref[name])
    for g, r in zip(grids, ref[name]):
        assert g["name"] == r["name"] and g["grid_count"] == len(ref[name])
        assert (g["grid_type"], g["grid_class"], g["codec"]) == (r["grid_type"], r["grid_class"], r["codec"])
        assert (g["grid_bytes"], g["file_bytes"], g["active_voxels"]) == (r["grid_size"], r["file_size"],
                                                                        r["voxel_count"])
        assert g["node_count"] == r["node_count"][:3] and g["tile_count"] == r["tile_count"]
        assert g["index_min"] + g["index_max"] == r["meta_index_bbox"]
        assert g["world_min"] + g["world_max"] == r["meta_world_bbox"]
        assert g["voxel_size"] == r["meta_voxel_size"]


def test_grid_lookup_by_name(files):
    assert nvdb.grid_index(files["multi.nvdb"], "block") == 1
    assert nvdb.grid_index(files["multi.nvdb"], "temperature") == 2
    with pytest.raises(KeyError):
        nvdb.grid_index(files["multi.nvdb"], "velocity")
    with pytest.raises(VptError, match="exceeds the grid count 3"):
        nvdb.file_info(files["multi.nvdb"], 3)


@pytest.mark.parametrize("name,index", FLOAT_GRIDS)
def test_grid_header_map_and_boxes(ref, files, name, index):
    r = ref[name][index]
    g = nvdb.grid_info(nvdb.read_grid(files[name], index))
    assert g["name"] == r["name"] and g["grid_type"] == 1
    assert g["index_min"] + g["index_max"] == r["index_bbox"]
    assert g["map_vec_d"] == r["map_vec_d"]
    assert np.array_equal(np.float32(g["map_vec_f"]), np.float32(r["map_vec_f"]))
    assert np.array_equal(np.float32(g["map_mat_f"])[[0, 4, 8]], np.float32(r["map_mat_f_diag"]))
    assert np.array_equal(np.float32(g["map_inv_mat_f"])[[0, 4, 8]], np.float32(r["map_inv_mat_f_diag"]))
    assert np.float32(g["background"]) == np.float32(r["background"])
    # renderer_scene.cpp:517-519: the clip box is the double world box rounded to float
    clip = np.float32(np.array(g["world_min"] + g["world_max"]))
    assert np.array_equal(clip, np.float32(r["clip_box_f"]))
    # the extent holds every voxel a lookup inside the clip box can read
    assert all(lo <= m - 2 and hi > x + 2 and lo % 8 == 0 and hi % 8 == 0
               for lo, hi, m, x in zip(g["extent_min"], g["extent_max"], g["index_min"], g["index_max"]))


@pytest.mark.parametrize("name,index", FLOAT_GRIDS)
def test_decoded_voxels_match_reference_accessor(ref, files, name, index):
    r = ref[name][index]
    buf = nvdb.read_grid(files[name], index)
    g = nvdb.grid_info(buf)
    origins, values = nvdb.decode_leaves(buf)
    assert len(origins) == g["flat_leaves"] and np.all(origins % 8 == 0)
    assert len({tuple(o) for o in origins}) == len(origins)  # one leaf per cell
    dense = dense_extent(origins, values, g["extent_min"], g["extent_max"])
    coords = np.array(r["coords"], dtype=np.int64).reshape(-1, 3)
    vals, inside = lookup(dense, g["extent_min"], coords)
    assert inside.mean() > 0.9
    np.testing.assert_array_equal(vals[inside], np.float32(r["values"])[inside])
    # every voxel of the index box grown by two: order-independent checksum and non-zero count
    b = r["checksum_box"]
    x, y, z = np.meshgrid(*[np.arange(b[a], b[a + 3] + 1) for a in range(3)], indexing="ij")
    xyz = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    v, ins = lookup(dense, g["extent_min"], xyz)
    assert ins.all()
    with np.errstate(over="ignore"):
        total = np.sum(voxel_hash(xyz[:, 0], xyz[:, 1], xyz[:, 2], v), dtype=np.uint64)
    assert int(total) == int(r["checksum"])
    assert int(np.count_nonzero(v)) == r["nonzero"]
    # the renderer's global majorant: max over [min, max) of the index box
    lo, hi = np.array(r["index_bbox"][:3]), np.array(r["index_bbox"][3:])
    e0 = np.array(g["extent_min"])
    sub = dense[tuple(slice(int(l - e), int(h - e)) for l, h, e in zip(lo, hi, e0))]
    assert np.float32(sub.max()) == np.float32(r["global_majorant"])


def test_tiles_become_constant_leaves(ref, files):
    """The "density" grid stores eight 8^3 blocks of 0.75 as lower-node tiles and "block" a 128^3
    region of 0.5 as an upper-node tile; the fog sphere's interior is tiles of 1.0."""
    buf = nvdb.read_grid(files["multi.nvdb"], "density")
    o, v = nvdb.decode_leaves(buf)
    g = nvdb.grid_info(buf)
    assert g["tile_count"][0] == 8 and len(o) == g["node_count"][0] + 8
    tiles = v[g["node_count"][0]:]
    assert np.all(tiles == np.float32(0.75))
    buf = nvdb.read_grid(files["multi.nvdb"], "block")
    o, v = nvdb.decode_leaves(buf)
    g = nvdb.grid_info(buf)
    n_leaf = g["node_count"][0]
    assert g["tile_count"][1] == 1 and np.all(v[n_leaf:] == np.float32(0.5))
    # the upper tile covers [128, 256) x [0, 128) x [0, 128), inside the extent: 16^3 leaves
    assert len(o) - n_leaf == 4096
    assert o[n_leaf:, 0].min() == 128 and o[n_leaf:, 0].max() == 248 and o[n_leaf:, 1:].max() == 120
    buf = nvdb.read_grid(files["sphere_fog.nvdb"])
    o, v = nvdb.decode_leaves(buf)
    g = nvdb.grid_info(buf)
    assert np.all(v[g["node_count"][0]:] == np.float32(1.0)) and g["tile_count"][0] > 0


def test_zip_grid_inflates_to_the_same_grid(files):
    a = nvdb.read_grid(files["sphere_fog.nvdb"])
    b = nvdb.read_grid(files["sphere_zip.nvdb"])
    assert a == b


@pytest.mark.parametrize("name,index", [("multi.nvdb", 0), ("sphere_fog.nvdb", 0)])
def test_trilinear_samples_match_reference(ref, files, name, index):
    """SampleFromVoxels<1> of the reference at index points, against the oracle's first-order
    sampler over the decoded extent (points shifted by the extent origin: 1e-6 relative)."""
    r = ref[name][index]
    buf = nvdb.read_grid(files[name], index)
    g = nvdb.grid_info(buf)
    o, v = nvdb.decode_leaves(buf)
    dense = dense_extent(o, v, g["extent_min"], g["extent_max"])
    sc = orc.make_scene(voxels=dense, voxel_size=1.0, origin=np.zeros(3, np.float32), density_coeff=1.0, albedo=1.0,
                        phase_kind=0, phase_param=0.0, env_rgb=None, width=1, height=1, cam_aspect=1.0,
                        cam_fovy=0.7, cam_pos=[0, 0, 3], cam_quat=[0, 0, 0, 1])
    pts = np.float32(r["sample_points"]).reshape(-1, 3) - np.float32(g["extent_min"])
    pts = np.ascontiguousarray(pts)
    out = np.zeros(len(pts), dtype=np.float32)
    orc.lib().orc_sample_density(sc.ref, orc.p(pts, orc.C.c_float), len(out), orc.p(out, orc.C.c_float))
    np.testing.assert_allclose(out, np.float32(r["sample_values"]), rtol=1e-6, atol=1e-6)


def test_refusals(files, tmp_path):
    temp = nvdb.read_grid(files["multi.nvdb"], "temperature")
    assert nvdb.grid_info(temp)["grid_type"] == 2
    with pytest.raises(VptError, match="grid type 2"):
        nvdb.decode_leaves(temp)
    good = nvdb.read_grid(files["sphere_fog.nvdb"])
    with pytest.raises(VptError, match="bad magic"):
        nvdb.grid_info(b"\0" * 8 + good[8:])
    with pytest.raises(VptError, match="buffer"):
        nvdb.grid_info(good[:500])
    with pytest.raises(VptError, match="shorter than the grid size|out of range|bad"):
        nvdb.decode_leaves(good[:len(good) // 2])
    # a child offset pointing outside the buffer is refused, not followed
    bad = bytearray(good)
    root = 672 + int(np.frombuffer(good[672 + 24:672 + 32], dtype="<u8")[0])
    bad[root + 64 + 8:root + 64 + 16] = np.int64(1 << 40).tobytes()
    with pytest.raises(VptError, match="upper-node reference"):
        nvdb.decode_leaves(bytes(bad))
    # a file whose segment header names the BLOSC codec
    raw = bytearray(files["sphere_zip.nvdb"].read_bytes())
    raw[14:16] = np.uint16(2).tobytes()
    p = tmp_path / "blosc.nvdb"
    p.write_bytes(bytes(raw))
    assert nvdb.file_info(p)["codec"] == 2
    with pytest.raises(ValueError, match="BLOSC"):
        nvdb.read_grid(p)
    p2 = tmp_path / "notnvdb.nvdb"
    p2.write_bytes(b"not a nanovdb file at all")
    with pytest.raises(VptError, match="bad magic"):
        nvdb.file_info(p2)
