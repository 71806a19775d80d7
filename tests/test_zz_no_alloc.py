"""The allocation-free tracer launch (vpt_launch_plain_noalloc) against the context-based one.

vpt_launch_plain_noalloc is for callers that cannot call cudaMalloc, such as a host renderer
whose device memory belongs to its own pool allocator: they pass every input and output as
device pointers and the launch keeps its scratch in a fixed __device__ array. This test builds
those caller-owned buffers (here with torch) from the same inputs a VptContext uses, calls the
entry point twice in a row, and checks the images against two vpt_launch_plain calls. It lives
in its own file, collected last, and passes in a fresh process or after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from rtc8_gb300 import _lib
from rtc8_gb300.renderer import Renderer, constant_environment, frame_params, setup_scene

from ._scenes import small_config_mode, volume_for

pytestmark = pytest.mark.gpu


def _leaf_layout(vox: np.ndarray):
    """Leaf table and packed 8^3 leaves (value order x<<6 | y<<3 | z) of a dense volume."""
    nx, ny, nz = vox.shape
    lx, ly, lz = [(d + 7) // 8 for d in vox.shape]
    pad = np.zeros((lx * 8, ly * 8, lz * 8), np.float32)
    pad[:nx, :ny, :nz] = vox
    leaves = pad.reshape(lx, 8, ly, 8, lz, 8).transpose(0, 2, 4, 1, 3, 5).reshape(lx * ly * lz, 512)
    active = leaves.max(axis=1) > 0
    table = np.where(active, np.cumsum(active) - 1, -1).astype(np.int32)
    return table, np.ascontiguousarray(leaves[active]), (lx, ly, lz)


def _caller_buffers(r: Renderer, cfg, vox):
    import torch

    dev = torch.device("cuda")
    table, values, (lx, ly, lz) = _leaf_layout(vox)
    cells = r.cell_majorants()              # 8^3-voxel cells: the DDA grid at majorant_cell_log2 = 3
    info = r.volume_info()
    env = constant_environment(cfg.env_constant)
    texels = np.concatenate([env, np.zeros(env.shape[:2] + (1,), np.float32)], axis=2)
    mips, minfo = r.importance_map()
    seeds = r.rng_states()
    npix = cfg.width * cfg.height
    bufs = {
        "table": torch.from_numpy(table).to(dev), "values": torch.from_numpy(values).to(dev),
        "maj": torch.from_numpy(cells).to(dev), "env": torch.from_numpy(np.ascontiguousarray(texels)).to(dev),
        "mips": torch.from_numpy(mips).to(dev), "rng": torch.from_numpy(seeds.view(np.int64)).to(dev),
        "sum": torch.zeros(3 * npix, dtype=torch.float64, device=dev),
        "mean": torch.zeros(3 * npix, dtype=torch.float32, device=dev),
    }
    a = _lib.VptNoAllocTrace()
    a.frame = frame_params(cfg)
    a.width, a.height = cfg.width, cfg.height
    a.leaf_table, a.leaf_values, a.majorants = (bufs[k].data_ptr() for k in ("table", "values", "maj"))
    a.nx, a.ny, a.nz = vox.shape
    a.mx, a.my, a.mz = lx, ly, lz
    a.voxel_size = 1.0 / vox.shape[0]
    a.origin[:] = [-0.5, -0.5, -0.5]
    a.global_majorant = info["global_majorant"]
    a.env_texels = bufs["env"].data_ptr()
    a.env_h, a.env_w = env.shape[:2]
    a.imp_mips = bufs["mips"].data_ptr()
    a.map_w, a.map_h, a.num_mips, a.imp_integral = minfo["map_w"], minfo["map_h"], minfo["num_mips"], minfo["integral"]
    a.rng, a.sum_rgb, a.mean_rgb = (bufs[k].data_ptr() for k in ("rng", "sum", "mean"))
    return a, bufs


@pytest.mark.parametrize("streams", [0, 1])
def test_noalloc_launch_matches_context_launch(cuda_device, streams):
    import torch

    cfg = small_config_mode(size=40, n=32).replace(rng_stream_mode=streams)
    assert cfg.majorant_cell_log2 == 3
    vox = volume_for(cfg)
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg, volume=vox)
    args, bufs = _caller_buffers(r, cfg, vox)
    lib = _lib.load()
    spp = 3
    for call in range(2):  # two calls in a row, continuing the accumulation and the streams
        args.spp, args.accum_base, args.stream_base = spp, call * spp, call * spp
        rc = lib.vpt_launch_plain_noalloc(C.byref(args), None)
        assert rc == 0, lib.vpt_last_error()
        r.launch_plain(spp)
    torch.cuda.synchronize()
    ref_sum, n = r.download_sum()
    assert n == 2 * spp
    got_sum = bufs["sum"].cpu().numpy().reshape(ref_sum.shape)
    got_mean = bufs["mean"].cpu().numpy().reshape(ref_sum.shape)
    assert got_sum.sum() > 0
    if streams == 0:
        # Same kernel, same inputs, one lane per pixel: identical bits.
        np.testing.assert_array_equal(got_sum, ref_sum)
        np.testing.assert_array_equal(bufs["rng"].cpu().numpy().view(np.uint64), r.rng_states())
    else:
        # FP64 atomics add a pixel's samples in launch-dependent order.
        np.testing.assert_allclose(got_sum, ref_sum, rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(got_mean, r.download_mean(), rtol=1e-6, atol=1e-9)
    r.close()


def test_noalloc_rejects_sizes_beyond_the_scratch(cuda_device):
    cfg = small_config_mode(size=16, n=16)
    vox = volume_for(cfg)
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg, volume=vox)
    args, bufs = _caller_buffers(r, cfg, vox)
    lib = _lib.load()
    args.spp = 4096 + 1
    assert lib.vpt_launch_plain_noalloc(C.byref(args), None) == -1
    assert b"VPT_NOALLOC_MAX_SPP" in lib.vpt_last_error()
    r.close()


def test_noalloc_reports_device_errors_in_the_callers_word(cuda_device):
    """A segment that hits its step cap sets VPT_DEVERR_STEP_CAP in the caller's error word, as
    vpt_get_device_errors reports it for a context launch."""
    import torch

    from ._scenes import small_reference_mode

    cfg = small_reference_mode(size=16, n=16, sigma=60.0).replace(max_steps_per_segment=3)
    vox = volume_for(cfg)
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg, volume=vox)
    args, bufs = _caller_buffers(r, cfg, vox)
    word = torch.zeros(1, dtype=torch.int32, device="cuda")
    args.device_errors = word.data_ptr()
    args.spp = 2
    lib = _lib.load()
    assert lib.vpt_launch_plain_noalloc(C.byref(args), None) == 0, lib.vpt_last_error()
    r.launch_plain(2)
    torch.cuda.synchronize()
    assert r.device_errors() & 0x1
    assert int(word.item()) == r.device_errors()
    r.close()


def test_noalloc_leaves_device_memory_unchanged(cuda_device):
    """After the first call (which looks the scratch address up), further calls change the
    device's free memory by nothing."""
    import torch

    cfg = small_config_mode(size=24, n=24)
    vox = volume_for(cfg)
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg, volume=vox)
    args, bufs = _caller_buffers(r, cfg, vox)
    lib = _lib.load()
    args.spp = 2
    assert lib.vpt_launch_plain_noalloc(C.byref(args), None) == 0, lib.vpt_last_error()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    for call in range(1, 4):
        args.accum_base, args.stream_base = 2 * call, 2 * call
        assert lib.vpt_launch_plain_noalloc(C.byref(args), None) == 0, lib.vpt_last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free_before
    assert bufs["sum"].sum().item() > 0
    r.close()
