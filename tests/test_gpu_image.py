"""The tone-map + 8-bit sRGB kernel on the GPU, through the C ABI, against the oracle's
restatement on the same mean image. The GPU evaluates powf/expf, the oracle std::pow/std::exp:
floats agree within 4e-6 relative (a few ulp), bytes within 1 where a value sits on a
quantisation step, and exactly for >= 99% of the channels."""
import ctypes as C

import numpy as np
import pytest

from oracle import orc
from rtc8_gb300 import _lib, image
from rtc8_gb300.renderer import Renderer, setup_scene

from ._scenes import small_config_mode

pytestmark = pytest.mark.gpu


def _rendered(cfg, spp=4):
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg)
    r.launch_plain(spp)
    r.synchronize()
    return r


@pytest.mark.parametrize("brightness", [1.0, 3.0])
def test_tonemap_kernel_matches_oracle(cuda_device, brightness):
    import torch

    cfg = small_config_mode(size=48, n=32)
    r = _rendered(cfg)
    mean = r.download_mean()
    # brighten part of the image so that the tone map's shoulder and the 255 clamp are exercised
    assert mean.max() > 0
    f32 = torch.zeros((cfg.height * cfg.width, 4), dtype=torch.float32, device="cuda")
    u8 = torch.zeros(cfg.height * cfg.width, dtype=torch.int32, device="cuda")
    _lib.check(r.lib.vpt_tonemap(r.ctx, None, brightness, _lib.VPT_SDR_SRGB, C.c_void_p(f32.data_ptr()),
                                 C.c_void_p(u8.data_ptr())), "vpt_tonemap")
    torch.cuda.synchronize()
    g_rgb = f32.cpu().numpy()
    g_rgba = u8.cpu().numpy().view(np.uint8).reshape(-1, 4)
    o_rgb, o_rgba = orc.tonemap(mean.reshape(-1, 3), brightness)
    np.testing.assert_allclose(g_rgb[:, :3], o_rgb, rtol=4e-6, atol=1e-7)
    assert np.all(g_rgb[:, 3] == 1.0)
    diff = np.abs(g_rgba.astype(np.int32) - o_rgba.astype(np.int32))
    assert diff.max() <= 1 and (diff == 0).mean() >= 0.99
    assert np.all(g_rgba[:, 3] == 255) and g_rgba[:, :3].max() > 100
    # the synchronous download runs the same kernel; flip-y writes the rows bottom-up
    img = r.image_rgba8(brightness)
    np.testing.assert_array_equal(img.reshape(-1, 4), g_rgba)
    flipped = r.image_rgba8(brightness, flip_y=True)
    np.testing.assert_array_equal(flipped, img[::-1])
    lin = r.image_rgba8(brightness, srgb=False)
    assert np.all(lin[..., :3] <= img[..., :3])
    r.close()


def test_png_frame_of_a_render(cuda_device, tmp_path):
    from .test_image_output import decode_png

    cfg = small_config_mode(size=32, n=32)
    r = _rendered(cfg, spp=2)
    p = tmp_path / "000.png"
    r.save_png(p)
    np.testing.assert_array_equal(decode_png(p.read_bytes()), r.image_rgba8())
    e = tmp_path / "output.exr"
    r.save_exr(e)
    assert e.read_bytes() == image.encode_exr(r.download_mean())
    r.close()


def test_environment_from_exr(cuda_device, tmp_path):
    """An EXR environment map uploads the same texels and importance map as the float array it
    was written from (half precision)."""
    from ._scenes import small_config_mode

    rng = np.random.default_rng(5)
    env = (rng.random((32, 64, 3)) * 3).astype(np.float32)
    p = image.write_exr(tmp_path / "env.exr", env, compression=image.EXR_ZIP)
    cfg = small_config_mode(size=16, n=16)
    a = Renderer(cfg.width, cfg.height)
    setup_scene(a, cfg)
    rgb = a.load_environment_exr(p)
    np.testing.assert_array_equal(rgb, env.astype(np.float16).astype(np.float32))
    b = Renderer(cfg.width, cfg.height)
    setup_scene(b, cfg)
    b.set_environment_rgb(env.astype(np.float16).astype(np.float32))
    ma, ia = a.importance_map()
    mb, ib = b.importance_map()
    np.testing.assert_array_equal(ma, mb)
    assert ia == ib
    np.testing.assert_array_equal(a.download_environment(64, 32), b.download_environment(64, 32))
    a.close()
    b.close()
