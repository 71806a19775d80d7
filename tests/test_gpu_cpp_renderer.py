"""The C++ host side (include/rtc8_vpt.hpp, rtc8::VolumeRenderer) driving the C ABI as a C++
renderer would: scene setup, a path-tracing launch, the accumulated mean and the tone-mapped
8-bit frame. Its output is bit-identical to the same calls through the Python binding (same
scene, seed and launch; the tracker is deterministic)."""
import shutil
import struct
import subprocess
from pathlib import Path

import ctypes as C
import numpy as np
import pytest

from rtc8_gb300 import build
from rtc8_gb300.configs import volume_box
from rtc8_gb300.renderer import Renderer, constant_environment, frame_params

from ._scenes import small_config_mode, volume_for

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

_SRC = r'''
#include "rtc8_vpt.hpp"
#include <cstdio>
#include <cstring>
#include <vector>

template <class T> static bool rd(FILE* f, T* p, size_t n) { return std::fread(p, sizeof(T), n, f) == n; }

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 2;
    int32_t h[8];
    float vs_origin[4];
    uint64_t seed = 0;
    uint32_t fp_size = 0;
    if (!rd(f, h, 8) || !rd(f, vs_origin, 4) || !rd(f, &seed, 1) || !rd(f, &fp_size, 1)) return 2;
    if (fp_size != sizeof(VptFrameParams)) return 3;
    VptFrameParams fp;
    if (!rd(f, reinterpret_cast<unsigned char*>(&fp), sizeof(fp))) return 2;
    const int32_t w = h[0], ht = h[1], nx = h[2], ny = h[3], nz = h[4], ew = h[5], eh = h[6], spp = h[7];
    std::vector<float> vox(size_t(nx) * ny * nz), env(size_t(ew) * eh * 3);
    if (!rd(f, vox.data(), vox.size()) || !rd(f, env.data(), env.size())) return 2;
    std::fclose(f);

    rtc8::VolumeRenderer r(w, ht);
    r.set_volume_dense(vox.data(), nx, ny, nz, vs_origin[0], vs_origin + 1);
    r.set_environment(env.data(), ew, eh);
    r.set_frame(fp);
    r.seed(seed);
    r.path_trace(nullptr, uint32_t(spp));
    r.synchronize(nullptr);
    const std::vector<float> mean = r.mean_rgb();
    const std::vector<uint32_t> rgba = r.image_rgba8(2.0f);
    const uint32_t errs = r.device_errors();
    f = std::fopen(argv[2], "wb");
    std::fwrite(mean.data(), sizeof(float), mean.size(), f);
    std::fwrite(rgba.data(), sizeof(uint32_t), rgba.size(), f);
    std::fwrite(&errs, sizeof(errs), 1, f);
    std::fclose(f);
    return 0;
}
'''


def test_cpp_volume_renderer_matches_python_binding(cuda_device, tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    cfg = small_config_mode(size=40, n=32)
    vox = np.ascontiguousarray(volume_for(cfg), dtype=np.float32)
    env = constant_environment(cfg.env_constant if cfg.env_constant is not None else 0.5)
    vs, origin = volume_box(cfg.volume)
    fp = frame_params(cfg)
    spp = 3
    blob = struct.pack("<8i", cfg.width, cfg.height, *vox.shape, env.shape[1], env.shape[0], spp)
    blob += struct.pack("<4f", vs, *origin) + struct.pack("<QI", cfg.rng_seed, C.sizeof(fp))
    blob += bytes(fp) + vox.tobytes() + np.ascontiguousarray(env, dtype=np.float32).tobytes()
    (tmp_path / "in.bin").write_bytes(blob)

    src = tmp_path / "render.cpp"
    src.write_text(_SRC)
    libdir = build.LIB.parent
    cuda_inc = Path(build.nvcc()).resolve().parent.parent / "include"
    exe = tmp_path / "render"
    subprocess.run([cxx, "-std=c++17", "-O1", "-I", str(ROOT / "include"), "-I", str(cuda_inc), str(src),
                    "-L", str(libdir), "-lrtc8_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    res = (tmp_path / "out.bin").read_bytes()
    npix = cfg.width * cfg.height
    mean_cpp = np.frombuffer(res[: 12 * npix], dtype=np.float32).reshape(cfg.height, cfg.width, 3)
    rgba_cpp = np.frombuffer(res[12 * npix: 16 * npix], dtype=np.uint32)
    errs_cpp = struct.unpack("<I", res[16 * npix:])[0]

    r = Renderer(cfg.width, cfg.height)
    r.set_volume_dense(vox, vs, origin)
    r.set_environment_rgb(env)
    r.set_frame(fp)
    r.seed_rng(cfg.rng_seed)
    r.launch_plain(spp)
    r.synchronize()
    mean = r.download_mean()
    rgba = r.image_rgba8(2.0).reshape(-1, 4)
    assert mean.max() > 0
    np.testing.assert_array_equal(mean_cpp, mean)
    np.testing.assert_array_equal(rgba_cpp.view(np.uint8).reshape(-1, 4), rgba)
    assert errs_cpp == r.device_errors() == 0
    r.close()
