"""The C-ABI library builds for sm_103a, loads, and exports every entry point of include/*.h.

No compute call is made here (this suite runs without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**\s*([a-z][a-z0-9_]*)\s*\(", text,
                             flags=re.M):
            names.append(m.group(1))
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from rtc8_gb300 import build

    path = build.build()
    return ctypes.CDLL(str(path))


def test_headers_declare_entry_points():
    names = declared_functions()
    assert "vpt_launch_plain" in names and "vpt_create" in names
    assert len(names) >= 25


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"missing exports: {missing}"


def test_python_binding_covers_every_symbol():
    from rtc8_gb300 import _lib

    missing = [n for n in declared_functions() if n not in _lib.EXPORTS]
    assert not missing, f"no ctypes declaration for: {missing}"


def test_library_built_for_sm_103a():
    from rtc8_gb300 import build

    assert "arch=compute_103a,code=sm_103a" in build.ARCH


def test_cpp_shim_compiles_links_and_checks_hashgrid_arguments(lib, tmp_path):
    """include/rtc8_nrc.hpp: the reference's rtc8::NeuralRadianceCache interface over the C ABI
    compiles and links as the renderer would use it, with the reference's own HashGrid call
    (renderer_scene.cpp:50); an out-of-range layer count throws the library's message before any
    device work, so this runs without a GPU (the GPU tests run the valid call)."""
    import shutil
    import subprocess

    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    src = tmp_path / "shim.cpp"
    src.write_text(
        '#include "rtc8_nrc.hpp"\n#include <cstdio>\n'
        "int main(int argc, char**) {\n  rtc8::NeuralRadianceCache cache;\n"
        "  if (argc > 1) cache.initialize(rtc8::PositionEncoding::HashGrid, 2, 0.01f);\n"
        "  try { cache.initialize(rtc8::PositionEncoding::HashGrid, 9, 1e-2f); }\n"
        '  catch (const std::exception& e) { std::puts(e.what()); return 0; }\n  return 1;\n}\n')
    from rtc8_gb300 import build

    libdir = build.LIB.parent
    exe = tmp_path / "shim"
    cuda_inc = Path(build.nvcc()).resolve().parent.parent / "include"
    subprocess.run([cxx, "-std=c++17", "-I", str(ROOT / "include"), "-I", str(cuda_inc), str(src), "-L", str(libdir),
                    "-lrtc8_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    assert "num_hidden_layers out of range" in out and "hash grid" in out


def test_cpp_renderer_header_compiles_and_orients_like_python(lib, tmp_path):
    """include/rtc8_vpt.hpp: rtc8::VolumeRenderer and look_at_quaternion compile and link; the
    camera quaternion equals the Python camera's (float32 rounding) for looks along the axes and
    the diagonals, and a bad image size throws with the library's message (no device work)."""
    import shutil
    import subprocess

    import numpy as np

    from rtc8_gb300 import build
    from rtc8_gb300.configs import look_at

    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    eyes = [(0.0, 0.0, 3.0), (3.0, 0.0, 0.0), (0.0, 0.0, -3.0), (-2.0, 0.5, 0.1), (1.7, 1.1, -2.3),
            (-1.0, -2.0, -1.5), (0.3, 0.2, 4.0)]
    src = tmp_path / "vpt_shim.cpp"
    calls = "\n".join(
        f"  rtc8::look_at_quaternion({{{e[0]!r}, {e[1]!r}, {e[2]!r}}}, {{0.0, 0.0, 0.0}}, {{0.0, 1.0, 0.0}}, q);\n"
        '  std::printf("%.9g %.9g %.9g %.9g\\n", q[0], q[1], q[2], q[3]);' for e in eyes)
    src.write_text(
        '#include "rtc8_vpt.hpp"\n#include <cstdio>\n'
        "int main() {\n  float q[4];\n" + calls + "\n"
        "  try { rtc8::VolumeRenderer r(0, 16); }\n"
        '  catch (const std::exception& e) { std::printf("%s\\n", e.what()); return 0; }\n  return 1;\n}\n')
    libdir = build.LIB.parent
    exe = tmp_path / "vpt_shim"
    cuda_inc = Path(build.nvcc()).resolve().parent.parent / "include"
    subprocess.run([cxx, "-std=c++17", "-Wall", "-Werror", "-I", str(ROOT / "include"), "-I", str(cuda_inc), str(src),
                    "-L", str(libdir), "-lrtc8_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    lines = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.splitlines()
    for e, line in zip(eyes, lines):
        q = np.array([float(v) for v in line.split()])
        want = look_at(e, (0.0, 0.0, 0.0)).astype(np.float32)
        np.testing.assert_allclose(q, want, atol=1.5e-7)
    assert "vpt_create" in lines[len(eyes)] and "bad arguments" in lines[len(eyes)]
