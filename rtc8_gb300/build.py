"""Builds the product library ``librtc8_gb300.so`` in-tree for sm_103a.

Each ``csrc/*.cu`` translation unit is compiled in parallel with nvcc and linked into one
shared library that exports the C ABI declared in ``include/rtc8_vpt.h`` and
``include/rtc8_nrc.h``. The tracker units are compiled without fused multiply-add
contraction so that path decisions follow the reference's float operation order.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "librtc8_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr",
          "-Xptxas", "-warn-spills"]
# Units whose float arithmetic must follow the reference's operation order: no FMA contraction,
# so products and sums round as in the oracle's restatement (compiled with -ffp-contract=off).
# The scene unit is among them so that the seeded fBm volumes equal the host generator's bit for bit.
NO_FMA_UNITS = {"vpt_tracer.cu", "vpt_post.cu", "vpt_wavefront.cu", "vpt_scene.cu"}
# The tracker units use the reference's own device arithmetic: it compiles its path-tracing
# programs and kernels with --use_fast_math (renderer/CMakeLists.txt:48, 65, 91), i.e. intrinsic
# transcendentals, approximate division and square root, denormals flushed. FMA contraction,
# which --use_fast_math would also switch on, stays off (the explicit -fmad=false after it wins).
FAST_MATH_UNITS = {"vpt_tracer.cu", "vpt_wavefront.cu"}
FAST_MATH = ["--use_fast_math", "-fmad=false"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build rtc8_gb300")
    return exe


def _compile(src: Path, verbose_ptxas: bool) -> tuple[Path, str]:
    obj = BUILD / (src.stem + ".o")
    cmd = [nvcc(), "-c", str(src), "-o", str(obj), *ARCH, *COMMON]
    if src.name in NO_FMA_UNITS:
        cmd += ["-fmad=false"]
    if src.name in FAST_MATH_UNITS:
        cmd += FAST_MATH
    if verbose_ptxas:
        cmd += ["-Xptxas", "-v"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build(force: bool = False, verbose_ptxas: bool = False, jobs: int | None = None) -> Path:
    srcs = sorted(CSRC.glob("*.cu"))
    deps = srcs + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted((PKG.parent / "include").glob("*.h"))
    if LIB.exists() and not force:
        lib_mtime = LIB.stat().st_mtime
        if all(p.stat().st_mtime <= lib_mtime for p in deps) and Path(__file__).stat().st_mtime <= lib_mtime:
            return LIB
    BUILD.mkdir(exist_ok=True)
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    logs = []
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose_ptxas), srcs))
    objs = [r[0] for r in results]
    logs = [r[1] for r in results if r[1]]
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc(), "-shared", "-o", str(tmp), *[str(o) for o in objs], *ARCH, "-cudart", "shared"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    if verbose_ptxas:
        for log in logs:
            sys.stderr.write(log)
    return LIB


SKY_TABLES = PKG / "data" / "hosek_tables.bin"


def generate_sky_tables(ref: Path, force: bool = False) -> Path | None:
    """Writes data/hosek_tables.bin (the Hosek-Wilkie 2013 spectral model's coefficient tables)
    from the model's C source in the reference checkout `ref` (ext/hosek_wilkie_2013), if that
    checkout is present; the file is generated, not committed. Returns its path or None."""
    src = ref / "ext" / "hosek_wilkie_2013" / "ArHosekSkyModel.c"
    if not src.exists():
        return SKY_TABLES if SKY_TABLES.exists() else None
    gen = PKG / "data" / "hosek_tables_gen.c"
    if SKY_TABLES.exists() and not force and SKY_TABLES.stat().st_mtime >= gen.stat().st_mtime:
        return SKY_TABLES
    BUILD.mkdir(exist_ok=True)
    exe = BUILD / "hosek_tables_gen"
    cc = os.environ.get("CC", "gcc")
    res = subprocess.run([cc, "-O1", "-w", "-std=gnu99", "-I", str(src.parent), str(gen), str(src), "-lm", "-o",
                          str(exe)], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"sky table generator failed to build:\n{res.stderr}")
    tmp = SKY_TABLES.with_suffix(".tmp")
    subprocess.run([str(exe), str(tmp)], check=True)
    os.replace(tmp, SKY_TABLES)
    return SKY_TABLES


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(LIB)
