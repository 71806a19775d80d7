"""Builds the oracle (test infrastructure only) into ``oracle/_build/liboracle.so``.

The restatement is plain C++ compiled with OpenMP and without floating-point contraction,
so the x86-64 development host and the aarch64 GPU host produce identical results.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"
LIB = OUT / "liboracle.so"
SRCS = [HERE / "vpt_oracle.cpp", HERE / "nrc_oracle.cpp", HERE / "nrc_setup_oracle.cpp", HERE / "scene_oracle.cpp"]
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math"]


def build(force: bool = False) -> Path:
    srcs = [s for s in SRCS if s.exists()]
    deps = srcs + sorted(HERE.glob("*.h"))
    if LIB.exists() and not force and all(d.stat().st_mtime <= LIB.stat().st_mtime for d in deps):
        return LIB
    OUT.mkdir(exist_ok=True)
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++"), *FLAGS, "-o", str(tmp), *[str(s) for s in srcs]]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
