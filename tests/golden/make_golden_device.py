"""Runs the reference's own device code on a GPU and records its answers as a golden fixture.

oracle/build_ref.sh (in a checkout with the reference next to it) compiles oracle/ref_kat_device.cu
— known-answer kernels around the reference's PCG32RNG, SchlickPhaseFunction,
HierarchicalImportanceMap, ImageBasedEnvironmentalLight, LambertBRDF, SimplePBR_BRDF and
offsetRayOrigin, plus the reference's own
importance-map kernels (renderer/gpu_kernels/compute_light_probs.cu) and radiance-cache set-up
kernels (renderer/gpu_kernels/nrc_set_up_kernels.cu) — to oracle/_ref/ref_kat_device.ptx. On a
GPU host this script builds oracle/kat_device_loader.cpp, feeds it seeded inputs and writes the
inputs and the reference's outputs to one compressed .npz:

    python tests/golden/make_golden_device.py --out <file.npz>

The committed copy is tests/golden/ref_device_kat.npz; tests/test_oracle_device_kat.py checks the
oracle against it on the CPU.
"""
from __future__ import annotations

import argparse
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
REF = ROOT / "oracle" / "_ref"
PTX = REF / "ref_kat_device.ptx"
LOADER = REF / "kat_device_loader"

# Radiance-cache set-up scenario: a 32x32 image, 64 training suffixes, 512 training vertices.
IMG_W, IMG_H = 32, 32
MAX_SUFFIX = 64
N_VERT = 512
INVALID = 0x3FFFFF


def build_loader() -> None:
    if LOADER.exists():
        return
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    subprocess.run([nvcc, "-std=c++17", "-O2", str(ROOT / "oracle" / "kat_device_loader.cpp"), "-o", str(LOADER),
                    "-lcuda"], check=True)


def queries(rng, n: int) -> np.ndarray:
    q = np.zeros((n, 14), np.float32)
    q[:, 0:3] = rng.random((n, 3))
    q[:, 3] = rng.random(n) * np.pi
    q[:, 4] = rng.random(n) * 2 * np.pi
    q[:, 5] = rng.random(n) * np.pi
    q[:, 6] = rng.random(n) * 2 * np.pi
    q[:, 7] = rng.random(n)
    q[:, 8:11] = rng.random((n, 3))
    q[:, 11:14] = rng.random((n, 3)) * 0.2
    return q


def make_inputs(rng) -> dict:
    d = {}
    d["pcg.states"] = rng.integers(0, 2 ** 63, 64, dtype=np.int64).view(np.uint64) * np.uint64(3)
    d["schlick.k"] = np.array([-0.9, -0.4, 0.0, 0.3, 0.8], np.float32)
    u = rng.random((256, 2)).astype(np.float32)
    u[:4] = [[0.0, 0.0], [0.5, 0.5], [0.999999, 0.25], [0.125, 0.999999]]
    d["schlick.u"] = u
    # A non-uniform environment: gamma-distributed texels, a few black ones, a bright spot.
    ew, eh = 64, 32
    env = rng.gamma(0.6, 1.0, (eh, ew, 3)).astype(np.float32)
    env[5, 10:14] = 0.0
    env[12:14, 40:43] *= 500.0
    d["env.dims"] = np.array([ew, eh], np.uint32)
    d["env.rgb"] = env
    ue = rng.random((1024, 2)).astype(np.float32)
    ue[:3] = [[0.0, 0.0], [0.5, 0.5], [0.999999, 0.999999]]
    d["env.u"] = ue
    # prepareNRC: previous frame made 40000 training records on an 8x8 training image.
    params = np.zeros(16, np.uint32)
    params[:12] = [IMG_W, IMG_H, MAX_SUFFIX, 1, 12345, 0, 40000, 8, 8, 3, N_VERT, N_VERT]
    params[12] = np.array([2.0], np.float32).view(np.uint32)[0]
    d["nrc.params"] = params
    # propagateRadianceValues: 64 suffixes, each the tail of a chain of up to 8 vertices.
    prev = np.full(N_VERT, INVALID, np.uint32)
    term_prev = np.full(MAX_SUFFIX, INVALID, np.uint32)
    v = 0
    for s in range(MAX_SUFFIX):
        length = int(rng.integers(0, 9)) if s % 7 else 0
        last = INVALID
        for _ in range(length):
            if v >= N_VERT:
                break
            prev[v] = last
            last = v
            v += 1
        term_prev[s] = last
    has_q = (rng.random(MAX_SUFFIX) < 0.7).astype(np.uint32)
    plen = rng.integers(0, 200, MAX_SUFFIX).astype(np.uint32)
    d["prop.term"] = np.concatenate([term_prev, has_q, plen])
    d["prop.inferred"] = (rng.standard_normal((MAX_SUFFIX, 3)) * 2).astype(np.float32)  # negatives clamp to 0
    d["prop.query"] = queries(rng, MAX_SUFFIX)
    d["prop.vtp"] = rng.random((N_VERT, 3)).astype(np.float32)
    d["prop.vprev"] = prev
    d["prop.target0"] = rng.random((N_VERT, 3)).astype(np.float32)
    q0 = queries(rng, N_VERT)
    q0[::37, 8:14] = 0.0                                     # zero reflectance: safeDivide gives 0
    d["prop.query0"] = q0
    # shuffleTrainingData: 512 records with unique positions, some invalid queries / targets.
    qs = queries(rng, N_VERT)
    qs[:, 0] = np.arange(N_VERT, dtype=np.float32) / N_VERT
    qs[3, 5] = np.nan
    qs[77, 9] = np.inf
    ts = (rng.random((N_VERT, 3)) * 4).astype(np.float32)
    ts[5, 1] = -1.0
    ts[6, 0] = np.nan
    ts[7] = [1e7, 3e6, 2.0]                                  # clamped to 1e6 after scaling
    d["shuf.query0"] = qs
    d["shuf.target0"] = ts
    # accumulateInferredRadianceValues on the 32x32 image (finite, non-negative contributions).
    npix = IMG_W * IMG_H
    d["acc.ttp"] = rng.random((npix, 3)).astype(np.float32)
    d["acc.hasq"] = (rng.random(npix) < 0.6).astype(np.uint32)
    d["acc.contrib"] = rng.random((npix, 3)).astype(np.float32)
    d["acc.inferred"] = (rng.standard_normal((npix, 3)) * 2).astype(np.float32)
    d["acc.query"] = queries(rng, npix)
    d["acc.prev"] = rng.random((npix, 3)).astype(np.float32)
    # Surface BSDFs (drawn after everything above, so the earlier inputs keep their values): the
    # materials' decoded values (8-bit sRGB base colour, 8-bit roughness / metallic), query
    # directions over both hemispheres including grazing ones, variates, second directions.
    raw = surface_materials()
    d["bsdf.raw"] = raw
    d["bsdf.params"] = decoded_bsdf_params(raw)
    nb = 512
    qd = rng.standard_normal((nb, 3))
    qd[:8, 2] = np.abs(qd[:8, 2]) * 1e-3
    d["bsdf.q"] = (qd / np.linalg.norm(qd, axis=1, keepdims=True)).astype(np.float32)
    ub = rng.random((nb, 2)).astype(np.float32)
    ub[:3] = [[0.0, 0.0], [0.5, 0.5], [0.999999, 0.999999]]
    d["bsdf.u"] = ub
    vd = rng.standard_normal((nb, 3))
    d["bsdf.v"] = (vd / np.linalg.norm(vd, axis=1, keepdims=True)).astype(np.float32)
    # offsetRayOrigin: points near and far from the origin, unit normals.
    npts = 256
    pts = (rng.standard_normal((npts, 3)) * np.where(rng.random((npts, 1)) < 0.3, 0.01, 10.0)).astype(np.float32)
    nrm = rng.standard_normal((npts, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    d["offset.pn"] = np.concatenate([pts, nrm.astype(np.float32)], axis=1)
    return d


def surface_materials() -> np.ndarray:
    """Raw materials (kind, base colour, roughness, metallic; the immediate values a scene gives):
    SimplePBR dielectrics from rough to smooth, metals, and Lambert."""
    return np.array([[0, 0.8, 0.8, 0.8, 0.5, 0.0], [0, 0.55, 0.6, 0.8, 0.3, 0.0], [0, 0.95, 0.75, 0.45, 0.2, 1.0],
                     [0, 0.2, 0.9, 0.3, 0.02, 0.0], [0, 0.9, 0.9, 0.9, 1.0, 0.5], [1, 0.75, 0.15, 0.12, 0.0, 0.0]],
                    np.float32)


def decoded_bsdf_params(raw: np.ndarray) -> np.ndarray:
    """The values the reference's 1x1 textures return: 8-bit truncation, sRGB decode of the colour
    (renderer_scene.cpp:860-900, 1202-1255), smoothness = min(1 - roughness, 0.999) (:1978)."""
    def unorm8(v):
        return np.minimum(np.floor(np.float32(255.0) * np.float32(v)), 255.0)

    out = []
    for kind, r, g, b, rough, metal in raw:
        c = unorm8(np.array([r, g, b])) / 255.0
        lin = np.where(c <= 0.04045, c / 12.92, ((c + 0.055) / 1.055) ** 2.4).astype(np.float32)
        smooth = np.float32(min(np.float32(1.0) - np.float32(unorm8(rough) / 255.0), np.float32(0.999)))
        out.append([kind, *lin, smooth, np.float32(unorm8(metal) / 255.0)])
    return np.array(out, np.float32)


OUTPUTS = {
    "sizes.out": np.uint32, "pcg.raw": np.uint32, "pcg.f01": np.float32, "schlick.out": np.float32,
    "env.out": np.float32, "env.integral": np.float32, "env.mips": np.float32,
    "prep.out": np.uint32, "prep.minmax": np.float32, "prep.avg": np.float32, "prep.term": np.uint32,
    "prop.target_out": np.float32, "shuf.query1": np.float32, "shuf.target1": np.float32,
    "shuf.minmax": np.float32, "shuf.avg": np.float32, "acc.out": np.float32, "bsdf.out": np.float32,
    "offset.out": np.float32,
}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    args = ap.parse_args()
    if not PTX.exists():
        print(f"{PTX} is missing: build it with oracle/build_ref.sh where the reference checkout is", file=sys.stderr)
        return 2
    build_loader()
    rng = np.random.default_rng(20261204)
    inputs = make_inputs(rng)
    with tempfile.TemporaryDirectory() as tmp:
        for name, arr in inputs.items():
            np.ascontiguousarray(arr).tofile(Path(tmp) / name)
        subprocess.run([str(LOADER), str(PTX), tmp], check=True)
        outputs = {name: np.fromfile(Path(tmp) / name, dtype=t) for name, t in OUTPUTS.items()}
    np.savez_compressed(args.out, **{"in:" + k: v for k, v in inputs.items()},
                        **{"out:" + k: v for k, v in outputs.items()})
    print("wrote", args.out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
