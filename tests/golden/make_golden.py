"""Regenerates the golden fixtures from programs built against the reference's own sources.

Run with the reference checkout in REF (default: a checkout named "reference" next to this
repository):

    python tests/golden/make_golden.py

It builds oracle/_ref/ with oracle/build_ref.sh and writes
  tests/golden/ref_basic_types.json   common/basic_types.{h,cpp} outputs (polar maps, frames,
                                      quaternion matrices, 16-band CIE CMF integrals)
  tests/golden/ref_nanovdb.json       NanoVDB 32.3 GridBuilder / SampleFromVoxels<1> / Ray::clip
  tests/golden/ref_hosek_kat.json     Hosek-Wilkie radiance at fixed angles (first sky entry)
  tests/golden/ref_hosek_states.json  Hosek-Wilkie model states and direct solar radiance at six
                                      further (elevation, turbidity, albedo) combinations
  tests/golden/nvdb/                  .nvdb files written by NanoVDB 32.3 io::writeGrid(s)
                                      (gzip-compressed when uncoded) and ref_nvdb_files.json,
                                      the reference's own reading of them
  rtc8_gb300/data/hosek_sky.json      per-band sky states used by the sky configurations
The fixtures are committed; the GPU host never reads the reference.
"""
from __future__ import annotations

import gzip
import json
import os
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
REF_BIN = ROOT / "oracle" / "_ref"
GOLDEN = ROOT / "tests" / "golden"
DATA = ROOT / "rtc8_gb300" / "data"

# (solar elevation deg, turbidity, ground albedo; negative = the renderer's per-band ramp)
SKY_REQUESTS = [(20.0, 3.0, 0.3), (30.0, 4.0, -1.0), (20.0, 4.0, -1.0)]
# More model states of the library, at other elevations, turbidities and albedos (fixture only).
SKY_CHECKS = [(5.0, 2.0, 0.1), (45.0, 6.5, -1.0), (70.0, 9.3, 0.8), (1.5, 10.0, 0.5), (88.0, 1.0, -1.0),
              (12.5, 3.7, 0.3)]


def run(name: str, *args: str) -> dict:
    out = subprocess.run([str(REF_BIN / name), *args], check=True, capture_output=True, text=True).stdout
    return json.loads(out)


def main() -> int:
    env = dict(os.environ)
    env.setdefault("REF", str(ROOT.parent / "reference"))
    subprocess.run(["bash", str(ROOT / "oracle" / "build_ref.sh")], check=True, env=env)
    basic = run("ref_kat_basic")
    (GOLDEN / "ref_basic_types.json").write_text(json.dumps(basic))
    nvdb = run("ref_kat_nanovdb")
    (GOLDEN / "ref_nanovdb.json").write_text(json.dumps(nvdb))
    args = [str(x) for req in SKY_REQUESTS for x in req]
    sky = run("ref_hosek_dump", *args)
    kat = sky["entries"][0].pop("radiance_kat")
    first = sky["entries"][0]
    (GOLDEN / "ref_hosek_kat.json").write_text(json.dumps({
        "elevation_deg": first["elevation_deg"], "turbidity": first["turbidity"], "albedo": first["albedo"],
        "band_theta_gamma_radiance": kat}))
    checks = run("ref_hosek_dump", *[str(x) for req in SKY_CHECKS for x in req])
    (GOLDEN / "ref_hosek_states.json").write_text(json.dumps(
        {"entries": [{k: e[k] for k in ("elevation_deg", "turbidity", "albedo", "states", "solar_kat")}
                     for e in checks["entries"]]}))
    for e in sky["entries"]:
        e.pop("solar_kat", None)
    nvdb_dir = GOLDEN / "nvdb"
    nvdb_dir.mkdir(exist_ok=True)
    with tempfile.TemporaryDirectory() as tmp:
        out = subprocess.run([str(REF_BIN / "ref_nvdb_files"), tmp], check=True, capture_output=True,
                             text=True).stdout
        (nvdb_dir / "ref_nvdb_files.json").write_text(json.dumps(json.loads(out)))
        for name in ("multi.nvdb", "sphere_fog.nvdb"):
            with open(Path(tmp) / name, "rb") as src, gzip.GzipFile(nvdb_dir / (name + ".gz"), "wb", 9,
                                                                     mtime=0) as dst:
                shutil.copyfileobj(src, dst)
        shutil.copy(Path(tmp) / "sphere_zip.nvdb", nvdb_dir / "sphere_zip.nvdb")
    DATA.mkdir(exist_ok=True)
    sky["cmf"] = basic["cmf_xs_ys_zs_centers_integral"]
    sky["source"] = ("Hosek-Wilkie 2013 v1.4a model states (arhosekskymodelstate_alloc_init) per renderer band, "
                     "and the renderer's 16-band CIE 1931 CMF integrals, generated by tests/golden/make_golden.py")
    (DATA / "hosek_sky.json").write_text(json.dumps(sky))
    print("wrote fixtures")
    return 0


if __name__ == "__main__":
    sys.exit(main())
