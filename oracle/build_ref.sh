#!/usr/bin/env bash
# Builds the known-answer programs that link the reference's own sources (read in place from
# the reference checkout, never copied) into oracle/_ref/. Needs the reference checkout, so it
# runs in the development container only; the fixtures these programs produce are committed
# under tests/golden/ and rtc8_gb300/data/ by tests/golden/make_golden.py.
#
#   REF=<path to the reference checkout> oracle/build_ref.sh
# (without REF: a checkout named "reference" next to this repository)
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${REF:-$(cd "$HERE/../.." && pwd)/reference}"
OUT="$HERE/_ref"
if [[ ! -d "$REF/common" ]]; then
    echo "reference checkout not found at $REF" >&2
    exit 2
fi
mkdir -p "$OUT"

# Hosek-Wilkie 2013 sky model (plain C) + the state dumper.
gcc -O2 -std=gnu99 -w -c "$REF/ext/hosek_wilkie_2013/ArHosekSkyModel.c" -o "$OUT/ArHosekSkyModel.o"
gcc -O2 -std=gnu99 -I "$REF/ext/hosek_wilkie_2013" "$HERE/ref_hosek_dump.c" "$OUT/ArHosekSkyModel.o" -lm \
    -o "$OUT/ref_hosek_dump"

# NanoVDB 32.3 grid builder, first-order sampler and ray clip.
g++ -O2 -std=c++17 -w -I "$REF/ext/nanovdb" "$HERE/ref_kat_nanovdb.cpp" -o "$OUT/ref_kat_nanovdb" -lpthread

# NanoVDB 32.3 file writer/reader fixtures (io::writeGrid(s), with the ZIP codec through zlib).
g++ -O2 -std=c++17 -w -DNANOVDB_USE_ZIP -I "$REF/ext/nanovdb" "$HERE/ref_nvdb_files.cpp" -o "$OUT/ref_nvdb_files" \
    -lpthread -lz

# common/basic_types.{h,cpp} host math (needs CUDA vector types, hence nvcc in host mode).
NVCC="${NVCC:-nvcc}"
"$NVCC" -std=c++17 -O2 -w -x cu -DCUDA_UTIL_DONT_USE_GL_INTEROP -I "$REF/common" "$HERE/ref_kat_basic.cu" "$REF/common/basic_types.cpp" \
    -o "$OUT/ref_kat_basic"
# Known-answer kernels over the reference's own device code (PTX, run on the GPU host by
# oracle/kat_device_loader.cpp): the reference's CUDA flags (renderer/CMakeLists.txt:37-51), with
# oracle/optix_stub standing in for the absent OptiX SDK headers.
"$NVCC" -ptx -std=c++17 -arch=compute_90 --use_fast_math -w -DCUDA_UTIL_DONT_USE_GL_INTEROP \
    -I "$HERE/optix_stub" -I "$REF" -I "$REF/common" -I "$REF/ext/nanovdb" \
    "$HERE/ref_kat_device.cu" -o "$OUT/ref_kat_device.ptx"
echo "built reference known-answer programs in $OUT"
