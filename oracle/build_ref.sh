#!/usr/bin/env bash
# Compiles parts of the reference, from its sources where they lie in the
# read-only reference checkout, into oracle/_ref/ (git-ignored).  Test
# infrastructure only: these libraries pin the oracle's restatements.
#   libref_bvh.so    the reference's BLAS / TLAS builders (bvh_builder.cpp,
#                    tlas_builder.cpp) with a malloc-backed arena header
#   libref_assets.so oracle/ref_assets.c on the reference's vendored cgltf / ufbx
#   libref_stb.so    oracle/ref_stb.c on the reference's vendored stb_image
#   libref_hlsl.so   the reference's traversal, intersection, sampling and
#                    shade-stage HLSL, rewritten by ref_hlsl/hlsl_to_cpp.py into
#                    oracle/_ref/hlsl/ and compiled with ref_hlsl/hlsl_shim.h
# Usage: oracle/build_ref.sh [reference_root]
#   reference_root defaults to $WF_REFERENCE_ROOT, else a checkout named
#   "reference" beside this repository.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${WF_REFERENCE_ROOT:-$HERE/../../reference}}"
OUT="$HERE/_ref"
if [ ! -f "$REF/source/renderer/bvh/bvh_builder.cpp" ]; then
  echo "reference sources not found under $REF; skipping" >&2
  exit 0
fi
mkdir -p "$OUT"
g++ -std=c++20 -O2 -ffp-contract=off -fPIC -shared -w \
  -I "$HERE/ref_shim" -I "$REF/source" -I "$REF/extern" \
  -o "$OUT/libref_bvh.so" \
  "$HERE/ref_driver.cpp" \
  "$REF/source/renderer/bvh/bvh_builder.cpp" \
  "$REF/source/renderer/bvh/tlas_builder.cpp"
echo "built $OUT/libref_bvh.so"
# The reference's scene loaders' libraries (cgltf, ufbx, vendored under
# extern/) behind oracle/ref_assets.c, a restatement of asset_loader.cpp's data
# extraction: pins wavefrontpathtracing_gb300.gltf / .fbx.
if [ -f "$REF/extern/ufbx/ufbx.c" ] && [ -f "$REF/extern/cgltf/cgltf.h" ]; then
  gcc -std=gnu11 -O1 -fPIC -shared -w -I "$REF/extern" \
    -o "$OUT/libref_assets.so" "$HERE/ref_assets.c" "$REF/extern/ufbx/ufbx.c" -lm
  echo "built $OUT/libref_assets.so"
fi
# The reference's image decoder (extern/stb/stb_image.h, vendored): pins the
# library's JPEG and Radiance HDR decoders.
if [ -f "$REF/extern/stb/stb_image.h" ]; then
  gcc -std=gnu11 -O2 -fPIC -shared -w -I "$REF/extern" \
    -o "$OUT/libref_stb.so" "$HERE/ref_stb.c" -lm
  echo "built $OUT/libref_stb.so"
fi
# The reference's compute shaders as C++: pins oracle/orc_impl.h (traversal and
# shading).  -ffp-contract=off keeps every float operation rounding as written
# (gcc would contract a*b+c into fma on aarch64).  liborc.so supplies the
# shim's sin / cos / atan2 / asin and texture filter.
if [ -f "$REF/source/renderer/shaders/wavefront/shade.hlsl" ]; then
  make -s -C "$HERE"
  python3 "$HERE/ref_hlsl/hlsl_to_cpp.py" "$REF" "$OUT/hlsl"
  g++ -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared -w \
    -I "$HERE/ref_hlsl" -I "$OUT/hlsl" \
    -o "$OUT/libref_hlsl.so" \
    "$HERE/ref_hlsl/ref_trace.cpp" "$HERE/ref_hlsl/ref_shade.cpp" \
    -L "$HERE/_build" -lorc -Wl,-rpath,'$ORIGIN/../_build'
  echo "built $OUT/libref_hlsl.so"
fi
