#!/usr/bin/env bash
# Compiles the reference's own BLAS/TLAS builder sources, where they lie in the
# read-only reference checkout, into oracle/_ref/libref_bvh.so (git-ignored).
# Test infrastructure only: it pins the oracle's restatement of the builders.
# Usage: oracle/build_ref.sh [reference_root]   (default /root/reference)
set -euo pipefail
REF="${1:-/root/reference}"
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
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
