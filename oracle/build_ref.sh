#!/usr/bin/env bash
# Compiles the reference's own sources for the host into oracle/_ref/ (test
# infrastructure only; see ref_harness.cpp).  Reads the read-only reference
# tree in place; copies nothing out of it.  Needs only g++.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
ref="${PCS_REFERENCE_ROOT:-/root/reference}"
if [ ! -d "$ref/src/gpu" ]; then
    echo "reference sources not found at $ref; skipping oracle/_ref" >&2
    exit 0
fi
out="$here/_ref"
mkdir -p "$out"
CXX="${CXX:-g++}"
flags=(-std=c++14 -O2 -fPIC -ffp-contract=off -fno-fast-math -w
       -I"$here/ref_shim" -I"$ref/src/gpu" -I"$ref/external")
srcs=("$here/ref_harness.cpp"
      "$ref/src/gpu/shared/input.cpp"
      "$ref/src/gpu/shared/output.cpp"
      "$ref/src/gpu/shared/common.cpp"
      "$ref/src/gpu/support/utility.cpp"
      "$ref/src/gpu/support/cuda_error.cpp"
      "$ref/external/tinyxml2/tinyxml2.cpp")
"$CXX" "${flags[@]}" -shared -o "$out/libpcsref.so" "${srcs[@]}"
# the tree these were compiled from, for the scripts that read its fixtures
# (oracle.reference_root())
printf '%s\n' "$ref" > "$out/reference_root"
echo "built $out/libpcsref.so"
