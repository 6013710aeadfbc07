#!/usr/bin/env bash
# Builds the reference's own distance kernel, cusim::K_distance
# (src/gpu/cusim/kernel-distance.inl), for sm_103a into oracle/_ref/kdist/
# (test infrastructure only; see ref_kdist.cu).  Two libraries:
#   libkdist_nofma.so  -fmad=false: every `a2 += dd*dd` is a separate IEEE
#                      multiply and add (the contract this library keeps)
#   libkdist_fma.so    nvcc's defaults, as the reference's premake5.lua:76
#                      compiles it (-O2, FMA contraction on)
#
#   build_ref_kdist.sh prepare   where the reference tree is present: writes
#                                oracle/_ref/kdist/kernel-distance.inl
#   build_ref_kdist.sh           prepares when it can, then builds both
#                                libraries with nvcc (run it on the machine
#                                with the GPU: host binaries do not move
#                                between machines)
#
# The prepared file is the reference's kernel-distance.inl with one change:
# warp_prefix's inline PTX `shfl.up.b32 d|p, a, b, 0;` (the pre-CUDA-9 form,
# which ptxas rejects for sm_70 and newer) becomes
# `shfl.sync.up.b32 d|p, a, b, 0, 0xffffffff;`, the same shuffle for a full
# warp.  It lives only under the git-ignored oracle/_ref/.
set -euo pipefail
here="$(cd "$(dirname "$0")" && pwd)"
out="$here/_ref/kdist"
ref="${PCS_REFERENCE_ROOT:-/root/reference}"
src="$ref/src/gpu/cusim/kernel-distance.inl"
if [ -f "$src" ]; then
    mkdir -p "$out"
    sed 's/shfl\.up\.b32 t0|valid, %0, \([0-9][0-9]*\), 0;/shfl.sync.up.b32 t0|valid, %0, \1, 0, 0xffffffff;/' \
        "$src" > "$out/kernel-distance.inl.tmp"
    n="$(grep -c 'shfl\.sync\.up\.b32' "$out/kernel-distance.inl.tmp" || true)"
    if [ "$n" != 5 ] || grep -q '"shfl\.up\.b32' "$out/kernel-distance.inl.tmp"; then
        echo "unexpected kernel-distance.inl: $n of 5 shuffles rewritten" >&2
        rm -f "$out/kernel-distance.inl.tmp"
        exit 1
    fi
    mv "$out/kernel-distance.inl.tmp" "$out/kernel-distance.inl"
fi
if [ "${1:-}" = prepare ]; then
    exit 0
fi
if [ ! -f "$out/kernel-distance.inl" ]; then
    echo "no prepared kernel-distance.inl under $out (the reference tree is needed once); skipping" >&2
    exit 0
fi
NVCC="${NVCC:-${CUDA_HOME:-/usr/local/cuda}/bin/nvcc}"
common=(-O2 -std=c++17 --expt-relaxed-constexpr -gencode arch=compute_103a,code=sm_103a
        -Xcompiler -fPIC -shared -I"$out" -w)
"$NVCC" "${common[@]}" -fmad=false -o "$out/libkdist_nofma.so" "$here/ref_kdist.cu" &
p1=$!
"$NVCC" "${common[@]}" -o "$out/libkdist_fma.so" "$here/ref_kdist.cu" &
p2=$!
wait "$p1"
wait "$p2"
echo "built $out/libkdist_nofma.so $out/libkdist_fma.so"
