#!/usr/bin/env bash
# Rebuilds the reference's own CUDA step (moonsh5009/MPS_CUDA) headless for sm_103a -- TEST
# INFRASTRUCTURE ONLY.  Output goes to oracle/_ref/ (git-ignored).
#
# 1. When the reference tree is present (MPS_REFERENCE, default /root/reference), refresh a
#    scripted copy of the sources the step needs into oracle/_ref/src (so that the same build
#    can run on a machine without the reference tree) and apply the edits below to the copy.
# 2. Compile the step's translation units with the headless stand-in headers of
#    oracle/ref_shim and link them with oracle/ref_driver.cu into one library per variant.
#
# Edits to the copy (never to the reference tree):
#  - MPSSPHKernel.cuh:18  `constexpr REAL NeighborSearch` -> `constexpr void NeighborSearch`
#    (the function returns nothing; g++ 13 rejects the missing return, MSVC accepted it).
#  - MPSSPHKernel.cuh:5   USE_CUBIC_KERNEL becomes overridable (-DUSE_CUBIC_KERNEL=1).
#  - MPSSPHDFSPHUtil.cu:333,419  the density (1e-4) and divergence (1e-3) tolerance literals
#    become overridable macros with the shipped values as defaults.
# Variants: "shipped" (poly6/spiky, shipped tolerances) and "config" (cubic spline, 1e-3/1e-3).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
REF="${MPS_REFERENCE:-/root/reference}"
NVCC="${NVCC:-nvcc}"
command -v "$NVCC" >/dev/null 2>&1 || NVCC=/usr/local/cuda/bin/nvcc

if [ -d "$REF/src/MPS_Computer" ]; then
    rm -rf "$OUT/src" "$OUT/include"
    mkdir -p "$OUT/src" "$OUT/include"
    cp -r "$REF/src/MPS_Computer" "$REF/src/MPS_Object" "$REF/src/MCUDA_Lib" "$OUT/src/"
    cp -r "$REF/include/glm" "$OUT/include/"
    K="$OUT/src/MPS_Computer/MPSSPHKernel.cuh"
    sed -i 's/constexpr REAL NeighborSearch/constexpr void NeighborSearch/' "$K"
    sed -i 's/^#define USE_CUBIC_KERNEL[[:space:]]*0/#ifndef USE_CUBIC_KERNEL\n#define USE_CUBIC_KERNEL 0\n#endif/' "$K"
    D="$OUT/src/MPS_Computer/MPSSPHDFSPHUtil.cu"
    sed -i 's/h_error.front() < 1.0e-4 \&\& l > 2u/h_error.front() < MPS_REF_CD_TOL \&\& l > 2u/' "$D"
    sed -i 's/h_error.front() < 1.0e-3 \&\& l > 1u/h_error.front() < MPS_REF_DF_TOL \&\& l > 1u/' "$D"
    sed -i '1i #ifndef MPS_REF_CD_TOL\n#define MPS_REF_CD_TOL 1.0e-4\n#endif\n#ifndef MPS_REF_DF_TOL\n#define MPS_REF_DF_TOL 1.0e-3\n#endif' "$D"
    grep -q "constexpr void NeighborSearch" "$K"
    grep -q "MPS_REF_CD_TOL && l > 2u" "$D"
    grep -q "MPS_REF_DF_TOL && l > 1u" "$D"
fi
if [ ! -d "$OUT/src/MPS_Computer" ]; then
    echo "reference sources unavailable (no $REF and no copy in $OUT/src)" >&2
    exit 2
fi
# without the reference tree, libraries built earlier from the copy are current
if [ ! -d "$REF/src/MPS_Computer" ] && [ -f "$OUT/shipped/libmpsref.so" ] && [ -f "$OUT/config/libmpsref.so" ]; then
    exit 0
fi

TUS="MPS_Computer/MPSSPHBaseUtil.cu MPS_Computer/MPSSPHDFSPHUtil.cu MPS_Computer/MPSSPHNonPressureUtil.cu MPS_Computer/MPSAdvectUtil.cu MPS_Object/MPSSpatialHash.cu"
COMMON=(-std=c++20 --extended-lambda "-D__declspec(x)=" -Xcompiler -fPIC -gencode arch=compute_103a,code=sm_103a -O3
        -w -I"$HERE/ref_shim" -I"$OUT/include" -I"$OUT/src")

build_variant() {
    local name="$1"; shift
    local dir="$OUT/$name"
    mkdir -p "$dir"
    local objs=()
    local pids=()
    for tu in $TUS ref_driver; do
        local src obj
        if [ "$tu" = ref_driver ]; then src="$HERE/ref_driver.cu"; else src="$OUT/src/$tu"; fi
        obj="$dir/$(basename "$tu").o"
        objs+=("$obj")
        "$NVCC" "${COMMON[@]}" "$@" -c "$src" -o "$obj" &
        pids+=($!)
    done
    for p in "${pids[@]}"; do wait "$p"; done
    "$NVCC" -gencode arch=compute_103a,code=sm_103a -shared -o "$dir/libmpsref.so" "${objs[@]}" -lcudart
}

build_variant shipped &
P1=$!
build_variant config -DUSE_CUBIC_KERNEL=1 -DMPS_REF_CD_TOL=1.0e-3 -DMPS_REF_DF_TOL=1.0e-3 &
P2=$!
wait $P1
wait $P2
ls -la "$OUT/shipped/libmpsref.so" "$OUT/config/libmpsref.so"
