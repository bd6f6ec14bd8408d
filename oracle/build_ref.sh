#!/usr/bin/env bash
# Test infrastructure: builds the reference's own implicit step, and the block-sparse
# CG of its FEM demo, headless, from the reference sources where they lie, into
# oracle/_ref/ (git-ignored; never committed).
#
#   OpenCloth_Implicit/OpenCloth_Implicit/main.cpp  -> _ref/imp_f32.cpp (generated copy)
#                                                  -> _ref/imp_f64.cpp (FP64 copy)
#   ref_harness.cpp + shim/GL/*.h + dep/glm          -> _ref/ref_step_f32, _ref/ref_step_f64
#   OpenCloth_CoRotated_Linear_FEM/.../main.cpp      -> _ref/fem_f32.cpp, _ref/fem_f64.cpp
#   fem_harness.cpp + shim/GL/*.h + dep/glm          -> _ref/fem_step_f32, _ref/fem_step_f64
#
# The FEM copy differs from the reference only in InitGL's mesh size (main.cpp:426,
# read from OC_FEM_X/OC_FEM_Y/OC_FEM_Z at start-up).
#
# The generated copies differ from the reference only where a compile-time constant
# has to become a run-time value (grid size main.cpp:60, CG EPS main.cpp:126 and i_max
# main.cpp:128, read from OC_NUMX/OC_NUMY/OC_EPS/OC_IMAX at start-up).  The FP64 copy
# additionally maps glm::vecN/matN -> glm::dvecN/dmatN, float -> double and strips the
# f suffix from floating literals.
#
# The reference tree is OC_REFERENCE_DIR when set, else a checkout named `reference`
# beside this repository (../reference from the repository root).  Exits 0 without
# building when the tree is absent.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${OC_REFERENCE_DIR:-$HERE/../../reference}"
SRC="$REF/OpenCloth_Implicit/OpenCloth_Implicit/main.cpp"
OUT="$HERE/_ref"
if [ ! -f "$SRC" ]; then
    echo "build_ref: reference source not present ($SRC); skipping"
    exit 0
fi
mkdir -p "$OUT"

sed -E \
    -e 's/^int numX = 20, numY=20;/int numX = oc_env_int("OC_NUMX", 20), numY = oc_env_int("OC_NUMY", 20);/' \
    -e 's/^const float EPS = 0\.001f;/const float EPS = oc_env_real("OC_EPS", 0.001f);/' \
    -e 's/^const int i_max = 10;/const int i_max = oc_env_int("OC_IMAX", 10);/' \
    "$SRC" > "$OUT/imp_f32.cpp"
for pat in 'oc_env_int("OC_NUMX"' 'oc_env_real("OC_EPS"' 'oc_env_int("OC_IMAX"'; do
    grep -qF "$pat" "$OUT/imp_f32.cpp" || { echo "build_ref: substitution failed: $pat" >&2; exit 1; }
done

sed -E \
    -e 's/glm::(vec|mat)([234])/glm::d\1\2/g' \
    -e 's/\bfloat\b/double/g' \
    -e 's/\b([0-9]+\.[0-9]*|[0-9]*\.[0-9]+)f\b/\1/g' \
    "$OUT/imp_f32.cpp" > "$OUT/imp_f64.cpp"

FEM_SRC="$REF/OpenCloth_CoRotated_Linear_FEM/OpenCloth_CoRotated_Linear_FEM/main.cpp"
sed -E \
    -e 's/^\tGenerateBlocks\(10,3,3,0\.1f,0\.1f,0\.1f\);/\tGenerateBlocks(oc_env_int("OC_FEM_X", 10), oc_env_int("OC_FEM_Y", 3), oc_env_int("OC_FEM_Z", 3), 0.1f, 0.1f, 0.1f);/' \
    "$FEM_SRC" > "$OUT/fem_f32.cpp"
grep -qF 'oc_env_int("OC_FEM_X"' "$OUT/fem_f32.cpp" || { echo "build_ref: FEM substitution failed" >&2; exit 1; }
sed -E \
    -e 's/glm::(vec|mat)([234])/glm::d\1\2/g' \
    -e 's/\bfloat\b/double/g' \
    -e 's/\b([0-9]+\.[0-9]*|[0-9]*\.[0-9]+)f\b/\1/g' \
    "$OUT/fem_f32.cpp" > "$OUT/fem_f64.cpp"

CXXFLAGS="-std=c++14 -O2 -ffp-contract=off -w -I$HERE/shim -I$REF/dep/glm -I$OUT -Dglm_core_func_integer"
g++ $CXXFLAGS -DOC_REAL=float '-DOC_REF_SOURCE="imp_f32.cpp"' "$HERE/ref_harness.cpp" -o "$OUT/ref_step_f32" &
g++ $CXXFLAGS -DOC_REAL=double '-DOC_REF_SOURCE="imp_f64.cpp"' "$HERE/ref_harness.cpp" -o "$OUT/ref_step_f64" &
g++ $CXXFLAGS -DOC_REAL=float '-DOC_FEM_SOURCE="fem_f32.cpp"' "$HERE/fem_harness.cpp" -o "$OUT/fem_step_f32" &
g++ $CXXFLAGS -DOC_REAL=double '-DOC_FEM_SOURCE="fem_f64.cpp"' "$HERE/fem_harness.cpp" -o "$OUT/fem_step_f64" &
wait %1 && wait %2 && wait %3 && wait %4
echo "build_ref: built $OUT/ref_step_f32 $OUT/ref_step_f64 $OUT/fem_step_f32 $OUT/fem_step_f64"
