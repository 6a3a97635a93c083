#!/usr/bin/env bash
# Host build of the reference's OWN projector, gateway and TV sources -- the
# strongest parity pin for the oracle (test infrastructure only).
#
# Compiles, straight from the reference checkout (ASDPOCS_REFERENCE_DIR, else
# a checkout named "reference" beside the repository), without copying any
# source into the repository:
#   * src/AxAtx/Ax_cone_gpu.cu lines 1-297 and 339-776 (device functions and
#     kernels; the cudaMalloc launchers are replaced by oracle/ref_shim_tail.inc)
#     with the host shim oracle/ref_shim_head.h, as one translation unit;
#   * src/AxAtx/Ax_main_test.cpp and Atx_main_test.cpp (mex gateways);
#   * src/tvmin/imgTVGradMin.cpp and imgTVGradMin3D.cpp (TV, OpenMP);
# against the stand-in mex API in oracle/mexstub, into oracle/_ref/libasdref.so.
# -ffp-contract=off gives the IEEE operation-by-operation float semantics that
# the oracle and the CUDA kernels also use.  Exits 0 without building when the
# reference checkout is absent (for example on a machine that only runs the
# prebuilt library).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${ASDPOCS_REFERENCE_DIR:-$HERE/../../reference}"
OUT="$HERE/_ref"
CU="$REF/src/AxAtx/Ax_cone_gpu.cu"
if [ ! -f "$CU" ]; then
  echo "build_ref: reference sources not found at $REF; skipped"
  exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
FLAGS=(-O2 -fPIC -ffp-contract=off -fopenmp -I "$HERE/mexstub")
{ sed -n '1,297p;339,776p' "$CU"; cat "$HERE/ref_shim_tail.inc"; } |
  "$CXX" "${FLAGS[@]}" -x c++ -include "$HERE/ref_shim_head.h" -c - -o "$OUT/ref_kernels.o" &
"$CXX" "${FLAGS[@]}" -DmexFunction=ref_mex_ax -c "$REF/src/AxAtx/Ax_main_test.cpp" -o "$OUT/ref_ax_gw.o" &
"$CXX" "${FLAGS[@]}" -DmexFunction=ref_mex_atx -c "$REF/src/AxAtx/Atx_main_test.cpp" -o "$OUT/ref_atx_gw.o" &
"$CXX" "${FLAGS[@]}" -DmexFunction=ref_mex_tv2d -DshowUsage=ref_tv2d_usage -c "$REF/src/tvmin/imgTVGradMin.cpp" -o "$OUT/ref_tv2d.o" &
"$CXX" "${FLAGS[@]}" -DmexFunction=ref_mex_tv3d -DshowUsage=ref_tv3d_usage -c "$REF/src/tvmin/imgTVGradMin3D.cpp" -o "$OUT/ref_tv3d.o" &
"$CXX" "${FLAGS[@]}" -c "$HERE/mexstub/mexstub.cpp" -o "$OUT/mexstub.o" &
wait
"$CXX" -shared -fopenmp -o "$OUT/libasdref.so" "$OUT"/ref_kernels.o "$OUT"/ref_ax_gw.o \
  "$OUT"/ref_atx_gw.o "$OUT"/ref_tv2d.o "$OUT"/ref_tv3d.o "$OUT"/mexstub.o
echo "build_ref: built $OUT/libasdref.so"
