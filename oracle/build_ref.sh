#!/usr/bin/env bash
# Builds the reference's own CUDA kernels (TEST INFRASTRUCTURE) from the sources
# where they lie, into oracle/_ref/ only:
#   ref_dcgrid.cubin   src/dcgrid/dcgrid_{fluid,multigrid_solver,structure,adaptation}.cu
#                      + src/utils/sim_utils.cu
#   ref_uniform.cubin  src/uniformgrid/uniformgrid_{fluid,structure}.cu + sim_utils.cu
#   ref_names.txt      mangled kernel names (from the host objects' symbol tables)
# Each cubin is one translation unit that #includes the reference .cu files by
# path. -fmad=false keeps the reference's float operations unfused, so its
# results are comparable bit for bit with the oracle's float mirror.
# Usage: build_ref.sh <reference tree>   (or REF=<reference tree> build_ref.sh)
# Needs the reference's sources and nvcc.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${1:-${REF:-}}"
OUT="$HERE/_ref"
NVCC="${NVCC:-nvcc}"
[ -n "$REF" ] || { echo "usage: $0 <reference tree>" >&2; exit 2; }
[ -d "$REF/src/dcgrid" ] || { echo "reference tree not found at $REF" >&2; exit 2; }
mkdir -p "$OUT"
FLAGS=(-std=c++17 -O3 -fmad=false -diag-suppress 2506,177,550 -include "$HERE/ref_shim/ref_prelude.h"
       -I"$HERE/ref_shim" -I"$REF/src" -I"$REF/src/utils" -I"$REF/include/cuda"
       -gencode arch=compute_103a,code=sm_103a)
cat > "$OUT/unity_dcgrid.cu" <<EOT
#include "$REF/src/utils/sim_utils.cu"
#include "$REF/src/dcgrid/dcgrid_fluid.cu"
#include "$REF/src/dcgrid/dcgrid_multigrid_solver.cu"
#include "$REF/src/dcgrid/dcgrid_structure.cu"
#include "$REF/src/dcgrid/dcgrid_adaptation.cu"
EOT
cat > "$OUT/unity_uniform.cu" <<EOT
#include "$REF/src/utils/sim_utils.cu"
#include "$REF/src/uniformgrid/uniformgrid_fluid.cu"
#include "$REF/src/uniformgrid/uniformgrid_structure.cu"
EOT
for u in dcgrid uniform; do
  "$NVCC" "${FLAGS[@]}" -cubin "$OUT/unity_$u.cu" -o "$OUT/ref_$u.cubin"
  "$NVCC" "${FLAGS[@]}" -rdc=true -c "$OUT/unity_$u.cu" -o "$OUT/unity_$u.o" 2>/dev/null
done
nm -g "$OUT/unity_dcgrid.o" "$OUT/unity_uniform.o" | awk '$3 ~ /^_Z[0-9]+k_(dcgrid|uniform)_/ {print $3}' | sort -u > "$OUT/ref_names.txt"
rm -f "$OUT"/unity_*.o "$OUT"/unity_*.cu
echo "built $(ls "$OUT"/*.cubin | wc -l) cubins, $(wc -l < "$OUT/ref_names.txt") kernels"
