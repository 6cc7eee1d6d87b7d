#!/usr/bin/env bash
# Builds oracle/_ref/libbkma_ref.so: the reference's own solver and config
# sources, compiled where they lie (read-only) with the host-only shim in
# oracle/ref_shim, plus oracle/ref_driver.cpp. Outputs only into oracle/_ref/.
# Needs the reference checkout (BKMA_REFERENCE_DIR, else the default below);
# exits 0 with a note when it is absent. Records the directory it used in
# oracle/_ref/reference_dir.txt (read by oracle.reference_dir()).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${BKMA_REFERENCE_DIR:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF/src/solvers/AdvectionSolver.hpp" ]; then
    echo "build_ref: reference sources not found at $REF; skipping"
    exit 0
fi
mkdir -p "$OUT"
CXX="${CXX:-g++}"
"$CXX" -std=c++17 -O2 -ffp-contract=off -fno-fast-math -fopenmp -fPIC -shared \
    -I "$HERE/ref_shim" -I "$REF/src" -I "$REF/src/config" \
    -I "$REF/src/solvers" -I "$REF/src/tools" \
    "$HERE/ref_driver.cpp" \
    "$REF/src/config/ConfigMap.cpp" \
    "$REF/src/config/AdvectionParams.cpp" \
    "$REF/src/config/Conv1dParams.cpp" \
    "$REF/src/config/inih/ini.cpp" \
    "$REF/src/config/inih/INIReader.cpp" \
    -o "$OUT/libbkma_ref.so.tmp"
mv "$OUT/libbkma_ref.so.tmp" "$OUT/libbkma_ref.so"
# where the sources were found, for the tests and fixture script that read them
printf '%s\n' "$REF" > "$OUT/reference_dir.txt"
echo "build_ref: $OUT/libbkma_ref.so"
