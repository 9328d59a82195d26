#!/bin/sh
# Builds oracle/_ref/ref_probe from the reference's own host sources where they
# lie (grids.cpp, r_lut.cpp, nist_loader.cpp; header-only host physics), and
# oracle/_ref/ref_writer_probe from its output writers.  Runs
# only where the reference tree is mounted; the output never leaves oracle/_ref.
set -e
# SM2D_REFERENCE names the root of the reference tree (its src/ and run_simulation.cpp).
[ -n "$SM2D_REFERENCE" ] || { echo "set SM2D_REFERENCE to the reference tree" >&2; exit 2; }
REF=$SM2D_REFERENCE
HERE=$(cd "$(dirname "$0")" && pwd)
[ -d "$REF/src" ] || { echo "reference tree not found at $REF" >&2; exit 1; }
mkdir -p "$HERE/_ref"
g++ -O2 -std=c++17 -ffp-contract=off -I"$REF/src/include" \
    "$REF/src/core/grids.cpp" "$REF/src/lut/r_lut.cpp" "$REF/src/lut/nist_loader.cpp" \
    "$HERE/ref_probe.cpp" -o "$HERE/_ref/ref_probe"
# the output writers and depth-dose metrics (run_simulation.cpp with its main
# renamed, deterministic_beam.cpp, bragg_peak.cpp)
g++ -O2 -std=c++17 -ffp-contract=off -I"$REF/src/include" -Dmain=reference_run_simulation_main \
    -c "$REF/run_simulation.cpp" -o "$HERE/_ref/run_simulation.o"
g++ -O2 -std=c++17 -ffp-contract=off -I"$REF/src/include" \
    "$REF/src/validation/deterministic_beam.cpp" "$REF/src/validation/bragg_peak.cpp" \
    "$REF/src/core/grids.cpp" "$REF/src/lut/r_lut.cpp" "$REF/src/lut/nist_loader.cpp" \
    "$HERE/_ref/run_simulation.o" "$HERE/ref_writer_probe.cpp" -o "$HERE/_ref/ref_writer_probe"
echo "$HERE/_ref/ref_probe"
