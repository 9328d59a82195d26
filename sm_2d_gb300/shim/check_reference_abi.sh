#!/bin/sh
# Checks the C++ drop-in layer against the SM_2D tree's own headers (run
# where SM2D_REFERENCE names that tree; writes only under shim/_build):
#   1. sm2d_ref_shim.cpp compiled against the tree's headers and against
#      include/sm2d_ref_types.hpp defines the same entry points with the same
#      mangled names, i.e. the same parameter types;
#   2. every exchanged type has the same size and member offsets both ways.
# Prints "abi ok" and exits 0 when both hold.
set -e
REF="${SM2D_REFERENCE:?set SM2D_REFERENCE to the SM_2D source tree}"
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(cd "$HERE/../.." && pwd)"
OUT="$HERE/_build"
CUDA="${CUDA_HOME:-/usr/local/cuda}"
mkdir -p "$OUT"
REFINC="-I$REF/src/include -I$REF/src/cuda -I$REF/src"
NVCC="$CUDA/bin/nvcc -gencode arch=compute_103a,code=sm_103a -x cu -std=c++17 -diag-suppress 20050,177"
$NVCC -c -DSM2D_SHIM_REFERENCE_HEADERS $REFINC -I"$ROOT/include" "$HERE/sm2d_ref_shim.cpp" -o "$OUT/shim_ref.o"
g++ -std=c++17 -c -I"$ROOT/include" -I"$CUDA/include" "$HERE/sm2d_ref_shim.cpp" -o "$OUT/shim_own.o"
nm -g --defined-only "$OUT/shim_ref.o" | awk '$2=="T"{print $3}' | grep sm_2d | sort > "$OUT/symbols_ref.txt"
nm -g --defined-only "$OUT/shim_own.o" | awk '$2=="T"{print $3}' | grep sm_2d | sort > "$OUT/symbols_own.txt"
diff "$OUT/symbols_ref.txt" "$OUT/symbols_own.txt"
test -s "$OUT/symbols_own.txt"
$NVCC -DSM2D_SHIM_REFERENCE_HEADERS $REFINC "$HERE/ref_layout_probe.cpp" -o "$OUT/probe_ref" -Xcompiler -Wno-invalid-offsetof
g++ -std=c++17 -Wno-invalid-offsetof -I"$ROOT/include" "$HERE/ref_layout_probe.cpp" -o "$OUT/probe_own"
"$OUT/probe_ref" > "$OUT/layout_ref.txt"
"$OUT/probe_own" > "$OUT/layout_own.txt"
diff "$OUT/layout_ref.txt" "$OUT/layout_own.txt"
echo "abi ok: $(wc -l < "$OUT/symbols_own.txt") entry points, $(wc -l < "$OUT/layout_own.txt") sizes and offsets"
