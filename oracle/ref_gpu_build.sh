#!/bin/sh
# The reference's own GPU build (its run_simulation command, K1-K6 kernels
# and host code) for sm_103a, for the golden fixtures of
# tests/golden/make_golden_gpu.py and the reference_gpu timing.  Two steps:
#
#   sh oracle/ref_gpu_build.sh stage   where SM2D_REFERENCE names the SM_2D tree:
#                                      copies the translation units its CMake
#                                      build lists (CMakeLists.txt: IMPL_CPU_SOURCES,
#                                      IMPL_CUDA_SOURCES, CUDA_KERNEL_SOURCES,
#                                      run_simulation.cpp), their headers and the
#                                      PSTAR table into oracle/_ref/tree (ignored
#                                      by git, carried to the GB300 host with the
#                                      checkout), unmodified
#   sh oracle/ref_gpu_build.sh build   compiles that copy with nvcc and g++
#                                      (separable compilation, as the CMake build
#                                      sets it) into oracle/_ref/gpu/run_simulation
#                                      and, with SM2D_ENABLE_DEBUG_DUMPS, into
#                                      oracle/_ref/gpu/run_simulation_dumps
#
# The reference's CMake build is not used (it needs GTest); this recipe
# compiles the same sources with the same definitions.
set -e
HERE=$(cd "$(dirname "$0")" && pwd)
TREE="$HERE/_ref/tree"
OUT="$HERE/_ref/gpu"
CUDA=${CUDA_HOME:-/usr/local/cuda}
CPU_SRC="src/utils/logger.cpp src/core/grids.cpp src/core/psi_storage.cpp src/core/buckets.cpp
 src/lut/nist_loader.cpp src/lut/r_lut.cpp src/boundary/boundaries.cpp src/boundary/loss_tracking.cpp
 src/audit/conservation.cpp src/audit/global_budget.cpp src/audit/reporting.cpp src/validation/bragg_peak.cpp
 src/validation/lateral_spread.cpp src/validation/deterministic_beam.cpp src/validation/determinism.cpp
 src/validation/validation_report.cpp src/source/pencil_source.cpp src/source/gaussian_source.cpp
 src/gpu/gpu_transport_runner.cpp src/utils/memory_tracker.cpp src/utils/cuda_pool.cpp
 src/perf/memory_profiler.cpp src/perf/kernel_profiler.cpp src/perf/occupancy_analyzer.cpp
 src/perf/fine_batch_planner.cpp src/perf/memory_preflight.cpp"
CU_SRC="src/cuda/kernels/k1_activemask.cu src/cuda/kernels/k2_coarsetransport.cu
 src/cuda/kernels/k3_finetransport.cu src/cuda/kernels/k4_transfer.cu src/cuda/kernels/k5_audit.cu
 src/cuda/kernels/k6_swap.cu src/cuda/gpu_transport_wrapper.cu src/cuda/k1k6_pipeline.cu"

case "$1" in
stage)
    REF=${SM2D_REFERENCE:?set SM2D_REFERENCE to the SM_2D source tree}
    rm -rf "$TREE"
    mkdir -p "$TREE"
    for f in $CPU_SRC $CU_SRC run_simulation.cpp; do
        mkdir -p "$TREE/$(dirname "$f")"
        cp "$REF/$f" "$TREE/$f"
    done
    cp -r "$REF/src/include" "$TREE/src/include"
    for d in device kernels; do cp -r "$REF/src/cuda/$d" "$TREE/src/cuda/"; done
    cp "$REF/src/cuda/"*.cuh "$TREE/src/cuda/"
    mkdir -p "$TREE/src/data/nist"
    cp "$REF/src/data/nist/pstar_water.txt" "$TREE/src/data/nist/"
    echo "staged $(find "$TREE" -type f | wc -l) files in $TREE"
    ;;
build)
    [ -f "$TREE/run_simulation.cpp" ] || { echo "stage the reference tree first" >&2; exit 1; }
    mkdir -p "$OUT"
    INC="-I$TREE/src/include -I$TREE/src/cuda -I$CUDA/include"
    for variant in plain dumps; do
        DEF="-DSM2D_HAS_CUDA"
        [ "$variant" = dumps ] && DEF="$DEF -DSM2D_ENABLE_DEBUG_DUMPS"
        OBJ="$OUT/obj_$variant"
        mkdir -p "$OBJ"
        pids=""
        for f in $CU_SRC; do
            "$CUDA/bin/nvcc" -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -rdc=true \
                --expt-relaxed-constexpr -diag-suppress 20050 $DEF $INC -c "$TREE/$f" \
                -o "$OBJ/$(basename "$f").o" &
            pids="$pids $!"
        done
        for f in $CPU_SRC run_simulation.cpp; do
            g++ -O2 -std=c++17 $DEF $INC -c "$TREE/$f" -o "$OBJ/$(basename "$f").o" &
            pids="$pids $!"
        done
        for p in $pids; do wait "$p"; done
        "$CUDA/bin/nvcc" -gencode arch=compute_103a,code=sm_103a -dlink "$OBJ"/*.cu.o -o "$OBJ/dlink.o"
        exe="$OUT/run_simulation"
        [ "$variant" = dumps ] && exe="$OUT/run_simulation_dumps"
        g++ "$OBJ"/*.o -o "$exe" -L"$CUDA/lib64" -L"$CUDA/targets/sbsa-linux/lib" \
            -L"$CUDA/targets/x86_64-linux/lib" -lcudart -lpthread
        echo "built $exe"
    done
    ;;
*)
    echo "usage: ref_gpu_build.sh stage|build" >&2
    exit 2
    ;;
esac
