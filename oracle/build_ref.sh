#!/bin/sh
# Builds oracle/_ref/ref_pipeline: the reference's own hot-path sources,
# compiled unmodified from the reference checkout, linked with the project's
# shims (oracle/ref_shims/) and CPU solver (oracle/solver.c); and
# oracle/_ref/ref_gds: the reference's GDSII database and saveToMesh
# (limboint.hpp) with the project's stand-in for Limbo's stream reader;
# oracle/_ref/ref_network: its output stage and .sim_input reader
# (solnoutclass.hpp) with stand-ins for Eigen and Parser-SPEF.
# Test infrastructure only; output stays in oracle/_ref/ (git-ignored).
# usage: oracle/build_ref.sh [reference_root]
#   (default: $G2P_REFERENCE_ROOT, else /root/reference)
set -e
REF=${1:-${G2P_REFERENCE_ROOT:-/root/reference}}
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
[ -f "$REF/src/fdtd.hpp" ] || { echo "reference sources not found under $REF" >&2; exit 1; }
mkdir -p "$OUT"
CXXFLAGS="-std=c++17 -O2 -ffp-contract=off -w -I$HERE/ref_shims -I$REF/src -I$HERE"
gcc -std=c11 -O2 -ffp-contract=off -c "$HERE/solver.c" -I"$HERE" -o "$OUT/solver.o" &
g++ $CXXFLAGS -c "$REF/src/mesh.cpp" -o "$OUT/mesh.o" &
g++ $CXXFLAGS -c "$REF/src/generateStiff.cpp" -o "$OUT/generateStiff.o" &
g++ $CXXFLAGS -c "$REF/src/matrixCon.cpp" -o "$OUT/matrixCon.o" &
g++ $CXXFLAGS -c "$HERE/ref_shims/mkl_sparse_shim.cpp" -o "$OUT/mkl_sparse_shim.o" &
g++ $CXXFLAGS -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o" &
g++ $CXXFLAGS -c "$HERE/ref_gds.cpp" -o "$OUT/ref_gds.o" &
wait
g++ -o "$OUT/ref_gds" "$OUT/ref_gds.o" "$OUT/mesh.o" "$OUT/mkl_sparse_shim.o" -lm
# oracle/_ref/ref_network: the reference's output stage and .sim_input
# reader (solnoutclass.hpp) against the project's Eigen and Parser-SPEF
# stand-ins; the writers read an uninitialised time_t, which
# -ftrivial-auto-var-init=zero makes the epoch
g++ $CXXFLAGS -ftrivial-auto-var-init=zero -c "$HERE/ref_network.cpp" -o "$OUT/ref_network.o"
g++ -o "$OUT/ref_network" "$OUT/ref_network.o" "$OUT/mkl_sparse_shim.o" -lm
g++ -o "$OUT/ref_pipeline" "$OUT/ref_harness.o" "$OUT/mesh.o" "$OUT/generateStiff.o" "$OUT/matrixCon.o" \
    "$OUT/mkl_sparse_shim.o" "$OUT/solver.o" -lm
# oracle/_ref/ref_pipeline_vh: the same harness with the reference's
# full-wave (Vh) path compiled in (oracle/ref_matrixcon_vh.cpp) and the
# dense LAPACK/PARDISO stand-ins; findVh.cpp supplies matrix_multi
g++ $CXXFLAGS -c "$HERE/ref_matrixcon_vh.cpp" -o "$OUT/matrixCon_vh.o" &
g++ $CXXFLAGS -DG2P_REF_VH -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness_vh.o" &
g++ $CXXFLAGS -c "$REF/src/findVh.cpp" -o "$OUT/findVh.o" &
g++ $CXXFLAGS -c "$HERE/lapacke_shim.cpp" -o "$OUT/lapacke_shim.o" &
wait
g++ -o "$OUT/ref_pipeline_vh" "$OUT/ref_harness_vh.o" "$OUT/mesh.o" "$OUT/generateStiff.o" "$OUT/matrixCon_vh.o" \
    "$OUT/findVh.o" "$OUT/mkl_sparse_shim.o" "$OUT/lapacke_shim.o" "$OUT/solver.o" -lm
echo "built $OUT/ref_pipeline_vh"
# oracle/_ref/ref_pipeline_gb300: the same harness with generateStiff,
# hypreSolve and paraGenerator taken from the library's reference-side shim
# (oracle/gb300_path.cpp), linked with libgds2para_gb300.so when it is built
LIB="$HERE/../gds2para_gb300/_build"
if [ -f "$LIB/libgds2para_gb300.so" ]; then
    g++ $CXXFLAGS -I"$HERE/../include" -c "$HERE/gb300_path.cpp" -o "$OUT/gb300_path.o" &
    g++ $CXXFLAGS -DG2P_REF_WITH_GB300_SHIM -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness_gb300.o" &
    wait
    g++ -o "$OUT/ref_pipeline_gb300" "$OUT/ref_harness_gb300.o" "$OUT/mesh.o" "$OUT/gb300_path.o" \
        "$OUT/mkl_sparse_shim.o" -L"$LIB" -lgds2para_gb300 -Wl,-rpath,"$LIB" -lm
    echo "built $OUT/ref_pipeline_gb300"
fi
echo "built $OUT/ref_pipeline $OUT/ref_gds $OUT/ref_network"
