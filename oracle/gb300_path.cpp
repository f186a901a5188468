// The translation unit a gds2Para maintainer adds to put the V0 path on the
// GPU: the reference's generateStiff (src/generateStiff.cpp:6), hypreSolve
// (src/hypreSolve.cpp:9) and paraGenerator (src/matrixCon.cpp:11), with
// their own prototypes, forwarded to the library through
// include/gds2para_gb300_shim.hpp.  TEST INFRASTRUCTURE here: oracle/build_ref.sh
// compiles it against the reference's own fdtd.hpp (which proves that the
// shim binds to the real fdtdMesh) and links oracle/_ref/ref_pipeline_gb300,
// the reference's harness with these three functions in place of the
// reference's generateStiff.cpp, its hypreSolve and matrixCon.cpp.
#include "fdtd.hpp"
#include "hypreSolver.h"
#include "gds2para_gb300_shim.hpp"

int generateStiff(fdtdMesh *sys) { return g2p_shim::generateStiff(sys); }

int hypreSolve(fdtdMesh *sys, myint *ARowId, myint *AColId, double *Aval, myint leng_A, double *bin, myint leng_v0,
               double *solution) {
    return g2p_shim::hypreSolve(sys, ARowId, AColId, Aval, leng_A, bin, leng_v0, solution);
}

int paraGenerator(fdtdMesh *sys, unordered_map<double, int> xi, unordered_map<double, int> yi,
                  unordered_map<double, int> zi) {
    return g2p_shim::paraGenerator(sys, xi, yi, zi);
}
