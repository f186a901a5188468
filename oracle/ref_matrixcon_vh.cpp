// TEST INFRASTRUCTURE: the reference's src/matrixCon.cpp compiled with its
// full-wave (Vh) path in.  The reference defines SKIP_VH in src/fdtd.hpp:76,
// which compiles out find_Vh(1000) (src/matrixCon.cpp:331-333) and the
// per-port, per-frequency Vh correction (src/matrixCon.cpp:609-805); this unit
// includes fdtd.hpp first, drops that definition (the header's include guard
// keeps it from coming back), and reports the V0 + Vh Z-parameters
// (PRINT_V0_Vh_Z_PARAM) instead of rescaling the V0 ones (PRINT_V0_Z_PARAM,
// whose print_z_V0 would overwrite every frequency after the first).  LAPACK
// and PARDISO come from oracle/ref_shims/lapacke_shim.cpp.  Built by
// oracle/build_ref.sh into oracle/_ref/ref_pipeline_vh.
#include "fdtd.hpp"
#undef SKIP_VH
#undef PRINT_V0_Z_PARAM
#define PRINT_V0_Vh_Z_PARAM
#include "matrixCon.cpp"
