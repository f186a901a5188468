/* Declaration shim for the HYPRE/MPI names matrixCon.cpp sees through
 * hypreSolver.h.  The solver behind hypreSolve() is the project's FP64 CPU
 * solver (oracle/solver.c); MPI is single-rank and its calls are no-ops.
 * Test infrastructure only. */
#ifndef G2P_ORACLE_HYPRE_SHIM_H
#define G2P_ORACLE_HYPRE_SHIM_H
typedef long long HYPRE_Int;
typedef double HYPRE_Complex;
typedef double HYPRE_Real;
typedef int MPI_Comm;
#define MPI_COMM_WORLD 0
extern "C" int MPI_Init(int *argc, char ***argv);
extern "C" int MPI_Finalize(void);
extern "C" int MPI_Comm_size(MPI_Comm, int *);
extern "C" int MPI_Comm_rank(MPI_Comm, int *);
#endif
