/* CPU oracle for the gds2Para extraction hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's algorithm, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * Nothing in the product (gds2para_gb300/) links, loads or calls it.
 *
 * Each function cites the reference file:line it restates.  It is pinned
 * against the reference's own sources compiled here (oracle/build_ref.sh ->
 * oracle/_ref) through the fixtures in tests/golden/. */
#ifndef G2P_ORACLE_H
#define G2P_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- sparse CSR in FP64, int64 indices (the reference's myint) ---- */
typedef struct {
    int64_t n, m;        /* rows, cols */
    int64_t *ptr;        /* [n+1] */
    int64_t *col;        /* [nnz] */
    double *val;         /* [nnz] */
} g2po_csr;

void g2po_csr_free(g2po_csr *A);

/* ---- solver: the stand-in for hypreSolve (hypreSolve.cpp:9-283) ----
 * Flexible GMRES(restart) right-preconditioned by one AMG V-cycle of
 * aggregation AMG with symmetric Gauss-Seidel smoothing (the single-rank
 * form of HYPRE's relax type 6).  As hypre_FlexGMRESModifyPCAMG
 * (hypreSolve.cpp:285-293) does, the V-cycle uses pc_mod_sweeps sweeps while
 * the relative residual is above pc_tol.  Convergence test: ||b-Ax|| <=
 * rtol*||b||, as HYPRE's FlexGMRES with a zero initial guess. */
typedef struct {
    int restart;        /* KDim, 10 in the reference (hypreSolve.cpp:211) */
    int maxit;          /* 100 in the reference (hypreSolver.h:11) */
    double rtol;        /* 1e-4 in the reference (hypreSolver.h:8) */
    double pc_tol;      /* 0.1 (hypreSolver.h:9) */
    int pc_mod_sweeps;  /* 10 (hypreSolver.h:10) */
    int coarse_size;    /* direct solve below this many rows */
    double strength;    /* aggregation strength threshold */
    int reuse_setup;    /* 0: rebuild the hierarchy on every solve, as the
                           reference does (hypreSolve.cpp:36-68,251); 1: build
                           once per matrix and reuse it across ports */
    int stop_after_solves;    /* paraGenerator timing samples: stop after this many solves (0 = all) */
} g2po_solver_opts;

typedef struct {
    int iterations;
    double rel_residual;
    int levels;
    int converged;
} g2po_solve_stats;

void g2po_solver_default_opts(g2po_solver_opts *o);
/* Solves A x = b; A given as row-sorted COO (hypreSolve's input form). */
int g2po_solve_coo(const int64_t *rows, const int64_t *cols, const double *vals, int64_t nnz,
                   const double *b, int64_t n, double *x, const g2po_solver_opts *o,
                   g2po_solve_stats *st);

/* ---- the mesh description consumed by the path (the fdtdMesh subset,
 *      fdtd.hpp:182-356, after meshAndMark and portSet) ---- */
typedef struct {
    int64_t nx, ny, nz;
    const double *xn, *yn, *zn;        /* node coordinates (m) */
    const double *stack_epsn;          /* [nz] stackEpsn (relative) */
    const double *stack_sign;          /* [nz] stackSign (S/m) */
    const int64_t *mark_node;          /* [N_node] conductor id (1-based) or 0 */
    const int64_t *mark_edge;          /* [N_edge] conductor id or 0 */
    int64_t num_cdt;
    const int32_t *mark_port;          /* [num_cdt] conductor[].markPort */
    const uint8_t *cdt_return;         /* [num_cdt] 1 if its PEC sets were taken (mesh.cpp:943-953) */
    int32_t num_ports;
    const int32_t *port_side_ptr;      /* [num_ports+1] */
    const int64_t *side_edge_ptr;      /* [num_sides+1] */
    const int64_t *side_edges;         /* portEdge, return -> supply */
    const double *side_area;           /* portArea */
    const int32_t *side_dir;           /* portDirection */
    double freq_start, freq_end, freq_unit;
    int32_t nfreq, freq_scale;
} g2po_mesh;

/* Index maps: PEC edge flags and mapEdge (fdtd.hpp:1444-1529, mesh.cpp:950-987).
 * map_edge[N_edge] receives the new index or -1; returns bden. */
int64_t g2po_index_maps(const g2po_mesh *m, int64_t *map_edge, uint8_t *pec_edge, uint8_t *pec_node);

/* Curl-curl stiffness S = Sh*Se^T/mu with PEC rows/cols removed
 * (generateStiff.cpp:6-565, :897-980).  CSR over the remapped edges. */
int g2po_stiffness(const g2po_mesh *m, const int64_t *map_edge, const uint8_t *pec_edge, g2po_csr *S);

/* V0 basis in the reference's COO order, rows = original edge indices. */
typedef struct {
    int64_t nnz, ncol;
    int64_t *row, *col;
    double *val, *aval;
    int64_t *map;          /* [N_node] column+1 or 0 */
} g2po_v0;
void g2po_v0_free(g2po_v0 *v);

int g2po_v0d(const g2po_mesh *m, const uint8_t *pec_node, g2po_v0 *v);   /* merge_v0d1 fdtd.hpp:1823-2774 */
int g2po_v0c(const g2po_mesh *m, const uint8_t *pec_node, g2po_v0 *v);   /* merge_v0c  fdtd.hpp:2866-3479 */
int g2po_ad(const g2po_mesh *m, const g2po_v0 *v, g2po_csr *A);         /* generateAd fdtd.hpp:2778-2862 */
int g2po_ac(const g2po_mesh *m, const g2po_v0 *v, g2po_csr *A);         /* generateAc fdtd.hpp:3481-3574 */

/* Whole V0 extraction (paraGenerator matrixCon.cpp:11-907 with the default
 * SKIP_VH path): Z[nfreq*P*P] (re, im interleaved) in sys->x's layout,
 * including print_z_V0's frequency rescale (fdtd.hpp:4249-4316). */
typedef struct {
    int64_t leng_v0d, leng_v0c, nnz_ad, nnz_ac, bden;
    int solves, total_iterations;
    double max_rel_residual;
    double t_assembly, t_setup, t_solve;     /* seconds */
    double t_each[3];                        /* first port's Ad, Ac, Ad solves incl. setup (s) */
} g2po_para_stats;
int g2po_para_generator(const g2po_mesh *m, const g2po_solver_opts *o, int max_ports,
                        double *z_out, g2po_para_stats *st);

/* The same extraction as a job whose ports can run on several host threads:
 * g2po_job_create does the assembly (index maps, V0d/Ad, V0c/Ac; the mesh
 * must outlive the job); g2po_job_port_stage runs port p's next solve
 * (0: Ad, 1: Ac, 2: Ad and the port's Z column), each with its own AMG setup
 * as hypreSolve does.  Calls for different ports may run concurrently;
 * calls for one port must be ordered.  g2po_job_z writes Z as
 * g2po_para_generator does. */
typedef struct g2po_job g2po_job;
g2po_job *g2po_job_create(const g2po_mesh *m, g2po_para_stats *st);
int g2po_job_port_stage(g2po_job *j, int port, const g2po_solver_opts *o, g2po_solve_stats *ss, double *t_setup);
void g2po_job_z(const g2po_job *j, double *z_out);
void g2po_job_destroy(g2po_job *j);

/* The full-wave (Vh) path, which the reference compiles out (SKIP_VH,
 * fdtd.hpp:76): g2po_job_enable_vh before any port's stages keeps the V0
 * fields it needs and builds S; g2po_find_vh restates find_Vh(k)
 * (fdtd.hpp:3577-3859) into vh (nr x mm complex, column-major, interleaved,
 * malloc'd; nr = N_edge - bden); g2po_job_vh_z restates the per-port,
 * per-frequency Vh correction (matrixCon.cpp:609-805) and
 * Construct_Z_V0_Vh (fdtd.hpp:4133-4170).  The dense eigen and linear
 * solves come from oracle/lapacke_shim.cpp. */
int g2po_job_enable_vh(g2po_job *j);
int64_t g2po_job_nr(const g2po_job *j);
int g2po_find_vh(g2po_job *j, int k, double **vh, int64_t *mm);
int g2po_job_vh_z(g2po_job *j, const double *vh, int64_t mm, double *z_vh, double *z_ref);

#ifdef __cplusplus
}
#endif
#endif
