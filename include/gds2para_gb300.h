/* gds2para_gb300 -- GB300-native (sm_103a) full-wave extraction hot path of
 * purdue-onchip/gds2Para behind a plain C ABI.
 *
 * The reference's C++ entry points on this path and their replacements:
 *
 *   fdtdMesh (src/fdtd.hpp:182-356)            -> g2p_mesh_desc + g2p_mesh
 *   setMapEdge/findBoundNodeEdge
 *            (src/fdtd.hpp:1444-1529)           -> g2p_index_maps
 *   generateStiff (src/generateStiff.cpp:6)    -> g2p_generate_stiff (+ g2p_export_stiff)
 *   merge_v0d1/generateAd, merge_v0c/generateAc
 *            (src/fdtd.hpp:1823-3574)           -> g2p_assemble_v0 (+ g2p_export_v0,
 *                                                  g2p_export_laplacian)
 *   hypreSolve (src/hypreSolve.cpp:9,
 *            src/hypreSolver.h:14)              -> g2p_hypre_solve, g2p_solver_*
 *   paraGenerator (src/matrixCon.cpp:11)       -> g2p_para_generator
 *   find_Vh (src/fdtd.hpp:3577)                -> g2p_find_vh (+ g2p_export_vh, g2p_set_vh)
 *   paraGenerator's full-wave part
 *            (src/matrixCon.cpp:609-805)        -> g2p_para_generator_vh
 *
 * Arrays in g2p_mesh_desc may live in host or device memory (they are
 * copied with unified addressing); every output buffer is a HOST pointer
 * owned by the caller; device memory is owned by the handles.  Every entry
 * point returns a g2p_status and never exits the process; g2p_last_error()
 * describes the most recent failure of the calling thread.  A handle must be
 * used by one host thread at a time.  The library runs on CUDA device 0 (or
 * the device current when the handle is created) and requires sm_103a. */
#ifndef GDS2PARA_GB300_H
#define GDS2PARA_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    G2P_OK = 0,
    G2P_ERR_INVALID = 1,        /* bad argument or inconsistent mesh description */
    G2P_ERR_CUDA = 2,           /* CUDA runtime failure (see g2p_last_error) */
    G2P_ERR_NOMEM = 3,          /* device (or, for find_Vh's eigenvectors, host) allocation failed */
    G2P_ERR_NOT_CONVERGED = 4,  /* solver hit maxit above rtol (result still written) */
    G2P_ERR_UNSUPPORTED = 5,    /* layout outside what the path handles (message says which) */
    G2P_ERR_STATE = 6,          /* a required earlier step has not run */
    G2P_ERR_ADMISSION = 7       /* job rejected: its device footprint exceeds the budget */
} g2p_status;

/* The fdtdMesh members the path reads, after meshAndMark and portSet
 * (src/mesh.cpp:5-1133,1196-1594).  Field meanings follow the reference:
 * node n = iz*N_node_s + ix*ny + iy; edges are numbered per z plane as
 * y-edges, x-edges, then z-edges (src/fdtd.hpp:4107-4130). */
typedef struct {
    int64_t nx, ny, nz;                /* node counts */
    const double *xn, *yn, *zn;        /* node coordinates (m) */
    const double *stack_epsn;          /* [nz] stackEpsn (relative permittivity) */
    const double *stack_sign;          /* [nz] stackSign (S/m) */
    const int64_t *mark_node;          /* [N_node] conductor id (1-based) or 0 */
    const int64_t *mark_edge;          /* [N_edge] conductor id or 0 */
    int64_t num_cdt;                   /* numCdt */
    const int32_t *mark_port;          /* [num_cdt] conductor[].markPort: -1 return, 0 passive, p+1 excited */
    const uint8_t *cdt_return;         /* [num_cdt] 1 if findBoundNodeEdge ran on it (src/mesh.cpp:943-953) */
    int32_t num_ports;
    const int32_t *port_side_ptr;      /* [num_ports+1] sides of each port */
    const int64_t *side_edge_ptr;      /* [num_sides+1] */
    const int64_t *side_edges;         /* portEdge, return -> supply */
    const double *side_area;           /* portArea */
    const int32_t *side_dir;           /* portDirection */
    double freq_start, freq_end, freq_unit;
    int32_t nfreq, freq_scale;         /* freqScale 1 linear, 0 logarithmic */
} g2p_mesh_desc;

typedef struct g2p_mesh g2p_mesh;
typedef struct g2p_solver g2p_solver;

/* G2P_PREC_FP64: the plain FP64 method.  G2P_PREC_MIXED: FP32 FGMRES and AMG
 * inside FP64 iterative refinement.  G2P_PREC_FP64_PC32: FP64 FGMRES whose
 * V-cycle preconditioner runs in FP32 (for operators whose conditioning
 * stalls FP32 Krylov solves). */
enum { G2P_PREC_FP64 = 0, G2P_PREC_MIXED = 1, G2P_PREC_FP64_PC32 = 2 };

typedef struct {
    int32_t precision;        /* G2P_PREC_FP64, G2P_PREC_MIXED or G2P_PREC_FP64_PC32 */
    int32_t restart;          /* FGMRES restart length (KDim) */
    int32_t maxit;            /* max FGMRES iterations (FP64) / refinement sweeps x inner (mixed) */
    double rtol;              /* ||b - A x|| <= rtol * ||b|| per right-hand side */
    int32_t smoother_degree;  /* Chebyshev degree of the AMG smoother */
    int32_t coarse_size;      /* dense LU below this many rows */
    double strength;          /* aggregation strength threshold */
    int32_t max_levels;
    double inner_rtol;        /* mixed: inner FP32 solve tolerance */
    int32_t inner_maxit;      /* mixed: inner FP32 iterations per refinement step */
    int32_t batch;            /* paraGenerator: 1 = all ports as one RHS block, 0 = port by
                                 port, n >= 2 = blocks of at most n ports */
    int32_t use_graphs;       /* 1 (default): each Arnoldi step (V-cycle, product,
                                 Gram-Schmidt, Givens) is captured as a CUDA graph on
                                 its second use and replayed; results are identical */
    int32_t autotune;         /* paraGenerator, 1: pick the block width of the port
                                 right-hand sides (all ports, or 8/16/32/64 at a time)
                                 and the Chebyshev degree (2, 3, 4) of the Ad solves by
                                 timing the first block's Ad solve with each, and the
                                 aggregation strength of Ac's AMG (strength / 2,
                                 strength, 2 strength) by timing its first Ac solve,
                                 once per grid shape and port count in the process
                                 (later jobs of that shape reuse the choice); 0
                                 (default): all ports, smoother_degree, Ac at
                                 min(2 strength, 0.1) */
    int32_t inner_restart;    /* mixed: restart length of the inner FP32 FGMRES (its
                                 basis is (2 inner_restart + 1) vectors of n x k; 0 =
                                 restart) */
} g2p_solver_params;

typedef struct {
    int32_t iterations;       /* total inner iterations (max over right-hand sides) */
    int32_t refinements;      /* outer FP64 refinement steps (mixed) */
    double rel_residual;      /* max over right-hand sides, FP64 true residual */
    int32_t levels;
    int32_t converged;
    int64_t coarse_rows;
    double setup_ms, solve_ms;
} g2p_solve_stats;

typedef struct {
    int64_t bden, leng_S, leng_v0d, leng_v0c, nnz_v0d, nnz_v0c, nnz_ad, nnz_ac;
} g2p_sizes;

typedef struct {
    g2p_sizes sizes;
    int32_t solves;           /* linear systems solved (3 per port) */
    int32_t total_iterations;
    double max_rel_residual;
    double assembly_ms, setup_ms, solve_ms, total_ms;
    int32_t ad_levels, ac_levels;
    int32_t rhs_block, ad_degree;    /* ports per block solve and Ad's Chebyshev degree used */
    double ac_strength;              /* aggregation strength threshold of Ac's AMG */
    int32_t ac_precision;            /* Ac's solver mode (G2P_PREC_*; tuned with autotune) */
    int32_t ac_iterations;           /* iterations of the Ac solves */
} g2p_extract_stats;

/* ---- library ---- */
const char *g2p_last_error(void);
const char *g2p_version(void);
/* parity_mode 1: the reference's hypreSolve settings (FlexGMRES KDim 10, 100
 * iterations, rtol 1e-4; src/hypreSolver.h:7-11); 0: the oracle settings
 * (FP64, rtol 1e-10). */
void g2p_default_params(g2p_solver_params *p, int32_t parity_mode);

/* ---- fdtdMesh ---- */
g2p_status g2p_mesh_create(const g2p_mesh_desc *desc, g2p_mesh **out);
g2p_status g2p_mesh_destroy(g2p_mesh *m);
g2p_status g2p_mesh_sizes(const g2p_mesh *m, g2p_sizes *out);

/* ---- index maps: setMapEdge / findBoundNodeEdge / LOWER_BOUNDARY_PEC
 * (src/fdtd.hpp:1444-1529, src/mesh.cpp:943-987).  map_edge (nullable) gets
 * N_edge values: the edge's index after PEC removal, or -1. ---- */
g2p_status g2p_index_maps(g2p_mesh *m, int64_t *bden, int64_t *map_edge);

/* ---- generateStiff (src/generateStiff.cpp:6-565): S = Sh*Se^T/mu over the
 * non-PEC edges, kept on the device as CSR.  g2p_export_stiff writes the
 * reference's COO (SRowId, SColId, Sval; leng_S entries). ---- */
g2p_status g2p_generate_stiff(g2p_mesh *m, int64_t *leng_S);
g2p_status g2p_export_stiff(g2p_mesh *m, int64_t *row, int64_t *col, double *val);

/* ---- V0 bases and Laplacians (src/fdtd.hpp:1823-3574).  which = 0 for
 * V0d/Ad, 1 for V0c/Ac.  g2p_export_v0 writes the COO of V0 (rows = original
 * edge index, in the reference's entry order) with its a-values and the node
 * map (column+1 or 0; N_node values); g2p_export_laplacian writes the
 * row-sorted COO the reference hands to hypreSolve. ---- */
g2p_status g2p_assemble_v0(g2p_mesh *m, g2p_sizes *out);
g2p_status g2p_export_v0(g2p_mesh *m, int32_t which, int64_t *row, int64_t *col, double *val, double *aval,
                         int64_t *map);
g2p_status g2p_export_laplacian(g2p_mesh *m, int32_t which, int64_t *row, int64_t *col, double *val);

/* ---- hypreSolve (src/hypreSolve.cpp:9): x = A^-1 b for a row-sorted COO A
 * (0-based int64), with the reference's parity settings.  Unlike the
 * reference it reports non-convergence (G2P_ERR_NOT_CONVERGED) instead of
 * returning 0 unconditionally; the solution is written either way. ---- */
g2p_status g2p_hypre_solve(const int64_t *ARowId, const int64_t *AColId, const double *Aval, int64_t leng_A,
                           const double *bin, int64_t leng_v0, double *solution);

/* Reusable AMG-FGMRES solver on one matrix (setup once, many solves). */
g2p_status g2p_solver_create(const int64_t *ARowId, const int64_t *AColId, const double *Aval, int64_t leng_A,
                             int64_t n, const g2p_solver_params *p, g2p_solver **out);
/* b, x: host, column-major n x nrhs. */
g2p_status g2p_solver_solve(g2p_solver *s, const double *b, double *x, int32_t nrhs, g2p_solve_stats *st);
g2p_status g2p_solver_destroy(g2p_solver *s);

/* ---- paraGenerator (src/matrixCon.cpp:11-907, default V0 path): per port
 * the three solves Ad, Ac, Ad, the back-projections and Construct_Z_V0
 * (src/fdtd.hpp:4173-4215), then print_z_V0's frequency rescale
 * (src/fdtd.hpp:4249-4316).  z_out (host) receives nfreq*P*P complex values
 * as interleaved (re, im) doubles in sys->x's layout, including the
 * reference's transposed storage of frequencies after the first.  Runs
 * g2p_index_maps and g2p_assemble_v0 first if they have not run. ---- */
g2p_status g2p_para_generator(g2p_mesh *m, const g2p_solver_params *p, double *z_out, g2p_extract_stats *st);

/* ---- full-wave (Vh) mode: find_Vh (src/fdtd.hpp:3577-3859) and the Vh
 * correction of paraGenerator (src/matrixCon.cpp:609-805) with
 * Construct_Z_V0_Vh (src/fdtd.hpp:4133-4170); the reference compiles this
 * path out (SKIP_VH, src/fdtd.hpp:76).
 * g2p_find_vh: k Arnoldi steps (modified Gram-Schmidt, on the device) on the
 * 2N operator [[0, I], [-D_eps^-1 S/s^2, -D_eps^-1 D_sig/s]], s = 1e14, the
 * Hessenberg eigenproblem on the host, and Vh = V(1:N,1:k) * (the
 * eigenvectors of the eigenvalues with |Im| > 1e-6, a conjugate pair giving
 * two columns).  *leng_vh = Vh's column count.  Needs g2p_generate_stiff.
 * g2p_export_vh: Vh (host or device), column-major N x leng_vh complex as
 * interleaved (re, im) doubles, N = leng_S's row count (non-PEC edges).
 * g2p_para_generator_vh: runs g2p_find_vh if it has not run, the V0 path
 * (z_v0, nullable, as g2p_para_generator writes it) keeping each port's V0
 * field directions, then per port and frequency the deflated Galerkin
 * correction; z_vh (host) receives nfreq*P*P complex values, entry
 * f*P*P + q + P*p for response port q and source port p, NOT rescaled or
 * transposed (print_z_V0_Vh's layout).  The reference's own output for the
 * first frequency adds Construct_Z_V0's value to this one (it accumulates
 * into sys->x without clearing it).  The 2 x 2 and leng_vh x leng_vh
 * complex solves run on the host, as LAPACK does them in the reference.
 * g2p_set_vh: installs a Vh computed elsewhere (same layout as
 * g2p_export_vh writes, leng_vh columns) in place of g2p_find_vh's, for
 * reuse across calls or for checking the correction stage on its own.
 * g2p_hessenberg_eig: eigenvalues (wr, wi) of the real upper Hessenberg
 * n x n matrix h (column-major; entries below the subdiagonal ignored), a
 * complex pair at consecutive positions, positive imaginary part first:
 * the library's dhseqr stand-in, exported for tests. ---- */
g2p_status g2p_find_vh(g2p_mesh *m, int32_t k, int64_t *leng_vh);
g2p_status g2p_export_vh(g2p_mesh *m, double *vh);
g2p_status g2p_set_vh(g2p_mesh *m, const double *vh, int64_t leng_vh);
g2p_status g2p_para_generator_vh(g2p_mesh *m, const g2p_solver_params *p, int32_t k, double *z_vh, double *z_v0,
                                 g2p_extract_stats *st);
g2p_status g2p_hessenberg_eig(int64_t n, const double *h, double *wr, double *wi);
/* g2p_stiff_apply: y = S x (x, y: host or device, leng_S's row count each)
 * by the assembled CSR (matrix_free = 0) or by the matrix-free curl-curl
 * stencil (1: face circulations then edge sums over full-grid arrays staged
 * by TMA tiles; the same coefficients as generateStiff, equal to rounding;
 * g2p_find_vh applies S this way).  *ms (nullable) receives the device time
 * of one product averaged over reps >= 1 repetitions. */
g2p_status g2p_stiff_apply(g2p_mesh *m, int32_t matrix_free, int32_t reps, const double *x, double *y, double *ms);

/* ---- diagnostics (no counterpart in the reference) ----
 * g2p_launch_count: kernels launched by the library so far in this process.
 * g2p_profile_begin/end: CUDA-event timing of the sparse matrix-multi-vector
 * kernel (the solves' dominant kernel) between the two calls: total device
 * milliseconds, algorithmic bytes (values + column indices + row offsets
 * read once, vectors read and written once) and launches.  Single-threaded
 * use only. */
int64_t g2p_launch_count(void);
void g2p_profile_begin(void);
g2p_status g2p_profile_end(double *kernel_ms, double *kernel_bytes, int64_t *launches);
/* Per-kernel device time of the last profiled interval, one line per kernel
 * ("name<TAB>launches<TAB>total_ms"); returns the full length, writes at most
 * cap-1 bytes plus a terminator. */
int64_t g2p_profile_report(char *buf, int64_t cap);
/* The short-row SpMM launches (k_spmm_sell) of the last profiled interval
 * in eight classes: FP32 operators then FP64 operators, each split by the
 * operator's rows (< 64k, < 256k, < 1M, >= 1M).
 * Writes device milliseconds, algorithmic bytes and launches per class
 * (arrays of 8). */
void g2p_profile_buckets(double *ms, double *bytes, int64_t *launches);

/* ---- conductor marking and ports: meshAndMark's findInsideCond and conductor
 * numbering (src/mesh.cpp:683-1020) and portSet (src/mesh.cpp:1196-1594) on
 * the structured grid already chosen (xn, yn, zn).  Conductors are boxes of
 * node indices (closed ranges; a later box overwrites an earlier one); the
 * z = 0 plane is the lower PEC boundary.  Outputs are the g2p_mesh_desc
 * fields: mark_node [N_node] and mark_edge [N_edge] (host or device
 * memory), num_cdt, and -- when num_ports > 0 -- mark_port and cdt_return
 * [max_cdt], side_edge_ptr [nsides + 1], side_edges [max_side_edges],
 * side_area and side_dir [nsides], nsides = port_side_ptr[num_ports].
 * Conductors are numbered 1.. in the order of their lowest node, as the
 * reference's labelling leaves them. ---- */
typedef struct { int64_t x0, x1, y0, y1, z0, z1; } g2p_box;
typedef struct { int64_t sx, sy, sz, rx, ry, rz; } g2p_port_side;   /* supply node -> return node */
g2p_status g2p_mesh_mark(int64_t nx, int64_t ny, int64_t nz, const double *xn, const double *yn, const double *zn,
                         const g2p_box *boxes, int64_t nbox, int32_t num_ports, const int32_t *port_side_ptr,
                         const g2p_port_side *sides, int64_t *mark_node, int64_t *mark_edge, int64_t *num_cdt,
                         int32_t *mark_port, uint8_t *cdt_return, int64_t max_cdt, int64_t *side_edge_ptr,
                         int64_t *side_edges, int64_t max_side_edges, double *side_area, int32_t *side_dir);

/* Conductor marking from polygons, the rest of meshAndMark and portSet
 * (findInsideCond, src/fdtd.hpp:534-826; the conductor numbering, port
 * placement and boundary marks of src/mesh.cpp:456-1020; portSet,
 * src/mesh.cpp:1196-1356) on the grid g2p_mesh_grid made from the same
 * polygons and port sides.  Polygons as g2p_polygons_get returns them, with
 * poly_z[2 * npoly] their (z bottom, z top) in metres from the stack layer of
 * their GDSII number (equal values: on no layer; such a polygon marks
 * nothing).  Port sides: side_coords[6 * nside] (supply x y z, return x y z,
 * metres) for the sides of port p at port_side_ptr[p] ..
 * port_side_ptr[p + 1] - 1, and side_dir_in[nside] (+1/-1).  A port end
 * outside every conductor moves along the port axis to the nearest
 * conductor node within 50 lines, as findPortNode moves it, and
 * side_coords is updated in place.  Outputs as g2p_mesh_mark. */
g2p_status g2p_mesh_mark_polygons(int64_t nx, int64_t ny, int64_t nz, const double *xn, const double *yn,
                                  const double *zn, int64_t npoly, const int64_t *vert_ptr, const double *vx,
                                  const double *vy, const double *poly_z, int32_t num_ports,
                                  const int32_t *port_side_ptr, double *side_coords, const int32_t *side_dir_in,
                                  int64_t *mark_node, int64_t *mark_edge, int64_t *num_cdt, int32_t *mark_port,
                                  uint8_t *cdt_return, int64_t max_cdt, int64_t *side_edge_ptr, int64_t *side_edges,
                                  int64_t max_side_edges, double *side_area, int32_t *side_dir);

/* ---- layout ingest (host code; the reference reads GDSII with Limbo into
 * AsciiDataBase and flattens it with saveToMesh, limboint.hpp:2823-3150,
 * TestMain.cpp:258-292) ----
 * g2p_gdsii_read flattens the file's last cell (the top cell) into the
 * conductor polygons the reference stores in fdtdMesh::conductorIn, in the
 * same order and with the same vertices (metres): boundaries, one rectangle
 * per path segment, boxes with BOXTYPE 0, then structure and array
 * references, recursively.  Polygons on the ignored GDSII layers are left
 * out.  g2p_polygons_get fills layer[npoly], vert_ptr[npoly + 1] (offsets of
 * each polygon's vertices) and x, y[nvert], sized by g2p_polygons_size. */
typedef struct g2p_polygons g2p_polygons;
g2p_status g2p_gdsii_read(const char *path, const int32_t *ignore_layers, int32_t n_ignore, g2p_polygons **out);
g2p_status g2p_polygons_size(const g2p_polygons *p, int64_t *npoly, int64_t *nvert);
g2p_status g2p_polygons_get(const g2p_polygons *p, int32_t *layer, int64_t *vert_ptr, double *x, double *y);
void g2p_polygons_free(g2p_polygons *p);

/* .sim_input reader (SolverDataBase::readSimInput, src/solnoutclass.hpp:
 * 5412-5886, as convertToFDTDMesh passes it on, :5894-5984).  Sizes: the
 * physically valid stack layers, the ports (sides with the same name form
 * one port) and their sides.  g2p_sim_input_get (any output may be null):
 * lim[6] (xlim1 xlim2 ylim1 ylim2 zlim1 zlim2, metres); units[4] = length
 * unit, freqUnit, freqStart, freqEnd (freqEnd = freqStart for one point);
 * freq_counts[2] = nfreq, freqScale; layers[4 * nlayer] = z begin, z end
 * (metres), eps_r, sigma and layer_gdsii[nlayer]; port_side_ptr[nport + 1],
 * side_coords[6 * nside] (supply x y z, return x y z, metres) and
 * side_dir[nside] (+1 when a supply coordinate exceeds the return's).  A
 * board-outline file in place of the x/y limits is G2P_ERR_UNSUPPORTED. */
typedef struct g2p_sim_input g2p_sim_input;
g2p_status g2p_sim_input_read(const char *path, g2p_sim_input **out);
g2p_status g2p_sim_input_sizes(const g2p_sim_input *s, int32_t *nlayer, int32_t *nport, int32_t *nside);
g2p_status g2p_sim_input_get(const g2p_sim_input *s, double *lim, double *units, int32_t *freq_counts,
                             double *layers, int32_t *layer_gdsii, int32_t *port_side_ptr, double *side_coords,
                             int32_t *side_dir);
void g2p_sim_input_free(g2p_sim_input *s);

/* The mesher's grid lines (meshAndMark, mesh.cpp:5-330): x/y lines from the
 * polygon vertices and port-side ends, merged and filled by the reference's
 * disMin/disMax rules against the limits lim[6] = {xlim1, xlim2, ylim1,
 * ylim2, zlim1, zlim2}; z lines from the stack layers and port sides; and
 * per cell layer the eps and sigma of the stack layer containing it, plus the
 * top surface (stack_epsn, stack_sign: nz entries).  Polygons as
 * g2p_polygons_get returns them; sides: 6 per port side (x1 y1 z1 x2 y2 z2);
 * stack: 4 per layer (z begin, z end, eps_r, sigma), all lengths in metres.
 * counts[3] = {nx, ny, nz} is always set; G2P_ERR_INVALID when nx or ny
 * exceeds cap_xy or nz exceeds cap_z. */
g2p_status g2p_mesh_grid(const double *lim, int64_t npoly, const int64_t *vert_ptr, const double *vx, const double *vy,
                         int32_t nside, const double *sides, int32_t nstack, const double *stack, int64_t cap_xy,
                         int64_t cap_z, double *xn, double *yn, double *zn, double *stack_epsn, double *stack_sign,
                         int64_t *counts);

/* ---- extraction service (no counterpart in the reference, which extracts
 * one layout per process) ----
 * A queue of extraction jobs, each the work of g2p_mesh_create +
 * g2p_generate_stiff + g2p_para_generator on its own layout.  While fewer
 * than max_active jobs run, the first queued job whose device footprint
 * estimate fits mem_budget_bytes minus the estimates of the running jobs
 * starts; a later job may pass one that does not fit yet at most
 * 2 * max_active times, after which the passed job holds the queue until it
 * fits (a job larger than the budget runs alone).  A job whose estimate with
 * all its ports in one block (batch 1) exceeds 2/3 of the budget runs them in
 * the widest power-of-two blocks that fit (one at a time if none does).
 * Each running job
 * has its own host thread, mesh handle and CUDA stream, so their kernels
 * overlap on the device; results do not depend on what else runs.  The
 * estimate is a size model scaled by the largest measured/model ratio of
 * jobs that ran alone (device pool high-water).  g2p_server_submit copies
 * the description's arrays (host or device) before it returns.
 * g2p_server_wait blocks until the job ends, writes Z as
 * g2p_para_generator does (z_out: nfreq*P*P complex, may be NULL), and
 * forgets the job.  Use one server from any number of host threads. */
typedef struct g2p_server g2p_server;
typedef struct {
    double queued_ms, run_ms, total_ms;          /* submit->start, start->end, submit->end */
    int64_t footprint_estimate, footprint_measured;   /* bytes; measured only when it ran alone */
    int32_t ran_alone;
} g2p_job_times;
g2p_status g2p_server_create(int64_t mem_budget_bytes, int32_t max_active, g2p_server **out);
g2p_status g2p_server_submit(g2p_server *s, const g2p_mesh_desc *desc, const g2p_solver_params *p, int64_t *job);
g2p_status g2p_server_wait(g2p_server *s, int64_t job, double *z_out, g2p_extract_stats *st, g2p_job_times *t);
/* Finishes the queued and running jobs, then frees the server. */
g2p_status g2p_server_destroy(g2p_server *s);

/* ---- edge map without device allocation (no counterpart in the
 * reference) ----
 * Same map_edge and bden as g2p_index_maps, on device pointers and without
 * a mesh handle, for callers that cannot let the library take device memory:
 * a host runtime whose own arena or caching allocator holds the device's
 * memory, or a per-layout loop on a fixed latency budget.  Its one temporary
 * (the scan's per-tile partial sums) is a static 256 KiB device buffer, so
 * it takes at most 67,106,816 edges (32,767 tiles of 2,048) and at most
 * 2^20 nodes along each axis, and returns G2P_ERR_INVALID, with the limit in
 * g2p_last_error, beyond either.
 * mark_edge [N_edge] and cdt_return [num_cdt] are inputs; map_edge [N_edge]
 * and bden [1] are outputs; all four must be device, managed or mapped
 * pinned host memory.  Nothing needs to be zeroed first.  Work is queued on
 * `stream` (a cudaStream_t; NULL = the default stream) and the call returns
 * without synchronizing.  The first call on each device also looks the
 * buffer's address up (cudaGetSymbolAddress, which can load the module):
 * make that first call outside any stream capture.  That address is kept
 * for the life of the process and does not survive cudaDeviceReset: do not
 * call this entry point on a device after resetting it.  All calls on one device
 * share the buffer, so two calls whose work can overlap on the device (other
 * streams, other host threads) race: order them on one stream or with
 * events. */
g2p_status g2p_map_edge_noalloc(int64_t nx, int64_t ny, int64_t nz, const int64_t *mark_edge,
                                const uint8_t *cdt_return, int64_t num_cdt, int64_t *map_edge,
                                int64_t *bden, void *stream);

/* ---- network parameters after paraGenerator ----
 * Matrices are nfreq blocks of nports x nports complex values, entry (i, j)
 * of frequency f at (f*nports + i)*nports + j as interleaved (re, im)
 * doubles: the order saveNetworkParam reads sys->x in
 * (src/solnoutclass.hpp:1394-1452), so g2p_para_generator's z_out is a
 * valid input.
 *
 * g2p_convert_param: convertParam (src/solnoutclass.hpp:1456-1610).  from and
 * to are 'Z', 'Y' or 'S'; Z <-> Y invert the matrix, the S conversions use
 * the ports' real source impedances z_source [nports] (> 0; may be NULL for
 * Z <-> Y).  Up to 64 ports; one GPU block per frequency.  in, out and
 * z_source may be host or device memory; in == out is allowed.  A singular
 * matrix returns G2P_ERR_INVALID (the reference carries on with Eigen's
 * result). */
g2p_status g2p_convert_param(char from, char to, int32_t nports, int32_t nfreq, const double *z_source,
                             const double *in, double *out);
/* g2p_write_touchstone: dumpTouchstone (src/solnoutclass.hpp:6118-6226), a
 * Touchstone 2.0 file; g2p_write_citi: dumpCITI
 * (src/solnoutclass.hpp:6040-6115), a CITIfile.  param is the matrices'
 * kind ('Z', 'Y' or 'S'), freqs [nfreq] in Hz, z_source [nports] the port
 * impedances, design the design name.  Host memory only; no GPU is used.
 * Unlike the reference, the time stamp is the current local time. */
g2p_status g2p_write_touchstone(const char *path, char param, int32_t nports, int32_t nfreq, const double *freqs,
                                const double *z_source, const double *p, const char *design);
g2p_status g2p_write_citi(const char *path, char param, int32_t nports, int32_t nfreq, const double *freqs,
                          const double *p, const char *design);
/* g2p_ybus_from_param: computeYBusFromParam(0) (src/solnoutclass.hpp:1662-1748,
 * dense build), which saveNetworkParam runs: nodal matrices G and C
 * [nports*nports, row-major, host] from the first frequency's matrix p0
 * (nports*nports complex, interleaved, host or device) at freq0 Hz.  As in
 * the reference, 'Z' takes the matrix itself as Y and 'Y' takes its inverse
 * (on the GPU); G = Re Y, C(i,j) = -1 / (Im Y(i,j) * 2 pi freq0).  'S'
 * returns G2P_ERR_UNSUPPORTED (the reference leaves Y empty there). */
g2p_status g2p_ybus_from_param(char param, int32_t nports, double freq0, const double *p0, double *G, double *C);
/* g2p_terminate_port: terminatePortZ / terminatePortY (src/solnoutclass.hpp:
 * 1767-1921) on the GPU: port `port` of Z- ('Z') or Y-parameters ('Y') loaded
 * by an impedance or admittance and reduced away (Kron reduction,
 * p'_ij = p_ij - p_ik p_kj / (p_kk + load) for i, j != k); out holds
 * nfreq (nports-1)^2 complex values.  As in the reference the load is
 * load[0] at the first frequency with its imaginary part scaled by f / f0
 * (nload must be 1 for a single frequency).  The reference's own version
 * assigns where it compares (`if (indi = indPort)`) and fills only the upper
 * triangle, so it never finishes for a port after the first and leaves the
 * lower triangle zero otherwise; this one reduces the whole matrix.
 * g2p_y_from_circuit: computeYParamFromCircuit (:1617-1678), Y_f = G +
 * j 2 pi f C for every frequency. */
g2p_status g2p_terminate_port(char param, int32_t nports, int32_t nfreq, const double *freqs, int32_t port,
                              int32_t nload, const double *load, const double *in, double *out);
g2p_status g2p_y_from_circuit(int32_t nports, int32_t nfreq, const double *freqs, const double *G, const double *C,
                              double *out);
/* g2p_write_xyce: dumpXyce / toXyce (src/solnoutclass.hpp:2094-2225,
 * 6032-6037), a SPICE subcircuit; g2p_write_spef: dumpSPEF / toSPEF
 * (src/solnoutclass.hpp:1972-2091, 6008-6030), an IEEE 1481-1998 SPEF file
 * with one net.  G and C as g2p_ybus_from_param writes them (symmetrised
 * inside, as makeGSym/makeCSym do); elements below save_thresh times the
 * matrix total are left out (the reference's WRITE_THRESH is 1e-5).
 * port_names [nports] are the subcircuit pins; port_dirs [nports] 'I', 'O'
 * or 'B' (NULL: all 'B').  Host memory only; no GPU is used.  The SPEF
 * layout is this writer's own (the reference prints through Parser-SPEF). */
g2p_status g2p_write_xyce(const char *path, const char *design, int32_t nports, const char *const *port_names,
                          double freq0, const double *G, const double *C, double save_thresh);
g2p_status g2p_write_spef(const char *path, const char *design, int32_t nports, const char *const *port_names,
                          const char *port_dirs, const double *G, const double *C, double save_thresh);

#ifdef __cplusplus
}
#endif
#endif
