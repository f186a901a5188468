// Device AMG-preconditioned flexible GMRES: the hypreSolve replacement.
#pragma once
#include <vector>
#include "internal.h"

namespace g2p {

constexpr int kLongRow = 64;
constexpr int kLongChunk = 512;     // entries per block in the long-row kernel
constexpr int kHugeRow = 256;       // rows above this are split into chunks; shorter long rows get a warp
constexpr int kMaxRhs = 256;

// Rows longer than kLongRow: the lumped conductor potentials of Ad and the
// wide rows of coarse Galerkin operators.  Rows of up to kHugeRow entries
// are listed in mid (one warp each); longer ones are split into chunks of
// kLongChunk entries (one block each).
struct LongRows {
    int32_t *rows = nullptr;     // [n] row ids
    int64_t n = 0;
    int32_t *mid = nullptr;      // [nmid] row ids of rows with at most kHugeRow entries
    int64_t nmid = 0;
    int32_t *crow = nullptr;     // [nchunk] index into rows
    int64_t *cbeg = nullptr;     // [nchunk] first entry
    int64_t *rcp = nullptr;      // [n+1] chunks of each long row
    int64_t nchunk = 0;
    double *partial = nullptr;   // [nchunk * kMaxRhs]
    int32_t *done = nullptr;     // [n] chunks finished per row; zero between launches
    void release(cudaStream_t s) {
        dfree(rows, s); dfree(crow, s); dfree(cbeg, s); dfree(rcp, s); dfree(partial, s); dfree(done, s);
        dfree(mid, s);
        n = nchunk = nmid = 0;
    }
};

// Multi-RHS vectors are row-interleaved: x[i * k + r].
template <class T>
struct Level {
    int64_t n = 0, nc = 0;
    Csr<T> A;                   // operator in working precision
    LongRows lr;
    T *dinv = nullptr;          // 1 / a_ii
    double lmax = 2.0;          // spectral radius estimate of D^-1 A
    int32_t *agg = nullptr;     // aggregate of each row (-1: none)
    Csr<T> P;                   // smoothed prolongation (n x nc)
    int64_t *rptr = nullptr;    // aggregate -> members (ascending)
    int32_t *rmem = nullptr;
    T *x = nullptr, *b = nullptr, *t0 = nullptr, *t1 = nullptr, *d = nullptr;
};

struct SolverConfig {
    int restart = 20;
    int maxit = 300;
    double rtol = 1e-10;
    int degree = 2;
    int coarse_size = 256;
    double strength = 0.04;
    int max_levels = 20;
    double cheb_ratio = 0.15;    // lower Chebyshev bound = ratio * lmax
    double cheb_upper = 1.05;    // upper Chebyshev bound = upper * lmax (lmax: Gershgorin)
    double psmooth = 4.0 / 3.0;  // prolongation smoothing weight = psmooth / lmax
    bool reorth = true;
    bool use_graphs = false;     // replay each Arnoldi step from a CUDA graph
    bool block = false;          // the k right-hand sides share one block Krylov space
};

// The fused coarse tail of the V-cycle (coarse.cu): levels of at most
// kFuseRows rows, down to the coarsest, in one cooperative launch.
constexpr int kFuseRows = 65536;
constexpr int kFuseMaxLevels = 24;
constexpr int kFuseMaxDeg = 8;

template <class T>
struct Hierarchy {
    std::vector<Level<T>> lv;
    double *cinv = nullptr;     // coarsest inverse (FP64, row-major)
    int64_t nc = 0;
    int kcap = 0;               // RHS capacity of the work vectors
    // fused coarse tail: first fused level (-1: none), the device table of
    // its levels, barrier words, grid size; fuse_off after a give-up
    int fuse_from = -1;
    void *fuse_tab = nullptr;
    unsigned *fuse_bar = nullptr;
    unsigned long long *fuse_trace = nullptr;   // G2P_FUSE_TRACE time stamps
    int fuse_blocks = 0;
    int fuse_cluster = 0;       // cluster form: CTAs of the one cluster (grid = cluster)
    bool fuse_off = false;
    bool fuse_failed = false;   // a fused launch could not be issued
    std::vector<double> fuse_key;
    void release(cudaStream_t s);
};

// First level of the fused tail for k right-hand sides, or -1 (the tail
// needs at least two levels and k <= 32; by default the cluster form for
// k <= 8 where none of its levels has long rows; G2P_FUSE=0/1/2: off / grid
// / cluster).
template <class T>
int coarse_fuse_level(const Hierarchy<T> &H, int k);
// Builds the device table of the fused levels for k right-hand sides (call
// outside stream capture; sets H.fuse_from, or leaves it -1).
template <class T>
g2p_status coarse_prepare(Hierarchy<T> &H, const SolverConfig &cfg, int k, cudaStream_t s);
// The V-cycle from level H.fuse_from down and up again, on that level's own
// b (in) and x (out).
template <class T>
void coarse_cycle(Hierarchy<T> &H, int k, cudaStream_t s);
// Whether a fused launch gave up since the last check; if so the fused path
// is switched off for this hierarchy (synchronizes s).
template <class T>
g2p_status coarse_gave_up(Hierarchy<T> &H, cudaStream_t s, bool *gave_up);

// FP64 hierarchy built from A64 (device CSR); an FP32 copy can be derived.
g2p_status amg_setup(const Csr<double> &A, const SolverConfig &cfg, cudaStream_t s, int64_t *scan_work_holder,
                     Hierarchy<double> &H);
g2p_status amg_to_float(const Hierarchy<double> &H, cudaStream_t s, Hierarchy<float> &F);

template <class T>
struct Krylov {
    int64_t n = 0;
    int k = 0, m = 0;
    T *V = nullptr, *Z = nullptr, *w = nullptr, *r = nullptr;
    double *H = nullptr, *cs = nullptr, *sn = nullptr, *g = nullptr, *y = nullptr;
    double *beta = nullptr, *bnorm = nullptr, *partial = nullptr, *hcol = nullptr;
    double *sc = nullptr;       // (m + 1) x k norms of the unnormalised basis vectors
    double *h_est = nullptr;    // pinned host copy of residual estimates
    // Arnoldi step j as a CUDA graph (captured on its second use), valid for
    // the block width, operator and preconditioner in graph_key
    struct Step {
        cudaGraphExec_t exec = nullptr;
        int64_t launches = 0;
        bool seen = false, failed = false;
    };
    std::vector<Step> steps;
    std::vector<const void *> graph_key;
    // block iteration (block_krylov.cu): device scratch, Gram-Schmidt
    // partial sums, pinned host copies; sized for bk right-hand sides, bm steps
    double *bdev = nullptr, *bpart = nullptr, *bhost = nullptr;
    int bk = 0, bm = 0;
    void drop_graphs();
    void release(cudaStream_t s);
};

struct SolveReport {
    int iterations = 0;
    double rel_residual = 0.0;
    bool converged = false;
};

// An FP32 V-cycle used as the preconditioner of an FP64 FGMRES: the basis
// vector is rounded to FP32, cycled through H (the hierarchy of the operator
// scaled by a power of two, which FGMRES does not need undone), and the
// result widened back.  lr: long rows of the FP64 operator; in, out: n * k
// FP32 work vectors.
struct F32Precond {
    Hierarchy<float> *H = nullptr;
    const LongRows *lr = nullptr;
    float *in = nullptr, *out = nullptr;
};

// FGMRES(m) right-preconditioned by one V-cycle per iteration, for k right-
// hand sides at once.  x holds the initial guess on entry.  With pc (FP64
// only) the V-cycle runs in FP32 on pc->H and H is not used.  op_lr: the long
// rows of A (default: those of pc, or of H's level 0, which must then have
// A's pattern).
// With cfg.block (and no pc, k in {2, 4, 8, 16, 32}, b and x 16-byte
// aligned) the solve is block FGMRES (block_fgmres).
template <class T>
g2p_status fgmres(const Csr<T> &A, Hierarchy<T> &H, Krylov<T> &K, const T *b, T *x, int k, const SolverConfig &cfg,
                  const double *bnorm_override, cudaStream_t s, SolveReport &rep, const F32Precond *pc = nullptr,
                  const LongRows *op_lr = nullptr);

// Block FGMRES(m) (block_krylov.cu): the k right-hand sides share one block
// Krylov space (block Arnoldi with block Gram-Schmidt and Cholesky QR, one
// V-cycle of the k columns per step, block Givens least squares on the
// host).  Same arguments and report as fgmres without pc.
template <class T>
bool block_krylov_supported(int k, const T *b, const T *x);
template <class T>
g2p_status block_fgmres(const Csr<T> &A, Hierarchy<T> &H, Krylov<T> &K, const T *b, T *x, int k,
                        const SolverConfig &cfg, const double *bnorm_override, cudaStream_t s, SolveReport &rep,
                        const LongRows *op_lr = nullptr);
// One V-cycle of H from level 0 (x = M^-1 b) for k right-hand sides.
template <class T>
void precond_vcycle(Hierarchy<T> &H, const SolverConfig &cfg, int k, cudaStream_t s, const T *b, T *x);
// r = b - A x for k right-hand sides (FP64 or FP32).
template <class T>
void spmm_residual(const Csr<T> &A, const LongRows &lr, const T *x, T *r, int k, const T *b, cudaStream_t s);

template <class T>
g2p_status krylov_alloc(Krylov<T> &K, int64_t n, int k, int m, cudaStream_t s);
template <class T>
g2p_status hierarchy_reserve(Hierarchy<T> &H, int k, cudaStream_t s);

// y = A x for k interleaved right-hand sides (FP64 or FP32).
template <class T>
void spmm(const Csr<T> &A, const LongRows &lr, const T *x, T *y, int k, cudaStream_t s);
// r = b - A x (FP64)
void residual64(const Csr<double> &A, const LongRows &lr, const double *b, const double *x, double *r, int k,
                cudaStream_t s);
// per-column 2-norms of an n x k interleaved block into out[k] (device)
template <class T>
void colnorms(const T *x, int64_t n, int k, double *partial, double *out, cudaStream_t s);

template <class T>
g2p_status find_long_rows(const Csr<T> &A, LongRows &lr, cudaStream_t s);
g2p_status copy_long_rows(const LongRows &src, LongRows &dst, cudaStream_t s);
// Sliced-ELL copy of the rows of A with at most maxlen (<= 254) entries.
template <class T>
g2p_status sell_build(Csr<T> &A, cudaStream_t s, int64_t maxlen = kLongRow);
template <class T>
g2p_status sell_refill(Csr<T> &A, cudaStream_t s);

}  // namespace g2p

struct g2p_solver {
    cudaStream_t stream = nullptr;
    bool owns_stream = false;
    g2p::SolverConfig cfg;
    int precision = 0;
    int inner_maxit = 40;
    int inner_restart = 10;
    double inner_rtol = 3e-3;
    g2p::Csr<double> A;                 // original FP64 operator
    g2p::LongRows lr;
    double cscale = 1.0;                // mixed: power-of-two scale of the FP32 operator
    g2p::Hierarchy<double> H64;
    g2p::Hierarchy<float> H32;
    g2p::Krylov<double> K64;
    g2p::Krylov<float> K32;
    int kcap = 0;
    // work
    double *xb = nullptr, *bb = nullptr, *rb = nullptr;
    float *rf = nullptr, *df = nullptr;
    int64_t *scan_work = nullptr;
    double setup_ms = 0;
    int levels = 0;
    int64_t coarse_rows = 0;
    bool fp64_vcycle = false;           // the FP32 V-cycle did not precondition A: FP64 hierarchy built
};
