// The coarse tail of the AMG V-cycle in one cooperative launch.
//
// Below a few tens of thousands of rows a level's kernels are latency-bound:
// each smoother step, residual, restriction and prolongation is a launch of a
// few microseconds of work behind several microseconds of launch and tail.
// k_coarse_cycle runs every level from the first small one down to the
// coarsest and back up in one persistent launch, with a grid-wide barrier
// between dependent phases instead of a launch.  The arithmetic is the
// V-cycle's (Chebyshev pre- and post-smoothing with the levels' own
// coefficients, residual, aggregate restriction, dense coarsest apply or
// smoothing, smoothed prolongation); the two Chebyshev iterates ping-pong
// between a level's x and t0 vectors, so a step needs one barrier.
//
// Two launch forms (G2P_FUSE=1 or 2; unset: the cluster form for blocks of
// at most 8 right-hand sides whose tail levels have no long rows):
// * grid: a cooperative launch over every SM, levels of up to kFuseRows
//   rows.  The barrier is an arrival counter with a bounded spin.  A block
//   that waits too long sets an abandon flag and returns, and every other
//   block returns at its next barrier; the flag is sticky, and the solver,
//   which checks it once per solve, then repeats that solve with the
//   launch-per-kernel V-cycle.
// * cluster: one thread-block cluster (16 CTAs where the part allows it,
//   else 8), levels of up to kClusterRows rows.  The barrier is the
//   hardware cluster barrier (barrier.cluster arrive.release /
//   wait.acquire): the cluster's CTAs are co-scheduled, so it needs no spin
//   and cannot give up, and it costs a fraction of a grid-wide barrier over
//   two dies.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "primitives.cuh"
#include "solver.h"

namespace g2p {

namespace {

constexpr int kFuseThreads = 512;
constexpr int kFuseLongRow = 64;       // longer rows take a warp
constexpr int kFuseSpin = 1 << 22;     // polls of >= 32 ns before a block gives up
constexpr int kFuseTraceLen = 512;     // phase time stamps kept by G2P_FUSE_TRACE
constexpr int64_t kClusterRows = 16384; // largest level of the cluster form (G2P_FUSE_ROWS overrides)

template <class T>
struct FuseLevel {
    int64_t n;
    const int64_t *ptr;
    const int32_t *col;
    const T *val;
    const T *dinv;
    T *b, *x, *t, *d;
    // members of the next level's rows (restriction) and the prolongation
    // from the next level
    const int64_t *rptr;
    const int32_t *rmem;
    const int64_t *pptr;
    const int32_t *pcol;
    const T *pval;
    // rows longer than kLongRow: those of at most kHugeRow entries take a
    // warp each; longer ones are split into chunks of kLongChunk entries
    // (one warp each, partial sums in `partial`), whose sums a second stage
    // adds in chunk order
    const int32_t *lrows;        // [nlong] all long rows
    int64_t nlong;
    const int32_t *mid;          // [nmid] rows of at most kHugeRow entries
    int64_t nmid;
    const int32_t *crow;         // [nchunk] index into lrows
    const int64_t *cbeg;         // [nchunk] first entry of the chunk
    const int64_t *rcp;          // [nlong + 1] chunks of each long row
    int64_t nchunk;
    double *partial;             // [nchunk * kMaxRhs]
    int deg;                     // Chebyshev degree of this level's smoother
    double inv_theta;
    double c1[kFuseMaxDeg], c2[kFuseMaxDeg];
};

enum { kResid = 0, kFirstAdd = 1, kStep = 2 };

// bar[0]: arrivals of this launch; bar[1]: this launch gave up; bar[2]:
// sticky "some launch gave up" for the solver.
__device__ __forceinline__ bool grid_sync(unsigned *bar, unsigned &phase, int spin_limit,
                                          unsigned long long *trace = nullptr) {
    __shared__ int quit;
    __syncthreads();
    if (trace && blockIdx.x == 0 && threadIdx.x == 0 && phase < kFuseTraceLen) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        trace[phase] = t;
    }
    ++phase;
    if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(&bar[0], 1u);
        const unsigned target = phase * gridDim.x;
        int q = 0, it = 0;
        while (*(volatile unsigned *)&bar[0] < target) {
            if (*(volatile unsigned *)&bar[1] || ++it > spin_limit) {
                atomicExch(&bar[1], 1u);
                atomicExch(&bar[2], 1u);
                q = 1;
                break;
            }
            __nanosleep(32);
        }
        __threadfence();
        quit = q;
    }
    __syncthreads();
    return quit == 0;
}

// Barrier of every thread of the cluster (the whole grid in the cluster
// form), with the memory ordering of a release/acquire pair at cluster scope.
__device__ __forceinline__ bool cluster_sync(unsigned &phase, unsigned long long *trace) {
    if (trace && blockIdx.x == 0 && threadIdx.x == 0 && phase < kFuseTraceLen) {
        unsigned long long t;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        trace[phase] = t;
    }
    ++phase;
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
    return true;
}

template <class T>
__device__ __forceinline__ void finish_row(int kind, const FuseLevel<T> &L, int it, int64_t t, T dinv_i, T s,
                                           const T *X, T *Y) {
    const T res = L.b[t] - s;
    if (kind == kResid) {
        Y[t] = res;
        return;
    }
    T dd;
    if (kind == kFirstAdd) dd = (T)L.inv_theta * dinv_i * res;
    else dd = (T)L.c1[it] * L.d[t] + (T)L.c2[it] * dinv_i * res;
    L.d[t] = dd;
    Y[t] = X[t] + dd;
}

// One smoother or residual phase on level L: s = (A X)[i, r] for every row
// and right-hand side, then the row's update into Y (X is only read).
// Short rows take KG lanes each (one per right-hand side); rows of up to
// kHugeRow entries a warp; longer rows are split into chunks, a warp each,
// whose partial sums spmm_phase_long adds after a barrier.
template <class T, int KG>
__device__ __forceinline__ void warp_row_sums(const FuseLevel<T> &L, int64_t q0, int64_t q1, const T *X, int k,
                                              int lane, double (&acc)[KG]) {
#pragma unroll
    for (int c = 0; c < KG; c++) acc[c] = 0;
    for (int64_t q = q0 + lane; q < q1; q += 32) {
        const double a = (double)L.val[q];
        const T *xr = X + (int64_t)L.col[q] * k;
#pragma unroll
        for (int c = 0; c < KG; c++)
            if (c < k) acc[c] += a * (double)xr[c];
    }
#pragma unroll
    for (int c = 0; c < KG; c++) acc[c] = warp_sum(acc[c]);
}

// acc[c] += a * x[c] for the k (<= KG) right-hand sides of one row of X,
// with 16-byte loads when the row is KG wide and 16-byte aligned
template <class T, int KG>
__device__ __forceinline__ void axpy_row(T a, const T *xr, int k, T (&acc)[KG]) {
    constexpr int V = 16 / sizeof(T);
    if (KG % V == 0 && k == KG) {
#pragma unroll
        for (int c = 0; c < KG; c += V) {
            if constexpr (sizeof(T) == 4) {
                const float4 v = *reinterpret_cast<const float4 *>(xr + c);
                acc[c] += a * v.x; acc[c + 1] += a * v.y; acc[c + 2] += a * v.z; acc[c + 3] += a * v.w;
            } else {
                const double2 v = *reinterpret_cast<const double2 *>(xr + c);
                acc[c] += a * v.x; acc[c + 1] += a * v.y;
            }
        }
    } else {
#pragma unroll
        for (int c = 0; c < KG; c++)
            if (c < k) acc[c] += a * xr[c];
    }
}

template <class T, int KG>
__device__ void spmm_phase(int kind, const FuseLevel<T> &L, int it, const T *X, T *Y, int k, int64_t g0, int64_t ng,
                           int r, int64_t warp, int64_t nwarps, int lane) {
    const int64_t n = L.n;
    // short rows: kEs lanes per row, each over every kEs-th entry and all
    // right-hand sides; the kEs lanes then add their sums (xor tree) and
    // each finishes the right-hand sides c with c % kEs == its lane
    constexpr int kEs = 4;
    const int e = lane & (kEs - 1);
    const unsigned gmask = 0xFu << (lane & ~(kEs - 1));
    const int64_t slot = warp * (32 / kEs) + (lane >> 2), nslot = nwarps * (32 / kEs);
    for (int64_t i = slot; i < n; i += nslot) {
        const int64_t s0 = L.ptr[i], s1 = L.ptr[i + 1];
        if (s1 - s0 > kLongRow) continue;
        T acc[KG];
#pragma unroll
        for (int c = 0; c < KG; c++) acc[c] = 0;
        for (int64_t q = s0 + e; q < s1; q += kEs) axpy_row<T, KG>(L.val[q], X + (int64_t)L.col[q] * k, k, acc);
#pragma unroll
        for (int c = 0; c < KG; c++) {
            acc[c] += __shfl_xor_sync(gmask, acc[c], 1);
            acc[c] += __shfl_xor_sync(gmask, acc[c], 2);
        }
        const T di = L.dinv[i];
#pragma unroll
        for (int c = 0; c < KG; c++)
            if (c < k && (c & (kEs - 1)) == e) finish_row<T>(kind, L, it, i * k + c, di, acc[c], X, Y);
    }
    // mid rows: a warp each, complete
    for (int64_t w = warp; w < L.nmid; w += nwarps) {
        const int64_t i = L.mid[w];
        double acc[KG];
        warp_row_sums<T, KG>(L, L.ptr[i], L.ptr[i + 1], X, k, lane, acc);
        T mine = 0;
#pragma unroll
        for (int c = 0; c < KG; c++)
            if (c == lane) mine = (T)acc[c];
        if (lane < k) finish_row<T>(kind, L, it, i * k + lane, L.dinv[i], mine, X, Y);
    }
    // chunks of the longest rows: a warp each, partial sums only
    for (int64_t c = warp; c < L.nchunk; c += nwarps) {
        const int64_t i = L.lrows[L.crow[c]];
        const int64_t q0 = L.cbeg[c], q1 = min(q0 + (int64_t)kLongChunk, L.ptr[i + 1]);
        double acc[KG];
        warp_row_sums<T, KG>(L, q0, q1, X, k, lane, acc);
#pragma unroll
        for (int cc = 0; cc < KG; cc++)
            if (cc == lane && lane < k) L.partial[c * kMaxRhs + lane] = acc[cc];
    }
}

// Second stage of a phase on a level with chunked rows: each such row's
// chunk partials added in chunk order, then the row's update.
template <class T, int KG>
__device__ void spmm_phase_long(int kind, const FuseLevel<T> &L, int it, const T *X, T *Y, int k, int64_t g0,
                                int64_t ng, int r) {
    for (int64_t l = g0; l < L.nlong; l += ng) {
        const int64_t c0 = L.rcp[l], c1 = L.rcp[l + 1];
        if (c1 == c0 || r >= k) continue;
        double s = 0;
        for (int64_t c = c0; c < c1; c++) s += __ldcg(L.partial + c * kMaxRhs + r);
        const int64_t i = L.lrows[l];
        finish_row<T>(kind, L, it, i * k + r, L.dinv[i], (T)s, X, Y);
    }
}

template <class T, int KG, bool CL>
__global__ void __launch_bounds__(kFuseThreads, 1) k_coarse_cycle(const FuseLevel<T> *__restrict__ lv, int nlev,
                                                               const double *__restrict__ cinv, int k, unsigned *bar,
                                                               int spin_limit, unsigned long long *trace) {
    const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nthreads = (int64_t)gridDim.x * blockDim.x;
    const int r = (int)(tid & (KG - 1));
    const int64_t g0 = tid / KG, ng = nthreads / KG;
    const int lane = threadIdx.x & 31;
    const int64_t warp = tid >> 5, nwarps = nthreads >> 5;
    unsigned phase = 0;
    T *cur[kFuseMaxLevels];
    auto sync = [&]() {
        if constexpr (CL) return cluster_sync(phase, trace);
        else return grid_sync(bar, phase, spin_limit, trace);
    };
    // a whole SpMM phase: rows, mid rows and chunks; then the chunked rows
    // after a barrier when the level has any
    auto spmm = [&](int kind, const FuseLevel<T> &L, int it, const T *X, T *Y) {
        spmm_phase<T, KG>(kind, L, it, X, Y, k, g0, ng, r, warp, nwarps, lane);
        if (L.nchunk == 0) return true;
        if (!sync()) return false;
        spmm_phase_long<T, KG>(kind, L, it, X, Y, k, g0, ng, r);
        return true;
    };
    // down: pre-smoothing from a zero guess, residual, restriction
    for (int l = 0; l + 1 < nlev; l++) {
        const FuseLevel<T> &L = lv[l];
        T *X = L.t, *Y = L.x;   // an odd number of swaps leaves the result in x
        if (l == 0) {           // coarser levels take this step with their restriction
            for (int64_t i = g0; i < L.n; i += ng) {
                if (r >= k) continue;
                const int64_t t = i * k + r;
                const T dd = (T)L.inv_theta * L.dinv[i] * L.b[t];
                L.d[t] = dd;
                X[t] = dd;
            }
            if (!sync()) return;
        }
        for (int it = 1; it < L.deg; it++) {
            if (!spmm(kStep, L, it, X, Y)) return;
            T *tmp = X; X = Y; Y = tmp;
            if (!sync()) return;
        }
        cur[l] = X;
        if (!spmm(kResid, L, 0, X, Y)) return;
        if (!sync()) return;
        // restriction, and the coarser level's first smoothing step from a
        // zero guess (row by row: d = x = D^-1 b / theta, x in its t vector)
        const FuseLevel<T> &C = lv[l + 1];
        const bool first = l + 2 < nlev || !cinv;
        for (int64_t I = g0; I < C.n; I += ng) {
            if (r >= k) continue;
            T acc = 0;
            for (int64_t m = L.rptr[I]; m < L.rptr[I + 1]; m++) acc += Y[(int64_t)L.rmem[m] * k + r];
            const int64_t t = I * k + r;
            C.b[t] = acc;
            if (first) {
                const T dd = (T)C.inv_theta * C.dinv[I] * acc;
                C.d[t] = dd;
                C.t[t] = dd;
            }
        }
        if (!sync()) return;
    }
    // coarsest: dense inverse or Chebyshev smoothing
    {
        const FuseLevel<T> &L = lv[nlev - 1];
        if (cinv) {
            // a warp per row: lane (jj, rr) takes columns jj, jj + 32 / KG, ...
            // for right-hand side rr, so each load instruction reads 32 / KG
            // whole rows of b; FP64 sums in four chains, then a fixed tree
            const int64_t n = L.n;
            constexpr int JS = 32 / KG;
            const int jj = lane / KG, rr = lane % KG;
            for (int64_t i = warp; i < n; i += nwarps) {
                const double *a = cinv + i * n;
                double acc[4] = {0, 0, 0, 0};
                if (rr < k) {
                    int64_t j = jj;
                    for (; j + 3 * JS < n; j += 4 * JS) {
#pragma unroll
                        for (int u = 0; u < 4; u++) acc[u] += a[j + u * JS] * (double)L.b[(j + u * JS) * k + rr];
                    }
                    for (; j < n; j += JS) acc[0] += a[j] * (double)L.b[j * k + rr];
                }
                double v = (acc[0] + acc[1]) + (acc[2] + acc[3]);
#pragma unroll
                for (int o = KG; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                if (jj == 0 && rr < k) L.x[i * k + rr] = (T)v;
            }
        } else {
            T *X = L.t, *Y = L.x;   // the first step came with the restriction
            for (int sweep = 0; sweep < 5; sweep++) {
                for (int it = sweep == 0 ? 1 : 0; it < L.deg; it++) {
                    if (!sync()) return;
                    if (!spmm(it == 0 ? kFirstAdd : kStep, L, it, X, Y)) return;
                    T *tmp = X; X = Y; Y = tmp;
                }
            }
        }
        if (!sync()) return;
    }
    // up: prolongation of the coarser level's result, post-smoothing
    for (int l = nlev - 2; l >= 0; l--) {
        const FuseLevel<T> &L = lv[l];
        const T *xc = lv[l + 1].x;
        T *X = cur[l], *Y = X == L.x ? L.t : L.x;
        for (int64_t i = g0; i < L.n; i += ng) {
            if (r >= k) continue;
            T acc = 0;
            for (int64_t q = L.pptr[i]; q < L.pptr[i + 1]; q++) acc += L.pval[q] * xc[(int64_t)L.pcol[q] * k + r];
            X[i * k + r] += acc;
        }
        for (int it = 0; it < L.deg; it++) {
            if (!sync()) return;
            if (!spmm(it == 0 ? kFirstAdd : kStep, L, it, X, Y)) return;
            T *tmp = X; X = Y; Y = tmp;
        }
        if (l > 0 && !sync()) return;
    }
    if (trace) sync();
}

// Chebyshev coefficients of the smoother on a level, as chebyshev() in
// solver.cu computes them: interval [ratio lmax, upper lmax], first step
// d = x = D^-1 b / theta, then d = c1 d + c2 D^-1 (b - A x).
template <class T>
void cheb_coefficients(FuseLevel<T> &f, double lmax_est, int deg, double ratio, double upper) {
    const double lmax = lmax_est * upper, lmin = lmax_est * ratio;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
    const double sigma = theta / delta;
    double rho = 1.0 / sigma;
    f.deg = deg;
    f.inv_theta = 1.0 / theta;
    for (int it = 0; it < kFuseMaxDeg; it++) f.c1[it] = f.c2[it] = 0;
    for (int it = 1; it < deg; it++) {
        const double rn = 1.0 / (2.0 * sigma - rho);
        f.c1[it] = rn * rho;
        f.c2[it] = 2.0 * rn / delta;
        rho = rn;
    }
}

template <class T>
using CoarseKernel = void (*)(const FuseLevel<T> *, int, const double *, int, unsigned *, int, unsigned long long *);

template <class T, bool CL>
CoarseKernel<T> coarse_kernel_of(int kg) {
    switch (kg) {
        case 1: return k_coarse_cycle<T, 1, CL>;
        case 2: return k_coarse_cycle<T, 2, CL>;
        case 4: return k_coarse_cycle<T, 4, CL>;
        case 8: return k_coarse_cycle<T, 8, CL>;
        case 16: return k_coarse_cycle<T, 16, CL>;
        default: return k_coarse_cycle<T, 32, CL>;
    }
}
template <class T>
CoarseKernel<T> coarse_kernel(int kg, bool cluster) {
    return cluster ? coarse_kernel_of<T, true>(kg) : coarse_kernel_of<T, false>(kg);
}

// G2P_FUSE: 0 = off, 1 = grid form, 2 = cluster form; unset = the cluster
// form where its levels have no long rows (-1)
int fuse_mode() {
    const char *e = getenv("G2P_FUSE");
    if (!e) return -1;
    const int m = atoi(e);
    return m == 1 || m == 2 ? m : 0;
}

}  // namespace

// The first level of the fused tail for k right-hand sides, or -1: the
// first level of at most kFuseRows (grid form) or kClusterRows (cluster
// form) rows, if at least one level lies below it.
template <class T>
int coarse_fuse_level(const Hierarchy<T> &H, int k) {
    if (k < 1 || k > 32 || H.lv.size() < 3) return -1;
    // the grid form measured slower than the launch-per-kernel cycle
    // replayed from CUDA graphs on the workloads here (a comparison switch)
    const int mode = fuse_mode();
    if (mode == 0 || H.fuse_off) return -1;
    int64_t rows = mode == 1 ? kFuseRows : kClusterRows;
    if (const char *r = getenv("G2P_FUSE_ROWS")) rows = std::max<int64_t>(1, atoll(r));
    const int nlev = (int)H.lv.size();
    for (int l = 1; l < nlev - 1; l++)
        if (H.lv[l].n <= rows) {
            if (nlev - l > kFuseMaxLevels) return -1;
            if (mode == -1) {
                // by default only for blocks of at most 8 right-hand sides and
                // where no fused level has long rows (measured: faster for Ac
                // on c2 and c1; slower at 32 right-hand sides (c3) and where
                // conductor rows need the whole GPU (Ad))
                if (k > 8) return -1;
                for (int q = l; q < nlev; q++)
                    if (H.lv[q].lr.n > 0) return -1;
            }
            return l;
        }
    return -1;
}

template <class T>
g2p_status coarse_prepare(Hierarchy<T> &H, const SolverConfig &cfg, int k, cudaStream_t s) {
    const int lc = coarse_fuse_level(H, k);
    H.fuse_from = -1;
    if (lc < 0) return G2P_OK;
    const int mode = fuse_mode();
    const std::vector<double> key = {(double)k, (double)H.kcap, (double)cfg.degree, cfg.cheb_ratio, cfg.cheb_upper,
                                     (double)lc, (double)mode};
    if (H.fuse_tab && H.fuse_key == key) {
        H.fuse_from = lc;
        return G2P_OK;
    }
    const int nlev = (int)H.lv.size();
    std::vector<FuseLevel<T>> tab(nlev - lc);
    for (int l = lc; l < nlev; l++) {
        Level<T> &L = H.lv[l];
        FuseLevel<T> &f = tab[l - lc];
        f.n = L.n;
        f.ptr = L.A.ptr; f.col = L.A.col; f.val = L.A.val;
        f.dinv = L.dinv;
        f.b = L.b; f.x = L.x; f.t = L.t0; f.d = L.d;
        const bool last = l == nlev - 1;
        f.rptr = last ? nullptr : L.rptr;
        f.rmem = last ? nullptr : L.rmem;
        f.pptr = last ? nullptr : L.P.ptr;
        f.pcol = last ? nullptr : L.P.col;
        f.pval = last ? nullptr : L.P.val;
        f.lrows = L.lr.rows;
        f.nlong = L.lr.n;
        f.mid = L.lr.mid;
        f.nmid = L.lr.nmid;
        f.crow = L.lr.crow;
        f.cbeg = L.lr.cbeg;
        f.rcp = L.lr.rcp;
        f.nchunk = L.lr.nchunk;
        f.partial = L.lr.partial;
        const int deg = last && !H.cinv ? 4 : cfg.degree;
        if (deg < 1 || deg > kFuseMaxDeg) return G2P_OK;
        cheb_coefficients(f, L.lmax, deg, cfg.cheb_ratio, cfg.cheb_upper);
    }
    if (!H.fuse_tab) {
        G2P_CUDA(cudaMalloc(&H.fuse_tab, sizeof(FuseLevel<T>) * kFuseMaxLevels));
        G2P_CUDA(cudaMalloc(&H.fuse_bar, sizeof(unsigned) * 4));
        G2P_CUDA(cudaMemsetAsync(H.fuse_bar, 0, sizeof(unsigned) * 4, s));
        if (getenv("G2P_FUSE_TRACE")) {
            G2P_CUDA(cudaMalloc(&H.fuse_trace, sizeof(unsigned long long) * kFuseTraceLen));
            G2P_CUDA(cudaMemsetAsync(H.fuse_trace, 0, sizeof(unsigned long long) * kFuseTraceLen, s));
        }
    }
    if (getenv("G2P_FUSE_TRACE"))
        for (int l = lc; l < nlev; l++)
            fprintf(stderr, "[g2p fuse] level %d: n=%lld nnz=%lld long=%lld mid=%lld chunks=%lld deg=%d%s\n", l,
                    (long long)H.lv[l].n, (long long)H.lv[l].A.nnz, (long long)H.lv[l].lr.n,
                    (long long)H.lv[l].lr.nmid, (long long)H.lv[l].lr.nchunk, tab[l - lc].deg,
                    l == nlev - 1 ? (H.cinv ? " (dense inverse)" : " (smoothed)") : "");
    G2P_CUDA(cudaMemcpyAsync(H.fuse_tab, tab.data(), sizeof(FuseLevel<T>) * tab.size(), cudaMemcpyHostToDevice, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    if (mode != 1) {
        // the largest cluster of these blocks that the part can place: 16
        // (non-portable) or 8
        const CoarseKernel<T> kfn = coarse_kernel<T>(pow2_ge(k), true);
        H.fuse_cluster = 0;
        for (int c : {16, 8}) {
            if (c > 8 && cudaFuncSetAttribute((const void *)kfn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                             cudaSuccess) {
                cudaGetLastError();
                continue;
            }
            cudaLaunchConfig_t lc_cfg = {};
            lc_cfg.gridDim = dim3((unsigned)c);
            lc_cfg.blockDim = dim3(kFuseThreads);
            cudaLaunchAttribute at;
            at.id = cudaLaunchAttributeClusterDimension;
            at.val.clusterDim.x = (unsigned)c;
            at.val.clusterDim.y = 1;
            at.val.clusterDim.z = 1;
            lc_cfg.attrs = &at;
            lc_cfg.numAttrs = 1;
            int nclusters = 0;
            if (cudaOccupancyMaxActiveClusters(&nclusters, (const void *)kfn, &lc_cfg) == cudaSuccess &&
                nclusters > 0) {
                H.fuse_cluster = c;
                break;
            }
            cudaGetLastError();
        }
        if (H.fuse_cluster == 0) return G2P_OK;
        H.fuse_blocks = H.fuse_cluster;
    } else {
        int dev = 0, per_sm = 0;
        G2P_CUDA(cudaGetDevice(&dev));
        G2P_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, coarse_kernel<T>(pow2_ge(k), false),
                                                               kFuseThreads, 0));
        int nsm = kSMs;
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        H.fuse_blocks = std::min(per_sm, 1) * nsm;
        H.fuse_cluster = 0;
        if (H.fuse_blocks < 1) return G2P_OK;
    }
    H.fuse_key = key;
    H.fuse_from = lc;
    return G2P_OK;
}

template <class T>
void coarse_cycle(Hierarchy<T> &H, int k, cudaStream_t s) {
    const int nlev = (int)H.lv.size() - H.fuse_from;
    int spin = kFuseSpin;
    if (const char *e = getenv("G2P_FUSE_SPIN_LIMIT")) spin = std::max(1, atoi(e));
    // arrivals and this launch's abandon flag start at zero; the sticky flag stays
    cudaMemsetAsync(H.fuse_bar, 0, sizeof(unsigned) * 2, s);
    const FuseLevel<T> *tab = static_cast<const FuseLevel<T> *>(H.fuse_tab);
    const double *cinv = H.cinv;
    unsigned *bar = H.fuse_bar;
    // G2P_FUSE_TRACE: block 0 stamps the global timer at every barrier
    unsigned long long *trace = getenv("G2P_FUSE_TRACE") ? H.fuse_trace : nullptr;
    void *args[] = {&tab, (void *)&nlev, &cinv, &k, &bar, &spin, &trace};
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)H.fuse_blocks);
    cfg.blockDim = dim3(kFuseThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr;
    const bool cluster = H.fuse_cluster > 0;
    if (cluster) {
        attr.id = cudaLaunchAttributeClusterDimension;
        attr.val.clusterDim.x = (unsigned)H.fuse_cluster;
        attr.val.clusterDim.y = 1;
        attr.val.clusterDim.z = 1;
    } else {
        attr.id = cudaLaunchAttributeCooperative;
        attr.val.cooperative = 1;
    }
    cfg.attrs = &attr;
    cfg.numAttrs = 1;
    g2p::kbegin(cluster ? "k_coarse_cycle<cluster>" : "k_coarse_cycle", s);
    if (cudaLaunchKernelExC(&cfg, (const void *)coarse_kernel<T>(pow2_ge(k), cluster), args) != cudaSuccess) {
        cudaGetLastError();
        H.fuse_failed = true;    // reported as a give-up: the solve is repeated unfused
    }
    g2p::kend(s);
}

template <class T>
g2p_status coarse_gave_up(Hierarchy<T> &H, cudaStream_t s, bool *gave_up) {
    *gave_up = false;
    if (!H.fuse_bar) return G2P_OK;
    if (H.fuse_trace && getenv("G2P_FUSE_TRACE")) {
        std::vector<unsigned long long> t(kFuseTraceLen);
        G2P_CUDA(cudaMemcpyAsync(t.data(), H.fuse_trace, sizeof(unsigned long long) * kFuseTraceLen,
                                 cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        fprintf(stderr, "[g2p fuse] phase durations of the last launch (us):");
        for (int i = 1; i < kFuseTraceLen && t[i] > t[i - 1]; i++) fprintf(stderr, " %.1f", (t[i] - t[i - 1]) * 1e-3);
        int last = 0;
        while (last + 1 < kFuseTraceLen && t[last + 1] > t[last]) last++;
        fprintf(stderr, "\n[g2p fuse] total %.1f us over %d barriers\n", (t[last] - t[0]) * 1e-3, last);
    }
    unsigned v = 0;
    G2P_CUDA(cudaMemcpyAsync(&v, H.fuse_bar + 2, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    if (v || H.fuse_failed) {
        *gave_up = true;
        H.fuse_off = true;
        H.fuse_failed = false;
        G2P_CUDA(cudaMemsetAsync(H.fuse_bar, 0, sizeof(unsigned) * 4, s));
    }
    return G2P_OK;
}

template int coarse_fuse_level<float>(const Hierarchy<float> &, int);
template int coarse_fuse_level<double>(const Hierarchy<double> &, int);
template g2p_status coarse_prepare<float>(Hierarchy<float> &, const SolverConfig &, int, cudaStream_t);
template g2p_status coarse_prepare<double>(Hierarchy<double> &, const SolverConfig &, int, cudaStream_t);
template void coarse_cycle<float>(Hierarchy<float> &, int, cudaStream_t);
template void coarse_cycle<double>(Hierarchy<double> &, int, cudaStream_t);
template g2p_status coarse_gave_up<float>(Hierarchy<float> &, cudaStream_t, bool *);
template g2p_status coarse_gave_up<double>(Hierarchy<double> &, cudaStream_t, bool *);

}  // namespace g2p
