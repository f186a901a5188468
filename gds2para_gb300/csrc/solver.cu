// AMG setup and application, multi-RHS sparse kernels, batched FGMRES.
//
// Replaces hypreSolve (hypreSolve.cpp:9-283): the reference solves each
// system with HYPRE FlexGMRES(10) preconditioned by one BoomerAMG V-cycle
// and rebuilds the hierarchy on every call.  Here the hierarchy is built on
// the device once per matrix:
//   * strength graph |a_ij| >= theta sqrt(|a_ii a_jj|) (rows longer than a
//     level-relative limit -- the lumped conductor potentials of Ad -- stay
//     singleton aggregates),
//   * aggregation from a distance-2 maximal independent set computed with
//     hashed priorities (two max-propagation sweeps per round), neighbours
//     joining the strongest root, distance-2 nodes joining a neighbour's
//     aggregate,
//   * smoothed prolongation P = (I - w D^-1 A) T of the piecewise-constant
//     aggregate basis T (w = 4 / (3 rho), rho the Gershgorin radius of
//     D^-1 A; long rows keep T), restriction by aggregate sums T^T, and the
//     Petrov-Galerkin coarse operator T^T A P formed as (T^T A) P, each
//     product by expand / stable radix sort / ordered reduce,
//   * Chebyshev smoothing on D^-1 A (bounds from the Gershgorin radius),
//   * an explicit FP64 inverse on the coarsest level.
// All right-hand sides of a block advance together through FGMRES.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <atomic>
#include <vector>

#include "primitives.cuh"

#include "solver.h"

namespace g2p {

// ------------------------------------------------------------ sparse kernels

// y = A x (or b - A x) for rows up to kLongRow entries.  Block shape
// (kx, 256/kx): threadIdx.x is the right-hand side, threadIdx.y the row.
template <class T>
__global__ void __launch_bounds__(256) k_spmm(int64_t n, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                                              const T *__restrict__ val, const T *__restrict__ x, T *__restrict__ y,
                                              int k, const T *__restrict__ b) {
    const int r = threadIdx.x;
    if (r >= k) return;
    G2P_FOR_ROWS(i, n) {
        int64_t s0 = ptr[i], s1 = ptr[i + 1];
        if (s1 - s0 > kLongRow) continue;
        T acc = 0;
        int64_t q = s0;
        // four independent gathers in flight per step
        for (; q + 4 <= s1; q += 4) {
            int32_t c0 = col[q], c1 = col[q + 1], c2 = col[q + 2], c3 = col[q + 3];
            T v0 = val[q], v1 = val[q + 1], v2 = val[q + 2], v3 = val[q + 3];
            T x0 = x[(int64_t)c0 * k + r], x1 = x[(int64_t)c1 * k + r];
            T x2 = x[(int64_t)c2 * k + r], x3 = x[(int64_t)c3 * k + r];
            acc += v0 * x0 + v1 * x1 + v2 * x2 + v3 * x3;
        }
        for (; q < s1; q++) acc += val[q] * x[(int64_t)col[q] * k + r];
        int64_t t = i * k + r;
        y[t] = b ? b[t] - acc : acc;
    }
}

// ---- sliced-ELL SpMM: one row per thread group, V right-hand sides per
// thread loaded as 16- or 8-byte vectors; the slice layout makes the column
// and value loads of a warp contiguous.
template <class T, int V>
struct XVec {
    T v[V];
    __device__ __forceinline__ void load(const T *__restrict__ p) {
        if constexpr (V * sizeof(T) >= 16) {
            constexpr int W = 16 / sizeof(T);
#pragma unroll
            for (int u = 0; u < V; u += W) {
                if constexpr (sizeof(T) == 4) {
                    float4 t = __ldg(reinterpret_cast<const float4 *>(p + u));
                    v[u] = t.x; v[u + 1] = t.y; v[u + 2] = t.z; v[u + 3] = t.w;
                } else {
                    double2 t = __ldg(reinterpret_cast<const double2 *>(p + u));
                    v[u] = t.x; v[u + 1] = t.y;
                }
            }
        } else if constexpr (V * sizeof(T) == 8 && sizeof(T) == 4) {
            float2 t = __ldg(reinterpret_cast<const float2 *>(p));
            v[0] = t.x; v[1] = t.y;
        } else {
#pragma unroll
            for (int u = 0; u < V; u++) v[u] = __ldg(p + u);
        }
    }
    // ordinary (coherent) load, for an output read back by the same thread
    __device__ __forceinline__ void load_plain(const T *p) {
#pragma unroll
        for (int u = 0; u < V; u++) v[u] = p[u];
    }
    __device__ __forceinline__ void store(T *__restrict__ p) const {
        if constexpr (V * sizeof(T) >= 16) {
            constexpr int W = 16 / sizeof(T);
#pragma unroll
            for (int u = 0; u < V; u += W) {
                if constexpr (sizeof(T) == 4) *reinterpret_cast<float4 *>(p + u) = make_float4(v[u], v[u + 1], v[u + 2], v[u + 3]);
                else *reinterpret_cast<double2 *>(p + u) = make_double2(v[u], v[u + 1]);
            }
        } else if constexpr (V * sizeof(T) == 8 && sizeof(T) == 4) {
            *reinterpret_cast<float2 *>(p) = make_float2(v[0], v[1]);
        } else {
#pragma unroll
            for (int u = 0; u < V; u++) p[u] = v[u];
        }
    }
};

constexpr int kSellUnroll = 8;

// The operand combined with the product, loaded before the gathers so its
// latency overlaps them: b (y = b - acc), the old y (accum: y = y + acc), or
// nothing (y = acc).
template <class T, int V>
__device__ __forceinline__ void spmm_pre(XVec<T, V> &pre, const T *y, const T *b, bool accum) {
    if (accum) pre.load_plain(y);
    else if (b) pre.load(b);
}
template <class T, int V>
__device__ __forceinline__ void spmm_out(T *y, bool has_b, bool accum, const XVec<T, V> &pre, const T (&acc)[V]) {
    XVec<T, V> out;
#pragma unroll
    for (int q = 0; q < V; q++) out.v[q] = accum ? pre.v[q] + acc[q] : (has_b ? pre.v[q] - acc[q] : acc[q]);
    out.store(y);
}

// Sum over the ES entry-split lanes of one row (lanes tpr apart within a
// group of G = tpr * ES consecutive lanes), in a fixed tree order.
template <class T, int V, int ES>
__device__ __forceinline__ void es_reduce(T (&acc)[V], int tpr) {
    if constexpr (ES > 1) {
        const int G = tpr * ES;
        const int lane = threadIdx.x + threadIdx.y * blockDim.x;   // blockDim.x == G divides 32
        const unsigned mask = G >= 32 ? 0xffffffffu : (((1u << G) - 1u) << ((lane & 31) & ~(G - 1)));
#pragma unroll
        for (int q = 0; q < V; q++)
            for (int o = tpr; o < G; o <<= 1) acc[q] += __shfl_xor_sync(mask, acc[q], o);
    }
}

// y = A x (or b - A x) over the short rows.  Block (tpr * ES, 256 / (tpr *
// ES)): the tpr = k / V threads of a row each own V consecutive right-hand
// sides, and ES of them (ES > 1 for wide operators) split the row's entries
// (entry j to lane j % ES), so a row of w entries costs w / ES dependent
// gathers per thread instead of w.
template <class T, int V, int ES>
__global__ void __launch_bounds__(256) k_spmm_sell(int64_t n, const int64_t *__restrict__ sptr,
                                                   const int32_t *__restrict__ scol, const T *__restrict__ sval,
                                                   const uint8_t *__restrict__ rlen, const T *__restrict__ x,
                                                   T *__restrict__ y, int k, const T *__restrict__ b, bool accum) {
    const int tpr = blockDim.x / ES;
    const int part = threadIdx.x % tpr, e = threadIdx.x / tpr;
    const int xo = part * V;
    G2P_FOR_ROWS(i, n) {
        const int lr = rlen[i];
        const bool longrow = lr == kSellLong;
        const int len = longrow ? 0 : lr;
        const int64_t base = sptr[i >> 5] + (i & 31);
        const int64_t t = i * k + xo;
        XVec<T, V> pre;
        if (!longrow && e == 0) spmm_pre<T, V>(pre, y + t, b ? b + t : nullptr, accum);
        T acc[V];
#pragma unroll
        for (int u = 0; u < V; u++) acc[u] = 0;
        for (int j0 = e; j0 < len; j0 += ES * kSellUnroll) {
            // all gathers of the chunk are issued before the first use; past
            // the row's end they repeat its first column and are not added
            int32_t c[kSellUnroll];
            T a[kSellUnroll];
#pragma unroll
            for (int u = 0; u < kSellUnroll; u++) {
                const bool in = j0 + ES * u < len;
                c[u] = in ? __ldg(scol + base + 32 * (int64_t)(j0 + ES * u)) : c[0];
                a[u] = in ? __ldg(sval + base + 32 * (int64_t)(j0 + ES * u)) : T(0);
            }
            XVec<T, V> xv[kSellUnroll];
#pragma unroll
            for (int u = 0; u < kSellUnroll; u++) xv[u].load(x + (int64_t)c[u] * k + xo);
#pragma unroll
            for (int u = 0; u < kSellUnroll; u++)
                if (j0 + ES * u < len) {
#pragma unroll
                    for (int w = 0; w < V; w++) acc[w] += a[u] * xv[u].v[w];
                }
        }
        es_reduce<T, V, ES>(acc, tpr);
        if (longrow || e != 0) continue;
        spmm_out<T, V>(y + t, b != nullptr, accum, pre, acc);
    }
}

// Sliced ELL for wide rows (more than one chunk of kSellUnroll entries),
// chunk-pipelined: the next chunk's column and value loads are issued while
// the current chunk's x gathers are in flight, so a row of c chunks exposes
// c + 1 memory round trips instead of 2 c.  Same summation order as
// k_spmm_sell with ES = 1.
template <class T, int V>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 1) k_spmm_sell_pipe(int64_t n, const int64_t *__restrict__ sptr,
                                                        const int32_t *__restrict__ scol, const T *__restrict__ sval,
                                                        const uint8_t *__restrict__ rlen, const T *__restrict__ x,
                                                        T *__restrict__ y, int k, const T *__restrict__ b, bool accum) {
    const int xo = threadIdx.x * V;
    G2P_FOR_ROWS(i, n) {
        const int lr = rlen[i];
        if (lr == kSellLong) continue;
        const int len = lr;
        const int64_t base = sptr[i >> 5] + (i & 31);
        const int64_t t = i * k + xo;
        XVec<T, V> pre;
        spmm_pre<T, V>(pre, y + t, b ? b + t : nullptr, accum);
        T acc[V];
#pragma unroll
        for (int u = 0; u < V; u++) acc[u] = 0;
        int32_t c[kSellUnroll];
        T a[kSellUnroll];
        auto fetch = [&](int j0) {
#pragma unroll
            for (int u = 0; u < kSellUnroll; u++) {
                const bool in = j0 + u < len;
                c[u] = in ? __ldg(scol + base + 32 * (int64_t)(j0 + u)) : c[0];
                a[u] = in ? __ldg(sval + base + 32 * (int64_t)(j0 + u)) : T(0);
            }
        };
        if (len > 0) fetch(0);
        for (int j0 = 0; j0 < len; j0 += kSellUnroll) {
            XVec<T, V> xv[kSellUnroll];
#pragma unroll
            for (int u = 0; u < kSellUnroll; u++) xv[u].load(x + (int64_t)c[u] * k + xo);
            T av[kSellUnroll];
#pragma unroll
            for (int u = 0; u < kSellUnroll; u++) av[u] = (j0 + u < len) ? a[u] : T(0);
            if (j0 + kSellUnroll < len) fetch(j0 + kSellUnroll);
#pragma unroll
            for (int u = 0; u < kSellUnroll; u++)
                if (j0 + u < len) {
#pragma unroll
                    for (int w = 0; w < V; w++) acc[w] += av[u] * xv[u].v[w];
                }
        }
        spmm_out<T, V>(y + t, b != nullptr, accum, pre, acc);
    }
}

// The same product on the uniform-width layout: the slot of entry j of row i
// is 32 (ell_w (i / 32) + j) + i % 32, so the only dependent loads are the
// column and value, then x.  Padding slots add 0 x_i.  ES as in k_spmm_sell.
template <class T, int V, int ES>
__global__ void __launch_bounds__(256) k_spmm_ell(int64_t n, int w, const int32_t *__restrict__ scol,
                                                  const T *__restrict__ sval, const T *__restrict__ x,
                                                  T *__restrict__ y, int k, const T *__restrict__ b, bool accum) {
    const int tpr = blockDim.x / ES;
    const int part = threadIdx.x % tpr, e = threadIdx.x / tpr;
    const int xo = part * V;
    G2P_FOR_ROWS(i, n) {
        const int64_t base = 32 * (int64_t)w * (i >> 5) + (i & 31);
        const int64_t t = i * k + xo;
        XVec<T, V> pre;
        if (e == 0) spmm_pre<T, V>(pre, y + t, b ? b + t : nullptr, accum);
        T acc[V];
#pragma unroll
        for (int u = 0; u < V; u++) acc[u] = 0;
        for (int j0 = e; j0 < w; j0 += ES * kSellUnroll) {
            int32_t c[kSellUnroll];
            T a[kSellUnroll];
#pragma unroll
            for (int u = 0; u < kSellUnroll; u++) {
                const bool in = j0 + ES * u < w;
                c[u] = in ? __ldg(scol + base + 32 * (int64_t)(j0 + ES * u)) : c[0];
                a[u] = in ? __ldg(sval + base + 32 * (int64_t)(j0 + ES * u)) : T(0);
            }
            XVec<T, V> xv[kSellUnroll];
#pragma unroll
            for (int u = 0; u < kSellUnroll; u++) xv[u].load(x + (int64_t)c[u] * k + xo);
#pragma unroll
            for (int u = 0; u < kSellUnroll; u++)
#pragma unroll
                for (int q = 0; q < V; q++) acc[q] += a[u] * xv[u].v[q];
        }
        es_reduce<T, V, ES>(acc, tpr);
        if (e != 0) continue;
        spmm_out<T, V>(y + t, b != nullptr, accum, pre, acc);
    }
}

// Uniform layout of width w <= kSellUnroll, persistent and software
// pipelined: each thread walks row groups with a grid stride and issues the
// next group's column and value loads before the current group's x gathers,
// so one memory round trip per group is exposed instead of two.
template <class T, int V>
__global__ void __launch_bounds__(256) k_spmm_ell_pipe(int64_t n, int w, const int32_t *__restrict__ scol,
                                                       const T *__restrict__ sval, const T *__restrict__ x,
                                                       T *__restrict__ y, int k, const T *__restrict__ b,
                                                       bool accum) {
    const int xo = threadIdx.x * V;
    const int64_t stride = (int64_t)gridDim.x * blockDim.y;
    int64_t i = blockIdx.x * (int64_t)blockDim.y + threadIdx.y;
    int32_t c[kSellUnroll];
    T a[kSellUnroll];
    auto fetch = [&](int64_t r) {
        const int64_t base = 32 * (int64_t)w * (r >> 5) + (r & 31);
#pragma unroll
        for (int u = 0; u < kSellUnroll; u++) {
            const bool in = u < w;
            c[u] = in ? __ldg(scol + base + 32 * (int64_t)u) : c[0];
            a[u] = in ? __ldg(sval + base + 32 * (int64_t)u) : T(0);
        }
    };
    if (i < n) fetch(i);
    for (; i < n; i += stride) {
        XVec<T, V> xv[kSellUnroll];
#pragma unroll
        for (int u = 0; u < kSellUnroll; u++) xv[u].load(x + (int64_t)c[u] * k + xo);
        T av[kSellUnroll];
#pragma unroll
        for (int u = 0; u < kSellUnroll; u++) av[u] = a[u];
        const int64_t t = i * k + xo;
        XVec<T, V> pre;
        spmm_pre<T, V>(pre, y + t, b ? b + t : nullptr, accum);
        if (i + stride < n) fetch(i + stride);
        T acc[V];
#pragma unroll
        for (int q = 0; q < V; q++) acc[q] = 0;
#pragma unroll
        for (int u = 0; u < kSellUnroll; u++)
#pragma unroll
            for (int q = 0; q < V; q++) acc[q] += av[u] * xv[u].v[q];
        spmm_out<T, V>(y + t, b != nullptr, accum, pre, acc);
    }
}

// Padding of the uniform layout: value 0 in every slot a row does not use
// (and in all slots of long rows), with the row's own first column -- a
// valid column also for a rectangular P, and one whose x row the thread
// gathers anyway, so padding adds no traffic and no shared hot spot.  An
// empty row uses column min(i, m - 1).
template <class T>
__global__ void k_ell_pad(int64_t n, int64_t m, int w, const uint8_t *__restrict__ rlen, int32_t *__restrict__ scol,
                          T *__restrict__ sval) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int len = rlen[i] == kSellLong ? 0 : rlen[i];
        const int64_t base = 32 * (int64_t)w * (i >> 5) + (i & 31);
        const int32_t pc = len > 0 ? scol[base] : (int32_t)(i < m ? i : m - 1);
        for (int j = len; j < w; j++) {
            scol[base + 32 * (int64_t)j] = pc;
            sval[base + 32 * (int64_t)j] = T(0);
        }
    }
}

__global__ void k_width_max(const int64_t *width, int64_t nslice, unsigned long long *mx) {
    unsigned long long m = 0;
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nslice; s += (int64_t)gridDim.x * blockDim.x)
        m = max(m, (unsigned long long)width[s]);
    if (m) atomicMax(mx, m);
}

__global__ void k_ell_sptr(int64_t *sptr, int64_t nslice, int64_t stride) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s <= nslice; s += (int64_t)gridDim.x * blockDim.x)
        sptr[s] = stride * s;
}

// Slice widths (entries of the slice's longest short row) and row lengths.
__global__ void k_sell_width(int64_t n, const int64_t *__restrict__ ptr, int64_t nslice, int64_t maxlen,
                             int64_t *__restrict__ width, uint8_t *__restrict__ rlen) {
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < nslice; s += (int64_t)gridDim.x * blockDim.x) {
        int64_t w = 0;
        for (int64_t i = 32 * s; i < 32 * s + 32 && i < n; i++) {
            int64_t l = ptr[i + 1] - ptr[i];
            if (l > maxlen) { rlen[i] = kSellLong; continue; }
            rlen[i] = (uint8_t)l;
            w = l > w ? l : w;
        }
        width[s] = 32 * w;
    }
}

template <class T>
__global__ void k_sell_fill(int64_t n, const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                            const T *__restrict__ val, const uint8_t *__restrict__ rlen, const int64_t *__restrict__ sptr,
                            int32_t *__restrict__ scol, T *__restrict__ sval) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int len = rlen[i];
        if (len == kSellLong) continue;
        const int64_t base = sptr[i >> 5] + (i & 31), p0 = ptr[i];
        for (int j = 0; j < len; j++) {
            scol[base + 32 * (int64_t)j] = col[p0 + j];
            sval[base + 32 * (int64_t)j] = val[p0 + j];
        }
    }
}

// Long rows: one block per chunk of kLongChunk entries writes its partial
// sums for every right-hand side; the block that finishes a row's last
// chunk adds the row's partials in chunk order (deterministic) and writes y.
template <class T>
__global__ void __launch_bounds__(256) k_spmm_long(const int32_t *__restrict__ rows, const int32_t *__restrict__ crow,
                                                   const int64_t *__restrict__ cbeg, const int64_t *__restrict__ rcp,
                                                   const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                                                   const T *__restrict__ val, const T *__restrict__ x, int k,
                                                   double *partial, int32_t *done, T *__restrict__ y,
                                                   const T *__restrict__ b) {
    __shared__ double sm[256];
    __shared__ int last;
    const int r = threadIdx.x, ty = threadIdx.y, ny = blockDim.y;
    const int l = crow[blockIdx.x];
    const int64_t row = rows[l];
    const int64_t q0 = cbeg[blockIdx.x], q1 = min(q0 + (int64_t)kLongChunk, ptr[row + 1]);
    // eight independent gathers in flight per thread
    T a[8];
#pragma unroll
    for (int u = 0; u < 8; u++) a[u] = 0;
    if (r < k) {
        int64_t q = q0 + ty;
        for (; q + 7 * ny < q1; q += 8 * ny) {
            int32_t c[8];
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) { c[u] = col[q + u * ny]; v[u] = val[q + u * ny]; }
#pragma unroll
            for (int u = 0; u < 8; u++) a[u] += v[u] * x[(int64_t)c[u] * k + r];
        }
        for (; q < q1; q += ny) a[0] += val[q] * x[(int64_t)col[q] * k + r];
    }
    // the block's entry lanes (threadIdx.y) combine in a fixed tree: xor
    // shuffles inside a warp, then the warps' sums in order (an FP64 chain
    // over all lanes costs microseconds on this part)
    const int tid = ty * blockDim.x + r, lane = tid & 31, wi = tid >> 5, kxb = blockDim.x;
    double v = (double)(((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7])));
    for (int off = kxb; off < 32; off <<= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int nw = (int)((blockDim.x * blockDim.y + 31) >> 5);
    const int slots = kxb < 32 ? nw : ny;                   // warps, or rows of the block when kxb >= 32
    if (kxb < 32 ? lane < kxb : true) sm[(kxb < 32 ? wi : ty) * kxb + r] = v;
    __syncthreads();
    if (ty == 0 && r < k) {
        double s = 0;
        for (int t = 0; t < slots; t++) s += sm[t * kxb + r];
        partial[(int64_t)blockIdx.x * kMaxRhs + r] = s;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0 && ty == 0) {
        const int nch = (int)(rcp[l + 1] - rcp[l]);
        last = atomicAdd(&done[l], 1) == nch - 1;
        if (last) done[l] = 0;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the row's chunk partials: thread ty adds chunks ty, ty + ny, ... in
    // order, then the same fixed tree as above over the entry lanes
    double s = 0;
    if (r < k)
        for (int64_t c = rcp[l] + ty; c < rcp[l + 1]; c += ny) s += __ldcg(partial + c * kMaxRhs + r);
    for (int off = kxb; off < 32; off <<= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
    if (kxb < 32 ? lane < kxb : true) sm[(kxb < 32 ? wi : ty) * kxb + r] = s;
    __syncthreads();
    if (ty != 0 || r >= k) return;
    double t = 0;
    for (int q = 0; q < slots; q++) t += sm[q * kxb + r];
    const int64_t o = row * k + r;
    y[o] = b ? (T)((double)b[o] - t) : (T)t;
}

// Rows of kLongRow < length <= kHugeRow: one warp per row.  Lane = (entry
// lane e, right-hand side r): kx = min(32, pow2 >= k) lanes cover the
// right-hand sides (looping when k > 32), 32 / kx lanes stride over the
// entries; a fixed shuffle tree adds the entry lanes.
template <class T>
__global__ void __launch_bounds__(256) k_spmm_mid(int64_t nmid, const int32_t *__restrict__ mid,
                                                  const int64_t *__restrict__ ptr, const int32_t *__restrict__ col,
                                                  const T *__restrict__ val, const T *__restrict__ x, int k, int kx,
                                                  T *__restrict__ y, const T *__restrict__ b) {
    // one block per row: thread (e, r) with r = tid % kx the right-hand side
    // and e = tid / kx one of 256 / kx entry lanes; entry lanes combine by a
    // fixed xor tree inside each warp, then the warps' sums in warp order
    __shared__ T wsum[8][32];
    const int tid = threadIdx.x, lane = tid & 31, wi = tid >> 5;
    const int r = tid % kx, e = tid / kx, ey = 256 / kx;
    const int64_t row = mid[blockIdx.x];
    const int64_t q0 = ptr[row], q1 = ptr[row + 1];
    for (int r0 = 0; r0 < k; r0 += kx) {
        const int rr = r0 + r;
        const bool on = rr < k;
        T a[8];
#pragma unroll
        for (int u = 0; u < 8; u++) a[u] = 0;
        if (on) {
            int64_t q = q0 + e;
            for (; q + 7 * ey < q1; q += 8 * ey) {
                int32_t c[8];
                T v[8];
#pragma unroll
                for (int u = 0; u < 8; u++) { c[u] = col[q + u * ey]; v[u] = val[q + u * ey]; }
#pragma unroll
                for (int u = 0; u < 8; u++) a[u] += v[u] * x[(int64_t)c[u] * k + rr];
            }
            for (; q < q1; q += ey) a[0] += val[q] * x[(int64_t)col[q] * k + rr];
        }
        T acc = ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
        for (int off = kx; off < 32; off <<= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
        if (lane < kx) wsum[wi][lane] = acc;
        __syncthreads();
        if (tid < kx && on) {
            T t = 0;
            for (int w = 0; w < 8; w++) t += wsum[w][tid];
            const int64_t o = row * k + rr;
            y[o] = b ? b[o] - t : t;
        }
        __syncthreads();
    }
}

// Event timing of the sparse matrix-multi-vector kernel (the dominant
// kernel of the solves) with its algorithmic bytes, enabled between
// g2p_profile_begin and g2p_profile_end.
struct KernelProfile {
    bool on = false;
    std::vector<cudaEvent_t> ev;
    size_t used = 0;
    double bytes = 0;
    int64_t launches = 0;
    std::vector<double> launch_bytes;   // per launch, for the size buckets
    std::vector<char> launch_f64;       // per launch: FP64 operator
    std::vector<int64_t> launch_rows;   // per launch: operator rows
};
static KernelProfile g_prof;
static double g_bucket_ms[8], g_bucket_bytes[8];
static int64_t g_bucket_n[8];

static void prof_event(cudaStream_t s) {
    if (g_prof.used == g_prof.ev.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        g_prof.ev.push_back(e);
    }
    cudaEventRecord(g_prof.ev[g_prof.used++], s);
}

// Right-hand sides per thread of the sliced-ELL kernel for k columns: one
// 16-byte load where k allows, so the threads of a row cover whole sectors.
template <class T>
static int sell_vec(int k) {
    int v = (int)(16 / sizeof(T));
    while (v > 1 && k % v) v >>= 1;
    return v;
}

// G2P_ELL_PIPE=0 selects the one-group-per-block kernel (for comparisons).
static bool pipe_ok() {
    static const bool on = [] {
        const char *e = getenv("G2P_ELL_PIPE");
        return e ? atoi(e) != 0 : true;
    }();
    return on;
}

// Profile name of a sparse-product launch: kernel, precision and operator size
// class (fine >= 1M rows, mid >= 64k rows, small).
static const char *spmm_name(int kind, bool f64, int64_t n) {
    static const char *names[4][2][3] = {
        {{"k_spmm_sell<f32,fine>", "k_spmm_sell<f32,mid>", "k_spmm_sell<f32,small>"},
         {"k_spmm_sell<f64,fine>", "k_spmm_sell<f64,mid>", "k_spmm_sell<f64,small>"}},
        {{"k_spmm_ell<f32,fine>", "k_spmm_ell<f32,mid>", "k_spmm_ell<f32,small>"},
         {"k_spmm_ell<f64,fine>", "k_spmm_ell<f64,mid>", "k_spmm_ell<f64,small>"}},
        {{"k_spmm_ell_pipe<f32,fine>", "k_spmm_ell_pipe<f32,mid>", "k_spmm_ell_pipe<f32,small>"},
         {"k_spmm_ell_pipe<f64,fine>", "k_spmm_ell_pipe<f64,mid>", "k_spmm_ell_pipe<f64,small>"}},
        {{"k_spmm_mid<f32,fine>", "k_spmm_mid<f32,mid>", "k_spmm_mid<f32,small>"},
         {"k_spmm_mid<f64,fine>", "k_spmm_mid<f64,mid>", "k_spmm_mid<f64,small>"}}};
    const int sc = n >= (1 << 20) ? 0 : n >= (1 << 16) ? 1 : 2;
    return names[kind][f64 ? 1 : 0][sc];
}

// Entry split for an operator of average slice width wavg: one chunk of
// kSellUnroll gathers per thread where possible, with tpr * ES <= 32 and tpr
// a power of two.
static int entry_split(double wavg, int tpr) {
    if (tpr & (tpr - 1)) return 1;
    int es = 1;
    while (es < 8 && wavg > kSellUnroll * es && tpr * es * 2 <= 32) es <<= 1;
    return es;
}

template <class T, int V, int ES>
static void launch_sell_es(const Csr<T> &A, const T *x, T *y, int k, const T *b, cudaStream_t s, bool accum,
                           const char *tag) {
    const int tpr = k / V;
    const int rows = 256 / (tpr * ES);
    int64_t g = (A.n + rows - 1) / rows;
    if (g > 0x7fffffffLL) g = 0x7fffffffLL;
    if (g < 1) g = 1;
    if (A.ell_w > 0)
        (g2p::kbegin(tag ? tag : spmm_name(1, sizeof(T) == 8, A.n), s),
         k_spmm_ell<T, V, ES><<<(unsigned)g, dim3(tpr * ES, rows), 0, s>>>(A.n, A.ell_w, A.scol, A.sval, x, y, k, b,
                                                                            accum),
         g2p::kend(s));
    else
        (g2p::kbegin(tag ? tag : spmm_name(0, sizeof(T) == 8, A.n), s),
         k_spmm_sell<T, V, ES><<<(unsigned)g, dim3(tpr * ES, rows), 0, s>>>(A.n, A.sptr, A.scol, A.sval, A.rlen, x, y,
                                                                             k, b, accum),
         g2p::kend(s));
}

template <class T, int V>
static void launch_sell(const Csr<T> &A, const T *x, T *y, int k, const T *b, cudaStream_t s, bool accum = false,
                        const char *tag = nullptr) {
    // one block per 256 / tpr rows, never grid-strided: blocks retire in row
    // order, so the rows in flight form one window and the x rows a stencil
    // shares (z-neighbours one layer apart) are still in L2 when reused
    const int tpr = k / V;
    const int rows = 256 / tpr;
    int64_t g = (A.n + rows - 1) / rows;
    if (g > 0x7fffffffLL) g = 0x7fffffffLL;
    if (g < 1) g = 1;
    if (A.ell_w > 0 && A.ell_w <= kSellUnroll && pipe_ok()) {
        // persistent: as many blocks as fit on the SMs at once
        // one value per instantiation, initialised once even with several host threads
        static const int resident = [tpr, rows] {
            int per_sm = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmm_ell_pipe<T, V>, tpr * rows, 0);
            return (per_sm > 0 ? per_sm : 4) * kSMs;
        }();
        const int64_t gp = std::min<int64_t>(g, resident);
        (g2p::kbegin(tag ? tag : spmm_name(2, sizeof(T) == 8, A.n), s),
         k_spmm_ell_pipe<T, V><<<(unsigned)gp, dim3(tpr, rows), 0, s>>>(A.n, A.ell_w, A.scol, A.sval, x, y, k, b, accum),
         g2p::kend(s));
    } else {
        // the entry split trades coalescing of the column and value loads for
        // shorter dependent chains: worth it only on small (latency-bound)
        // operators
        const double wavg = A.n > 0 ? (double)A.sell_slots / (32.0 * (double)((A.n + 31) / 32)) : 0.0;
        if (A.n >= (1 << 16) && A.ell_w == 0 && wavg > kSellUnroll) {
            // wide rows on a large operator: chunk-pipelined, coalesced loads
            (g2p::kbegin(tag ? tag : spmm_name(0, sizeof(T) == 8, A.n), s),
             k_spmm_sell_pipe<T, V><<<(unsigned)g, dim3(tpr, rows), 0, s>>>(A.n, A.sptr, A.scol, A.sval, A.rlen, x, y,
                                                                           k, b, accum),
             g2p::kend(s));
            return;
        }
        switch (A.n < (1 << 16) ? entry_split(wavg, tpr) : 1) {
            case 8: launch_sell_es<T, V, 8>(A, x, y, k, b, s, accum, tag); break;
            case 4: launch_sell_es<T, V, 4>(A, x, y, k, b, s, accum, tag); break;
            case 2: launch_sell_es<T, V, 2>(A, x, y, k, b, s, accum, tag); break;
            default: launch_sell_es<T, V, 1>(A, x, y, k, b, s, accum, tag); break;
        }
    }
}

// A side stream per launching stream (and host thread) for the long-row
// kernels of coarse operators, with the fork and join events.
struct SideStream {
    cudaStream_t side = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr;
    bool ok = false;
};
struct SideStreams {
    std::vector<std::pair<cudaStream_t, SideStream>> tab;
    ~SideStreams() {
        // errors at process exit (runtime already unloading) are ignored
        for (auto &e : tab)
            if (e.second.ok) {
                cudaEventDestroy(e.second.fork);
                cudaEventDestroy(e.second.join);
                cudaStreamDestroy(e.second.side);
            }
        cudaGetLastError();
    }
};
static SideStream *side_stream_of(cudaStream_t s) {
    thread_local SideStreams held;
    auto &tab = held.tab;
    for (auto &e : tab)
        if (e.first == s) return e.second.ok ? &e.second : nullptr;
    if (tab.size() >= 64) return nullptr;      // many launching streams: keep their long rows in line
    SideStream ss;
    ss.ok = cudaStreamCreateWithFlags(&ss.side, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&ss.fork, cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&ss.join, cudaEventDisableTiming) == cudaSuccess;
    if (!ss.ok) cudaGetLastError();
    tab.emplace_back(s, ss);
    return ss.ok ? &tab.back().second : nullptr;
}

// G2P_LONG_FORK=0 keeps the long-row kernels behind the short-row kernel on
// the launching stream (comparison).  Read at the start of each solve
// (refresh_long_fork), not per launch.
static std::atomic<bool> g_long_fork{true};
static void refresh_long_fork() {
    const char *e = getenv("G2P_LONG_FORK");
    g_long_fork = e ? atoi(e) != 0 : true;
}
static bool long_fork_on() { return g_long_fork.load(std::memory_order_relaxed); }

template <class T>
void spmm_b(const Csr<T> &A, const LongRows &lr, const T *x, T *y, int k, const T *b, cudaStream_t s) {
    bool prof = g_prof.on && g_prof.used + 2 <= (size_t)1 << 20;
    // coarse operators with long rows (conductor potentials): the long-row
    // kernels run on a side stream beside the short-row kernel and join
    // before the next launch.  Only with the sliced-ELL short-row kernels,
    // which leave the long rows of y alone (the uniform-width kernels write
    // every row and rely on the long-row kernels coming after them); not on
    // operators of 1M rows or more, whose persistent kernel wants every SM;
    // not while kernels are being timed one by one.
    SideStream *fork = nullptr;
    if ((lr.nmid > 0 || lr.nchunk > 0) && A.sptr != nullptr && A.ell_w == 0 && A.n < (1 << 20) && !prof &&
        !kprof_on() && long_fork_on())
        fork = side_stream_of(s);
    cudaStream_t sl = s;
    if (fork) {
        if (cudaEventRecord(fork->fork, s) == cudaSuccess && cudaStreamWaitEvent(fork->side, fork->fork, 0) == cudaSuccess) {
            sl = fork->side;
        } else {
            cudaGetLastError();
            fork = nullptr;
        }
    }
    if (fork) {
        dim3 lblk = row_block(k);
        if (lr.nmid > 0) {
            const int kx = k >= 32 ? 32 : pow2_ge(k);
            (g2p::kbegin(spmm_name(3, sizeof(T) == 8, A.n), sl),
             k_spmm_mid<T><<<(unsigned)lr.nmid, 256, 0, sl>>>(lr.nmid, lr.mid, A.ptr, A.col, A.val, x, k, kx, y, b), g2p::kend(sl));
        }
        if (lr.nchunk > 0)
            (g2p::kbegin(sizeof(T) == 8 ? "k_spmm_long<f64,coarse>" : "k_spmm_long<f32,coarse>", sl),
             k_spmm_long<T><<<(unsigned)lr.nchunk, lblk, 0, sl>>>(lr.rows, lr.crow, lr.cbeg, lr.rcp, A.ptr, A.col, A.val, x, k, lr.partial, lr.done, y, b), g2p::kend(sl));
        cudaEventRecord(fork->join, sl);
    }
    const bool sell = A.sptr != nullptr;
    if (prof) {
        // the events bracket the short-row launch itself, inside the
        // per-kernel profiler's own events (see the kbracket hooks below)
        if (sell)
            g_prof.bytes += (double)A.short_nnz * (sizeof(T) + 4) + (double)A.n + (double)((A.n + 31) / 32) * 8 +
                            (double)A.n * k * sizeof(T) * (b ? 3 : 2);
        else
            g_prof.bytes += (double)A.nnz * (sizeof(T) + 4) + (double)(A.n + 1) * 8 +
                            (double)A.n * k * sizeof(T) * (b ? 3 : 2);
        g_prof.launches++;
        const double lb = sell ? (double)A.short_nnz * (sizeof(T) + 4) + (double)A.n + (double)((A.n + 31) / 32) * 8 +
                                     (double)A.n * k * sizeof(T) * (b ? 3 : 2)
                               : (double)A.nnz * (sizeof(T) + 4) + (double)(A.n + 1) * 8 +
                                     (double)A.n * k * sizeof(T) * (b ? 3 : 2);
        g_prof.launch_bytes.push_back(lb);
        g_prof.launch_f64.push_back(sizeof(T) == 8);
        g_prof.launch_rows.push_back(A.n);
    }
    dim3 blk = row_block(k);
    if (prof) {
        kbracket_begin = prof_event;
        kbracket_end = prof_event;
    }
    if (sell) {
        // vector width only where every x row, y row and b row is aligned to it
        int v = sell_vec<T>(k);
        auto aligned = [&](const void *p) {
            size_t w = (size_t)v * sizeof(T) >= 16 ? 16 : (size_t)v * sizeof(T);
            return p == nullptr || ((uintptr_t)p % w) == 0;
        };
        while (v > 1 && !(aligned(x) && aligned(y) && aligned(b))) v >>= 1;
        switch (v) {
            case 8: launch_sell<T, 8>(A, x, y, k, b, s); break;
            case 4: launch_sell<T, 4>(A, x, y, k, b, s); break;
            case 2: launch_sell<T, 2>(A, x, y, k, b, s); break;
            default: launch_sell<T, 1>(A, x, y, k, b, s); break;
        }
    } else {
        (g2p::kbegin("k_spmm", s), k_spmm<T><<<row_grid(A.n, k, 152LL * 48), blk, 0, s>>>(A.n, A.ptr, A.col, A.val, x, y, k, b), g2p::kend(s));
    }
    if (prof) {
        kbracket_begin = nullptr;
        kbracket_end = nullptr;
    }
    if (fork) {
        cudaStreamWaitEvent(s, fork->join, 0);
        return;
    }
    if (lr.nmid > 0) {
        const int kx = k >= 32 ? 32 : pow2_ge(k);
        (g2p::kbegin(spmm_name(3, sizeof(T) == 8, A.n), s),
         k_spmm_mid<T><<<(unsigned)lr.nmid, 256, 0, s>>>(lr.nmid, lr.mid, A.ptr, A.col, A.val, x, k, kx, y, b), g2p::kend(s));
    }
    if (lr.nchunk > 0) {
        (g2p::kbegin(A.n >= (1 << 20) ? (sizeof(T) == 8 ? "k_spmm_long<f64,fine>" : "k_spmm_long<f32,fine>")
                                      : (sizeof(T) == 8 ? "k_spmm_long<f64,coarse>" : "k_spmm_long<f32,coarse>"), s),
         k_spmm_long<T><<<(unsigned)lr.nchunk, blk, 0, s>>>(lr.rows, lr.crow, lr.cbeg, lr.rcp, A.ptr, A.col, A.val, x, k, lr.partial, lr.done, y, b), g2p::kend(s));
    }
}

// x += P xc with the sliced-ELL copy of P (every row of P is short).
template <class T>
static void prolong_sell(const Csr<T> &P, const T *xc, T *x, int k, cudaStream_t s) {
    int v = sell_vec<T>(k);
    auto aligned = [&](const void *p) {
        size_t w = (size_t)v * sizeof(T) >= 16 ? 16 : (size_t)v * sizeof(T);
        return ((uintptr_t)p % w) == 0;
    };
    while (v > 1 && !(aligned(xc) && aligned(x))) v >>= 1;
    const char *tag = sizeof(T) == 8 ? "k_prolong_sell<f64>" : "k_prolong_sell<f32>";
    switch (v) {
        case 8: launch_sell<T, 8>(P, xc, x, k, nullptr, s, true, tag); break;
        case 4: launch_sell<T, 4>(P, xc, x, k, nullptr, s, true, tag); break;
        case 2: launch_sell<T, 2>(P, xc, x, k, nullptr, s, true, tag); break;
        default: launch_sell<T, 1>(P, xc, x, k, nullptr, s, true, tag); break;
    }
}

template <class T>
void spmm(const Csr<T> &A, const LongRows &lr, const T *x, T *y, int k, cudaStream_t s) {
    spmm_b<T>(A, lr, x, y, k, nullptr, s);
}
template void spmm<double>(const Csr<double> &, const LongRows &, const double *, double *, int, cudaStream_t);
template void spmm<float>(const Csr<float> &, const LongRows &, const float *, float *, int, cudaStream_t);

void residual64(const Csr<double> &A, const LongRows &lr, const double *b, const double *x, double *r, int k,
                cudaStream_t s) {
    spmm_b<double>(A, lr, x, r, k, b, s);
}

__global__ void k_mark_long(int64_t n, const int64_t *ptr, int64_t *flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = (ptr[i + 1] - ptr[i]) > kLongRow ? 1 : 0;
}
__global__ void k_list_long(int64_t n, const int64_t *ptr, const int64_t *pos, int32_t *rows) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if ((ptr[i + 1] - ptr[i]) > kLongRow) rows[pos[i]] = (int32_t)i;
}

__global__ void k_long_extent(int64_t nl, const int32_t *rows, const int64_t *ptr, int64_t *ext) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nl; i += (int64_t)gridDim.x * blockDim.x) {
        ext[2 * i] = ptr[rows[i]];
        ext[2 * i + 1] = ptr[rows[i] + 1];
    }
}

template <class T>
g2p_status find_long_rows(const Csr<T> &A, LongRows &lr, cudaStream_t s) {
    lr.release(s);
    int64_t *pos, *work;
    int64_t n = A.n;
    G2P_TRY(dalloc(&pos, n + 1, s));
    G2P_TRY(dalloc(&work, scan_work_size(n + 1) + 4, s));
    const int64_t *p = A.ptr;
    auto op = [p, n] __device__(int64_t i) -> int64_t { return i < n ? ((p[i + 1] - p[i]) > kLongRow ? 1 : 0) : 0; };
    G2P_TRY(exclusive_scan(op, n + 1, pos, work, s));
    int64_t nl = 0;
    G2P_CUDA(cudaMemcpyAsync(&nl, pos + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    if (nl > 0) {
        G2P_TRY(dalloc(&lr.rows, nl, s));
        (g2p::kbegin("k_list_long", s), k_list_long<<<grid_for(n), kThreads, 0, s>>>(n, A.ptr, pos, lr.rows), g2p::kend(s));
        // chunk table on the host from the long rows' extents (one copy)
        int64_t *ext;
        G2P_TRY(dalloc(&ext, 2 * nl, s));
        (g2p::kbegin("k_long_extent", s), k_long_extent<<<grid_for(nl), kThreads, 0, s>>>(nl, lr.rows, A.ptr, ext), g2p::kend(s));
        std::vector<int64_t> be(2 * nl);
        G2P_CUDA(cudaMemcpyAsync(be.data(), ext, sizeof(int64_t) * 2 * nl, cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        dfree(ext, s);
        std::vector<int32_t> crow, mid;
        std::vector<int64_t> cbeg, rcp(nl + 1, 0);
        std::vector<int32_t> rows(nl);
        G2P_CUDA(cudaMemcpyAsync(rows.data(), lr.rows, sizeof(int32_t) * nl, cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        for (int64_t l = 0; l < nl; l++) {
            if (be[2 * l + 1] - be[2 * l] <= kHugeRow) mid.push_back(rows[l]);
            else
                for (int64_t q = be[2 * l]; q < be[2 * l + 1]; q += kLongChunk) { crow.push_back((int32_t)l); cbeg.push_back(q); }
            rcp[l + 1] = (int64_t)crow.size();
        }
        lr.n = nl;
        lr.nchunk = (int64_t)crow.size();
        lr.nmid = (int64_t)mid.size();
        if (const char *e = getenv("G2P_DEBUG"))
            if (atoi(e) >= 2)
                fprintf(stderr, "[g2p long rows] n=%lld nnz=%lld long=%lld mid=%lld chunks=%lld\n", (long long)n,
                        (long long)A.nnz, (long long)nl, (long long)lr.nmid, (long long)lr.nchunk);
        G2P_TRY(dalloc(&lr.mid, lr.nmid, s));
        if (lr.nmid) G2P_CUDA(cudaMemcpyAsync(lr.mid, mid.data(), sizeof(int32_t) * lr.nmid, cudaMemcpyHostToDevice, s));
        G2P_TRY(dalloc(&lr.crow, lr.nchunk, s));
        G2P_TRY(dalloc(&lr.cbeg, lr.nchunk, s));
        G2P_TRY(dalloc(&lr.rcp, nl + 1, s));
        G2P_TRY(dalloc(&lr.partial, lr.nchunk * kMaxRhs, s));
        G2P_TRY(dalloc(&lr.done, nl, s));
        G2P_CUDA(cudaMemsetAsync(lr.done, 0, sizeof(int32_t) * nl, s));
        G2P_CUDA(cudaMemcpyAsync(lr.crow, crow.data(), sizeof(int32_t) * lr.nchunk, cudaMemcpyHostToDevice, s));
        G2P_CUDA(cudaMemcpyAsync(lr.cbeg, cbeg.data(), sizeof(int64_t) * lr.nchunk, cudaMemcpyHostToDevice, s));
        G2P_CUDA(cudaMemcpyAsync(lr.rcp, rcp.data(), sizeof(int64_t) * (nl + 1), cudaMemcpyHostToDevice, s));
        G2P_CUDA(cudaStreamSynchronize(s));
    }
    dfree(pos, s); dfree(work, s);
    return G2P_OK;
}
template g2p_status find_long_rows<double>(const Csr<double> &, LongRows &, cudaStream_t);
template g2p_status find_long_rows<float>(const Csr<float> &, LongRows &, cudaStream_t);

g2p_status copy_long_rows(const LongRows &src, LongRows &dst, cudaStream_t s) {
    dst.release(s);
    if (src.n == 0) return G2P_OK;
    dst.n = src.n; dst.nchunk = src.nchunk;
    G2P_TRY(dalloc(&dst.rows, src.n, s)); G2P_TRY(dalloc(&dst.crow, src.nchunk, s));
    G2P_TRY(dalloc(&dst.cbeg, src.nchunk, s)); G2P_TRY(dalloc(&dst.rcp, src.n + 1, s));
    G2P_TRY(dalloc(&dst.partial, src.nchunk * kMaxRhs, s));
    G2P_TRY(dalloc(&dst.done, src.n, s));
    dst.nmid = src.nmid;
    G2P_TRY(dalloc(&dst.mid, src.nmid, s));
    if (src.nmid) G2P_CUDA(cudaMemcpyAsync(dst.mid, src.mid, sizeof(int32_t) * src.nmid, cudaMemcpyDeviceToDevice, s));
    G2P_CUDA(cudaMemsetAsync(dst.done, 0, sizeof(int32_t) * src.n, s));
    G2P_CUDA(cudaMemcpyAsync(dst.rows, src.rows, sizeof(int32_t) * src.n, cudaMemcpyDeviceToDevice, s));
    G2P_CUDA(cudaMemcpyAsync(dst.crow, src.crow, sizeof(int32_t) * src.nchunk, cudaMemcpyDeviceToDevice, s));
    G2P_CUDA(cudaMemcpyAsync(dst.cbeg, src.cbeg, sizeof(int64_t) * src.nchunk, cudaMemcpyDeviceToDevice, s));
    G2P_CUDA(cudaMemcpyAsync(dst.rcp, src.rcp, sizeof(int64_t) * (src.n + 1), cudaMemcpyDeviceToDevice, s));
    return G2P_OK;
}

// Sliced-ELL copy of A's short rows (kept beside the CSR).
template <class T>
g2p_status sell_build(Csr<T> &A, cudaStream_t s, int64_t maxlen) {
    A.release_sell(s);
    const int64_t n = A.n, nslice = (n + 31) / 32;
    int64_t *width, *work;
    G2P_TRY(dalloc(&width, nslice + 1, s));
    G2P_TRY(dalloc(&work, scan_work_size(nslice + 1) + 4, s));
    G2P_TRY(dalloc(&A.rlen, n, s));
    G2P_TRY(dalloc(&A.sptr, nslice + 1, s));
    (g2p::kbegin("k_sell_width", s), k_sell_width<<<grid_for(nslice), kThreads, 0, s>>>(n, A.ptr, nslice, maxlen, width, A.rlen), g2p::kend(s));
    const int64_t *wp = width;
    auto op = [wp, nslice] __device__(int64_t i) -> int64_t { return i < nslice ? wp[i] : 0; };
    G2P_TRY(exclusive_scan(op, nslice + 1, A.sptr, work, s));
    unsigned long long *dmax;
    G2P_TRY(dalloc(&dmax, 1, s));
    G2P_CUDA(cudaMemsetAsync(dmax, 0, sizeof(unsigned long long), s));
    (g2p::kbegin("k_width_max", s), k_width_max<<<grid_for(nslice), kThreads, 0, s>>>(width, nslice, dmax), g2p::kend(s));
    int64_t slots = 0;
    unsigned long long hmax = 0;
    G2P_CUDA(cudaMemcpyAsync(&slots, A.sptr + nslice, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaMemcpyAsync(&hmax, dmax, sizeof(hmax), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    dfree(width, s); dfree(work, s); dfree(dmax, s);
    // one width for all slices when that costs at most a quarter more slots
    const int64_t wmax = (int64_t)hmax / 32;
    const bool uniform = wmax > 0 && 32 * wmax * nslice <= slots + slots / 4;
    if (uniform) {
        (g2p::kbegin("k_ell_sptr", s), k_ell_sptr<<<grid_for(nslice + 1), kThreads, 0, s>>>(A.sptr, nslice, 32 * wmax), g2p::kend(s));
        slots = 32 * wmax * nslice;
        A.ell_w = (int32_t)wmax;
    }
    A.sell_slots = slots;
    if (const char *e = getenv("G2P_DEBUG"))
        if (atoi(e) >= 2)
            fprintf(stderr, "[g2p sell] n=%lld nnz=%lld slots=%lld wmax=%lld uniform=%d\n", (long long)n,
                    (long long)A.nnz, (long long)slots, (long long)wmax, (int)uniform);
    G2P_TRY(dalloc(&A.scol, slots, s));
    G2P_TRY(dalloc(&A.sval, slots, s));
    (g2p::kbegin("k_sell_fill", s), k_sell_fill<T><<<grid_for(n), kThreads, 0, s>>>(n, A.ptr, A.col, A.val, A.rlen, A.sptr, A.scol, A.sval), g2p::kend(s));
    if (uniform)
        (g2p::kbegin("k_ell_pad", s), k_ell_pad<T><<<grid_for(n), kThreads, 0, s>>>(n, A.m, A.ell_w, A.rlen, A.scol, A.sval), g2p::kend(s));
    // entries of the long rows are not in the copy
    int64_t *lp, *lw;
    G2P_TRY(dalloc(&lp, n + 1, s));
    G2P_TRY(dalloc(&lw, scan_work_size(n + 1) + 4, s));
    const int64_t *pp = A.ptr;
    auto lop = [pp, n, maxlen] __device__(int64_t i) -> int64_t {
        if (i >= n) return 0;
        int64_t l = pp[i + 1] - pp[i];
        return l > maxlen ? 0 : l;
    };
    G2P_TRY(exclusive_scan(lop, n + 1, lp, lw, s));
    G2P_CUDA(cudaMemcpyAsync(&A.short_nnz, lp + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    dfree(lp, s); dfree(lw, s);
    G2P_CUDA(cudaGetLastError());
    return G2P_OK;
}
template g2p_status sell_build<double>(Csr<double> &, cudaStream_t, int64_t);
template g2p_status sell_build<float>(Csr<float> &, cudaStream_t, int64_t);

// New values, same pattern: rewrites the sliced-ELL copy's values from A.val
// (padding and long rows are untouched).
template <class T>
g2p_status sell_refill(Csr<T> &A, cudaStream_t s) {
    if (!A.sptr) return G2P_OK;
    (g2p::kbegin("k_sell_fill", s), k_sell_fill<T><<<grid_for(A.n), kThreads, 0, s>>>(A.n, A.ptr, A.col, A.val, A.rlen, A.sptr, A.scol, A.sval), g2p::kend(s));
    G2P_CUDA(cudaGetLastError());
    return G2P_OK;
}
template g2p_status sell_refill<double>(Csr<double> &, cudaStream_t);

// ------------------------------------------- 16-byte chunks of k-interleaved blocks
// A block of k right-hand sides is stored row-major (entry (i, r) at i*k + r).
// When k is a power-of-two multiple of the chunk width C = 16 / sizeof(T) and
// at most kVecMaxK, the kernels below move 16 bytes per thread and access
// instead of one element: cpr = k / C chunks per row, and a thread's chunk
// column stays fixed across its grid-stride loop (the stride is a multiple
// of cpr).  Other widths use the per-element kernels.
constexpr int kVecMaxK = 64;
template <class T> struct Chunk;
template <> struct Chunk<float> {
    static constexpr int C = 4;
    float v[4];
    __device__ __forceinline__ void ld(const float *p) {
        const float4 t = __ldg(reinterpret_cast<const float4 *>(p)); v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
    __device__ __forceinline__ void ldc(const float *p) {
        const float4 t = *reinterpret_cast<const float4 *>(p); v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
    __device__ __forceinline__ void st(float *p) const { *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]); }
};
template <> struct Chunk<double> {
    static constexpr int C = 2;
    double v[2];
    __device__ __forceinline__ void ld(const double *p) {
        const double2 t = __ldg(reinterpret_cast<const double2 *>(p)); v[0] = t.x; v[1] = t.y;
    }
    __device__ __forceinline__ void ldc(const double *p) {
        const double2 t = *reinterpret_cast<const double2 *>(p); v[0] = t.x; v[1] = t.y;
    }
    __device__ __forceinline__ void st(double *p) const { *reinterpret_cast<double2 *>(p) = make_double2(v[0], v[1]); }
};

template <class T>
static inline int chunk_cpr(int k) {
    constexpr int C = Chunk<T>::C;
    if (k % C != 0 || k > kVecMaxK) return 0;
    const int cpr = k / C;
    return (cpr & (cpr - 1)) == 0 ? cpr : 0;
}
static inline unsigned chunk_grid(int64_t nq) {
    int64_t b = (nq + 255) / 256;
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152LL * 16));
}
#define G2P_FOR_CHUNKS(q, nq) \
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < (nq); q += (int64_t)gridDim.x * blockDim.x)

// dst = src / h[col] (0 where h = 0): the Krylov start and Arnoldi normalisation
template <class T>
__global__ void __launch_bounds__(256) k_scale_cols_v(int64_t nq, int cpr, const double *h, const T *src, T *dst) {
    constexpr int C = Chunk<T>::C;
    const int cc = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) & (cpr - 1));
    T inv[C];
#pragma unroll
    for (int u = 0; u < C; u++) {
        const double b = h[cc * C + u];
        inv[u] = b > 0 ? (T)(1.0 / b) : (T)0;
    }
    G2P_FOR_CHUNKS(q, nq) {
        Chunk<T> a;
        a.ld(src + q * C);
#pragma unroll
        for (int u = 0; u < C; u++) a.v[u] *= inv[u];
        a.st(dst + q * C);
    }
}

// w -= sum_j h[j*k + col] V_j, h staged in shared memory
template <class T>
__global__ void __launch_bounds__(256) k_maxpy_v(int64_t nq, int cpr, int k, int J, const T *V, const double *h, T *w) {
    constexpr int C = Chunk<T>::C;
    extern __shared__ unsigned char smraw[];
    T *hs = reinterpret_cast<T *>(smraw);
    for (int t = threadIdx.x; t < J * k; t += blockDim.x) hs[t] = (T)h[t];
    __syncthreads();
    const int cc = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) & (cpr - 1));
    const int64_t nk = nq * C;
    G2P_FOR_CHUNKS(q, nq) {
        Chunk<T> acc;
        acc.ldc(w + q * C);
        for (int j = 0; j < J; j++) {
            Chunk<T> v;
            v.ld(V + (int64_t)j * nk + q * C);
            const T *hj = hs + j * k + cc * C;
#pragma unroll
            for (int u = 0; u < C; u++) acc.v[u] -= hj[u] * v.v[u];
        }
        acc.st(w + q * C);
    }
}

// The unnormalised Arnoldi basis (W_i = s_i V_i, s_i = |W_i| per column):
// out = w - sum_i c[i*k + col] W_i, the next basis vector as it stands, and
// the block partial sums of its squared columns (so no separate norm pass
// and no normalised copy).  c staged in shared memory.
template <int GC, class T>
__device__ __forceinline__ void chunk_col_reduce(const T (&v)[GC], double *sm, int cpr, int k, int C, int gvalid,
                                                 int64_t gbase, double *partial);
template <class T>
__global__ void __launch_bounds__(256) k_maxpy_norm_v(int64_t nq, int cpr, int k, int J, const T *V, const double *c,
                                                      const T *w, T *out, double *partial) {
    constexpr int C = Chunk<T>::C;
    extern __shared__ unsigned char smraw[];
    __shared__ double sm[8 * C * 16];
    T *hs = reinterpret_cast<T *>(smraw);
    for (int t = threadIdx.x; t < J * k; t += blockDim.x) hs[t] = (T)c[t];
    __syncthreads();
    const int cc = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) & (cpr - 1));
    const int64_t nk = nq * C;
    T sq[C];
#pragma unroll
    for (int u = 0; u < C; u++) sq[u] = 0;
    G2P_FOR_CHUNKS(q, nq) {
        Chunk<T> acc;
        acc.ld(w + q * C);
        for (int j = 0; j < J; j++) {
            Chunk<T> v;
            v.ld(V + (int64_t)j * nk + q * C);
            const T *hj = hs + j * k + cc * C;
#pragma unroll
            for (int u = 0; u < C; u++) acc.v[u] -= hj[u] * v.v[u];
        }
        acc.st(out + q * C);
#pragma unroll
        for (int u = 0; u < C; u++) sq[u] += acc.v[u] * acc.v[u];
    }
    chunk_col_reduce<C>(sq, sm, cpr, k, C, 1, 0, partial);
}

// From the dots d_i = W_i . w (w = A M^-1 W_j): the Hessenberg entries
// h_i = d_i / (s_i s_j), in place, and the update coefficients
// c_i = d_i / s_i^2 (zero for a zero column)
__global__ void k_unnorm_coef(int k, int j, const double *sc, double *h, double *c) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (j + 1) * k) return;
    const int i = t / k, r = t - i * k;
    const double si = sc[i * k + r], sj = sc[j * k + r], d = h[t];
    c[t] = si > 0 ? d / (si * si) : 0.0;
    h[t] = si > 0 && sj > 0 ? d / (si * sj) : 0.0;
}

// h_{j+1,j} = s_{j+1} / s_j
__global__ void k_unnorm_hnorm(int k, int j, const double *sc, double *hnorm) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= k) return;
    const double sj = sc[j * k + r];
    hnorm[r] = sj > 0 ? sc[(j + 1) * k + r] / sj : 0.0;
}

// Chebyshev: d = theta^-1 D^-1 b, x = d (or x += d)
// Chebyshev first step: d = D^-1 b / theta, x = d (or x += d with add).
// STX / STD: whether x and d are stored (a zero-guess smoother of degree >= 2
// keeps its first iterate in d only; a last step's d is never read).
template <class T, bool STX, bool STD>
__global__ void __launch_bounds__(256) k_cheb_first_v(int64_t nq, int shift, const T *dinv, const T *b, T *x, T *d,
                                                      double inv_theta, bool add) {
    constexpr int C = Chunk<T>::C;
    G2P_FOR_CHUNKS(q, nq) {
        const T di = (T)inv_theta * dinv[q >> shift];
        Chunk<T> bb, dd;
        bb.ld(b + q * C);
#pragma unroll
        for (int u = 0; u < C; u++) dd.v[u] = di * bb.v[u];
        if (STD) dd.st(d + q * C);
        if (add) {
            Chunk<T> xx;
            xx.ldc(x + q * C);
#pragma unroll
            for (int u = 0; u < C; u++) xx.v[u] += dd.v[u];
            xx.st(x + q * C);
        } else if (STX) {
            dd.st(x + q * C);
        }
    }
}

// Chebyshev: d = c1 d + c2 D^-1 res ; x += d.  XD: the iterate is d itself
// (the step after a zero-guess first step that stored d only), so x is
// written but not read; STD: whether d is stored.
template <class T, bool XD, bool STD>
__global__ void __launch_bounds__(256) k_cheb_step_v(int64_t nq, int shift, const T *dinv, const T *res, T *x, T *d,
                                                     double c1, double c2) {
    constexpr int C = Chunk<T>::C;
    const T a = (T)c1, bcoef = (T)c2;
    G2P_FOR_CHUNKS(q, nq) {
        const T di = bcoef * dinv[q >> shift];
        Chunk<T> rr, dd, xx;
        rr.ld(res + q * C);
        dd.ldc(d + q * C);
        if (XD) xx = dd;
        else xx.ldc(x + q * C);
#pragma unroll
        for (int u = 0; u < C; u++) {
            const T t = a * dd.v[u] + di * rr.v[u];
            dd.v[u] = t;
            xx.v[u] += t;
        }
        if (STD) dd.st(d + q * C);
        xx.st(x + q * C);
    }
}

// b_c[I] = sum over the members of I of res (members ascending)
template <class T>
__global__ void __launch_bounds__(256) k_restrict_v(int64_t nc, int shift, int k, const int64_t *rptr,
                                                    const int32_t *rmem, const T *res, T *bc) {
    constexpr int C = Chunk<T>::C;
    const int64_t nq = nc << shift;
    G2P_FOR_CHUNKS(q, nq) {
        const int64_t I = q >> shift;
        const int off = (int)(q & ((1 << shift) - 1)) * C;
        Chunk<T> acc;
#pragma unroll
        for (int u = 0; u < C; u++) acc.v[u] = 0;
        for (int64_t m = rptr[I]; m < rptr[I + 1]; m++) {
            Chunk<T> v;
            v.ld(res + (int64_t)rmem[m] * k + off);
#pragma unroll
            for (int u = 0; u < C; u++) acc.v[u] += v.v[u];
        }
        acc.st(bc + q * C);
    }
}

// Per-column sums over the rows of a (cpr, 256 / cpr) block, cpr <= 16: G
// groups of C columns per thread.  Lanes of a warp that share a chunk column
// combine by xor shuffles, then the eight warps' sums are added in order.
// Result (g, column c) -> partial[(g * k + c) * gridDim.x + blockIdx.x].
template <int GC, class T>
__device__ __forceinline__ void chunk_col_reduce(const T (&v)[GC], double *sm, int cpr, int k, int C, int gvalid,
                                                 int64_t gbase, double *partial) {
    const int tid = threadIdx.y * cpr + threadIdx.x, lane = tid & 31, warp = tid >> 5;
#pragma unroll
    for (int e = 0; e < GC; e++) {
        double x = (double)v[e];
        for (int o = cpr; o < 32; o <<= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane < cpr) sm[(warp * GC + e) * cpr + lane] = x;
    }
    __syncthreads();
    for (int idx = tid; idx < GC * cpr; idx += 256) {
        const int e = idx / cpr, cc = idx % cpr;
        const int g = e / C, u = e % C;
        if (g < gvalid) {
            double acc = 0;
            for (int w = 0; w < 8; w++) acc += sm[(w * GC + e) * cpr + cc];
            partial[((gbase + g) * k + cc * C + u) * gridDim.x + blockIdx.x] = acc;
        }
    }
    __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(256) k_colsq_partial_v(const T *x, int64_t n, int k, double *partial) {
    constexpr int C = Chunk<T>::C;
    __shared__ double sm[8 * C * 16];
    const int cpr = blockDim.x, cc = threadIdx.x, ny = blockDim.y;
    T acc[C];
#pragma unroll
    for (int u = 0; u < C; u++) acc[u] = 0;
    for (int64_t i = blockIdx.x * (int64_t)ny + threadIdx.y; i < n; i += (int64_t)gridDim.x * ny) {
        Chunk<T> a;
        a.ld(x + i * k + cc * C);
#pragma unroll
        for (int u = 0; u < C; u++) acc[u] += a.v[u] * a.v[u];
    }
    chunk_col_reduce<C>(acc, sm, cpr, k, C, 1, 0, partial);
}

// Dots of basis vectors j0 .. j0 + G - 1 with w.  G is a compile-time count
// (one launch per group of at most 8, see mdot), so exactly G products per
// element are issued: an FP64 dot is bound by the FP64 pipe on this part.
template <class T, int G>
__global__ void __launch_bounds__(256) k_mdot_partial_v(const T *V, int64_t n, int j0, const T *w, int k,
                                                        double *partial) {
    constexpr int C = Chunk<T>::C, GC = G * C;
    __shared__ double sm[8 * GC * 16];
    const int cpr = blockDim.x, cc = threadIdx.x, ny = blockDim.y;
    const int64_t nk = n * k;
    T acc[GC];          // acc[g * C + u]
#pragma unroll
    for (int e = 0; e < GC; e++) acc[e] = 0;
    for (int64_t i = blockIdx.x * (int64_t)ny + threadIdx.y; i < n; i += (int64_t)gridDim.x * ny) {
        const int64_t t = i * k + cc * C;
        Chunk<T> ww;
        ww.ld(w + t);
#pragma unroll
        for (int g = 0; g < G; g++) {
            Chunk<T> vv;
            vv.ld(V + (int64_t)(j0 + g) * nk + t);
#pragma unroll
            for (int u = 0; u < C; u++) acc[g * C + u] += vv.v[u] * ww.v[u];
        }
    }
    chunk_col_reduce<GC>(acc, sm, cpr, k, C, G, j0, partial);
}

// --------------------------------------------------------------- reductions
// Deterministic per-column sums of squares: block partials, then an ordered
// final pass.
constexpr int kRedBlocks = 152 * 4;
constexpr int64_t kMaxDenseCoarse = 768;

// Block shape (kx, 256 / kx) with kx the power of two >= k: threadIdx.x is
// the right-hand side, threadIdx.y strides over rows, so every thread keeps
// one column's partial sum and the block reduces in a fixed order.

// Sums G per-thread values over the threads of a (kx, 256 / kx) block that
// share column r, in a fixed order: xor shuffles inside each warp, then the
// warps' (or, for kx >= 32, the rows') sums one after another.  sm holds
// G * 256 doubles; the result for (g, r) lands in sm[g * 256 + r].
template <int G>
__device__ __forceinline__ void block_col_reduce(double (&v)[G], double *sm) {
    const int kx = blockDim.x, r = threadIdx.x, ty = threadIdx.y;
    const int tid = ty * kx + r, lane = tid & 31, warp = tid >> 5;
    if (kx < 32) {
        for (int o = kx; o < 32; o <<= 1)
#pragma unroll
            for (int g = 0; g < G; g++) v[g] += __shfl_xor_sync(0xffffffffu, v[g], o);
    }
    const int slots = kx < 32 ? 8 : (int)blockDim.y;      // warps, or rows of the block
    const bool rep = kx < 32 ? lane < kx : true;
    const int slot = kx < 32 ? warp : ty;
    if (rep)
#pragma unroll
        for (int g = 0; g < G; g++) sm[(g * slots + slot) * kx + r] = v[g];
    __syncthreads();
    double out[G];
    if (tid < kx) {
#pragma unroll
        for (int g = 0; g < G; g++) {
            double acc = 0;
            for (int q = 0; q < slots; q++) acc += sm[(g * slots + q) * kx + r];
            out[g] = acc;
        }
    }
    __syncthreads();
    if (tid < kx)
#pragma unroll
        for (int g = 0; g < G; g++) sm[g * 256 + r] = out[g];
    __syncthreads();
}

template <class T>
__global__ void __launch_bounds__(256) k_colsq_partial(const T *x, int64_t n, int k, double *partial) {
    __shared__ double sm[256];
    const int r = threadIdx.x, ty = threadIdx.y, ny = blockDim.y;
    T acc = 0;
    if (r < k)
        for (int64_t i = blockIdx.x * (int64_t)ny + ty; i < n; i += (int64_t)gridDim.x * ny) {
            T v = x[i * k + r];
            acc += v * v;
        }
    double v[1] = {(double)acc};
    block_col_reduce<1>(v, sm);
    if (ty == 0 && r < k) partial[(int64_t)r * gridDim.x + blockIdx.x] = sm[r];
}

// One warp per output: lane l adds partials l, l + 32, ... in order, then a
// fixed xor tree combines the lanes (an FP64 add chain over all nb partials
// in one thread costs tens of microseconds on this part).
constexpr int kReduceWarps = 8;
__global__ void __launch_bounds__(32 * kReduceWarps) k_reduce_partials(const double *partial, int nb, int cnt,
                                                                       double *out, bool take_sqrt) {
    const int c = blockIdx.x * kReduceWarps + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (c >= cnt) return;
    const double *p = partial + (int64_t)c * nb;
    double s = 0;
    for (int b = lane; b < nb; b += 32) s += p[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) out[c] = take_sqrt ? sqrt(s) : s;
}
static inline unsigned reduce_grid(int cnt) { return (unsigned)((cnt + kReduceWarps - 1) / kReduceWarps); }

template <class T>
void colnorms(const T *x, int64_t n, int k, double *partial, double *out, cudaStream_t s) {
    const int cpr = chunk_cpr<T>(k);
    if (cpr && cpr <= 16) {
        (g2p::kbegin("k_colsq_partial", s), k_colsq_partial_v<T><<<kRedBlocks, dim3(cpr, 256 / cpr), 0, s>>>(x, n, k, partial), g2p::kend(s));
    } else {
        int kx = pow2_ge(k);
        dim3 blk(kx, 256 / kx);
        (g2p::kbegin("k_colsq_partial", s), k_colsq_partial<T><<<kRedBlocks, blk, 0, s>>>(x, n, k, partial), g2p::kend(s));
    }
    (g2p::kbegin("k_reduce_partials", s), k_reduce_partials<<<reduce_grid(k), 32 * kReduceWarps, 0, s>>>(partial, kRedBlocks, k, out, true), g2p::kend(s));
}
template void colnorms<double>(const double *, int64_t, int, double *, double *, cudaStream_t);
template void colnorms<float>(const float *, int64_t, int, double *, double *, cudaStream_t);

// dots[j*k + r] = <V_j[:, r], w[:, r]> for j < J, eight basis vectors per pass
// over w; block partials are reduced in a fixed order.
constexpr int kDotGroup = 8;
template <class T, int G>
__global__ void __launch_bounds__(256) k_mdot_partial(const T *V, int64_t n, int j0, const T *w, int k,
                                                      double *partial) {
    __shared__ double sm[G][256];
    const int r = threadIdx.x, ty = threadIdx.y, ny = blockDim.y;
    const int64_t nk = n * k;
    T acc[G];
#pragma unroll
    for (int g = 0; g < G; g++) acc[g] = 0;
    if (r < k)
        for (int64_t i = blockIdx.x * (int64_t)ny + ty; i < n; i += (int64_t)gridDim.x * ny) {
            int64_t t = i * k + r;
            T wv = w[t];
#pragma unroll
            for (int g = 0; g < G; g++) acc[g] += V[(int64_t)(j0 + g) * nk + t] * wv;
        }
    double v[G];
#pragma unroll
    for (int g = 0; g < G; g++) v[g] = (double)acc[g];
    block_col_reduce<G>(v, &sm[0][0]);
    for (int idx = ty * blockDim.x + r; idx < G * (int)blockDim.x; idx += blockDim.x * blockDim.y) {
        int g = idx / blockDim.x, rr = idx % blockDim.x;
        if (rr < k) partial[((int64_t)(j0 + g) * k + rr) * gridDim.x + blockIdx.x] = sm[g][rr];
    }
}

// w -= sum_j h[j*k + r] V_j ; also h_acc += h (for reorthogonalisation)
template <class T>
__global__ void __launch_bounds__(256) k_maxpy(const T *V, int64_t n, int J, const double *h, int k, T *w) {
    const int r = threadIdx.x;
    if (r >= k) return;
    const int64_t nk = n * k;
    T hr[64];
    for (int j = 0; j < J; j++) hr[j] = (T)h[j * k + r];
    G2P_FOR_ROWS(i, n) {
        int64_t t = i * k + r;
        T acc = w[t];
        for (int j = 0; j < J; j++) acc -= hr[j] * V[(int64_t)j * nk + t];
        w[t] = acc;
    }
}

// ---------------------------------------------------------------- smoothing
template <class T>
__global__ void k_cheb_first(int64_t n, int k, const T *dinv, const T *b, T *x, T *d, double inv_theta, bool add) {
    const int r = threadIdx.x;
    if (r >= k) return;
    G2P_FOR_ROWS(i, n) {
        // add == false: x0 = 0 so the residual is b; add == true: b holds b - A x
        int64_t t = i * k + r;
        T dd = (T)inv_theta * dinv[i] * b[t];
        d[t] = dd;
        x[t] = add ? x[t] + dd : dd;
    }
}

// d = c1 d + c2 D^-1 (b - A x) with t = b - A x precomputed; x += d
template <class T>
__global__ void k_cheb_step(int64_t n, int k, const T *dinv, const T *res, T *x, T *d, double c1, double c2) {
    const int r = threadIdx.x;
    if (r >= k) return;
    const T a = (T)c1, b = (T)c2;
    G2P_FOR_ROWS(i, n) {
        int64_t t = i * k + r;
        T dd = a * d[t] + b * dinv[i] * res[t];
        d[t] = dd;
        x[t] = x[t] + dd;
    }
}

template <class T>
static void chebyshev(Level<T> &L, int deg, double ratio, double upper, const T *b, T *x, bool zero_guess, int k,
                      cudaStream_t s) {
    double lmax = L.lmax * upper, lmin = L.lmax * ratio;
    double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
    double sigma = theta / delta, rho = 1.0 / sigma;
    unsigned g = row_grid(L.n, k);
    dim3 blk = row_block(k);
    const int cpr = chunk_cpr<T>(k);
    const int64_t nq = L.n * cpr;
    const int shift = cpr ? __builtin_ctz(cpr) : 0;
    // the chunked kernels store only what later steps read: a zero-guess
    // first step of a smoother of degree >= 2 leaves its iterate in d alone
    // (x == d there), and the last step does not store d (the next smoother
    // call starts it afresh); the arithmetic is unchanged
    auto first = [&](const T *src, bool add, bool stx, bool std_) {
        const double it_ = 1.0 / theta;
        if (cpr) {
            g2p::kbegin("k_cheb_first", s);
            const unsigned cg = chunk_grid(nq);
            if (stx && std_) k_cheb_first_v<T, true, true><<<cg, 256, 0, s>>>(nq, shift, L.dinv, src, x, L.d, it_, add);
            else if (stx) k_cheb_first_v<T, true, false><<<cg, 256, 0, s>>>(nq, shift, L.dinv, src, x, L.d, it_, add);
            else k_cheb_first_v<T, false, true><<<cg, 256, 0, s>>>(nq, shift, L.dinv, src, x, L.d, it_, add);
            g2p::kend(s);
        } else {
            (g2p::kbegin("k_cheb_first", s), k_cheb_first<T><<<g, blk, 0, s>>>(L.n, k, L.dinv, src, x, L.d, it_, add), g2p::kend(s));
        }
    };
    bool x_in_d = false;
    if (zero_guess) {
        x_in_d = cpr && deg >= 2;
        first(b, false, !x_in_d, deg >= 2);
    } else {
        spmm_b<T>(L.A, L.lr, x, L.t0, k, b, s);
        first(L.t0, true, true, deg >= 2);
    }
    for (int it = 1; it < deg; it++) {
        spmm_b<T>(L.A, L.lr, x_in_d ? L.d : x, L.t0, k, b, s);
        double rn = 1.0 / (2.0 * sigma - rho);
        const double c1 = rn * rho, c2 = 2.0 * rn / delta;
        const bool last = it == deg - 1;
        if (cpr) {
            g2p::kbegin("k_cheb_step", s);
            const unsigned cg = chunk_grid(nq);
            if (x_in_d && last) k_cheb_step_v<T, true, false><<<cg, 256, 0, s>>>(nq, shift, L.dinv, L.t0, x, L.d, c1, c2);
            else if (x_in_d) k_cheb_step_v<T, true, true><<<cg, 256, 0, s>>>(nq, shift, L.dinv, L.t0, x, L.d, c1, c2);
            else if (last) k_cheb_step_v<T, false, false><<<cg, 256, 0, s>>>(nq, shift, L.dinv, L.t0, x, L.d, c1, c2);
            else k_cheb_step_v<T, false, true><<<cg, 256, 0, s>>>(nq, shift, L.dinv, L.t0, x, L.d, c1, c2);
            g2p::kend(s);
        } else {
            (g2p::kbegin("k_cheb_step", s), k_cheb_step<T><<<g, blk, 0, s>>>(L.n, k, L.dinv, L.t0, x, L.d, c1, c2), g2p::kend(s));
        }
        x_in_d = false;
        rho = rn;
    }
}

// b_c[I] = sum over members i of I of (b_i - (A x)_i)  (t0 holds b - A x)
template <class T>
__global__ void k_restrict(int64_t nc, int k, const int64_t *rptr, const int32_t *rmem, const T *res, T *bc) {
    const int r = threadIdx.x;
    if (r >= k) return;
    G2P_FOR_ROWS(I, nc) {
        T acc = 0;
        for (int64_t q = rptr[I]; q < rptr[I + 1]; q++) acc += res[(int64_t)rmem[q] * k + r];
        bc[I * k + r] = acc;
    }
}


// x = A_c^-1 b on the coarsest level: one warp per (row, right-hand side);
// lane l takes columns l, l + 32, ... and a fixed xor tree combines them.
template <class T>
__global__ void __launch_bounds__(256) k_dense_apply(int64_t n, int k, const double *Ainv, const T *b, T *x) {
    const int64_t wid = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= n * k) return;
    const int64_t i = wid / k;
    const int r = (int)(wid % k);
    const double *a = Ainv + i * n;
    double acc = 0;
    for (int64_t j = lane; j < n; j += 32) acc += a[j] * (double)b[j * k + r];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (lane == 0) x[i * k + r] = (T)acc;
}

template <class T>
__global__ void k_prolong_csr(int64_t n, int k, const int64_t *ptr, const int32_t *col, const T *val, const T *xc, T *x) {
    const int r = threadIdx.x;
    if (r >= k) return;
    G2P_FOR_ROWS(i, n) {
        int64_t t = i * k + r;
        T acc = x[t];
        for (int64_t q = ptr[i]; q < ptr[i + 1]; q++) acc += val[q] * xc[(int64_t)col[q] * k + r];
        x[t] = acc;
    }
}

// One V-cycle on level l: x = M_l^-1 b.  Level 0 runs on the caller's
// vectors (the Krylov basis vector in, the preconditioned vector out), the
// coarser levels on their own work vectors.
// x += y over n * k entries
template <class T>
__global__ void k_vec_add(int64_t nk, const T *y, T *x) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x)
        x[i] += y[i];
}

template <class T>
static void vcycle(Hierarchy<T> &H, const SolverConfig &cfg, int l, int k, cudaStream_t s, const T *b, T *x) {
    if (l > 0 && l == H.fuse_from) {       // b, x are the level's own vectors
        coarse_cycle<T>(H, k, s);
        return;
    }
    Level<T> &L = H.lv[l];
    if (l == (int)H.lv.size() - 1) {
        if (H.cinv) (g2p::kbegin("k_dense_apply", s), k_dense_apply<T><<<(unsigned)((L.n * k * 32 + 255) / 256), 256, 0, s>>>(L.n, k, H.cinv, b, x), g2p::kend(s));
        else {
            chebyshev<T>(L, 4, cfg.cheb_ratio, cfg.cheb_upper, b, x, true, k, s);
            for (int q = 0; q < 4; q++) chebyshev<T>(L, 4, cfg.cheb_ratio, cfg.cheb_upper, b, x, false, k, s);
        }
        return;
    }
    chebyshev<T>(L, cfg.degree, cfg.cheb_ratio, cfg.cheb_upper, b, x, true, k, s);
    spmm_b<T>(L.A, L.lr, x, L.t0, k, b, s);
    Level<T> &C = H.lv[l + 1];
    if (const int cpr = chunk_cpr<T>(k))
        (g2p::kbegin("k_restrict", s), k_restrict_v<T><<<chunk_grid(C.n * cpr), 256, 0, s>>>(C.n, __builtin_ctz(cpr), k, L.rptr, L.rmem, L.t0, C.b), g2p::kend(s));
    else
        (g2p::kbegin("k_restrict", s), k_restrict<T><<<row_grid(C.n, k), row_block(k), 0, s>>>(C.n, k, L.rptr, L.rmem, L.t0, C.b), g2p::kend(s));
    vcycle<T>(H, cfg, l + 1, k, s, C.b, C.x);
    // G2P_COARSE_CYCLES=n (comparison): n - 1 further cycles of the first
    // coarse level on its residual, through the fine level's scratch
    // vectors (free between restriction and prolongation)
    if (l == 0 && H.lv.size() > 2) {
        static const int extra = getenv("G2P_COARSE_CYCLES") ? atoi(getenv("G2P_COARSE_CYCLES")) - 1 : 0;
        for (int c = 0; c < extra; c++) {
            spmm_b<T>(C.A, C.lr, C.x, L.t0, k, C.b, s);
            vcycle<T>(H, cfg, l + 1, k, s, L.t0, L.d);
            (g2p::kbegin("k_vec_add", s), k_vec_add<T><<<grid_for(C.n * k), kThreads, 0, s>>>(C.n * k, L.d, C.x), g2p::kend(s));
        }
    }
    if (L.P.sptr) prolong_sell<T>(L.P, C.x, x, k, s);
    else (g2p::kbegin("k_prolong_csr", s), k_prolong_csr<T><<<row_grid(L.n, k), row_block(k), 0, s>>>(L.n, k, L.P.ptr, L.P.col, L.P.val, C.x, x), g2p::kend(s));
    chebyshev<T>(L, cfg.degree, cfg.cheb_ratio, cfg.cheb_upper, b, x, false, k, s);
}

// ------------------------------------------------------------- AMG setup
// Position of the diagonal in row i (columns ascending; linear fallback).
__device__ __forceinline__ int64_t diag_pos(const int64_t *ptr, const int32_t *col, int64_t i) {
    int64_t lo = ptr[i], hi = ptr[i + 1] - 1;
    while (lo <= hi) {
        int64_t mid = (lo + hi) >> 1;
        int32_t c = col[mid];
        if (c == i) return mid;
        if (c < i) lo = mid + 1; else hi = mid - 1;
    }
    for (int64_t q = ptr[i]; q < ptr[i + 1]; q++) if (col[q] == i) return q;
    return -1;
}

__global__ void k_diag(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, double *diag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t q = diag_pos(ptr, col, i);
        diag[i] = q >= 0 ? val[q] : 0.0;
    }
}

// 1/a_ii and the Gershgorin radius max_i sum_j |a_ij| / |a_ii| of D^-1 A;
// rows longer than kLongRow are summed by k_gersh_long.
// Non-negative doubles order like their bit patterns, so a maximum can be
// kept as an unsigned integer; one atomic per warp.
__device__ __forceinline__ void warp_atomic_max(unsigned long long *dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    if ((threadIdx.x & 31) == 0 && v) atomicMax(dst, v);
}

__global__ void k_dinv_gersh(int64_t n, const int64_t *ptr, const double *val, const double *diag, double *dinv,
                             unsigned long long *lmax_bits) {
    unsigned long long m = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double d = diag[i];
        if (d == 0.0) d = 1.0;
        dinv[i] = 1.0 / d;
        if (ptr[i + 1] - ptr[i] > kLongRow) continue;
        double s = 0;
        for (int64_t q = ptr[i]; q < ptr[i + 1]; q++) s += fabs(val[q]);
        const unsigned long long b = (unsigned long long)__double_as_longlong(s / fabs(d));
        m = b > m ? b : m;
    }
    warp_atomic_max(lmax_bits, m);
}

__global__ void __launch_bounds__(256) k_gersh_long(const int32_t *rows, const int64_t *ptr, const double *val,
                                                    const double *diag, unsigned long long *lmax_bits) {
    __shared__ double sm[256];
    int64_t i = rows[blockIdx.x];
    double s = 0;
    for (int64_t q = ptr[i] + threadIdx.x; q < ptr[i + 1]; q += blockDim.x) s += fabs(val[q]);
    sm[threadIdx.x] = s;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sm[threadIdx.x] += sm[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double d = diag[i];
        if (d == 0.0) d = 1.0;
        atomicMax(lmax_bits, (unsigned long long)__double_as_longlong(sm[0] / fabs(d)));
    }
}

// row containing entry q (ptr ascending)
__device__ __forceinline__ int64_t row_of(const int64_t *ptr, int64_t n, int64_t q) {
    int64_t lo = 0, hi = n - 1;
    while (lo < hi) {
        int64_t mid = (lo + hi + 1) >> 1;
        if (ptr[mid] <= q) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
    return x;
}

// strong(i, q) for entry q of row i
__device__ __forceinline__ bool strong(int64_t i, int64_t q, const int32_t *col, const double *val, const double *diag,
                                       const uint8_t *dense, double theta) {
    int32_t j = col[q];
    if (j == i || dense[j]) return false;
    return fabs(val[q]) >= theta * sqrt(fabs(diag[i] * diag[j]));
}

// dense flag and eligibility (state): 0 out/ineligible, 1 undecided
__global__ void k_agg_init(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, const double *diag,
                           int64_t lim, double theta, uint8_t *dense, uint64_t *T) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dense[i] = (ptr[i + 1] - ptr[i]) > lim ? 1 : 0;
}

// Strong-connection mask per entry, evaluated once per level:
// |a_ij| >= theta sqrt(|a_ii a_jj|), j != i, j not dense.  Dense rows are
// left unwritten; every reader skips them.
__global__ void k_strong_mask(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, const double *diag,
                              double theta, const uint8_t *dense, uint8_t *sm) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (dense[i]) continue;
        for (int64_t q = ptr[i]; q < ptr[i + 1]; q++) sm[q] = strong(i, q, col, val, diag, dense, theta) ? 1 : 0;
    }
}

__global__ void k_agg_state(int64_t n, const int64_t *ptr, const uint8_t *sm, const uint8_t *dense, uint64_t *T) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        bool elig = false;
        if (!dense[i])
            for (int64_t q = ptr[i]; q < ptr[i + 1]; q++)
                if (sm[q]) { elig = true; break; }
        uint64_t st = elig ? 1ull : 0ull;
        T[i] = (st << 62) | ((uint64_t)(hash32((uint32_t)i * 2654435761u + 12345u) & 0x3fffffffu) << 32) | (uint64_t)(uint32_t)i;
    }
}

__global__ void k_mis_max(int64_t n, const int64_t *ptr, const int32_t *col, const uint8_t *sm, const uint8_t *dense,
                          const uint64_t *in, uint64_t *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t m = in[i];
        if (!dense[i])
            for (int64_t q = ptr[i]; q < ptr[i + 1]; q++)
                if (sm[q]) { uint64_t v = in[col[q]]; m = v > m ? v : m; }
        out[i] = m;
    }
}

__global__ void k_mis_update(int64_t n, uint64_t *T, const uint64_t *M, int *undecided) {
    int cnt = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t t = T[i];
        if ((t >> 62) != 1) continue;
        uint64_t m = M[i];
        if (m == t) T[i] = (t & ~(3ull << 62)) | (2ull << 62);           // IN
        else if ((m >> 62) == 2) T[i] = t & ~(3ull << 62);              // OUT (state 0)
        else cnt++;
    }
    if (cnt) atomicAdd(undecided, cnt);
}

// roots: IN nodes and dense rows
__global__ void k_root_flag(int64_t n, const uint64_t *T, const uint8_t *dense, int64_t *flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = ((T[i] >> 62) == 2 || dense[i]) ? 1 : 0;
}

__global__ void k_agg_phase1(int64_t n, const int64_t *ptr, const int32_t *col, const uint8_t *sm, const uint8_t *dense,
                             const uint64_t *T, const int64_t *rootid, int32_t *agg1) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        uint64_t t = T[i];
        if ((t >> 62) == 2 || dense[i]) { agg1[i] = (int32_t)rootid[i]; continue; }
        // eligible nodes were set IN or OUT; an OUT node with a strong root
        // neighbour joins the highest-priority one
        uint64_t best = 0;
        int64_t bj = -1;
        for (int64_t q = ptr[i]; q < ptr[i + 1]; q++) {
            if (!sm[q]) continue;
            uint64_t v = T[col[q]];
            if ((v >> 62) == 2 && v > best) { best = v; bj = col[q]; }
        }
        agg1[i] = bj >= 0 ? (int32_t)rootid[bj] : -2;
    }
}

__global__ void k_agg_phase2(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, const uint8_t *sm,
                             const int32_t *agg1, int32_t *agg) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t a = agg1[i];
        if (a != -2) { agg[i] = a; continue; }
        bool elig = false;
        double best = -1;
        int32_t ba = -1;
        for (int64_t q = ptr[i]; q < ptr[i + 1]; q++) {
            if (!sm[q]) continue;
            elig = true;
            int32_t aj = agg1[col[q]];
            if (aj >= 0 && fabs(val[q]) > best) { best = fabs(val[q]); ba = aj; }
        }
        agg[i] = elig ? ba : -1;
    }
}

// RAP of the piecewise-constant prolongation: expand (agg_i, agg_j, a_ij)
__global__ void k_rap_count(int64_t n, const int64_t *ptr, const int32_t *col, const int32_t *agg, int64_t *cnt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = 0;
        if (agg[i] >= 0)
            for (int64_t q = ptr[i]; q < ptr[i + 1]; q++) c += agg[col[q]] >= 0;
        cnt[i] = c;
    }
}

__global__ void k_rap_expand(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, const int32_t *agg,
                             const int64_t *off, uint64_t nc, uint64_t *keys, double *vals) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t ai = agg[i];
        if (ai < 0) continue;
        int64_t o = off[i];
        for (int64_t q = ptr[i]; q < ptr[i + 1]; q++) {
            int32_t aj = agg[col[q]];
            if (aj < 0) continue;
            keys[o] = (uint64_t)ai * nc + (uint64_t)aj;
            vals[o] = val[q];
            o++;
        }
    }
}

__global__ void k_heads64(const uint64_t *keys, int64_t n, int64_t *head) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        head[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

// Segmented sums of the sorted expansion, deterministic: segments of at
// most kSegShort entries are summed in order by one thread, longer ones
// (the coarse conductor couplings) by a block in a fixed tree order.
constexpr int64_t kSegShort = 32;

__global__ void k_seg_start(const int64_t *head, const int64_t *segid, int64_t ne, int64_t nseg, int64_t *sstart) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ne; i += (int64_t)gridDim.x * blockDim.x)
        if (head[i]) sstart[segid[i]] = i;
    if (blockIdx.x == 0 && threadIdx.x == 0) sstart[nseg] = ne;
}

__global__ void k_seg_short(const uint64_t *keys, const double *vals, int64_t nseg, const int64_t *sstart, uint64_t nc,
                            int32_t *ocol, double *oval, int64_t *longlist, unsigned long long *nlong) {
    for (int64_t sg = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sg < nseg; sg += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = sstart[sg], e = sstart[sg + 1];
        ocol[sg] = (int32_t)(keys[b] % nc);
        if (e - b <= kSegShort) {
            double acc = 0;
            for (int64_t j = b; j < e; j++) acc += vals[j];
            oval[sg] = acc;
        } else {
            longlist[atomicAdd(nlong, 1ull)] = sg;
        }
    }
}

__global__ void __launch_bounds__(256) k_seg_long(const double *vals, const int64_t *sstart, const int64_t *longlist,
                                                  const unsigned long long *nlong, double *oval) {
    __shared__ double sm[256];
    const int64_t nl = (int64_t)*nlong;
    for (int64_t li = blockIdx.x; li < nl; li += gridDim.x) {
        const int64_t sg = longlist[li];
        const int64_t b = sstart[sg], e = sstart[sg + 1];
        double acc = 0;
        for (int64_t j = b + threadIdx.x; j < e; j += 256) acc += vals[j];
        sm[threadIdx.x] = acc;
        __syncthreads();
        for (int w = 128; w > 0; w >>= 1) {
            if (threadIdx.x < w) sm[threadIdx.x] += sm[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) oval[sg] = sm[0];
        __syncthreads();
    }
}

// Row offsets of the reduced matrix: keys are sorted by (row, column).
__global__ void k_seg_rowptr(const uint64_t *keys, const int64_t *sstart, int64_t nseg, uint64_t nc, int64_t nrows,
                             int64_t *ptr) {
    for (int64_t sg = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sg <= nseg; sg += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = sg < nseg ? (int64_t)(keys[sstart[sg]] / nc) : nrows;
        const int64_t rp = sg > 0 ? (int64_t)(keys[sstart[sg - 1]] / nc) : -1;
        for (int64_t a = rp + 1; a <= r; a++) ptr[a] = sg;
    }
}

__global__ void k_agg_key(int64_t n, const int32_t *agg, const int64_t *pos, uint32_t *key, int32_t *node) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (agg[i] >= 0) { key[pos[i]] = (uint32_t)agg[i]; node[pos[i]] = (int32_t)i; }
}

__global__ void k_member_ptr(int64_t m, const uint32_t *skey, int64_t nc, int64_t *rptr) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= m; i += (int64_t)gridDim.x * blockDim.x) {
        // rptr[a] = first position with key >= a
        if (i == 0) { for (int64_t a = 0; a <= (m > 0 ? skey[0] : nc - 1) && a < nc; a++) rptr[a] = 0; }
        else if (i == m) { for (int64_t a = skey[m - 1] + 1; a <= nc; a++) rptr[a] = m; }
        else if (skey[i] != skey[i - 1]) { for (int64_t a = skey[i - 1] + 1; a <= skey[i]; a++) rptr[a] = i; }
    }
}

__global__ void k_dense_fill(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, double *Dm) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int64_t q = ptr[i]; q < ptr[i + 1]; q++) Dm[i * n + col[q]] += val[q];
}

// Gauss-Jordan inversion with partial pivoting.  Step kk reads (a_in,
// inv_in) and writes (a_out, inv_out), so no block waits on another within a
// step: block i owns row i, repeats the (cheap) pivot search of column kk
// itself -- largest |a_ik|, i >= kk, the first one on ties -- and writes its
// row after the swap of rows kk and p and the elimination.  Columns of a at
// or left of kk are never read again and are not written.  bv, bi: 256
// doubles and indices of shared memory.
__device__ __forceinline__ void gj_step(const double *a_in, const double *inv_in, double *a_out, double *inv_out,
                                        int64_t n, int64_t kk, int *singular, double *bv, int64_t *bi) {
    const int t = threadIdx.x;
    double mv = -1.0;
    int64_t mi = n;
    for (int64_t r = kk + t; r < n; r += blockDim.x) {
        const double v = fabs(a_in[r * n + kk]);
        if (v > mv) { mv = v; mi = r; }
    }
    bv[t] = mv; bi[t] = mi;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o && (bv[t + o] > bv[t] || (bv[t + o] == bv[t] && bi[t + o] < bi[t]))) { bv[t] = bv[t + o]; bi[t] = bi[t + o]; }
        __syncthreads();
    }
    const int64_t p = bi[0];
    double pval = a_in[p * n + kk];
    if (pval == 0.0) {
        if (blockIdx.x == 0 && t == 0) *singular = 1;
        pval = 1e-300;
    }
    const int64_t i = blockIdx.x;
    const int64_t src = i == kk ? p : (i == p ? kk : i);     // row i after the swap
    const double f = i == kk ? 0.0 : a_in[src * n + kk];
    for (int64_t c = kk + 1 + t; c < n; c += blockDim.x) {
        const double pr = a_in[p * n + c] / pval;
        a_out[i * n + c] = i == kk ? pr : a_in[src * n + c] - f * pr;
    }
    for (int64_t c = t; c < n; c += blockDim.x) {
        const double pr = inv_in[p * n + c] / pval;
        inv_out[i * n + c] = i == kk ? pr : inv_in[src * n + c] - f * pr;
    }
}

// One launch per pivot step over the whole GPU.
__global__ void __launch_bounds__(256) k_gj_step(const double *__restrict__ a_in, const double *__restrict__ inv_in,
                                                 double *__restrict__ a_out, double *__restrict__ inv_out, int64_t n,
                                                 int64_t kk, int *singular) {
    __shared__ double bv[256];
    __shared__ int64_t bi[256];
    gj_step(a_in, inv_in, a_out, inv_out, n, kk, singular, bv, bi);
}

// All n pivot steps in one cooperative launch (one block per row, every
// block resident), with a grid-wide barrier between steps instead of a
// launch.  Buffers ping-pong as in the per-step loop; the inverse ends in
// inv1 when n is odd, inv0 otherwise.  flags[0] is the singular flag,
// flags[1] the barrier's arrival count and flags[2] set when a block gave up
// waiting (bounded spin: spin_limit polls of 64 ns or more), in which case
// the caller recomputes with one launch per pivot.
constexpr int kGjSpinLimit = 1 << 22;
__global__ void __launch_bounds__(256) k_gj_coop(double *a0, double *inv0, double *a1, double *inv1, int64_t n,
                                                 int *flags, int spin_limit) {
    __shared__ double bv[256];
    __shared__ int64_t bi[256];
    __shared__ int quit;
    const int t = threadIdx.x;
    unsigned *arrived = reinterpret_cast<unsigned *>(flags + 1);
    volatile int *abandon = flags + 2;
    for (int64_t kk = 0; kk < n; kk++) {
        const bool odd = kk & 1;
        gj_step(odd ? a1 : a0, odd ? inv1 : inv0, odd ? a0 : a1, odd ? inv0 : inv1, n, kk, flags, bv, bi);
        // grid barrier: every block's writes of step kk before any read of step kk+1
        __syncthreads();
        if (t == 0) {
            __threadfence();
            atomicAdd(arrived, 1u);
            const unsigned target = (unsigned)((kk + 1) * gridDim.x);
            int it = 0, q = 0;
            while (*(volatile unsigned *)arrived < target) {
                if (*abandon || ++it > spin_limit) { *abandon = 1; q = 1; break; }
                __nanosleep(64);
            }
            __threadfence();
            quit = q;
        }
        __syncthreads();
        if (quit) return;
    }
}

__global__ void k_identity(double *m, int64_t n) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n * n; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = t / n;
        m[t] = (t - r * n == r) ? 1.0 : 0.0;
    }
}


// Smoothed prolongation row i: T row plus -w/a_ii * sum_j a_ij T row j,
// columns deduplicated in first-seen order then sorted.
constexpr int kPsMax = kLongRow + 1;
__device__ __forceinline__ int ps_row(int64_t i, const int64_t *ptr, const int32_t *col, const double *val,
                                      const double *diag, const int32_t *agg, double w, int32_t *cols, double *vals) {
    int nr = 0;
    int32_t ai = agg[i];
    if (ai >= 0) { cols[0] = ai; vals[0] = 1.0; nr = 1; }
    int64_t s0 = ptr[i], s1 = ptr[i + 1];
    if (s1 - s0 > kLongRow || diag[i] == 0.0) return nr;
    double f = -w / diag[i];
    for (int64_t q = s0; q < s1; q++) {
        int32_t aj = agg[col[q]];
        if (aj < 0) continue;
        int t = 0;
        while (t < nr && cols[t] != aj) t++;
        if (t == nr) { cols[nr] = aj; vals[nr] = 0.0; nr++; }
        vals[t] += f * val[q];
    }
    for (int a = 1; a < nr; a++) {
        int32_t c = cols[a]; double v = vals[a];
        int b = a - 1;
        while (b >= 0 && cols[b] > c) { cols[b + 1] = cols[b]; vals[b + 1] = vals[b]; b--; }
        cols[b + 1] = c; vals[b + 1] = v;
    }
    return nr;
}

__global__ void k_ps_count(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, const double *diag,
                           const int32_t *agg, double w, int64_t *cnt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t cols[kPsMax];
        double vals[kPsMax];
        cnt[i] = ps_row(i, ptr, col, val, diag, agg, w, cols, vals);
    }
}

__global__ void k_ps_fill(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, const double *diag,
                          const int32_t *agg, double w, const int64_t *pptr, int32_t *pcol, double *pval) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int32_t cols[kPsMax];
        double vals[kPsMax];
        int nr = ps_row(i, ptr, col, val, diag, agg, w, cols, vals);
        int64_t o = pptr[i];
        for (int t = 0; t < nr; t++) { pcol[o + t] = cols[t]; pval[o + t] = vals[t]; }
    }
}

// (T^T A): rows of A summed by aggregate; key agg(i) * n + j
__global__ void k_ta_count(int64_t n, const int64_t *ptr, const int32_t *agg, int64_t *cnt) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        cnt[i] = agg[i] >= 0 ? ptr[i + 1] - ptr[i] : 0;
}
__global__ void k_ta_expand(int64_t n, int64_t nnz, const int64_t *ptr, const int32_t *col, const double *val,
                            const int32_t *agg, const int64_t *off, uint64_t ncols, uint64_t *keys, double *vals) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x) {
        int64_t i = row_of(ptr, n, q);
        int32_t a = agg[i];
        if (a < 0) continue;
        int64_t o = off[i] + (q - ptr[i]);
        keys[o] = (uint64_t)a * ncols + (uint64_t)col[q];
        vals[o] = val[q];
    }
}
// (T^T A) P: key I * nc + J
// (T^T A) P, one thread per entry of B = T^T A; off[q] = output offset
__global__ void k_bp_expand(int64_t nr, int64_t nnzb, const int64_t *bptr, const int32_t *bcol, const double *bval,
                            const int64_t *pptr, const int32_t *pcol, const double *pval, const int64_t *off,
                            uint64_t nc, uint64_t *keys, double *vals) {
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < nnzb; q += (int64_t)gridDim.x * blockDim.x) {
        int64_t I = row_of(bptr, nr, q);
        int64_t j = bcol[q];
        double b = bval[q];
        int64_t o = off[q];
        for (int64_t t = pptr[j]; t < pptr[j + 1]; t++, o++) {
            keys[o] = (uint64_t)I * nc + (uint64_t)pcol[t];
            vals[o] = b * pval[t];
        }
    }
}

template <class T>
void Hierarchy<T>::release(cudaStream_t s) {
    if (fuse_tab) cudaFree(fuse_tab);
    if (fuse_bar) cudaFree(fuse_bar);
    if (fuse_trace) cudaFree(fuse_trace);
    fuse_tab = nullptr;
    fuse_bar = nullptr;
    fuse_trace = nullptr;
    fuse_from = -1;
    fuse_key.clear();
    for (auto &L : lv) {
        L.A.release(s);
        L.P.release(s);
        L.lr.release(s); dfree(L.dinv, s); dfree(L.agg, s); dfree(L.rptr, s); dfree(L.rmem, s);
        dfree(L.x, s); dfree(L.b, s); dfree(L.t0, s); dfree(L.t1, s); dfree(L.d, s);
    }
    lv.clear();
    dfree(cinv, s);
    kcap = 0;
}
template struct Hierarchy<double>;
template struct Hierarchy<float>;

static int key_bits(uint64_t v) {
    int b = 0;
    while (b < 64 && (v >> b) != 0) b++;
    return b < 8 ? 8 : ((b + 7) / 8) * 8;
}

// Sorted, ordered reduction of expanded (key, value) pairs into a CSR with
// nrows rows and key = row * ncols + col.
static g2p_status esc_to_csr(uint64_t *&k0, double *&v0, int64_t ne, int64_t nrows, int64_t ncols, cudaStream_t s,
                             Csr<double> &out) {
    uint64_t *k1;
    double *v1;
    G2P_TRY(dalloc(&k1, ne, s));
    G2P_TRY(dalloc(&v1, ne, s));
    int64_t *counts, *work;
    int64_t wn = scan_work_size(std::max(sort_counts_size(ne), ne + 1) + nrows + 1) + 8;
    G2P_TRY(dalloc(&counts, sort_counts_size(ne), s));
    G2P_TRY(dalloc(&work, wn, s));
    bool in1 = false;
    G2P_TRY(radix_sort_pairs(k0, v0, k1, v1, ne, key_bits((uint64_t)nrows * (uint64_t)ncols), counts, work, &in1, s));
    dfree(counts, s);
    uint64_t *sk = in1 ? k1 : k0;
    double *sv = in1 ? v1 : v0;
    int64_t *head, *segid;
    G2P_TRY(dalloc(&head, ne + 1, s));
    G2P_TRY(dalloc(&segid, ne + 1, s));
    (g2p::kbegin("k_heads64", s), k_heads64<<<grid_for(ne), kThreads, 0, s>>>(sk, ne, head), g2p::kend(s));
    const int64_t *hp = head;
    auto hop = [hp, ne] __device__(int64_t i) -> int64_t { return i < ne ? hp[i] : 0; };
    G2P_TRY(exclusive_scan(hop, ne + 1, segid, work, s));
    int64_t nseg = 0;
    G2P_CUDA(cudaMemcpyAsync(&nseg, segid + ne, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    out.n = nrows; out.m = ncols; out.nnz = nseg;
    G2P_TRY(dalloc(&out.col, nseg, s)); G2P_TRY(dalloc(&out.val, nseg, s)); G2P_TRY(dalloc(&out.ptr, nrows + 1, s));
    int64_t *sstart, *longlist;
    unsigned long long *nlong;
    G2P_TRY(dalloc(&sstart, nseg + 1, s));
    G2P_TRY(dalloc(&longlist, ne / (kSegShort + 1) + 1, s));
    G2P_TRY(dalloc(&nlong, 1, s));
    G2P_CUDA(cudaMemsetAsync(nlong, 0, sizeof(unsigned long long), s));
    (g2p::kbegin("k_seg_start", s), k_seg_start<<<grid_for(ne), kThreads, 0, s>>>(head, segid, ne, nseg, sstart), g2p::kend(s));
    (g2p::kbegin("k_seg_short", s), k_seg_short<<<grid_for(nseg), kThreads, 0, s>>>(sk, sv, nseg, sstart, (uint64_t)ncols, out.col, out.val, longlist, nlong), g2p::kend(s));
    (g2p::kbegin("k_seg_long", s), k_seg_long<<<kSMs * 4, 256, 0, s>>>(sv, sstart, longlist, nlong, out.val), g2p::kend(s));
    if (nseg > 0) {
        (g2p::kbegin("k_seg_rowptr", s), k_seg_rowptr<<<grid_for(nseg + 1), kThreads, 0, s>>>(sk, sstart, nseg, (uint64_t)ncols, nrows, out.ptr), g2p::kend(s));
    } else {
        G2P_CUDA(cudaMemsetAsync(out.ptr, 0, sizeof(int64_t) * (nrows + 1), s));
    }
    G2P_CUDA(cudaStreamSynchronize(s));
    dfree(sstart, s); dfree(longlist, s); dfree(nlong, s);
    dfree(head, s); dfree(segid, s); dfree(work, s);
    dfree(k0, s); dfree(k1, s); dfree(v0, s); dfree(v1, s);
    k0 = nullptr; v0 = nullptr;
    return G2P_OK;
}

// Row lengths -> offsets (exclusive scan); returns the total.
static g2p_status offsets_of(const int64_t *cnt, int64_t n, int64_t *off, cudaStream_t s, int64_t *total) {
    int64_t *work;
    G2P_TRY(dalloc(&work, scan_work_size(n + 1) + 4, s));
    auto op = [cnt, n] __device__(int64_t i) -> int64_t { return i < n ? cnt[i] : 0; };
    G2P_TRY(exclusive_scan(op, n + 1, off, work, s));
    G2P_CUDA(cudaMemcpyAsync(total, off + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    dfree(work, s);
    return G2P_OK;
}

// ---- Galerkin product A_c = T^T A P, one coarse row per warp: shared-
// memory hash tables accumulate B = T^T A's row (member rows in ascending
// order, one row at a time) and then A_c's row (B's entries in ascending
// column order, one at a time), so every sum is taken in a fixed order.
// Only the unique columns are sorted.  Rows whose unique columns overflow
// the table are flagged and built by expand-sort-compress over those rows.
constexpr int kRapTable = 256;            // hash slots per warp (power of two)
constexpr int kRapWarps = 4;              // warps per block (24 KB of shared memory)
struct RapWarpMem {
    int32_t hkey[kRapTable];
    double hval[kRapTable];
    int32_t bcol[kRapTable];
    double bval[kRapTable];
    int32_t flag;
};

template <class F>
__global__ void k_for_each(int64_t n, F f) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) f(i);
}

// w1 = entries of a member row, w2 = its products with the rows of P (rows
// longer than kLongRow: w2 from k_rap_rowcount_long)
__global__ void k_rap_rowcount(int64_t n, const int64_t *ptr, const int32_t *col, const int32_t *agg,
                               const int64_t *pptr, int64_t *w1, int64_t *w2) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t a = 0, b = 0;
        if (agg[i] >= 0) {
            a = ptr[i + 1] - ptr[i];
            if (a <= kLongRow)
                for (int64_t q = ptr[i]; q < ptr[i + 1]; q++) b += pptr[col[q] + 1] - pptr[col[q]];
        }
        w1[i] = a;
        w2[i] = b;
    }
}
__global__ void __launch_bounds__(256) k_rap_rowcount_long(const int32_t *rows, const int64_t *ptr, const int32_t *col,
                                                           const int32_t *agg, const int64_t *pptr, int64_t *w2) {
    __shared__ int64_t sm[8];
    const int64_t i = rows[blockIdx.x];
    if (agg[i] < 0) return;
    int64_t b = 0;
    for (int64_t q = ptr[i] + threadIdx.x; q < ptr[i + 1]; q += blockDim.x) b += pptr[col[q] + 1] - pptr[col[q]];
    for (int o = 16; o > 0; o >>= 1) b += __shfl_xor_sync(0xffffffffu, b, o);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = b;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sm[w];
        w2[i] = t;
    }
}
// m1 = member entries, m2 = product count (bounds of B's and A_c's row)
__global__ void k_rap_aggcount(int64_t nc, const int64_t *rptr, const int32_t *rmem, const int64_t *w1,
                               const int64_t *w2, int64_t *m1, int64_t *m2) {
    for (int64_t I = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; I < nc; I += (int64_t)gridDim.x * blockDim.x) {
        int64_t a = 0, b = 0;
        for (int64_t q = rptr[I]; q < rptr[I + 1]; q++) { a += w1[rmem[q]]; b += w2[rmem[q]]; }
        m1[I] = a;
        m2[I] = b;
    }
}

// Adds v to key's slot (inserting the key); false when the table is full.
// The lanes of one call hold distinct keys.
__device__ __forceinline__ bool rap_add(RapWarpMem &w, int32_t key, double v) {
    static_assert(kRapTable == 256, "hash shift below assumes 256 slots");
    uint32_t h = ((uint32_t)key * 2654435761u) >> (32 - 8);
    for (int probe = 0; probe < kRapTable; probe++) {
        const uint32_t slot = (h + probe) & (kRapTable - 1);
        const int32_t old = atomicCAS(&w.hkey[slot], -1, key);
        if (old == -1 || old == key) {
            w.hval[slot] += v;
            return true;
        }
    }
    return false;
}

// Compacts the table into (bcol, bval) sorted by column; returns the count.
__device__ int rap_collect(RapWarpMem &w) {
    const int lane = threadIdx.x & 31;
    int n = 0;
    for (int s0 = 0; s0 < kRapTable; s0 += 32) {
        const int slot = s0 + lane;
        const bool used = w.hkey[slot] != -1;
        const unsigned b = __ballot_sync(0xffffffffu, used);
        if (used) {
            const int o = n + __popc(b & ((1u << lane) - 1u));
            w.bcol[o] = w.hkey[slot];
            w.bval[o] = w.hval[slot];
        }
        n += __popc(b);
    }
    int np = 1;
    while (np < n) np <<= 1;
    for (int t = n + lane; t < np; t += 32) { w.bcol[t] = 0x7fffffff; w.bval[t] = 0; }
    __syncwarp();
    for (int kk = 2; kk <= np; kk <<= 1)
        for (int j = kk >> 1; j > 0; j >>= 1) {
            for (int i = lane; i < np; i += 32) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const int32_t a = w.bcol[i], c = w.bcol[ixj];
                    if ((a > c) == ((i & kk) == 0)) {
                        w.bcol[i] = c; w.bcol[ixj] = a;
                        const double t = w.bval[i]; w.bval[i] = w.bval[ixj]; w.bval[ixj] = t;
                    }
                }
            }
            __syncwarp();
        }
    return n;
}

__device__ __forceinline__ void rap_clear(RapWarpMem &w) {
    const int lane = threadIdx.x & 31;
    for (int t = lane; t < kRapTable; t += 32) { w.hkey[t] = -1; w.hval[t] = 0; }
    if (lane == 0) w.flag = 0;
    __syncwarp();
}

__global__ void __launch_bounds__(32 * kRapWarps) k_rap_hash(int64_t nc, const int64_t *m1, const int64_t *rptr, const int32_t *rmem,
                                                             const int64_t *aptr, const int32_t *acol,
                                                             const double *aval, const int64_t *pptr,
                                                             const int32_t *pcol, const double *pval,
                                                             const int64_t *off2, int32_t *tcol, double *tval,
                                                             int64_t *nnz, uint8_t *over) {
    __shared__ RapWarpMem mem[kRapWarps];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    RapWarpMem &w = mem[warp];
    for (int64_t I = (int64_t)blockIdx.x * kRapWarps + warp; I < nc; I += (int64_t)gridDim.x * kRapWarps) {
        // a member row longer than the table cannot fit (its columns are
        // distinct): such rows (conductor potentials) go to the sort path
        if (m1[I] > kRapTable) {
            bool longrow = false;
            for (int64_t q = rptr[I] + lane; q < rptr[I + 1]; q += 32)
                longrow |= aptr[rmem[q] + 1] - aptr[rmem[q]] > kRapTable;
            if (__any_sync(0xffffffffu, longrow)) { if (lane == 0) over[I] = 1; __syncwarp(); continue; }
        }
        // ---- B row I: member rows in ascending order, one at a time
        rap_clear(w);
        bool ok = true;
        for (int64_t q = rptr[I]; q < rptr[I + 1] && ok; q++) {
            const int64_t i = rmem[q], b0 = aptr[i], len = aptr[i + 1] - b0;
            for (int64_t t0 = 0; t0 < len && ok; t0 += 32) {
                const int64_t t = t0 + lane;
                const bool fit = t >= len || rap_add(w, acol[b0 + t], aval[b0 + t]);
                ok = __all_sync(0xffffffffu, fit);
            }
            __syncwarp();
        }
        if (!ok) { if (lane == 0) over[I] = 1; __syncwarp(); continue; }
        const int nb = rap_collect(w);
        // ---- A_c row I: B's entries in ascending column order, one at a time
        for (int t = lane; t < kRapTable; t += 32) { w.hkey[t] = -1; w.hval[t] = 0; }
        __syncwarp();
        for (int r = 0; r < nb && ok; r++) {
            const int64_t j = w.bcol[r], pb = pptr[j], pl = pptr[j + 1] - pb;
            const double bv = w.bval[r];
            for (int64_t t0 = 0; t0 < pl && ok; t0 += 32) {
                const int64_t t = t0 + lane;
                const bool fit = t >= pl || rap_add(w, pcol[pb + t], bv * pval[pb + t]);
                ok = __all_sync(0xffffffffu, fit);
            }
            __syncwarp();
        }
        if (!ok) { if (lane == 0) over[I] = 1; __syncwarp(); continue; }
        const int nout = rap_collect(w);
        const int64_t o = off2[I];
        for (int t = lane; t < nout; t += 32) { tcol[o + t] = w.bcol[t]; tval[o + t] = w.bval[t]; }
        if (lane == 0) { nnz[I] = nout; over[I] = 0; }
        __syncwarp();
    }
}

// Expansion of T^T A for the listed aggregates: keys h * n + column in
// member-then-entry order, one block per aggregate.
__global__ void __launch_bounds__(256) k_rap_expand_list(const int64_t *list, const int64_t *off, const int64_t *rptr,
                                                         const int32_t *rmem, const int64_t *aptr, const int32_t *acol,
                                                         const double *aval, uint64_t n, uint64_t *keys, double *vals) {
    const int64_t h = blockIdx.x, I = list[h];
    int64_t o = off[h];
    for (int64_t q = rptr[I]; q < rptr[I + 1]; q++) {
        const int64_t i = rmem[q], b0 = aptr[i], len = aptr[i + 1] - b0;
        for (int64_t t = threadIdx.x; t < len; t += blockDim.x) {
            keys[o + t] = (uint64_t)h * n + (uint64_t)acol[b0 + t];
            vals[o + t] = aval[b0 + t];
        }
        o += len;
    }
}
// Row h of the listed aggregates' product to its place among the coarse
// rows, one block per row (these rows are the long ones).
__global__ void k_rap_place(const int64_t *list, const int64_t *cptr, const int32_t *ccol, const double *cval,
                            const int64_t *off2, int32_t *tcol, double *tval, int64_t *nnz) {
    const int64_t h = blockIdx.x, I = list[h], b = cptr[h], len = cptr[h + 1] - b, o = off2[I];
    for (int64_t t = threadIdx.x; t < len; t += blockDim.x) { tcol[o + t] = ccol[b + t]; tval[o + t] = cval[b + t]; }
    if (threadIdx.x == 0) nnz[I] = len;
}
// Coarse rows to their final places: one warp per row of at most kRapTable
// entries (the table's rows); longer rows by k_rap_compact_list.
__global__ void k_rap_compact(int64_t nc, const int64_t *off2, const int64_t *ptr, const int32_t *tcol,
                              const double *tval, int32_t *col, double *val) {
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    for (int64_t I = w; I < nc; I += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const int64_t src = off2[I], dst = ptr[I], len = ptr[I + 1] - dst;
        if (len > kRapTable) continue;
        for (int64_t t = lane; t < len; t += 32) { col[dst + t] = tcol[src + t]; val[dst + t] = tval[src + t]; }
    }
}
__global__ void k_rap_compact_list(const int64_t *list, const int64_t *off2, const int64_t *ptr, const int32_t *tcol,
                                   const double *tval, int32_t *col, double *val) {
    const int64_t I = list[blockIdx.x], src = off2[I], dst = ptr[I], len = ptr[I + 1] - dst;
    if (len <= kRapTable) return;
    for (int64_t t = threadIdx.x; t < len; t += blockDim.x) { col[dst + t] = tcol[src + t]; val[dst + t] = tval[src + t]; }
}

// Indices I with flag[I] != 0, ascending; returns their count.
static g2p_status list_flagged(const uint8_t *flag, int64_t n, cudaStream_t s, int64_t **list, int64_t *count) {
    int64_t *pos, *work;
    G2P_TRY(dalloc(&pos, n + 1, s));
    G2P_TRY(dalloc(&work, scan_work_size(n + 1) + 4, s));
    auto op = [flag, n] __device__(int64_t i) -> int64_t { return i < n ? (flag[i] ? 1 : 0) : 0; };
    G2P_TRY(exclusive_scan(op, n + 1, pos, work, s));
    G2P_CUDA(cudaMemcpyAsync(count, pos + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    G2P_TRY(dalloc(list, std::max<int64_t>(*count, 1), s));
    int64_t *lp = *list;
    const int64_t *pp = pos;
    auto put = [flag, pp, lp] __device__(int64_t i) { if (flag[i]) lp[pp[i]] = i; };
    (g2p::kbegin("k_list_flagged", s), k_for_each<<<grid_for(n), kThreads, 0, s>>>(n, put), g2p::kend(s));
    dfree(pos, s); dfree(work, s);
    return G2P_OK;
}

// A_c = T^T A P: per coarse row in shared memory, and by expand-sort-
// compress over the rows whose unique columns overflow the table.
static g2p_status rap_rows(const Level<double> &L, int64_t n, int64_t nc, cudaStream_t s, Csr<double> &out) {
    int64_t *w1, *w2, *m1, *m2;
    G2P_TRY(dalloc(&w1, n, s)); G2P_TRY(dalloc(&w2, n, s));
    G2P_TRY(dalloc(&m1, nc, s)); G2P_TRY(dalloc(&m2, nc, s));
    (g2p::kbegin("k_rap_rowcount", s), k_rap_rowcount<<<grid_for(n), kThreads, 0, s>>>(n, L.A.ptr, L.A.col, L.agg, L.P.ptr, w1, w2), g2p::kend(s));
    if (L.lr.n > 0)
        (g2p::kbegin("k_rap_rowcount_long", s), k_rap_rowcount_long<<<(unsigned)L.lr.n, 256, 0, s>>>(L.lr.rows, L.A.ptr, L.A.col, L.agg, L.P.ptr, w2), g2p::kend(s));
    (g2p::kbegin("k_rap_aggcount", s), k_rap_aggcount<<<grid_for(nc), kThreads, 0, s>>>(nc, L.rptr, L.rmem, w1, w2, m1, m2), g2p::kend(s));
    dfree(w1, s); dfree(w2, s);
    int64_t *off2, ne2 = 0;
    G2P_TRY(dalloc(&off2, nc + 1, s));
    G2P_TRY(offsets_of(m2, nc, off2, s, &ne2));
    dfree(m2, s);
    int32_t *tcol;
    double *tval;
    int64_t *nnzr;
    uint8_t *over;
    G2P_TRY(dalloc(&tcol, std::max<int64_t>(ne2, 1), s)); G2P_TRY(dalloc(&tval, std::max<int64_t>(ne2, 1), s));
    G2P_TRY(dalloc(&nnzr, nc, s)); G2P_TRY(dalloc(&over, nc, s));
    {
        const int64_t g = std::min<int64_t>((nc + kRapWarps - 1) / kRapWarps, (int64_t)kSMs * 64);
        (g2p::kbegin("k_rap_hash", s), k_rap_hash<<<(unsigned)std::max<int64_t>(g, 1), 32 * kRapWarps, 0, s>>>(
             nc, m1, L.rptr, L.rmem, L.A.ptr, L.A.col, L.A.val, L.P.ptr, L.P.col, L.P.val, off2, tcol, tval, nnzr, over),
         g2p::kend(s));
    }
    int64_t *hl, nh = 0;
    G2P_TRY(list_flagged(over, nc, s, &hl, &nh));
    dfree(over, s);
    if (nh > 0) {
        // B_h = T^T A over the flagged aggregates (rows renumbered 0..nh-1)
        int64_t *cnt, *off1, ne1 = 0;
        G2P_TRY(dalloc(&cnt, nh, s)); G2P_TRY(dalloc(&off1, nh + 1, s));
        const int64_t *hp = hl, *m1p = m1;
        int64_t *cp = cnt;
        auto gcnt = [hp, m1p, cp] __device__(int64_t h) { cp[h] = m1p[hp[h]]; };
        (g2p::kbegin("k_rap_hcount", s), k_for_each<<<grid_for(nh), kThreads, 0, s>>>(nh, gcnt), g2p::kend(s));
        G2P_TRY(offsets_of(cnt, nh, off1, s, &ne1));
        dfree(cnt, s);
        uint64_t *ek0;
        double *ev0;
        G2P_TRY(dalloc(&ek0, std::max<int64_t>(ne1, 1), s)); G2P_TRY(dalloc(&ev0, std::max<int64_t>(ne1, 1), s));
        (g2p::kbegin("k_rap_expand_list", s), k_rap_expand_list<<<(unsigned)nh, 256, 0, s>>>(hl, off1, L.rptr, L.rmem, L.A.ptr, L.A.col, L.A.val, (uint64_t)n, ek0, ev0), g2p::kend(s));
        dfree(off1, s);
        Csr<double> B;
        G2P_TRY(esc_to_csr(ek0, ev0, ne1, nh, n, s, B));
        // C_h = B_h P
        int64_t *off, ne = 0;
        G2P_TRY(dalloc(&off, B.nnz + 1, s));
        {
            int64_t *wk;
            G2P_TRY(dalloc(&wk, scan_work_size(B.nnz + 1) + 4, s));
            const int32_t *bc = B.col;
            const int64_t *pp = L.P.ptr;
            int64_t nb = B.nnz;
            auto pop = [bc, pp, nb] __device__(int64_t q) -> int64_t { return q < nb ? pp[bc[q] + 1] - pp[bc[q]] : 0; };
            G2P_TRY(exclusive_scan(pop, nb + 1, off, wk, s));
            G2P_CUDA(cudaMemcpyAsync(&ne, off + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
            G2P_CUDA(cudaStreamSynchronize(s));
            dfree(wk, s);
        }
        G2P_TRY(dalloc(&ek0, std::max<int64_t>(ne, 1), s)); G2P_TRY(dalloc(&ev0, std::max<int64_t>(ne, 1), s));
        (g2p::kbegin("k_bp_expand", s), k_bp_expand<<<grid_for(B.nnz), kThreads, 0, s>>>(nh, B.nnz, B.ptr, B.col, B.val, L.P.ptr, L.P.col, L.P.val, off, (uint64_t)nc, ek0, ev0), g2p::kend(s));
        dfree(off, s);
        B.release(s);
        Csr<double> Ch;
        G2P_TRY(esc_to_csr(ek0, ev0, ne, nh, nc, s, Ch));
        (g2p::kbegin("k_rap_place", s), k_rap_place<<<(unsigned)nh, 256, 0, s>>>(hl, Ch.ptr, Ch.col, Ch.val, off2, tcol, tval, nnzr), g2p::kend(s));
        Ch.release(s);
    }
    dfree(m1, s);
    out.n = nc; out.m = nc;
    G2P_TRY(dalloc(&out.ptr, nc + 1, s));
    int64_t nnz = 0;
    G2P_TRY(offsets_of(nnzr, nc, out.ptr, s, &nnz));
    out.nnz = nnz;
    G2P_TRY(dalloc(&out.col, std::max<int64_t>(nnz, 1), s)); G2P_TRY(dalloc(&out.val, std::max<int64_t>(nnz, 1), s));
    (g2p::kbegin("k_rap_compact", s), k_rap_compact<<<grid_for(nc * 32), kThreads, 0, s>>>(nc, off2, out.ptr, tcol, tval, out.col, out.val), g2p::kend(s));
    // rows longer than the table come only from the flagged aggregates
    if (nh > 0)
        (g2p::kbegin("k_rap_compact_list", s), k_rap_compact_list<<<(unsigned)nh, 256, 0, s>>>(hl, off2, out.ptr, tcol, tval, out.col, out.val), g2p::kend(s));
    dfree(hl, s);
    dfree(off2, s); dfree(tcol, s); dfree(tval, s); dfree(nnzr, s);
    return G2P_OK;
}

// Host wall time of setup phases, printed with G2P_DEBUG >= 2 (synchronizes).
struct PhaseClock {
    bool on = false;
    std::chrono::steady_clock::time_point t0;
    PhaseClock() {
        const char *e = getenv("G2P_DEBUG");
        on = e && atoi(e) >= 2;
        t0 = std::chrono::steady_clock::now();
    }
    void mark(const char *what, int level, cudaStream_t s) {
        if (!on) return;
        cudaStreamSynchronize(s);
        auto t = std::chrono::steady_clock::now();
        fprintf(stderr, "[g2p setup] L%d %-14s %8.3f ms\n", level, what,
                std::chrono::duration<double, std::milli>(t - t0).count());
        t0 = t;
    }
};

g2p_status amg_setup(const Csr<double> &A0, const SolverConfig &cfg, cudaStream_t s, int64_t *, Hierarchy<double> &H) {
    PhaseClock pc_;
    H.release(s);
    // level 0 owns a copy of the operator
    Level<double> L0;
    L0.n = A0.n;
    L0.A.n = L0.A.m = A0.n; L0.A.nnz = A0.nnz;
    G2P_TRY(dalloc(&L0.A.ptr, A0.n + 1, s)); G2P_TRY(dalloc(&L0.A.col, A0.nnz, s)); G2P_TRY(dalloc(&L0.A.val, A0.nnz, s));
    G2P_CUDA(cudaMemcpyAsync(L0.A.ptr, A0.ptr, sizeof(int64_t) * (A0.n + 1), cudaMemcpyDeviceToDevice, s));
    G2P_CUDA(cudaMemcpyAsync(L0.A.col, A0.col, sizeof(int32_t) * A0.nnz, cudaMemcpyDeviceToDevice, s));
    G2P_CUDA(cudaMemcpyAsync(L0.A.val, A0.val, sizeof(double) * A0.nnz, cudaMemcpyDeviceToDevice, s));
    H.lv.push_back(L0);
    int64_t *work = nullptr;
    int64_t work_n = 0;
    auto need_work = [&](int64_t n) -> g2p_status {
        int64_t w = scan_work_size(n) + 8;
        if (w > work_n) { dfree(work, s); G2P_TRY(dalloc(&work, w, s)); work_n = w; }
        return G2P_OK;
    };
    int *d_int = nullptr;
    unsigned long long *d_lmax = nullptr;
    G2P_TRY(dalloc(&d_int, 4, s));
    G2P_TRY(dalloc(&d_lmax, 1, s));
    for (int l = 0;; l++) {
        Level<double> &L = H.lv[l];
        int64_t n = L.n;
        double *diag;
        G2P_TRY(dalloc(&diag, n, s));
        G2P_TRY(dalloc(&L.dinv, n, s));
        (g2p::kbegin("k_diag", s), k_diag<<<grid_for(n), kThreads, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, diag), g2p::kend(s));
        G2P_CUDA(cudaMemsetAsync(d_lmax, 0, sizeof(unsigned long long), s));
        pc_.mark("start", l, s);
        G2P_TRY(find_long_rows<double>(L.A, L.lr, s));   // synchronizes
        pc_.mark("long rows", l, s);
        (g2p::kbegin("k_dinv_gersh", s), k_dinv_gersh<<<grid_for(n), kThreads, 0, s>>>(n, L.A.ptr, L.A.val, diag, L.dinv, d_lmax), g2p::kend(s));
        if (L.lr.n > 0) (g2p::kbegin("k_gersh_long", s), k_gersh_long<<<(unsigned)L.lr.n, 256, 0, s>>>(L.lr.rows, L.A.ptr, L.A.val, diag, d_lmax), g2p::kend(s));
        unsigned long long lb = 0;
        G2P_CUDA(cudaMemcpyAsync(&lb, d_lmax, sizeof(lb), cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        double lm;
        memcpy(&lm, &lb, sizeof(lm));
        L.lmax = lm > 0 ? lm : 2.0;
        pc_.mark("gershgorin", l, s);
        bool last = n <= cfg.coarse_size || l + 1 >= cfg.max_levels;
        if (!last) {
            // ---- aggregation
            int64_t lim = 32 + 4 * (L.A.nnz / (n > 0 ? n : 1));
            uint8_t *dense;
            uint64_t *T, *M1, *M2;
            G2P_TRY(dalloc(&dense, n, s)); G2P_TRY(dalloc(&T, n, s)); G2P_TRY(dalloc(&M1, n, s)); G2P_TRY(dalloc(&M2, n, s));
            unsigned g = grid_for(n);
            (g2p::kbegin("k_agg_init", s), k_agg_init<<<g, kThreads, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, diag, lim, cfg.strength, dense, T), g2p::kend(s));
            uint8_t *smask;
            G2P_TRY(dalloc(&smask, L.A.nnz, s));
            (g2p::kbegin("k_strong_mask", s), k_strong_mask<<<g, kThreads, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, diag, cfg.strength, dense, smask), g2p::kend(s));
            (g2p::kbegin("k_agg_state", s), k_agg_state<<<g, kThreads, 0, s>>>(n, L.A.ptr, smask, dense, T), g2p::kend(s));
            for (int round = 0; round < 200; round++) {
                (g2p::kbegin("k_mis_max", s), k_mis_max<<<g, kThreads, 0, s>>>(n, L.A.ptr, L.A.col, smask, dense, T, M1), g2p::kend(s));
                (g2p::kbegin("k_mis_max", s), k_mis_max<<<g, kThreads, 0, s>>>(n, L.A.ptr, L.A.col, smask, dense, M1, M2), g2p::kend(s));
                G2P_CUDA(cudaMemsetAsync(d_int, 0, sizeof(int), s));
                (g2p::kbegin("k_mis_update", s), k_mis_update<<<g, kThreads, 0, s>>>(n, T, M2, d_int), g2p::kend(s));
                int und = 0;
                G2P_CUDA(cudaMemcpyAsync(&und, d_int, sizeof(int), cudaMemcpyDeviceToHost, s));
                G2P_CUDA(cudaStreamSynchronize(s));
                if (und == 0) break;
            }
            pc_.mark("mis", l, s);
            int64_t *rootid;
            G2P_TRY(dalloc(&rootid, n + 1, s));
            G2P_TRY(need_work(n + 1));
            {
                const uint64_t *Tp = T;
                const uint8_t *dp = dense;
                auto rop = [Tp, dp, n] __device__(int64_t i) -> int64_t {
                    return i < n ? (((Tp[i] >> 62) == 2 || dp[i]) ? 1 : 0) : 0;
                };
                G2P_TRY(exclusive_scan(rop, n + 1, rootid, work, s));
            }
            int64_t nc = 0;
            G2P_CUDA(cudaMemcpyAsync(&nc, rootid + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
            int32_t *agg1;
            G2P_TRY(dalloc(&agg1, n, s));
            G2P_TRY(dalloc(&L.agg, n, s));
            (g2p::kbegin("k_agg_phase1", s), k_agg_phase1<<<g, kThreads, 0, s>>>(n, L.A.ptr, L.A.col, smask, dense, T, rootid, agg1), g2p::kend(s));
            (g2p::kbegin("k_agg_phase2", s), k_agg_phase2<<<g, kThreads, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, smask, agg1, L.agg), g2p::kend(s));
            G2P_CUDA(cudaStreamSynchronize(s));
            dfree(agg1, s); dfree(rootid, s); dfree(dense, s); dfree(smask, s); dfree(T, s); dfree(M1, s); dfree(M2, s);
            pc_.mark("aggregates", l, s);
            if (nc == 0 || nc > (n * 9) / 10) {
                dfree(L.agg, s);
                last = true;
            } else {
                // ---- member lists (aggregate -> rows, ascending)
                int64_t *pos;
                G2P_TRY(dalloc(&pos, n + 1, s));
                const int32_t *ag = L.agg;
                auto mop = [ag, n] __device__(int64_t i) -> int64_t { return i < n ? (ag[i] >= 0 ? 1 : 0) : 0; };
                G2P_TRY(exclusive_scan(mop, n + 1, pos, work, s));
                int64_t nm = 0;
                G2P_CUDA(cudaMemcpyAsync(&nm, pos + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
                G2P_CUDA(cudaStreamSynchronize(s));
                uint32_t *k0, *k1;
                int32_t *v0, *v1;
                G2P_TRY(dalloc(&k0, nm, s)); G2P_TRY(dalloc(&k1, nm, s)); G2P_TRY(dalloc(&v0, nm, s)); G2P_TRY(dalloc(&v1, nm, s));
                (g2p::kbegin("k_agg_key", s), k_agg_key<<<g, kThreads, 0, s>>>(n, L.agg, pos, k0, v0), g2p::kend(s));
                int64_t *counts;
                G2P_TRY(dalloc(&counts, sort_counts_size(nm), s));
                G2P_TRY(need_work(sort_counts_size(nm)));
                bool in1 = false;
                G2P_TRY(radix_sort_pairs(k0, v0, k1, v1, nm, key_bits((uint64_t)nc), counts, work, &in1, s));
                dfree(counts, s);
                G2P_TRY(dalloc(&L.rptr, nc + 1, s));
                (g2p::kbegin("k_member_ptr", s), k_member_ptr<<<grid_for(nm + 1), kThreads, 0, s>>>(nm, in1 ? k1 : k0, nc, L.rptr), g2p::kend(s));
                L.rmem = in1 ? v1 : v0;
                dfree(in1 ? v0 : v1, s);
                dfree(k0, s); dfree(k1, s); dfree(pos, s);
                pc_.mark("members", l, s);
                // ---- smoothed prolongation P = (I - w D^-1 A) T
                double w = cfg.psmooth / L.lmax;
                int64_t *pc;
                G2P_TRY(dalloc(&pc, n + 1, s));
                G2P_TRY(dalloc(&L.P.ptr, n + 1, s));
                (g2p::kbegin("k_ps_count", s), k_ps_count<<<g, kThreads, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, diag, L.agg, w, pc), g2p::kend(s));
                int64_t pnnz = 0;
                G2P_TRY(offsets_of(pc, n, L.P.ptr, s, &pnnz));
                dfree(pc, s);
                L.P.n = n; L.P.m = nc; L.P.nnz = pnnz;
                G2P_TRY(dalloc(&L.P.col, pnnz, s)); G2P_TRY(dalloc(&L.P.val, pnnz, s));
                (g2p::kbegin("k_ps_fill", s), k_ps_fill<<<g, kThreads, 0, s>>>(n, L.A.ptr, L.A.col, L.A.val, diag, L.agg, w, L.P.ptr, L.P.col, L.P.val), g2p::kend(s));
                pc_.mark("prolongation", l, s);
                // ---- A_c = T^T A P: per coarse row in shared memory, or
                // (G2P_RAP_ESC=1, for comparisons) by expand-sort-compress over
                // all rows
                Level<double> C;
                C.n = nc;
                if (!getenv("G2P_RAP_ESC")) {
                    G2P_TRY(rap_rows(L, n, nc, s, C.A));
                } else {
                    // ---- B = T^T A (nc x n)
                    int64_t *cnt, *off;
                    G2P_TRY(dalloc(&cnt, n + 1, s)); G2P_TRY(dalloc(&off, n + 1, s));
                    (g2p::kbegin("k_ta_count", s), k_ta_count<<<g, kThreads, 0, s>>>(n, L.A.ptr, L.agg, cnt), g2p::kend(s));
                    int64_t ne = 0;
                    G2P_TRY(offsets_of(cnt, n, off, s, &ne));
                    uint64_t *ek0;
                    double *ev0;
                    G2P_TRY(dalloc(&ek0, ne, s)); G2P_TRY(dalloc(&ev0, ne, s));
                    (g2p::kbegin("k_ta_expand", s), k_ta_expand<<<grid_for(L.A.nnz), kThreads, 0, s>>>(n, L.A.nnz, L.A.ptr, L.A.col, L.A.val, L.agg, off, (uint64_t)n, ek0, ev0), g2p::kend(s));
                    dfree(cnt, s); dfree(off, s);
                    Csr<double> B;
                    G2P_TRY(esc_to_csr(ek0, ev0, ne, nc, n, s, B));
                    pc_.mark("T^T A", l, s);
                    // ---- A_c = B P (nc x nc), entry-parallel over B
                    G2P_TRY(dalloc(&off, B.nnz + 1, s));
                    {
                        int64_t *wk;
                        G2P_TRY(dalloc(&wk, scan_work_size(B.nnz + 1) + 4, s));
                        const int32_t *bc = B.col;
                        const int64_t *pp = L.P.ptr;
                        int64_t nb = B.nnz;
                        auto pop = [bc, pp, nb] __device__(int64_t q) -> int64_t { return q < nb ? pp[bc[q] + 1] - pp[bc[q]] : 0; };
                        G2P_TRY(exclusive_scan(pop, nb + 1, off, wk, s));
                        G2P_CUDA(cudaMemcpyAsync(&ne, off + nb, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
                        G2P_CUDA(cudaStreamSynchronize(s));
                        dfree(wk, s);
                    }
                    G2P_TRY(dalloc(&ek0, ne, s)); G2P_TRY(dalloc(&ev0, ne, s));
                    (g2p::kbegin("k_bp_expand", s), k_bp_expand<<<grid_for(B.nnz), kThreads, 0, s>>>(nc, B.nnz, B.ptr, B.col, B.val, L.P.ptr, L.P.col, L.P.val, off, (uint64_t)nc, ek0, ev0), g2p::kend(s));
                    dfree(off, s);
                    B.release(s);
                    G2P_TRY(esc_to_csr(ek0, ev0, ne, nc, nc, s, C.A));
                }
                L.nc = nc;
                H.lv.push_back(C);
                pc_.mark("galerkin", l, s);
            }
        }
        dfree(diag, s);
        if (last) {
            Level<double> &Cl = H.lv[l];
            int64_t nn = Cl.n;
            H.nc = nn;
            if (nn > kMaxDenseCoarse || nn == 0) break;   // coarsest level solved by smoothing
            double *Dm;
            G2P_TRY(dalloc(&Dm, nn * nn, s));
            G2P_TRY(dalloc(&H.cinv, nn * nn, s));
            G2P_CUDA(cudaMemsetAsync(Dm, 0, sizeof(double) * nn * nn, s));
            (g2p::kbegin("k_dense_fill", s), k_dense_fill<<<grid_for(nn), kThreads, 0, s>>>(nn, Cl.A.ptr, Cl.A.col, Cl.A.val, Dm), g2p::kend(s));
            G2P_CUDA(cudaMemsetAsync(d_int, 0, 3 * sizeof(int), s));
            {
                double *a1, *i0, *i1;
                G2P_TRY(dalloc(&a1, nn * nn, s)); G2P_TRY(dalloc(&i0, nn * nn, s)); G2P_TRY(dalloc(&i1, nn * nn, s));
                (g2p::kbegin("k_identity", s), k_identity<<<grid_for(nn * nn), kThreads, 0, s>>>(i0, nn), g2p::kend(s));
                double *ain = Dm, *aout = a1, *iin = i0, *iout = i1;
                // one cooperative launch when every row's block fits on the
                // device at once, else (or with G2P_GJ_STEPS=1, for
                // comparisons) one launch per pivot
                int coop_attr = 0, dev = 0, per_sm = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&coop_attr, cudaDevAttrCooperativeLaunch, dev);
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gj_coop, 256, 0);
                bool coop = false;
                if (coop_attr && (int64_t)per_sm * kSMs >= nn && !getenv("G2P_GJ_STEPS")) {
                    int64_t nn_arg = nn;
                    // G2P_GJ_SPIN_LIMIT (comparisons only) shortens the
                    // barrier's patience so that the give-up path runs
                    int spin = kGjSpinLimit;
                    if (const char *e = getenv("G2P_GJ_SPIN_LIMIT")) spin = std::max(1, atoi(e));
                    void *args[] = {&ain, &iin, &aout, &iout, &nn_arg, &d_int, &spin};
                    g2p::kbegin("k_gj_coop", s);
                    coop = cudaLaunchCooperativeKernel((void *)k_gj_coop, dim3((unsigned)nn), dim3(256), args, 0, s) == cudaSuccess;
                    g2p::kend(s);
                    if (coop) {
                        int gave_up = 0;
                        G2P_CUDA(cudaMemcpyAsync(&gave_up, d_int + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
                        G2P_CUDA(cudaStreamSynchronize(s));
                        if (gave_up) {           // start again from A and I
                            if (getenv("G2P_DEBUG"))
                                fprintf(stderr, "[g2p] coarse inverse (n=%lld): the cooperative launch's barrier gave "
                                                "up; recomputed with one launch per pivot\n", (long long)nn);
                            coop = false;
                            G2P_CUDA(cudaMemsetAsync(d_int, 0, sizeof(int), s));
                            G2P_CUDA(cudaMemsetAsync(Dm, 0, sizeof(double) * nn * nn, s));
                            (g2p::kbegin("k_dense_fill", s), k_dense_fill<<<grid_for(nn), kThreads, 0, s>>>(nn, Cl.A.ptr, Cl.A.col, Cl.A.val, Dm), g2p::kend(s));
                            (g2p::kbegin("k_identity", s), k_identity<<<grid_for(nn * nn), kThreads, 0, s>>>(i0, nn), g2p::kend(s));
                        } else if (nn & 1) {
                            std::swap(ain, aout);
                            std::swap(iin, iout);
                        }
                    } else {
                        cudaGetLastError();
                    }
                }
                for (int64_t kk = 0; kk < nn && !coop; kk++) {
                    (g2p::kbegin("k_gj_step", s), k_gj_step<<<(unsigned)nn, 256, 0, s>>>(ain, iin, aout, iout, nn, kk, d_int), g2p::kend(s));
                    std::swap(ain, aout);
                    std::swap(iin, iout);
                }
                G2P_CUDA(cudaMemcpyAsync(H.cinv, iin, sizeof(double) * nn * nn, cudaMemcpyDeviceToDevice, s));
                G2P_CUDA(cudaStreamSynchronize(s));
                dfree(a1, s); dfree(i0, s); dfree(i1, s);
            }
            dfree(Dm, s);
            pc_.mark("coarse inverse", l, s);
            break;
        }
    }
    dfree(d_int, s); dfree(d_lmax, s); dfree(work, s);
    G2P_CUDA(cudaGetLastError());
    G2P_CUDA(cudaStreamSynchronize(s));
    return G2P_OK;
}

__global__ void k_d2f(const double *in, float *out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (float)in[i];
}

g2p_status amg_to_float(const Hierarchy<double> &H, cudaStream_t s, Hierarchy<float> &F) {
    F.release(s);
    for (size_t l = 0; l < H.lv.size(); l++) {
        const Level<double> &L = H.lv[l];
        Level<float> f;
        f.n = L.n; f.nc = L.nc; f.lmax = L.lmax;
        f.A.n = f.A.m = L.A.n; f.A.nnz = L.A.nnz;
        // structure is shared by copying (owned separately for simple release)
        G2P_TRY(dalloc(&f.A.ptr, L.A.n + 1, s)); G2P_TRY(dalloc(&f.A.col, L.A.nnz, s)); G2P_TRY(dalloc(&f.A.val, L.A.nnz, s));
        G2P_CUDA(cudaMemcpyAsync(f.A.ptr, L.A.ptr, sizeof(int64_t) * (L.A.n + 1), cudaMemcpyDeviceToDevice, s));
        G2P_CUDA(cudaMemcpyAsync(f.A.col, L.A.col, sizeof(int32_t) * L.A.nnz, cudaMemcpyDeviceToDevice, s));
        (g2p::kbegin("k_d2f", s), k_d2f<<<grid_for(L.A.nnz), kThreads, 0, s>>>(L.A.val, f.A.val, L.A.nnz), g2p::kend(s));
        G2P_TRY(dalloc(&f.dinv, L.n, s));
        (g2p::kbegin("k_d2f", s), k_d2f<<<grid_for(L.n), kThreads, 0, s>>>(L.dinv, f.dinv, L.n), g2p::kend(s));
        G2P_TRY(copy_long_rows(L.lr, f.lr, s));
        if (L.P.ptr) {
            f.P.n = L.P.n; f.P.m = L.P.m; f.P.nnz = L.P.nnz;
            G2P_TRY(dalloc(&f.P.ptr, L.P.n + 1, s)); G2P_TRY(dalloc(&f.P.col, L.P.nnz, s)); G2P_TRY(dalloc(&f.P.val, L.P.nnz, s));
            G2P_CUDA(cudaMemcpyAsync(f.P.ptr, L.P.ptr, sizeof(int64_t) * (L.P.n + 1), cudaMemcpyDeviceToDevice, s));
            G2P_CUDA(cudaMemcpyAsync(f.P.col, L.P.col, sizeof(int32_t) * L.P.nnz, cudaMemcpyDeviceToDevice, s));
            (g2p::kbegin("k_d2f", s), k_d2f<<<grid_for(L.P.nnz), kThreads, 0, s>>>(L.P.val, f.P.val, L.P.nnz), g2p::kend(s));
        }
        if (L.agg) {
            G2P_TRY(dalloc(&f.agg, L.n, s));
            G2P_CUDA(cudaMemcpyAsync(f.agg, L.agg, sizeof(int32_t) * L.n, cudaMemcpyDeviceToDevice, s));
            G2P_TRY(dalloc(&f.rptr, L.nc + 1, s));
            G2P_CUDA(cudaMemcpyAsync(f.rptr, L.rptr, sizeof(int64_t) * (L.nc + 1), cudaMemcpyDeviceToDevice, s));
            int64_t nm = 0;
            G2P_CUDA(cudaMemcpyAsync(&nm, L.rptr + L.nc, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
            G2P_CUDA(cudaStreamSynchronize(s));
            G2P_TRY(dalloc(&f.rmem, nm, s));
            G2P_CUDA(cudaMemcpyAsync(f.rmem, L.rmem, sizeof(int32_t) * nm, cudaMemcpyDeviceToDevice, s));
        }
        F.lv.push_back(f);
    }
    F.nc = H.nc;
    if (H.cinv) {
        G2P_TRY(dalloc(&F.cinv, H.nc * H.nc, s));
        G2P_CUDA(cudaMemcpyAsync(F.cinv, H.cinv, sizeof(double) * H.nc * H.nc, cudaMemcpyDeviceToDevice, s));
    }
    G2P_CUDA(cudaStreamSynchronize(s));
    return G2P_OK;
}

template <class T>
g2p_status hierarchy_reserve(Hierarchy<T> &H, int k, cudaStream_t s) {
    if (k <= H.kcap) return G2P_OK;
    for (size_t l = 0; l < H.lv.size(); l++) {
        Level<T> &L = H.lv[l];
        dfree(L.x, s); dfree(L.b, s); dfree(L.t0, s); dfree(L.t1, s); dfree(L.d, s);
        // level 0 works on the Krylov vectors directly and needs no x, b
        if (l > 0) { G2P_TRY(dalloc(&L.x, L.n * k, s)); G2P_TRY(dalloc(&L.b, L.n * k, s)); }
        G2P_TRY(dalloc(&L.t0, L.n * k, s)); G2P_TRY(dalloc(&L.d, L.n * k, s));
    }
    H.kcap = k;
    return G2P_OK;
}
template g2p_status hierarchy_reserve<double>(Hierarchy<double> &, int, cudaStream_t);
template g2p_status hierarchy_reserve<float>(Hierarchy<float> &, int, cudaStream_t);

// ------------------------------------------------------------------- FGMRES
template <class T>
void Krylov<T>::drop_graphs() {
    for (auto &st : steps)
        if (st.exec) cudaGraphExecDestroy(st.exec);
    steps.clear();
    graph_key.clear();
}

template <class T>
void Krylov<T>::release(cudaStream_t s) {
    drop_graphs();
    dfree(V, s); dfree(Z, s); dfree(w, s); dfree(r, s);
    dfree(H, s); dfree(cs, s); dfree(sn, s); dfree(g, s); dfree(y, s);
    dfree(beta, s); dfree(bnorm, s); dfree(partial, s); dfree(hcol, s); dfree(sc, s);
    if (h_est) cudaFreeHost(h_est);
    h_est = nullptr;
    dfree(bdev, s); dfree(bpart, s);
    if (bhost) cudaFreeHost(bhost);
    bhost = nullptr;
    bk = 0; bm = 0;
    n = 0; k = 0; m = 0;
}
template struct Krylov<double>;
template struct Krylov<float>;

template <class T>
g2p_status krylov_alloc(Krylov<T> &K, int64_t n, int k, int m, cudaStream_t s) {
    if (K.n == n && K.k >= k && K.m >= m) return G2P_OK;
    K.release(s);
    K.n = n; K.k = k; K.m = m;
    G2P_TRY(dalloc(&K.V, n * k * (m + 1), s));
    G2P_TRY(dalloc(&K.Z, n * k * m, s));
    G2P_TRY(dalloc(&K.w, n * k, s));
    G2P_TRY(dalloc(&K.r, n * k, s));
    G2P_TRY(dalloc(&K.H, (int64_t)k * (m + 1) * m, s));
    G2P_TRY(dalloc(&K.cs, (int64_t)k * m, s));
    G2P_TRY(dalloc(&K.sn, (int64_t)k * m, s));
    G2P_TRY(dalloc(&K.g, (int64_t)k * (m + 1), s));
    G2P_TRY(dalloc(&K.y, (int64_t)k * m, s));
    G2P_TRY(dalloc(&K.beta, k, s));
    G2P_TRY(dalloc(&K.bnorm, k, s));
    G2P_TRY(dalloc(&K.partial, (int64_t)kRedBlocks * k * (m + 2), s));
    G2P_TRY(dalloc(&K.hcol, (int64_t)k * (2 * m + 4), s));
    G2P_TRY(dalloc(&K.sc, (int64_t)k * (m + 1), s));
    G2P_CUDA(cudaMallocHost(&K.h_est, sizeof(double) * 2 * k));
    return G2P_OK;
}
template g2p_status krylov_alloc<double>(Krylov<double> &, int64_t, int, int, cudaStream_t);
template g2p_status krylov_alloc<float>(Krylov<float> &, int64_t, int, int, cudaStream_t);

template <class T>
__global__ void k_start(int64_t n, int k, const T *r, const double *beta, T *v0) {
    const int rr = threadIdx.x;
    if (rr >= k) return;
    double b = beta[rr];
    const T inv = b > 0 ? (T)(1.0 / b) : (T)0;
    G2P_FOR_ROWS(i, n) {
        int64_t t = i * k + rr;
        v0[t] = r[t] * inv;
    }
}

// hcol = [dots (j+1 per rhs); norm]; form V_{j+1}, update H, Givens, g
template <class T>
__global__ void k_arnoldi_finish(int64_t n, int k, const double *hnorm, const T *w, T *vnext) {
    const int r = threadIdx.x;
    if (r >= k) return;
    double h = hnorm[r];
    const T inv = h > 0 ? (T)(1.0 / h) : (T)0;
    G2P_FOR_ROWS(i, n) {
        int64_t t = i * k + r;
        vnext[t] = w[t] * inv;
    }
}

__global__ void k_givens(int k, int m, int j, const double *hdots, const double *hnorm, double *H, double *cs, double *sn,
                         double *g, const double *bnorm, double *est) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= k) return;
    double *Hr = H + (int64_t)r * (m + 1) * m;    // column-major (m+1) x m
    for (int i = 0; i <= j; i++) Hr[j * (m + 1) + i] = hdots[i * k + r];
    Hr[j * (m + 1) + j + 1] = hnorm[r];
    double *c = cs + (int64_t)r * m, *s = sn + (int64_t)r * m, *gr = g + (int64_t)r * (m + 1);
    for (int i = 0; i < j; i++) {
        double a = Hr[j * (m + 1) + i], b = Hr[j * (m + 1) + i + 1];
        Hr[j * (m + 1) + i] = c[i] * a + s[i] * b;
        Hr[j * (m + 1) + i + 1] = -s[i] * a + c[i] * b;
    }
    double a = Hr[j * (m + 1) + j], b = Hr[j * (m + 1) + j + 1];
    double rr = sqrt(a * a + b * b);
    c[j] = rr != 0 ? a / rr : 1.0;
    s[j] = rr != 0 ? b / rr : 0.0;
    Hr[j * (m + 1) + j] = rr;
    Hr[j * (m + 1) + j + 1] = 0.0;
    gr[j + 1] = -s[j] * gr[j];
    gr[j] = c[j] * gr[j];
    double bn = bnorm[r];
    est[r] = bn > 0 ? fabs(gr[j + 1]) / bn : 0.0;
}

__global__ void k_g_init(int k, int m, const double *beta, double *g) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= k) return;
    for (int i = 0; i <= m; i++) g[(int64_t)r * (m + 1) + i] = 0.0;
    g[(int64_t)r * (m + 1)] = beta[r];
}

__global__ void k_backsolve(int k, int m, int j, const double *H, const double *g, double *y) {
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= k) return;
    const double *Hr = H + (int64_t)r * (m + 1) * m;
    const double *gr = g + (int64_t)r * (m + 1);
    double *yr = y + (int64_t)r * m;
    for (int i = j - 1; i >= 0; i--) {
        double sacc = gr[i];
        for (int q = i + 1; q < j; q++) sacc -= Hr[q * (m + 1) + i] * yr[q];
        double d = Hr[i * (m + 1) + i];
        yr[i] = d != 0 ? sacc / d : 0.0;
    }
}

// x += sum_i Z_i y_i, and y is laid out [r * m + i]
template <class T>
__global__ void k_xupdate(int64_t n, int k, int m, int j, const T *Z, const double *y, T *x, const double *sc) {
    const int r = threadIdx.x;
    if (r >= k) return;
    const int64_t nk = n * k;
    T yr[64];
    // with the unnormalised basis Z_q holds s_q M^-1 V_q: its weight is y_q / s_q
    for (int q = 0; q < j; q++) {
        const double yq = y[(int64_t)r * m + q];
        const double sq = sc ? sc[(int64_t)q * k + r] : 1.0;
        yr[q] = (T)(sc ? (sq > 0 ? yq / sq : 0.0) : yq);
    }
    G2P_FOR_ROWS(i, n) {
        int64_t t = i * k + r;
        T acc = x[t];
        for (int q = 0; q < j; q++) acc += Z[(int64_t)q * nk + t] * yr[q];
        x[t] = acc;
    }
}

template <class T>
static void mdot(const T *V, int64_t n, int J, const T *w, int k, double *partial, double *out, cudaStream_t s) {
    const int cpr = chunk_cpr<T>(k);
    const bool vec = cpr && cpr <= 16;
    const dim3 vblk(vec ? cpr : 1, vec ? 256 / cpr : 1);
    const int kx = pow2_ge(k);
    const dim3 blk(kx, 256 / kx);
    for (int j0 = 0; j0 < J; j0 += kDotGroup) {
        const int g = J - j0 < kDotGroup ? J - j0 : kDotGroup;
        g2p::kbegin("k_mdot_partial", s);
#define G2P_MDOT_CASE(G)                                                                                  \
    case G:                                                                                               \
        if (vec) k_mdot_partial_v<T, G><<<kRedBlocks, vblk, 0, s>>>(V, n, j0, w, k, partial);             \
        else k_mdot_partial<T, G><<<kRedBlocks, blk, 0, s>>>(V, n, j0, w, k, partial);                    \
        break;
        switch (g) {
            G2P_MDOT_CASE(1) G2P_MDOT_CASE(2) G2P_MDOT_CASE(3) G2P_MDOT_CASE(4)
            G2P_MDOT_CASE(5) G2P_MDOT_CASE(6) G2P_MDOT_CASE(7) default: G2P_MDOT_CASE(8)
        }
#undef G2P_MDOT_CASE
        g2p::kend(s);
    }
    (g2p::kbegin("k_reduce_partials", s), k_reduce_partials<<<reduce_grid(J * k), 32 * kReduceWarps, 0, s>>>(partial, kRedBlocks, J * k, out, false), g2p::kend(s));
}

__global__ void k_add_vec(double *a, const double *b, int n) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] += b[i];
}

__global__ void k_d_to_f(int64_t nk, const double *a, float *b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (float)a[i];
}
__global__ void k_f_to_d(int64_t nk, const float *a, double *b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nk; i += (int64_t)gridDim.x * blockDim.x)
        b[i] = (double)a[i];
}

template <class T>
g2p_status fgmres(const Csr<T> &A, Hierarchy<T> &H, Krylov<T> &K, const T *b, T *x, int k, const SolverConfig &cfg,
                  const double *bnorm_override, cudaStream_t s, SolveReport &rep, const F32Precond *pc,
                  const LongRows *op_lr) {
    refresh_long_fork();
    if (cfg.block && !pc && block_krylov_supported<T>(k, b, x))
        return block_fgmres<T>(A, H, K, b, x, k, cfg, bnorm_override, s, rep, op_lr);
    const int64_t n = A.n, nk = n * k;
    const int m = cfg.restart;
    if (k < 1 || k > kMaxRhs) { set_last_message("block of %d right-hand sides (1..%d supported)", k, kMaxRhs); return G2P_ERR_INVALID; }
    if (pc && !std::is_same<T, double>::value) { set_last_message("FP32 preconditioning of an FP32 solve"); return G2P_ERR_INVALID; }
    G2P_TRY(krylov_alloc<T>(K, n, k, m, s));
    if (pc) G2P_TRY(hierarchy_reserve<float>(*pc->H, k, s));
    else G2P_TRY(hierarchy_reserve<T>(H, k, s));
    int fuse_from;
    if (pc) {
        G2P_TRY(coarse_prepare<float>(*pc->H, cfg, k, s));
        fuse_from = pc->H->fuse_from;
    } else {
        G2P_TRY(coarse_prepare<T>(H, cfg, k, s));
        fuse_from = H.fuse_from;
    }
    const LongRows &lr0 = op_lr ? *op_lr : (pc ? *pc->lr : H.lv[0].lr);
    // FP32 solves keep the basis unnormalised (W_0 = r, W_{j+1} = the
    // orthogonalised remainder, their column norms in K.sc): no norm pass and
    // no normalised copy per step.  Chunked vectors, Gram-Schmidt once.  The
    // V-cycle is linear, so Z_j holds s_j M^-1 V_j and w = A Z_j carries s_j;
    // the preconditioned operator is near the identity there, so the norms
    // stay of the order of the residual's.  Not in FP64: its Gram-Schmidt is
    // bound by the FP64 pipe, which the fused norm loads further (measured
    // slower); nor with an FP32 preconditioner of the scaled operator, whose
    // outputs are off the basis' scale by that factor per step.
    // (G2P_UNNORM_BASIS=0: the normalised basis, comparison)
    const char *une = getenv("G2P_UNNORM_BASIS");
    const bool unnorm_on = une ? atoi(une) != 0 : true;
    const bool unnorm = unnorm_on && sizeof(T) == 4 && chunk_cpr<T>(k) != 0 && !cfg.reorth;
    // CUDA graphs of the Arnoldi steps: off while kernels are being timed;
    // rebuilt when the block width, operator or preconditioner changes
    const bool graphs = cfg.use_graphs && !kprof_on() && !g_prof.on;
    if (graphs) {
        const void *hier = pc ? (const void *)pc->H : (const void *)&H;
        const int kcap = pc ? pc->H->kcap : H.kcap;
        const std::vector<const void *> key = {(const void *)(intptr_t)k, (const void *)A.val, hier,
                                               (const void *)(intptr_t)kcap, (const void *)(intptr_t)cfg.degree,
                                               (const void *)(intptr_t)cfg.reorth, pc ? (const void *)pc->in : nullptr,
                                               (const void *)(intptr_t)fuse_from, (const void *)(intptr_t)unnorm,
                                               (const void *)(intptr_t)long_fork_on()};
        if (K.graph_key != key || (int)K.steps.size() != m) {
            K.drop_graphs();
            K.graph_key = key;
            K.steps.resize(m);
        }
    }
    const unsigned rg = row_grid(n, k);
    const dim3 rb = row_block(k);
    const int cpr = chunk_cpr<T>(k);
    const int64_t nq = n * cpr;
    auto maxpy = [&](const double *h, int J) {
        if (cpr)
            (g2p::kbegin("k_maxpy", s), k_maxpy_v<T><<<chunk_grid(nq), 256, sizeof(T) * J * k, s>>>(nq, cpr, k, J, K.V, h, K.w), g2p::kend(s));
        else
            (g2p::kbegin("k_maxpy", s), k_maxpy<T><<<rg, rb, 0, s>>>(K.V, n, J, h, k, K.w), g2p::kend(s));
    };
    if (bnorm_override) G2P_CUDA(cudaMemcpyAsync(K.bnorm, bnorm_override, sizeof(double) * k, cudaMemcpyDeviceToDevice, s));
    else colnorms<T>(b, n, k, K.partial, K.bnorm, s);
    int it = 0;
    rep.converged = false;
    double *dots2 = K.hcol + (int64_t)k * (m + 1);
    T *const r0 = unnorm ? K.V : K.r;
    for (;;) {
        // r = b - A x ; beta = ||r||
        spmm_b<T>(A, lr0, x, r0, k, b, s);
        colnorms<T>(r0, n, k, K.partial, K.beta, s);
        G2P_CUDA(cudaMemcpyAsync(K.h_est, K.beta, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaMemcpyAsync(K.h_est + k, K.bnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        double worst = 0;
        for (int r = 0; r < k; r++) {
            double bn = K.h_est[k + r];
            double rel = bn > 0 ? K.h_est[r] / bn : 0.0;
            worst = std::max(worst, rel);
        }
        rep.rel_residual = worst;
        if (worst <= cfg.rtol) { rep.converged = true; break; }
        if (it >= cfg.maxit) break;
        if (unnorm) G2P_CUDA(cudaMemcpyAsync(K.sc, K.beta, sizeof(double) * k, cudaMemcpyDeviceToDevice, s));
        else if (cpr) (g2p::kbegin("k_start", s), k_scale_cols_v<T><<<chunk_grid(nq), 256, 0, s>>>(nq, cpr, K.beta, K.r, K.V), g2p::kend(s));
        else (g2p::kbegin("k_start", s), k_start<T><<<rg, rb, 0, s>>>(n, k, K.r, K.beta, K.V), g2p::kend(s));
        (g2p::kbegin("k_g_init", s), k_g_init<<<(k + 63) / 64, 64, 0, s>>>(k, m, K.beta, K.g), g2p::kend(s));
        int j = 0;
        for (; j < m && it < cfg.maxit; j++) {
            T *Vj = K.V + (int64_t)j * nk, *Zj = K.Z + (int64_t)j * nk;
            auto step = [&]() {
                // Z_j = M^-1 V_j (one V-cycle, in place on the basis vectors)
                if constexpr (std::is_same<T, double>::value) {
                    if (pc) {
                        (g2p::kbegin("k_d_to_f", s), k_d_to_f<<<grid_for(nk), kThreads, 0, s>>>(nk, Vj, pc->in), g2p::kend(s));
                        vcycle<float>(*pc->H, cfg, 0, k, s, pc->in, pc->out);
                        (g2p::kbegin("k_f_to_d", s), k_f_to_d<<<grid_for(nk), kThreads, 0, s>>>(nk, pc->out, Zj), g2p::kend(s));
                    } else {
                        vcycle<T>(H, cfg, 0, k, s, Vj, Zj);
                    }
                } else {
                    vcycle<T>(H, cfg, 0, k, s, Vj, Zj);
                }
                spmm<T>(A, lr0, Zj, K.w, k, s);
                double *est = K.y;        // scratch for the estimates (k values)
                if (unnorm) {
                    // classical Gram-Schmidt once against the unnormalised basis
                    mdot<T>(K.V, n, j + 1, K.w, k, K.partial, K.hcol, s);
                    const int nc = (j + 1) * k;
                    (g2p::kbegin("k_unnorm_coef", s), k_unnorm_coef<<<(nc + 127) / 128, 128, 0, s>>>(k, j, K.sc, K.hcol, dots2), g2p::kend(s));
                    const unsigned cg = chunk_grid(nq);
                    (g2p::kbegin("k_maxpy_norm", s),
                     k_maxpy_norm_v<T><<<cg, 256, sizeof(T) * nc, s>>>(nq, cpr, k, j + 1, K.V, dots2, K.w, K.V + (int64_t)(j + 1) * nk, K.partial),
                     g2p::kend(s));
                    (g2p::kbegin("k_reduce_partials", s), k_reduce_partials<<<reduce_grid(k), 32 * kReduceWarps, 0, s>>>(K.partial, (int)cg, k, K.sc + (int64_t)(j + 1) * k, true), g2p::kend(s));
                    (g2p::kbegin("k_unnorm_hnorm", s), k_unnorm_hnorm<<<(k + 63) / 64, 64, 0, s>>>(k, j, K.sc, K.beta), g2p::kend(s));
                    (g2p::kbegin("k_givens", s), k_givens<<<(k + 63) / 64, 64, 0, s>>>(k, m, j, K.hcol, K.beta, K.H, K.cs, K.sn, K.g, K.bnorm, est), g2p::kend(s));
                    cudaMemcpyAsync(K.h_est, est, sizeof(double) * k, cudaMemcpyDeviceToHost, s);
                    return;
                }
                // classical Gram-Schmidt, optionally twice
                mdot<T>(K.V, n, j + 1, K.w, k, K.partial, K.hcol, s);
                maxpy(K.hcol, j + 1);
                if (cfg.reorth) {
                    mdot<T>(K.V, n, j + 1, K.w, k, K.partial, dots2, s);
                    maxpy(dots2, j + 1);
                    (g2p::kbegin("k_add_vec", s), k_add_vec<<<((j + 1) * k + 255) / 256, 256, 0, s>>>(K.hcol, dots2, (j + 1) * k), g2p::kend(s));
                }
                double *hnorm = K.beta;   // reuse
                colnorms<T>(K.w, n, k, K.partial, hnorm, s);
                if (cpr) (g2p::kbegin("k_arnoldi_finish", s), k_scale_cols_v<T><<<chunk_grid(nq), 256, 0, s>>>(nq, cpr, hnorm, K.w, K.V + (int64_t)(j + 1) * nk), g2p::kend(s));
                else (g2p::kbegin("k_arnoldi_finish", s), k_arnoldi_finish<T><<<rg, rb, 0, s>>>(n, k, hnorm, K.w, K.V + (int64_t)(j + 1) * nk), g2p::kend(s));
                (g2p::kbegin("k_givens", s), k_givens<<<(k + 63) / 64, 64, 0, s>>>(k, m, j, K.hcol, hnorm, K.H, K.cs, K.sn, K.g, K.bnorm, est), g2p::kend(s));
                cudaMemcpyAsync(K.h_est, est, sizeof(double) * k, cudaMemcpyDeviceToHost, s);
            };
            if (graphs) {
                auto &st = K.steps[j];
                if (st.exec) {
                    G2P_CUDA(cudaGraphLaunch(st.exec, s));
                    launch_add(st.launches);
                } else if (st.seen && !st.failed) {
                    // second use of step j: capture it, then replay
                    const int64_t n0 = launch_count();
                    cudaGraph_t gr = nullptr;
                    bool ok = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
                    if (ok) step();
                    ok = cudaStreamEndCapture(s, &gr) == cudaSuccess && ok && gr != nullptr;
                    if (ok) ok = cudaGraphInstantiate(&st.exec, gr, 0) == cudaSuccess;
                    if (gr) cudaGraphDestroy(gr);
                    st.launches = launch_count() - n0;
                    launch_add(-st.launches);
                    if (ok) {
                        G2P_CUDA(cudaGraphLaunch(st.exec, s));
                        launch_add(st.launches);
                    } else {
                        cudaGetLastError();
                        st.exec = nullptr;
                        st.failed = true;
                        step();
                    }
                } else {
                    st.seen = true;
                    step();
                }
            } else {
                step();
            }
            G2P_CUDA(cudaGetLastError());
            G2P_CUDA(cudaStreamSynchronize(s));
            it++;
            double worst = 0;
            for (int r = 0; r < k; r++) worst = std::max(worst, K.h_est[r]);
            if (worst <= cfg.rtol) { j++; break; }
        }
        (g2p::kbegin("k_backsolve", s), k_backsolve<<<(k + 63) / 64, 64, 0, s>>>(k, m, j, K.H, K.g, K.y), g2p::kend(s));
        (g2p::kbegin("k_xupdate", s), k_xupdate<T><<<rg, rb, 0, s>>>(n, k, m, j, K.Z, K.y, x, unnorm ? K.sc : nullptr), g2p::kend(s));
    }
    rep.iterations = it;
    G2P_CUDA(cudaGetLastError());
    return G2P_OK;
}
template <class T>
void precond_vcycle(Hierarchy<T> &H, const SolverConfig &cfg, int k, cudaStream_t s, const T *b, T *x) {
    vcycle<T>(H, cfg, 0, k, s, b, x);
}
template void precond_vcycle<double>(Hierarchy<double> &, const SolverConfig &, int, cudaStream_t, const double *,
                                     double *);
template void precond_vcycle<float>(Hierarchy<float> &, const SolverConfig &, int, cudaStream_t, const float *,
                                    float *);

template <class T>
void spmm_residual(const Csr<T> &A, const LongRows &lr, const T *x, T *r, int k, const T *b, cudaStream_t s) {
    spmm_b<T>(A, lr, x, r, k, b, s);
}
template void spmm_residual<double>(const Csr<double> &, const LongRows &, const double *, double *, int,
                                    const double *, cudaStream_t);
template void spmm_residual<float>(const Csr<float> &, const LongRows &, const float *, float *, int, const float *,
                                   cudaStream_t);

template g2p_status fgmres<double>(const Csr<double> &, Hierarchy<double> &, Krylov<double> &, const double *, double *,
                                   int, const SolverConfig &, const double *, cudaStream_t, SolveReport &,
                                   const F32Precond *, const LongRows *);
template g2p_status fgmres<float>(const Csr<float> &, Hierarchy<float> &, Krylov<float> &, const float *, float *, int,
                                  const SolverConfig &, const double *, cudaStream_t, SolveReport &, const F32Precond *,
                                  const LongRows *);

}  // namespace g2p

extern "C" void g2p_profile_begin(void) {
    g2p::kprof_set(true);
    g2p::g_prof.on = true;
    g2p::g_prof.used = 0;
    g2p::g_prof.bytes = 0;
    g2p::g_prof.launches = 0;
    g2p::g_prof.launch_bytes.clear();
    g2p::g_prof.launch_f64.clear();
    g2p::g_prof.launch_rows.clear();
}

extern "C" g2p_status g2p_profile_end(double *kernel_ms, double *kernel_bytes, int64_t *launches) {
    using namespace g2p;
    g_prof.on = false;
    kprof_set(false);
    G2P_TRY(kprof_collect());
    double ms = 0;
    // classes of the SpMM launches by operator rows: < 64k, < 256k, < 1M, >= 1M
    // (the last one is the fine level of the workloads here)
    const double edges[] = {0, 65536, 262144, 1048576, 1e30};
    double bms[8] = {0}, bby[8] = {0};
    int64_t bn[8] = {0};
    for (size_t i = 0; i + 1 < g_prof.used; i += 2) {
        float t = 0;
        G2P_CUDA(cudaEventElapsedTime(&t, g_prof.ev[i], g_prof.ev[i + 1]));
        ms += t;
        const size_t li = i / 2;
        if (li < g_prof.launch_bytes.size()) {
            const double lb = g_prof.launch_bytes[li];
            const double rows = (double)g_prof.launch_rows[li];
            const int o = g_prof.launch_f64[li] ? 4 : 0;
            for (int q = 0; q < 4; q++)
                if (rows >= edges[q] && rows < edges[q + 1]) { bms[o + q] += t; bby[o + q] += lb; bn[o + q]++; }
        }
    }
    for (int q = 0; q < 8; q++) { g_bucket_ms[q] = bms[q]; g_bucket_bytes[q] = bby[q]; g_bucket_n[q] = bn[q]; }
    const char *bname[4] = {"rows<64k", "rows<256k", "rows<1M", "rows>=1M"};
    for (int q = 0; q < 8; q++)
        if (bn[q]) {
            char nm[96];
            snprintf(nm, sizeof nm, "spmm_%s[%s]@%.0fGB/s", q < 4 ? "f32" : "f64", bname[q % 4],
                     bms[q] > 0 ? bby[q] / (bms[q] * 1e6) : 0.0);
            kprof_add_total(nm, bn[q], bms[q]);
        }
    if (kernel_ms) *kernel_ms = ms;
    if (kernel_bytes) *kernel_bytes = g_prof.bytes;
    if (launches) *launches = g_prof.launches;
    g_prof.used = 0;
    return G2P_OK;
}

extern "C" void g2p_profile_buckets(double *ms, double *bytes, int64_t *launches) {
    for (int q = 0; q < 8; q++) {
        if (ms) ms[q] = g2p::g_bucket_ms[q];
        if (bytes) bytes[q] = g2p::g_bucket_bytes[q];
        if (launches) launches[q] = g2p::g_bucket_n[q];
    }
}
