// Block FGMRES(m) for k right-hand sides that share one block Krylov space.
//
// The reference solves one right-hand side per HYPRE call (FlexGMRES(10)
// with a BoomerAMG V-cycle, hypreSolve.cpp:209-253).  The lock-step solver
// in solver.cu runs k independent recurrences side by side; here the k
// columns of each Arnoldi step are orthogonalised against, and searched
// over, the whole block basis, so every right-hand side sees k directions
// per V-cycle:
//
//   R0 = B - A X = V_0 B0                       (two-pass Cholesky QR)
//   Z_j = M^-1 V_j ; W = A Z_j
//   H_ij = V_i^T W, W -= V_i H_ij  (i <= j)     (block classical Gram-Schmidt, twice)
//   W = V_{j+1} H_{j+1,j}                        (two-pass Cholesky QR)
//   min_Y || E1 B0 - Hbar Y ||_F                 (Givens rotations on the host)
//   X += [Z_0 .. Z_J-1] Y
//
// Vectors are n x k blocks with the right-hand sides interleaved (element
// i * k + r), as everywhere in the solver.  A thread covers an S x S tile of
// the k x k products of one row (S = min(k, 4)), so the contractions read
// every vector once from HBM and issue 16 FMAs per two 16-byte loads; block
// partial sums are reduced in a fixed order (results are deterministic and
// graph replays are bit-identical).
//
// Rank deficiency: a column whose Cholesky pivot falls below tol times its
// Gram diagonal is taken as dependent on the columns before it; its basis
// vector is set to zero and its row of R to zero, so later steps carry a
// narrower block and the least-squares problem leaves that index out.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "block_lsq.h"
#include "solver.h"

namespace g2p {

namespace {

constexpr int kBRedBlocks = 152 * 4;

template <class T, int S>
__device__ __forceinline__ void vload(const T *p, T (&o)[S]) {
    if constexpr (S == 4 && sizeof(T) == 4) {
        const float4 v = *reinterpret_cast<const float4 *>(p);
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    } else if constexpr (S == 4 && sizeof(T) == 8) {
        const double2 a = *reinterpret_cast<const double2 *>(p), b = *reinterpret_cast<const double2 *>(p + 2);
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
    } else if constexpr (S == 2 && sizeof(T) == 4) {
        const float2 v = *reinterpret_cast<const float2 *>(p);
        o[0] = v.x; o[1] = v.y;
    } else if constexpr (S == 2 && sizeof(T) == 8) {
        const double2 v = *reinterpret_cast<const double2 *>(p);
        o[0] = v.x; o[1] = v.y;
    } else {
#pragma unroll
        for (int u = 0; u < S; u++) o[u] = p[u];
    }
}

template <class T, int S>
__device__ __forceinline__ void vstore(T *p, const T (&o)[S]) {
    if constexpr (S == 4 && sizeof(T) == 4) {
        *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
    } else if constexpr (S == 4 && sizeof(T) == 8) {
        *reinterpret_cast<double2 *>(p) = make_double2(o[0], o[1]);
        *reinterpret_cast<double2 *>(p + 2) = make_double2(o[2], o[3]);
    } else if constexpr (S == 2 && sizeof(T) == 4) {
        *reinterpret_cast<float2 *>(p) = make_float2(o[0], o[1]);
    } else if constexpr (S == 2 && sizeof(T) == 8) {
        *reinterpret_cast<double2 *>(p) = make_double2(o[0], o[1]);
    } else {
#pragma unroll
        for (int u = 0; u < S; u++) p[u] = o[u];
    }
}

template <int K>
struct Tile {
    static constexpr int S = K < 4 ? K : 4;       // tile edge
    static constexpr int NB = K / S;              // tiles per row edge
    static constexpr int TPR = NB * NB;           // threads per row in the k x k products
    static constexpr int RL = 256 / TPR;          // rows a block covers per pass
    static constexpr int SLOTS = TPR < 32 ? 8 : RL;
};

// Basis blocks per pass over W in the products: at most 32 accumulators
// (two blocks of 128-register threads per SM without spills) and the
// block's partial sums within 32 KB.
template <class T, int K>
constexpr int bdot_group() {
    constexpr int S = Tile<K>::S;
    constexpr int regs = 32 / (S * S);
    constexpr int smem = 32768 / (Tile<K>::SLOTS * K * K * 8);
    constexpr int g = regs < smem ? regs : smem;
    return g < 1 ? 1 : (g > 8 ? 8 : g);
}

// partial[((j0 + g) * K * K + p * K + q) * gridDim.x + block] = this block's
// share of sum_i V_{j0+g}[i, p] * W[i, q], for g < gact.
template <class T, int K, int GM>
__global__ void __launch_bounds__(256, 2) k_bdot_partial(const T *__restrict__ V, int64_t ldv, int j0, int gact,
                                                      const T *__restrict__ W, int64_t n, double *__restrict__ partial) {
    using Tl = Tile<K>;
    constexpr int S = Tl::S, NB = Tl::NB, TPR = Tl::TPR, RL = Tl::RL, SLOTS = Tl::SLOTS;
    extern __shared__ double bsm[];     // SLOTS * GM * K * K
    const int t = threadIdx.x, sub = t % TPR, lr = t / TPR, a = sub / NB, bq = sub % NB;
    T acc[GM][S][S];
#pragma unroll
    for (int g = 0; g < GM; g++)
#pragma unroll
        for (int p = 0; p < S; p++)
#pragma unroll
            for (int q = 0; q < S; q++) acc[g][p][q] = 0;
    for (int64_t i = blockIdx.x * (int64_t)RL + lr; i < n; i += (int64_t)gridDim.x * RL) {
        T w[S];
        vload<T, S>(W + i * K + bq * S, w);
#pragma unroll
        for (int g = 0; g < GM; g++) {
            if (g < gact) {
                T v[S];
                vload<T, S>(V + (int64_t)(j0 + g) * ldv + i * K + a * S, v);
#pragma unroll
                for (int p = 0; p < S; p++)
#pragma unroll
                    for (int q = 0; q < S; q++) acc[g][p][q] = fma(v[p], w[q], acc[g][p][q]);
            }
        }
    }
    // warp sums one value at a time (FP64 copies of all accumulators at
    // once would double the registers)
    const int lane = t & 31, warp = t >> 5;
    const bool rep = TPR < 32 ? lane < TPR : true;
    const int slot = TPR < 32 ? warp : lr;
#pragma unroll
    for (int g = 0; g < GM; g++)
#pragma unroll
        for (int p = 0; p < S; p++)
#pragma unroll
            for (int q = 0; q < S; q++) {
                double v = (double)acc[g][p][q];
                if constexpr (TPR < 32) {
#pragma unroll
                    for (int o = TPR; o < 32; o <<= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
                }
                if (rep && g < gact) bsm[(slot * GM + g) * K * K + (a * S + p) * K + bq * S + q] = v;
            }
    __syncthreads();
    for (int o = t; o < gact * K * K; o += blockDim.x) {
        const int g = o / (K * K), e = o - g * K * K;
        double s = 0;
        for (int q = 0; q < SLOTS; q++) s += bsm[(q * GM + g) * K * K + e];
        partial[((int64_t)(j0 + g) * K * K + e) * gridDim.x + blockIdx.x] = s;
    }
}

// out[c] = sum of partial[c * nb ..] in a fixed order (and add_to[c] += it).
__global__ void __launch_bounds__(256) k_bred(const double *partial, int nb, int cnt, double *out, double *add_to) {
    const int c = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (c >= cnt) return;
    const double *p = partial + (int64_t)c * nb;
    double s = 0;
    for (int b = lane; b < nb; b += 32) s += p[b];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) {
        out[c] = s;
        if (add_to) add_to[c] += s;
    }
}

// out[i, q] = (ACC ? out[i, q] : 0) + sign * sum_{g < J} sum_p X_g[i, p] C[(g K + p) K + q]
// (X_g = X + g * ldx).  out must not alias any X_g.
template <class T, int K, bool ACC>
__global__ void __launch_bounds__(256) k_bcomb(const T *__restrict__ X, int64_t ldx, int J, const double *__restrict__ C,
                                               double sign, T *__restrict__ out, int64_t n) {
    constexpr int S = Tile<K>::S, NB = Tile<K>::NB, RL = 256 / NB;
    extern __shared__ __align__(16) unsigned char bcsm[];
    T *c = reinterpret_cast<T *>(bcsm);
    for (int o = threadIdx.x; o < J * K * K; o += blockDim.x) c[o] = (T)(sign * C[o]);
    __syncthreads();
    const int bq = threadIdx.x % NB, lr = threadIdx.x / NB;
    for (int64_t i = blockIdx.x * (int64_t)RL + lr; i < n; i += (int64_t)gridDim.x * RL) {
        T acc[S];
        if constexpr (ACC) {
            vload<T, S>(out + i * K + bq * S, acc);
        } else {
#pragma unroll
            for (int q = 0; q < S; q++) acc[q] = 0;
        }
        for (int g = 0; g < J; g++) {
            const T *xr = X + (int64_t)g * ldx + i * K;
            const T *cg = c + g * K * K + bq * S;
#pragma unroll
            for (int p0 = 0; p0 < K; p0 += S) {
                T v[S];
                vload<T, S>(xr + p0, v);
#pragma unroll
                for (int pp = 0; pp < S; pp++)
#pragma unroll
                    for (int q = 0; q < S; q++) acc[q] = fma(v[pp], cg[(p0 + pp) * K + q], acc[q]);
            }
        }
        vstore<T, S>(out + i * K + bq * S, acc);
    }
}

// Cholesky factor R (upper, G = R^T R) of a K x K Gram matrix, its inverse M
// with the columns of dependent pivots zeroed, and Rout = R * Rprev (or R).
// One warp; lane q owns column q.
template <int K>
__global__ void __launch_bounds__(32) k_bchol(const double *G, double tol, const double *Rprev, double *Rout,
                                              double *M) {
    __shared__ double R[K][K], Mi[K][K];
    __shared__ int dep[K];
    const int q = threadIdx.x;
    for (int o = q; o < K * K; o += 32) (&R[0][0])[o] = 0.0;
    __syncwarp();
    for (int p = 0; p < K; p++) {
        const double gpp = G[p * K + p];
        double dd = gpp;
        for (int t = 0; t < p; t++) dd -= R[t][p] * R[t][p];
        const bool bad = !(gpp > 0.0) || !(dd > tol * gpp);
        const double rpp = bad ? 0.0 : sqrt(dd);
        if (q < K && q > p && !bad) {
            double s = G[p * K + q];
            for (int t = 0; t < p; t++) s -= R[t][p] * R[t][q];
            R[p][q] = s / rpp;
        }
        if (q == p) {
            R[p][p] = rpp;
            dep[p] = bad ? 1 : 0;
        }
        __syncwarp();
    }
    if (q < K) {
        // column q of the inverse of R with unit pivots in the dependent rows
        for (int i = q; i >= 0; i--) {
            double s = i == q ? 1.0 : 0.0;
            for (int t = i + 1; t <= q; t++) s -= R[i][t] * Mi[t][q];
            Mi[i][q] = s / (dep[i] ? 1.0 : R[i][i]);
        }
        for (int i = 0; i < K; i++) M[i * K + q] = dep[q] || i > q ? 0.0 : Mi[i][q];
        for (int p = 0; p < K; p++) {
            double s;
            if (Rprev) {
                s = 0.0;
                for (int t = p; t <= q; t++) s += R[p][t] * Rprev[t * K + q];
            } else {
                s = R[p][q];
            }
            Rout[p * K + q] = s;
        }
    }
}

// Device scratch of the block iteration (doubles, in K.bdev):
//   hcol  (m + 2) K^2   block column of the Hessenberg matrix (dots, then R)
//   dots2 (m + 1) K^2   second Gram-Schmidt pass
//   G, R1, M1, M2, R0   K^2 each
//   Y     m K^2         least-squares solution
struct BlockLayout {
    int64_t hcol, dots2, G, R1, M1, M2, R0, Y, total;
    BlockLayout(int k, int m) {
        const int64_t kk = (int64_t)k * k;
        hcol = 0;
        dots2 = hcol + (m + 2) * kk;
        G = dots2 + (m + 1) * kk;
        R1 = G + kk;
        M1 = R1 + kk;
        M2 = M1 + kk;
        R0 = M2 + kk;
        Y = R0 + kk;
        total = Y + (int64_t)m * kk;
    }
};

template <class T>
g2p_status block_alloc(Krylov<T> &K, int k, int m, cudaStream_t s) {
    if (K.bdev && K.bk >= k && K.bm >= m) return G2P_OK;
    dfree(K.bdev, s);
    dfree(K.bpart, s);
    if (K.bhost) cudaFreeHost(K.bhost);
    K.bhost = nullptr;
    const int kk = std::max(k, K.bk), mm = std::max(m, K.bm);
    BlockLayout L(kk, mm);
    G2P_TRY(dalloc(&K.bdev, L.total, s));
    G2P_TRY(dalloc(&K.bpart, (int64_t)kBRedBlocks * (mm + 1) * kk * kk, s));
    G2P_CUDA(cudaMallocHost(&K.bhost, sizeof(double) * (size_t)L.total));
    K.bk = kk;
    K.bm = mm;
    return G2P_OK;
}

template <class T, int K>
struct BlockOps {
    static constexpr int GM = bdot_group<T, K>();
    static constexpr double tol = sizeof(T) == 4 ? 1e-5 : 1e-12;

    // out[0 .. J K^2) = [V_0 .. V_{J-1}]^T W  (and add_to += out)
    static void dots(const T *V, int64_t ldv, int J, const T *W, int64_t n, double *partial, double *out,
                     double *add_to, cudaStream_t s) {
        const size_t sm = sizeof(double) * Tile<K>::SLOTS * GM * K * K;
        for (int j0 = 0; j0 < J; j0 += GM) {
            const int ga = std::min(GM, J - j0);
            (kbegin("k_bdot_partial", s),
             k_bdot_partial<T, K, GM><<<kBRedBlocks, 256, sm, s>>>(V, ldv, j0, ga, W, n, partial), kend(s));
        }
        const int cnt = J * K * K;
        (kbegin("k_bred", s), k_bred<<<(cnt + 7) / 8, 256, 0, s>>>(partial, kBRedBlocks, cnt, out, add_to), kend(s));
    }

    // out (+)= sign * [X_0 .. X_{J-1}] C, in launches whose coefficients fit
    // in 48 KB of shared memory
    static void comb(const T *X, int64_t ldx, int J, const double *C, double sign, T *out, int64_t n, bool acc,
                     cudaStream_t s) {
        const int jc = std::max(1, (int)(49152 / (sizeof(T) * K * K)));
        constexpr int RL = 256 / Tile<K>::NB;
        const unsigned grid = (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + RL - 1) / RL, 152LL * 8));
        for (int g0 = 0; g0 < J; g0 += jc) {
            const int gj = std::min(jc, J - g0);
            const size_t sm = sizeof(T) * (size_t)gj * K * K;
            const T *Xg = X + (int64_t)g0 * ldx;
            const double *Cg = C + (int64_t)g0 * K * K;
            if (acc || g0 > 0)
                (kbegin("k_bcomb", s), k_bcomb<T, K, true><<<grid, 256, sm, s>>>(Xg, ldx, gj, Cg, sign, out, n), kend(s));
            else
                (kbegin("k_bcomb", s), k_bcomb<T, K, false><<<grid, 256, sm, s>>>(Xg, ldx, gj, Cg, sign, out, n), kend(s));
        }
    }

    // X = out * Rdst with out's columns orthonormal (two Cholesky-QR passes
    // through tmp); Rdst (device, K x K) upper triangular.
    static void qr(const T *X, T *tmp, T *out, int64_t n, double *partial, double *bdev, const BlockLayout &L,
                   double *Rdst, cudaStream_t s) {
        dots(X, 0, 1, X, n, partial, bdev + L.G, nullptr, s);
        (kbegin("k_bchol", s), k_bchol<K><<<1, 32, 0, s>>>(bdev + L.G, tol, nullptr, bdev + L.R1, bdev + L.M1), kend(s));
        comb(X, 0, 1, bdev + L.M1, 1.0, tmp, n, false, s);
        dots(tmp, 0, 1, tmp, n, partial, bdev + L.G, nullptr, s);
        (kbegin("k_bchol", s), k_bchol<K><<<1, 32, 0, s>>>(bdev + L.G, tol, bdev + L.R1, Rdst, bdev + L.M2), kend(s));
        comb(tmp, 0, 1, bdev + L.M2, 1.0, out, n, false, s);
    }
};

template <class T, int KB>
g2p_status run_block(const Csr<T> &A, Hierarchy<T> &H, Krylov<T> &K, const T *b, T *x, const SolverConfig &cfg,
                     const double *bnorm_override, cudaStream_t s, SolveReport &rep, const LongRows &lr0) {
    using Ops = BlockOps<T, KB>;
    const int k = KB, m = cfg.restart;
    const int64_t n = A.n, nk = n * k;
    G2P_TRY(block_alloc<T>(K, k, m, s));
    const BlockLayout L(K.bk, K.bm);
    double *bdev = K.bdev, *bhost = K.bhost;
    const bool graphs = cfg.use_graphs && !kprof_on();
    if (graphs) {
        const std::vector<const void *> key = {(const void *)(intptr_t)k, (const void *)A.val, (const void *)&H,
                                               (const void *)(intptr_t)H.kcap, (const void *)(intptr_t)cfg.degree,
                                               (const void *)(intptr_t)cfg.reorth, (const void *)(intptr_t)-1,
                                               (const void *)(intptr_t)H.fuse_from};
        if (K.graph_key != key || (int)K.steps.size() != m) {
            K.drop_graphs();
            K.graph_key = key;
            K.steps.resize(m);
        }
    }
    if (bnorm_override) G2P_CUDA(cudaMemcpyAsync(K.bnorm, bnorm_override, sizeof(double) * k, cudaMemcpyDeviceToDevice, s));
    else colnorms<T>(b, n, k, K.partial, K.bnorm, s);
    BlockLSQ ls;
    std::vector<double> res(k), Y;
    int it = 0;
    rep.converged = false;
    for (;;) {
        spmm_residual<T>(A, lr0, x, K.r, k, b, s);
        colnorms<T>(K.r, n, k, K.partial, K.beta, s);
        G2P_CUDA(cudaMemcpyAsync(K.h_est, K.beta, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaMemcpyAsync(K.h_est + k, K.bnorm, sizeof(double) * k, cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        double worst = 0;
        for (int r = 0; r < k; r++) {
            const double bn = K.h_est[k + r];
            worst = std::max(worst, bn > 0 ? K.h_est[r] / bn : 0.0);
        }
        rep.rel_residual = worst;
        if (worst <= cfg.rtol) { rep.converged = true; break; }
        if (it >= cfg.maxit) break;
        std::vector<double> bn(K.h_est + k, K.h_est + 2 * k);
        // R0 = V_0 B0
        Ops::qr(K.r, K.w, K.V, n, K.bpart, bdev, L, bdev + L.R0, s);
        G2P_CUDA(cudaMemcpyAsync(bhost + L.R0, bdev + L.R0, sizeof(double) * k * k, cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        ls.reset(k, m, bhost + L.R0);
        int j = 0;
        for (; j < m && it < cfg.maxit; j++) {
            T *Vj = K.V + (int64_t)j * nk, *Zj = K.Z + (int64_t)j * nk;
            double *hcol = bdev + L.hcol;
            auto step = [&]() {
                precond_vcycle<T>(H, cfg, k, s, Vj, Zj);
                spmm<T>(A, lr0, Zj, K.w, k, s);
                Ops::dots(K.V, nk, j + 1, K.w, n, K.bpart, hcol, nullptr, s);
                Ops::comb(K.V, nk, j + 1, hcol, -1.0, K.w, n, true, s);
                if (cfg.reorth) {
                    Ops::dots(K.V, nk, j + 1, K.w, n, K.bpart, bdev + L.dots2, hcol, s);
                    Ops::comb(K.V, nk, j + 1, bdev + L.dots2, -1.0, K.w, n, true, s);
                }
                Ops::qr(K.w, K.r, K.V + (int64_t)(j + 1) * nk, n, K.bpart, bdev, L,
                        hcol + (int64_t)(j + 1) * k * k, s);
                cudaMemcpyAsync(bhost + L.hcol, hcol, sizeof(double) * (size_t)(j + 2) * k * k, cudaMemcpyDeviceToHost,
                                s);
            };
            if (graphs) {
                auto &st = K.steps[j];
                if (st.exec) {
                    G2P_CUDA(cudaGraphLaunch(st.exec, s));
                    launch_add(st.launches);
                } else if (st.seen && !st.failed) {
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
            ls.add_block(j, bhost + L.hcol, res.data());
            double w2 = 0;
            for (int r = 0; r < k; r++) w2 = std::max(w2, bn[r] > 0 ? res[r] / bn[r] : 0.0);
            if (w2 <= cfg.rtol) { j++; break; }
        }
        if (j == 0) break;
        // X += [Z_0 .. Z_{j-1}] Y
        const int nc = j * k;
        Y.assign((size_t)nc * k, 0.0);
        ls.solve(nc, Y.data());
        std::memcpy(bhost + L.Y, Y.data(), sizeof(double) * Y.size());
        G2P_CUDA(cudaMemcpyAsync(bdev + L.Y, bhost + L.Y, sizeof(double) * Y.size(), cudaMemcpyHostToDevice, s));
        Ops::comb(K.Z, nk, j, bdev + L.Y, 1.0, x, n, true, s);
    }
    rep.iterations = it;
    G2P_CUDA(cudaGetLastError());
    return G2P_OK;
}

}  // namespace

template <class T>
bool block_krylov_supported(int k, const T *b, const T *x) {
    if (k != 2 && k != 4 && k != 8 && k != 16 && k != 32) return false;
    // the tile loads are 16-byte vectors (8-byte for k = 2 in FP32)
    const uintptr_t al = (uintptr_t)std::min<size_t>(16, sizeof(T) * std::min(k, 4));
    return (uintptr_t)b % al == 0 && (uintptr_t)x % al == 0;
}
template bool block_krylov_supported<double>(int, const double *, const double *);
template bool block_krylov_supported<float>(int, const float *, const float *);

template <class T>
g2p_status block_fgmres(const Csr<T> &A, Hierarchy<T> &H, Krylov<T> &K, const T *b, T *x, int k,
                        const SolverConfig &cfg, const double *bnorm_override, cudaStream_t s, SolveReport &rep,
                        const LongRows *op_lr) {
    if (!block_krylov_supported<T>(k, b, x)) {
        set_last_message("block Krylov solve of %d right-hand sides (2, 4, 8, 16 or 32 supported)", k);
        return G2P_ERR_INVALID;
    }
    G2P_TRY(krylov_alloc<T>(K, A.n, k, cfg.restart, s));
    G2P_TRY(hierarchy_reserve<T>(H, k, s));
    G2P_TRY(coarse_prepare<T>(H, cfg, k, s));
    const LongRows &lr0 = op_lr ? *op_lr : H.lv[0].lr;
    switch (k) {
        case 2: return run_block<T, 2>(A, H, K, b, x, cfg, bnorm_override, s, rep, lr0);
        case 4: return run_block<T, 4>(A, H, K, b, x, cfg, bnorm_override, s, rep, lr0);
        case 8: return run_block<T, 8>(A, H, K, b, x, cfg, bnorm_override, s, rep, lr0);
        case 16: return run_block<T, 16>(A, H, K, b, x, cfg, bnorm_override, s, rep, lr0);
        default: return run_block<T, 32>(A, H, K, b, x, cfg, bnorm_override, s, rep, lr0);
    }
}
template g2p_status block_fgmres<double>(const Csr<double> &, Hierarchy<double> &, Krylov<double> &, const double *,
                                         double *, int, const SolverConfig &, const double *, cudaStream_t,
                                         SolveReport &, const LongRows *);
template g2p_status block_fgmres<float>(const Csr<float> &, Hierarchy<float> &, Krylov<float> &, const float *,
                                        float *, int, const SolverConfig &, const double *, cudaStream_t,
                                        SolveReport &, const LongRows *);

}  // namespace g2p
