// The full-wave (Vh) mode on the device: find_Vh (src/fdtd.hpp:3577-3859)
// and the per-port, per-frequency Vh correction of the V0 field
// (src/matrixCon.cpp:609-805) with Construct_Z_V0_Vh (src/fdtd.hpp:
// 4133-4170).  The reference compiles all of it out (SKIP_VH,
// src/fdtd.hpp:76); this is its algorithm, kept step for step:
//
//  * find_Vh: k Arnoldi steps with modified Gram-Schmidt on the 2N operator
//    [[0, I], [-D_eps^-1 S / s^2, -D_eps^-1 D_sig / s]] (s = 1e14), the
//    eigenvalues of the k x k Hessenberg matrix (Francis double-shift QR,
//    host), the right eigenvectors of those with |Im| > 1e-6 (inverse
//    iteration, host; a conjugate pair gives two columns), and
//    Vh = V(1:N, 1:k) * eigenvectors on the device.
//  * per port and frequency: Vh' = Vh - u0 ((u0a^H A u0) \ (u0a^H A Vh))
//    with A = -w^2 D_eps + i w D_sig and u0, u0a the port's V0 field
//    directions; the Galerkin system Vh'^H (S + A) Vh' y = Vh'^H (-i w J -
//    A u); final x = u + Vh' y; Z from the port edges.
//
// Device work: the operator products, the Arnoldi vectors, the Vh products
// and the mm x mm Galerkin matrix.  Host work, as the reference does it with
// LAPACK: the k x k eigenproblem, the 2 x 2 and mm x mm complex solves.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstring>
#include <thread>
#include <vector>

#include "primitives.cuh"
#include "solver.h"

namespace g2p {

typedef std::complex<double> cd;

struct FullWave {
    int64_t nr = 0, mm = 0;
    int32_t *map_r = nullptr;      // non-PEC edge index -> edge
    double *vh = nullptr;          // [mm][nr] complex (re, im interleaved)
    bool active = false;           // the V0 path keeps the ports' fields
    // per port: u0, u0a ([2][nr] real) and yd ([ne] complex), device
    std::vector<double *> u0, u0a, yd;
    void release_ports(cudaStream_t s) {
        for (auto *p : u0) dfree(p, s);
        for (auto *p : u0a) dfree(p, s);
        for (auto *p : yd) dfree(p, s);
        u0.clear(); u0a.clear(); yd.clear();
    }
    void release(cudaStream_t s) {
        release_ports(s);
        dfree(map_r, s);
        dfree(vh, s);
        nr = mm = 0;
    }
};

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kSigmaCu = 5.8e+7;      // SIGMA, src/fdtd.hpp:50 (the Vh products' conductivity)
constexpr int kFwThreads = 256;

__global__ void k_fw_map_r(int64_t ne, const int32_t *map_edge, int32_t *map_r) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x)
        if (map_edge[e] >= 0) map_r[map_edge[e]] = (int32_t)e;
}

// w = B^-1 A v for the 2N operator (src/fdtd.hpp:3593-3609), row by row in
// the order of S's entries
__global__ void k_fw_apply(int64_t nr, const int64_t *ptr, const int32_t *col, const double *val, const int32_t *map_r,
                           const int32_t *mark_edge, const double *epsn, const double *sign, int64_t L, double eps0,
                           double scale, const double *v, double *w) {
    const double s2 = scale * scale;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = map_r[r];
        const double eps = epsn[e / L];
        double acc = 0;
        for (int64_t q = ptr[r]; q < ptr[r + 1]; q++) acc += -val[q] * v[col[q]] / (eps * eps0 * s2);
        if (mark_edge[e] != 0) acc += -v[nr + r] * sign[e / L] / (eps * eps0 * scale);
        w[r] = v[nr + r];
        w[nr + r] = acc;
    }
}

// The same product with S v already in t (the matrix-free stencil):
// w[r] = v[nr + r]; w[nr + r] = -t[r] / (eps eps0 s^2) (+ the conductor term)
__global__ void k_fw_apply_sv(int64_t nr, const double *t, const int32_t *map_r, const int32_t *mark_edge,
                              const double *epsn, const double *sign, int64_t L, double eps0, double scale,
                              const double *v, double *w) {
    const double s2 = scale * scale;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = map_r[r];
        const double eps = epsn[e / L];
        double acc = -t[r] / (eps * eps0 * s2);
        if (mark_edge[e] != 0) acc += -v[nr + r] * sign[e / L] / (eps * eps0 * scale);
        w[r] = v[nr + r];
        w[nr + r] = acc;
    }
}

// Block partial sums of x . y (FP64), a fixed tree per block.
__global__ void __launch_bounds__(kFwThreads) k_fw_dot(int64_t n, const double *x, const double *y, double *partial) {
    __shared__ double sm[kFwThreads / 32];
    double acc = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        acc += x[i] * y[i];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < kFwThreads / 32; w++) t += sm[w];
        partial[blockIdx.x] = t;
    }
}

// w -= h x, then block partial sums of y . w
__global__ void __launch_bounds__(kFwThreads) k_fw_axpy_dot(int64_t n, const double *h, const double *x, double *w,
                                                            const double *y, double *partial) {
    __shared__ double sm[kFwThreads / 32];
    const double hv = *h;
    double acc = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double wi = w[i] - hv * x[i];
        w[i] = wi;
        acc += y[i] * wi;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w2 = 0; w2 < kFwThreads / 32; w2++) t += sm[w2];
        partial[blockIdx.x] = t;
    }
}

// One whole modified Gram-Schmidt step of find_Vh in one launch, for an
// operator of at most 4 * 1024 rows: the same arithmetic, in the same order,
// as k_fw_dot, then per basis vector k_fw_finish and k_fw_axpy_dot, then
// the norm and k_fw_scale, launched on a grid of kFwNb blocks of kFwThreads
// threads.  Those kernels give row e to thread e % 256 of block e / 256;
// this block of 1024 threads plays four such blocks at a time (group g =
// tid / 256 is block 4 r + g in round r), keeps its rows of w in registers,
// and reduces each emulated block's eight warp sums and then the block
// partials exactly as those kernels do.  Blocks past the rows contribute
// zero partials, which leave the sums unchanged.  The result (hcol, the
// norm, the next basis vector) is bit-identical, in 2 launches per step
// instead of 2 j + 3.
constexpr int kFwNb = 152 * 4;
template <int R>
__global__ void __launch_bounds__(1024) k_fw_mgs_step(int64_t n, int j, const double *V, double *w, double *hcol,
                                                      double *hn, double *vout) {
    __shared__ double sm[4 * R][kFwThreads / 32];
    __shared__ double pval;
    const int tid = threadIdx.x, g = tid >> 8, t = tid & 255, wg = t >> 5;
    const int nbv = (int)((n + kFwThreads - 1) / kFwThreads);
    auto row = [&](int r) -> int64_t { return (int64_t)(4 * r + g) * kFwThreads + t; };
    // the emulated blocks' sums of their eight warp sums (k_fw_dot's block
    // partials), and the sum over the blocks as k_fw_finish adds them: lane l
    // takes block l (at most 16 blocks here), then the xor tree
    auto finish = [&]() -> double {
        __syncthreads();
        if (tid < 32) {
            double acc = 0;
            for (int q = tid; q < nbv; q += 32) {
                double tt = 0;
                for (int u = 0; u < kFwThreads / 32; u++) tt += sm[q][u];
                acc += tt;
            }
            acc = warp_sum(acc);
            if (tid == 0) pval = acc;
        }
        __syncthreads();
        return pval;
    };
    double wv[R], xv[R], yv[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
        const bool in = row(r) < n;
        wv[r] = in ? w[row(r)] : 0.0;
        xv[r] = in ? V[row(r)] : 0.0;
        yv[r] = in && j > 1 ? V[n + row(r)] : 0.0;
    }
    // p = V_0 . w (k_fw_dot)
#pragma unroll
    for (int r = 0; r < R; r++) {
        double acc = 0;
        if (row(r) < n) acc += xv[r] * wv[r];
        acc = warp_sum(acc);
        if ((tid & 31) == 0) sm[4 * r + g][wg] = acc;
    }
    double p = finish();
    for (int i = 0; i < j; i++) {
        const double hv = p;
        if (tid == 0) hcol[i] = hv;
        const bool more = i + 1 < j;
        // V_{i+2}, for the next projection, while this one's sums run
        double zv[R];
#pragma unroll
        for (int r = 0; r < R; r++) zv[r] = (i + 2 < j && row(r) < n) ? V[(int64_t)(i + 2) * n + row(r)] : 0.0;
        // w -= h V_i, then the partials of y . w with y = V_{i+1}, or w
        // itself after the last basis vector (k_fw_axpy_dot)
#pragma unroll
        for (int r = 0; r < R; r++) {
            double acc = 0;
            if (row(r) < n) {
                const double wi = wv[r] - hv * xv[r];
                wv[r] = wi;
                acc += (more ? yv[r] : wi) * wi;
            }
            acc = warp_sum(acc);
            if ((tid & 31) == 0) sm[4 * r + g][wg] = acc;
        }
#pragma unroll
        for (int r = 0; r < R; r++) {
            xv[r] = yv[r];
            yv[r] = zv[r];
        }
        p = finish();
    }
    const double nrm = sqrt(p);
    if (tid == 0) *hn = nrm;
#pragma unroll
    for (int r = 0; r < R; r++)
        if (row(r) < n) {
            w[row(r)] = wv[r];
            vout[row(r)] = wv[r] / nrm;
        }
}

// out = sum of the nb partials (one warp, fixed tree); sqrt when asked
__global__ void k_fw_finish(const double *partial, int nb, double *out, int take_sqrt) {
    double acc = 0;
    for (int i = threadIdx.x; i < nb; i += 32) acc += partial[i];
    acc = warp_sum(acc);
    if (threadIdx.x == 0) *out = take_sqrt ? sqrt(acc) : acc;
}

__global__ void k_fw_scale(int64_t n, const double *w, const double *nrm, double *out) {
    const double d = *nrm;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = w[i] / d;
}

__global__ void k_fw_fill(int64_t n, double *x, double v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] = v;
}

// Vh[c][r] = sum_in V[in][r] v[c][in] (V real, v complex: [mm][k])
__global__ void k_fw_vh(int64_t nr, int64_t n2, int k, int64_t mm, const double *V, const double *v, double *vh) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nr * mm; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = t / nr, r = t - c * nr;
        double re = 0, im = 0;
        for (int in = 0; in < k; in++) {
            const double a = V[(int64_t)in * n2 + r];
            re += a * v[2 * (c * k + in)];
            im += a * v[2 * (c * k + in) + 1];
        }
        vh[2 * t] = re;
        vh[2 * t + 1] = im;
    }
}

// (-w^2 D_eps + i w D_sig) x on non-PEC edge r, as the Vh products write it
// (src/matrixCon.cpp:625-634): eps of layer (e + N_edge_v) / L, SIGMA.
struct DiagOp {
    const int32_t *map_r, *mark_edge;
    const double *epsn;
    int64_t nv, L;
    double eps0, freq;
    __device__ __forceinline__ void operator()(int64_t r, double xr, double xi, double &yr, double &yi) const {
        const int64_t e = map_r[r];
        const double eps = epsn[(e + nv) / L];
        const double w2 = -freq * freq * 4 * (kPi * kPi);
        if (mark_edge[e] != 0) {
            yr = xr * w2 * eps * eps0 - 2 * kPi * freq * xi * kSigmaCu;
            yi = xr * (freq * 2 * kPi) * kSigmaCu - xi * (freq * freq * 4 * (kPi * kPi)) * eps * eps0;
        } else {
            yr = xr * w2 * eps * eps0;
            yi = -xi * (freq * freq * 4 * (kPi * kPi)) * eps * eps0;
        }
    }
};

// out[a][c] = sum_r u[a][r] * D(x[c][r]) for a < 2 (u real, x complex or
// real), one block per column c; the block's partial sums combine in a
// fixed tree.  out is column-major 2 x ncol complex: (c * 2 + a) re, im.
__global__ void __launch_bounds__(kFwThreads) k_fw_proj2(int64_t nr, const double *u, const double *x, int x_real,
                                                         DiagOp D, double *out) {
    __shared__ double sm[4][kFwThreads / 32];
    const int64_t c = blockIdx.x;
    double a0r = 0, a0i = 0, a1r = 0, a1i = 0;
    for (int64_t r = threadIdx.x; r < nr; r += blockDim.x) {
        double xr, xi;
        if (x_real) { xr = x[c * nr + r]; xi = 0; }
        else { xr = x[2 * (c * nr + r)]; xi = x[2 * (c * nr + r) + 1]; }
        double yr, yi;
        D(r, xr, xi, yr, yi);
        const double u0 = u[r], u1 = u[nr + r];
        a0r += u0 * yr; a0i += u0 * yi;
        a1r += u1 * yr; a1i += u1 * yi;
    }
    a0r = warp_sum(a0r); a0i = warp_sum(a0i); a1r = warp_sum(a1r); a1i = warp_sum(a1i);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { sm[0][w] = a0r; sm[1][w] = a0i; sm[2][w] = a1r; sm[3][w] = a1i; }
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0;
        for (int q = 0; q < kFwThreads / 32; q++) t += sm[threadIdx.x][q];
        const int a = threadIdx.x >> 1, ri = threadIdx.x & 1;
        out[(c * 2 + a) * 2 + ri] = t;
    }
}

// Vh'[c][r] = Vh[c][r] - (u0[0][r] yn[c][0] + u0[1][r] yn[c][1])
__global__ void k_fw_deflate(int64_t nr, int64_t mm, const double *vh, const double *u0, const double *yn, double *vhd) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nr * mm; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = t / nr, r = t - c * nr;
        const double u_0 = u0[r], u_1 = u0[nr + r];
        const double mr = u_0 * yn[4 * c] + u_1 * yn[4 * c + 2];
        const double mi = u_0 * yn[4 * c + 1] + u_1 * yn[4 * c + 3];
        vhd[2 * t] = vh[2 * t] - mr;
        vhd[2 * t + 1] = vh[2 * t + 1] - mi;
    }
}

// T[c][r] = (S Vh')[c][r] + (-w^2 D_eps + i w D_sig) Vh'[c][r] with the
// products' own expression (src/matrixCon.cpp:699-720)
__global__ void k_fw_spmm(int64_t nr, int64_t mm, const int64_t *ptr, const int32_t *col, const double *val, DiagOp D,
                          const double *x, double *T) {
    const double w2 = -((D.freq * 2 * kPi) * (D.freq * 2 * kPi));
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nr * mm; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t c = t / nr, r = t - c * nr;
        const double *xc = x + 2 * c * nr;
        double re = 0, im = 0;
        for (int64_t q = ptr[r]; q < ptr[r + 1]; q++) {
            re += val[q] * xc[2 * col[q]];
            im += val[q] * xc[2 * col[q] + 1];
        }
        const int64_t e = D.map_r[r];
        const double eps = D.epsn[(e + D.nv) / D.L];
        const double xr = xc[2 * r], xi = xc[2 * r + 1];
        if (D.mark_edge[e] != 0) {
            re += w2 * eps * D.eps0 * xr - D.freq * 2 * kPi * kSigmaCu * xi;
            im += w2 * eps * D.eps0 * xi + D.freq * 2 * kPi * kSigmaCu * xr;
        } else {
            re += w2 * eps * D.eps0 * xr;
            im += w2 * eps * D.eps0 * xi;
        }
        T[2 * t] = re;
        T[2 * t + 1] = im;
    }
}

// G[c2][c1] = sum_r conj(X[c1][r]) Y[c2][r]: a tile of 16 x 16 outputs per
// block, r in chunks of 32 staged in shared memory
constexpr int kGt = 16, kGr = 32;
__global__ void __launch_bounds__(kGt * kGt) k_fw_gram(int64_t nr, int64_t mm, const double *X, const double *Y,
                                                       double *G) {
    __shared__ double xs[kGt][kGr][2], ys[kGt][kGr][2];
    const int tx = threadIdx.x % kGt, ty = threadIdx.x / kGt;
    const int64_t c1 = (int64_t)blockIdx.x * kGt + tx, c2 = (int64_t)blockIdx.y * kGt + ty;
    double re = 0, im = 0;
    for (int64_t r0 = 0; r0 < nr; r0 += kGr) {
        for (int q = threadIdx.x; q < kGt * kGr; q += kGt * kGt) {
            const int cc = q / kGr, rr = q % kGr;
            const int64_t r = r0 + rr;
            const int64_t a = (int64_t)blockIdx.x * kGt + cc, b = (int64_t)blockIdx.y * kGt + cc;
            const bool in = r < nr;
            xs[cc][rr][0] = in && a < mm ? X[2 * (a * nr + r)] : 0;
            xs[cc][rr][1] = in && a < mm ? X[2 * (a * nr + r) + 1] : 0;
            ys[cc][rr][0] = in && b < mm ? Y[2 * (b * nr + r)] : 0;
            ys[cc][rr][1] = in && b < mm ? Y[2 * (b * nr + r) + 1] : 0;
        }
        __syncthreads();
#pragma unroll 8
        for (int rr = 0; rr < kGr; rr++) {
            const double ar = xs[tx][rr][0], ai = xs[tx][rr][1], br = ys[ty][rr][0], bi = ys[ty][rr][1];
            re += ar * br + ai * bi;
            im += ar * bi - ai * br;
        }
        __syncthreads();
    }
    if (c1 < mm && c2 < mm) {
        G[2 * (c2 * mm + c1)] = re;
        G[2 * (c2 * mm + c1) + 1] = im;
    }
}

// rhs[c] = Vh'[c]^H (J' - A u), one block per column: J' has -i w on the
// port's edges; A u is the products' expression on yd (matrixCon.cpp:744-755)
__global__ void __launch_bounds__(kFwThreads) k_fw_rhs(int64_t nr, const double *X, const double *Jr, const double *yd,
                                                       DiagOp D, double fsf, double *rhs) {
    __shared__ double sm[2][kFwThreads / 32];
    const int64_t c = blockIdx.x;
    const double w2 = -((D.freq * 2 * kPi) * (D.freq * 2 * kPi));
    double sr = 0, si = 0;
    for (int64_t r = threadIdx.x; r < nr; r += blockDim.x) {
        const int64_t e = D.map_r[r];
        const double eps = D.epsn[(e + D.nv) / D.L];
        const double yr = yd[2 * e], yi = yd[2 * e + 1];
        double tr, ti;
        if (D.mark_edge[e] != 0) {
            tr = w2 * eps * D.eps0 * yr - D.freq * 2 * kPi * kSigmaCu * yi * fsf;
            ti = D.freq * 2 * kPi * kSigmaCu * yr + w2 * eps * D.eps0 * yi * fsf;
        } else {
            tr = w2 * eps * D.eps0 * yr;
            ti = w2 * eps * D.eps0 * yi * fsf;
        }
        // b = J' - A u; J' is (0, -w) on the port's edges
        const double br = -tr, bi = (Jr[r] != 0 ? -D.freq * 2 * kPi : 0.0) - ti;
        const double ar = X[2 * (c * nr + r)], ai = X[2 * (c * nr + r) + 1];
        sr += ar * br + ai * bi;
        si += ar * bi - ai * br;
    }
    sr = warp_sum(sr); si = warp_sum(si);
    if ((threadIdx.x & 31) == 0) { sm[0][threadIdx.x >> 5] = sr; sm[1][threadIdx.x >> 5] = si; }
    __syncthreads();
    if (threadIdx.x < 2) {
        double t = 0;
        for (int q = 0; q < kFwThreads / 32; q++) t += sm[threadIdx.x][q];
        rhs[2 * c + threadIdx.x] = t;
    }
}

// final x[r] = u[r] (frequency-scaled imaginary part) + sum_c Vh'[c][r] y[c]
__global__ void k_fw_final(int64_t nr, int64_t mm, const double *X, const double *y, const double *yd, const int32_t *map_r,
                           double fsf, double *out) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        double re = 0, im = 0;
        for (int64_t c = 0; c < mm; c++) {
            const double ar = X[2 * (c * nr + r)], ai = X[2 * (c * nr + r) + 1];
            re += ar * y[2 * c] - ai * y[2 * c + 1];
            im += ai * y[2 * c] + ar * y[2 * c + 1];
        }
        const int64_t e = map_r[r];
        out[2 * r] = yd[2 * e] + re;
        out[2 * r + 1] = yd[2 * e + 1] * fsf + im;
    }
}

// u0, u0a columns and yd of one port from its V0 fields (matrixCon.cpp:
// 414-430, 545-576); the norms over all edges come in norms[4]
__global__ void k_fw_fields(int64_t nr, int64_t ne, int k, int r0, const int32_t *map_r, const double *yd1,
                            const double *ydat, const double *yd2, const double *yc, const double *yd2a,
                            const double *yca, const double *norms, double *u0, double *u0a, double *yd) {
    const double n1 = norms[0], n1a = norms[1], n2 = norms[2], n2a = norms[3];
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t e = map_r[r], t = e * k + r0;
        u0[r] = yd1[t] / n1;
        u0a[r] = ydat[t] / n1a;
        u0[nr + r] = (yd2[t] + yc[t]) / n2;
        u0a[nr + r] = (yd2a[t] + yca[t]) / n2a;
    }
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t t = e * k + r0;
        yd[2 * e] = (yd2[t] - 0.0) + yc[t];
        yd[2 * e + 1] = 0.0 - yd1[t];
    }
}

// block partials of sum_e a[e, r0]^2, or of sum_e (a + b)[e, r0]^2
__global__ void __launch_bounds__(kFwThreads) k_fw_norm2(int64_t ne, int k, int r0, const double *a, const double *b,
                                                         double *partial) {
    __shared__ double sm[kFwThreads / 32];
    double acc = 0;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x) {
        const double v = b ? a[e * k + r0] + b[e * k + r0] : a[e * k + r0];
        acc += v * v;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w = 0; w < kFwThreads / 32; w++) t += sm[w];
        partial[blockIdx.x] = t;
    }
}

// ----------------------------------------------------------------- host
// Eigenvalues of a real upper Hessenberg matrix (column-major, destroyed):
// Francis double-shift QR iteration with deflation on negligible
// subdiagonal entries and exceptional shifts every ten iterations.  A
// complex pair is stored at consecutive positions, positive imaginary part
// first.  Returns 0, or the number of unconverged eigenvalues.
int hqr_eigenvalues(int64_t n, double *a, double *wr, double *wi) {
    auto A = [&](int64_t i, int64_t j) -> double & { return a[i + j * n]; };
    double norm = 0;
    for (int64_t j = 0; j < n; j++)
        for (int64_t i = 0; i <= std::min(j + 1, n - 1); i++) norm += std::fabs(A(i, j));
    const double ulp = 2.220446049250313e-16;
    double shifted = 0;
    int64_t hi = n - 1;
    int64_t iters = 0;
    while (hi >= 0) {
        int64_t lo = hi;
        while (lo >= 1) {
            double s = std::fabs(A(lo - 1, lo - 1)) + std::fabs(A(lo, lo));
            if (s == 0) s = norm;
            if (std::fabs(A(lo, lo - 1)) <= ulp * s) { A(lo, lo - 1) = 0; break; }
            lo--;
        }
        const double x = A(hi, hi);
        if (lo == hi) {
            wr[hi] = x + shifted; wi[hi] = 0;
            hi--; iters = 0;
            continue;
        }
        const double y = A(hi - 1, hi - 1), w = A(hi, hi - 1) * A(hi - 1, hi);
        if (lo == hi - 1) {
            const double p = 0.5 * (y - x), q = p * p + w, z = std::sqrt(std::fabs(q));
            if (q >= 0) {
                const double zz = p + std::copysign(z, p);
                wr[hi - 1] = wr[hi] = x + zz + shifted;
                if (zz != 0) wr[hi] = x - w / zz + shifted;
                wi[hi - 1] = wi[hi] = 0;
            } else {
                wr[hi - 1] = wr[hi] = x + p + shifted;
                wi[hi - 1] = z; wi[hi] = -z;
            }
            hi -= 2; iters = 0;
            continue;
        }
        if (iters >= 60 * std::max<int64_t>(n, 1)) return (int)(hi + 1);
        double sx = x, sy = y, sw = w;
        if (iters > 0 && iters % 10 == 0) {
            shifted += x;
            for (int64_t i = 0; i <= hi; i++) A(i, i) -= x;
            const double s = std::fabs(A(hi, hi - 1)) + std::fabs(A(hi - 1, hi - 2));
            sx = sy = 0.75 * s;
            sw = -0.4375 * s * s;
        }
        iters++;
        int64_t m = hi - 2;
        double p = 0, q = 0, r = 0;
        for (; m >= lo; m--) {
            const double z = A(m, m), rr = sx - z, ss = sy - z;
            p = (rr * ss - sw) / A(m + 1, m) + A(m, m + 1);
            q = A(m + 1, m + 1) - z - rr - ss;
            r = A(m + 2, m + 1);
            const double s = std::fabs(p) + std::fabs(q) + std::fabs(r);
            p /= s; q /= s; r /= s;
            if (m == lo) break;
            const double u = std::fabs(A(m, m - 1)) * (std::fabs(q) + std::fabs(r));
            const double v = std::fabs(p) * (std::fabs(A(m - 1, m - 1)) + std::fabs(z) + std::fabs(A(m + 1, m + 1)));
            if (u <= ulp * v) break;
        }
        for (int64_t i = m + 2; i <= hi; i++) {
            A(i, i - 2) = 0;
            if (i != m + 2) A(i, i - 3) = 0;
        }
        for (int64_t k = m; k <= hi - 1; k++) {
            const bool last = k == hi - 1;
            if (k != m) {
                p = A(k, k - 1); q = A(k + 1, k - 1); r = last ? 0 : A(k + 2, k - 1);
                const double xs = std::fabs(p) + std::fabs(q) + std::fabs(r);
                if (xs == 0) continue;
                p /= xs; q /= xs; r /= xs;
            }
            const double s = std::copysign(std::sqrt(p * p + q * q + r * r), p);
            if (k == m) {
                if (lo != m) A(k, k - 1) = -A(k, k - 1);
            } else {
                const double xs = std::fabs(A(k, k - 1)) + std::fabs(A(k + 1, k - 1)) + (last ? 0.0 : std::fabs(A(k + 2, k - 1)));
                A(k, k - 1) = -s * xs;
            }
            p += s;
            const double vx = p / s, vy = q / s, vz = r / s;
            q /= p; r /= p;
            for (int64_t j = k; j < n; j++) {
                double t = A(k, j) + q * A(k + 1, j);
                if (!last) { t += r * A(k + 2, j); A(k + 2, j) -= t * vz; }
                A(k + 1, j) -= t * vy;
                A(k, j) -= t * vx;
            }
            for (int64_t i = 0; i <= std::min(hi, k + 3); i++) {
                double t = vx * A(i, k) + vy * A(i, k + 1);
                if (!last) { t += vz * A(i, k + 2); A(i, k + 2) -= t * r; }
                A(i, k + 1) -= t * q;
                A(i, k) -= t;
            }
        }
    }
    return 0;
}

// Eigenvector of the real upper Hessenberg h (column-major) for lambda:
// three steps of inverse iteration on h - lambda I (one row interchange
// per column in its LU), scaled so that the largest |re| + |im| is 1.
// a * b by the textbook formula (the library's operator calls a routine that
// recovers infinities from NaN results, several times slower; the values
// here are finite)
static inline cd cmul(cd a, cd b) {
    return cd(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
}

std::vector<cd> hessenberg_eigvec(int64_t n, const double *h, cd lambda, double hnorm) {
    std::vector<cd> a((size_t)(n * n), cd(0));
    auto A = [&](int64_t i, int64_t j) -> cd & { return a[(size_t)(i + j * n)]; };
    for (int64_t j = 0; j < n; j++)
        for (int64_t i = 0; i <= std::min(j + 1, n - 1); i++) A(i, j) = cd(h[i + j * n]);
    const double tiny = 1e-13 * std::max(hnorm, 1e-300);
    for (int64_t i = 0; i < n; i++) A(i, i) -= lambda + cd(tiny, 0);
    std::vector<char> swp((size_t)n, 0);
    std::vector<cd> mul((size_t)n, cd(0));
    for (int64_t k = 0; k + 1 < n; k++) {
        if (std::abs(A(k + 1, k)) > std::abs(A(k, k))) {
            swp[(size_t)k] = 1;
            for (int64_t j = k; j < n; j++) std::swap(A(k, j), A(k + 1, j));
        }
        if (A(k, k) == cd(0)) A(k, k) = cd(tiny, 0);
        const cd f = A(k + 1, k) / A(k, k);
        mul[(size_t)k] = f;
        for (int64_t j = k + 1; j < n; j++) A(k + 1, j) -= cmul(f, A(k, j));
    }
    if (A(n - 1, n - 1) == cd(0)) A(n - 1, n - 1) = cd(tiny, 0);
    std::vector<cd> x((size_t)n, cd(1.0 / std::sqrt((double)n), 0));
    for (int it = 0; it < 3; it++) {
        for (int64_t k = 0; k + 1 < n; k++) {
            if (swp[(size_t)k]) std::swap(x[(size_t)k], x[(size_t)k + 1]);
            x[(size_t)k + 1] -= cmul(mul[(size_t)k], x[(size_t)k]);
        }
        for (int64_t k = n - 1; k >= 0; k--) {
            x[(size_t)k] /= A(k, k);
            for (int64_t i = 0; i < k; i++) x[(size_t)i] -= cmul(A(i, k), x[(size_t)k]);
        }
        double mx = 0;
        for (auto &v : x) mx = std::max(mx, std::abs(v));
        if (mx == 0 || !std::isfinite(mx)) break;
        for (auto &v : x) v /= mx;
    }
    double big = 0;
    for (auto &v : x) big = std::max(big, std::fabs(v.real()) + std::fabs(v.imag()));
    if (big > 0)
        for (auto &v : x) v /= big;
    return x;
}

// a x = b for one right-hand side (complex, column-major n x n), partial
// pivoting; a and b overwritten
int complex_solve(int64_t n, std::vector<cd> &a, std::vector<cd> &b) {
    auto A = [&](int64_t i, int64_t j) -> cd & { return a[(size_t)(i + j * n)]; };
    for (int64_t k = 0; k < n; k++) {
        int64_t p = k;
        double mv = std::abs(A(k, k));
        for (int64_t i = k + 1; i < n; i++)
            if (std::abs(A(i, k)) > mv) { mv = std::abs(A(i, k)); p = i; }
        if (mv == 0) return (int)(k + 1);
        if (p != k) {
            for (int64_t j = 0; j < n; j++) std::swap(A(k, j), A(p, j));
            std::swap(b[(size_t)k], b[(size_t)p]);
        }
        const cd d = A(k, k);
        for (int64_t i = k + 1; i < n; i++) {
            const cd f = A(i, k) / d;
            if (f == cd(0)) continue;
            for (int64_t j = k + 1; j < n; j++) A(i, j) -= f * A(k, j);
            b[(size_t)i] -= f * b[(size_t)k];
        }
    }
    for (int64_t k = n - 1; k >= 0; k--) {
        cd s = b[(size_t)k];
        for (int64_t j = k + 1; j < n; j++) s -= A(k, j) * b[(size_t)j];
        b[(size_t)k] = s / A(k, k);
    }
    return 0;
}

unsigned fw_grid(int64_t n) { return grid_for(n, kFwThreads, 152LL * 8); }

}  // namespace

void fullwave_release(FullWave *fw, cudaStream_t s) {
    if (!fw) return;
    fw->release(s);
    delete fw;
}

bool fullwave_active(const FullWave *fw) { return fw && fw->active; }

// The V0 path's hook: the fields of ports p0 .. p0 + kk - 1 (interleaved
// [e * kk + r] blocks: yd1 = V0d y0d, ydat = V0da y0d, yd2, yc, and the
// a-value products yd2a, yca) become u0, u0a and yd per port.
g2p_status fullwave_keep_ports(g2p_mesh *m, int p0, int kk, const double *yd1, const double *ydat, const double *yd2,
                               const double *yc, const double *yd2a, const double *yca) {
    FullWave &F = *m->fw;
    cudaStream_t s = m->stream;
    const int64_t ne = m->d.N_edge, nr = F.nr;
    const int nb = 152 * 4;
    double *partial, *norms;
    G2P_TRY(dalloc(&partial, nb, s));
    G2P_TRY(dalloc(&norms, 4, s));
    for (int r = 0; r < kk; r++) {
        const int p = p0 + r;
        if ((int)F.u0.size() <= p) { F.u0.resize(p + 1, nullptr); F.u0a.resize(p + 1, nullptr); F.yd.resize(p + 1, nullptr); }
        G2P_TRY(dalloc(&F.u0[p], 2 * nr, s));
        G2P_TRY(dalloc(&F.u0a[p], 2 * nr, s));
        G2P_TRY(dalloc(&F.yd[p], 2 * ne, s));
        const double *pairs[4][2] = {{yd1, nullptr}, {ydat, nullptr}, {yd2, yc}, {yd2a, yca}};
        for (int q = 0; q < 4; q++) {
            (kbegin("k_fw_norm2", s), k_fw_norm2<<<nb, kFwThreads, 0, s>>>(ne, kk, r, pairs[q][0], pairs[q][1], partial), kend(s));
            (kbegin("k_fw_finish", s), k_fw_finish<<<1, 32, 0, s>>>(partial, nb, norms + q, 1), kend(s));
        }
        (kbegin("k_fw_fields", s), k_fw_fields<<<fw_grid(std::max(nr, ne)), kFwThreads, 0, s>>>(nr, ne, kk, r, F.map_r, yd1, ydat, yd2, yc, yd2a, yca, norms, F.u0[p], F.u0a[p], F.yd[p]), kend(s));
    }
    G2P_CUDA(cudaStreamSynchronize(s));
    dfree(partial, s);
    dfree(norms, s);
    return G2P_OK;
}

// The Vh correction of every port at every frequency and its Z entries:
// z[f][q + P p] complex, Construct_Z_V0_Vh into zeros.
g2p_status fullwave_z(g2p_mesh *m, const std::vector<double> &freqs, double *z) {
    FullWave &F = *m->fw;
    cudaStream_t s = m->stream;
    const Dims &d = m->d;
    const int P = m->num_ports;
    const int64_t nr = F.nr, mm = F.mm;
    std::memset(z, 0, sizeof(double) * 2 * freqs.size() * P * P);
    if (mm == 0) return G2P_OK;
    double *vhd, *T, *G, *yr2, *tmp4, *yn, *rhs, *sol, *fx, *Jr;
    G2P_TRY(dalloc(&vhd, 2 * nr * mm, s));
    G2P_TRY(dalloc(&T, 2 * nr * mm, s));
    G2P_TRY(dalloc(&G, 2 * mm * mm, s));
    G2P_TRY(dalloc(&yr2, 4 * mm, s));
    G2P_TRY(dalloc(&tmp4, 8, s));
    G2P_TRY(dalloc(&yn, 4 * mm, s));
    G2P_TRY(dalloc(&rhs, 2 * mm, s));
    G2P_TRY(dalloc(&sol, 2 * mm, s));
    G2P_TRY(dalloc(&fx, 2 * nr, s));
    G2P_TRY(dalloc(&Jr, nr, s));
    std::vector<double> h_y(4 * mm), h_t4(8), h_G(2 * mm * mm), h_rhs(2 * mm), h_fx(2 * nr);
    std::vector<int32_t> map_edge_h(d.N_edge);
    G2P_CUDA(cudaMemcpyAsync(map_edge_h.data(), m->map_edge, sizeof(int32_t) * d.N_edge, cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    g2p_status st = G2P_OK;
    for (int p = 0; p < P && st == G2P_OK; p++) {
        // J' marks the port's edges (any side's edge; J is nonzero there)
        std::vector<double> jr(nr, 0.0);
        for (int sd = m->port_side_ptr[p]; sd < m->port_side_ptr[p + 1]; sd++)
            for (int64_t q = m->side_edge_ptr[sd]; q < m->side_edge_ptr[sd + 1]; q++) {
                const int64_t e = m->side_edges[q];
                if (map_edge_h[e] >= 0) jr[map_edge_h[e]] = m->side_dir[sd];
            }
        G2P_CUDA(cudaMemcpyAsync(Jr, jr.data(), sizeof(double) * nr, cudaMemcpyHostToDevice, s));
        double cur = 0.;
        for (int sd = m->port_side_ptr[p]; sd < m->port_side_ptr[p + 1]; sd++) cur += m->side_area[sd];
        for (size_t fi = 0; fi < freqs.size(); fi++) {
            const double freq = freqs[fi];
            const double fsf = m->freq_start * m->freq_unit / freq;
            DiagOp D{F.map_r, m->mark_edge, m->epsn, d.Nv, d.L, m->k.eps0, freq};
            // (u0a^H A Vh) and (u0a^H A u0), then the 2 x 2 solves on the host
            (kbegin("k_fw_proj2", s), k_fw_proj2<<<(unsigned)mm, kFwThreads, 0, s>>>(nr, F.u0a[p], F.vh, 0, D, yr2), kend(s));
            (kbegin("k_fw_proj2", s), k_fw_proj2<<<2, kFwThreads, 0, s>>>(nr, F.u0a[p], F.u0[p], 1, D, tmp4), kend(s));
            G2P_CUDA(cudaMemcpyAsync(h_y.data(), yr2, sizeof(double) * 4 * mm, cudaMemcpyDeviceToHost, s));
            G2P_CUDA(cudaMemcpyAsync(h_t4.data(), tmp4, sizeof(double) * 8, cudaMemcpyDeviceToHost, s));
            G2P_CUDA(cudaStreamSynchronize(s));
            for (int64_t c = 0; c < mm; c++) {
                std::vector<cd> a2 = {cd(h_t4[0], h_t4[1]), cd(h_t4[2], h_t4[3]), cd(h_t4[4], h_t4[5]), cd(h_t4[6], h_t4[7])};
                std::vector<cd> b2 = {cd(h_y[4 * c], h_y[4 * c + 1]), cd(h_y[4 * c + 2], h_y[4 * c + 3])};
                if (complex_solve(2, a2, b2) != 0) {
                    set_last_message("full-wave: singular 2 x 2 deflation system");
                    st = G2P_ERR_INVALID;
                    break;
                }
                h_y[4 * c] = b2[0].real(); h_y[4 * c + 1] = b2[0].imag();
                h_y[4 * c + 2] = b2[1].real(); h_y[4 * c + 3] = b2[1].imag();
            }
            if (st != G2P_OK) break;
            G2P_CUDA(cudaMemcpyAsync(yn, h_y.data(), sizeof(double) * 4 * mm, cudaMemcpyHostToDevice, s));
            (kbegin("k_fw_deflate", s), k_fw_deflate<<<fw_grid(nr * mm), kFwThreads, 0, s>>>(nr, mm, F.vh, F.u0[p], yn, vhd), kend(s));
            (kbegin("k_fw_spmm", s), k_fw_spmm<<<fw_grid(nr * mm), kFwThreads, 0, s>>>(nr, mm, m->S.ptr, m->S.col, m->S.val, D, vhd, T), kend(s));
            dim3 gg((unsigned)((mm + kGt - 1) / kGt), (unsigned)((mm + kGt - 1) / kGt));
            (kbegin("k_fw_gram", s), k_fw_gram<<<gg, kGt * kGt, 0, s>>>(nr, mm, vhd, T, G), kend(s));
            (kbegin("k_fw_rhs", s), k_fw_rhs<<<(unsigned)mm, kFwThreads, 0, s>>>(nr, vhd, Jr, F.yd[p], D, fsf, rhs), kend(s));
            G2P_CUDA(cudaMemcpyAsync(h_G.data(), G, sizeof(double) * 2 * mm * mm, cudaMemcpyDeviceToHost, s));
            G2P_CUDA(cudaMemcpyAsync(h_rhs.data(), rhs, sizeof(double) * 2 * mm, cudaMemcpyDeviceToHost, s));
            G2P_CUDA(cudaStreamSynchronize(s));
            std::vector<cd> Am((size_t)(mm * mm)), bv((size_t)mm);
            for (int64_t i = 0; i < mm * mm; i++) Am[(size_t)i] = cd(h_G[2 * i], h_G[2 * i + 1]);
            for (int64_t i = 0; i < mm; i++) bv[(size_t)i] = cd(h_rhs[2 * i], h_rhs[2 * i + 1]);
            if (complex_solve(mm, Am, bv) != 0) {
                set_last_message("full-wave: singular Galerkin system");
                st = G2P_ERR_INVALID;
                break;
            }
            for (int64_t i = 0; i < mm; i++) { h_rhs[2 * i] = bv[(size_t)i].real(); h_rhs[2 * i + 1] = bv[(size_t)i].imag(); }
            G2P_CUDA(cudaMemcpyAsync(sol, h_rhs.data(), sizeof(double) * 2 * mm, cudaMemcpyHostToDevice, s));
            (kbegin("k_fw_final", s), k_fw_final<<<fw_grid(nr), kFwThreads, 0, s>>>(nr, mm, vhd, sol, F.yd[p], F.map_r, fsf, fx), kend(s));
            G2P_CUDA(cudaMemcpyAsync(h_fx.data(), fx, sizeof(double) * 2 * nr, cudaMemcpyDeviceToHost, s));
            G2P_CUDA(cudaStreamSynchronize(s));
            // Construct_Z_V0_Vh: the response port's first side
            for (int q = 0; q < P; q++) {
                const int sd = m->port_side_ptr[q];
                double re = 0, im = 0;
                for (int64_t t = m->side_edge_ptr[sd]; t < m->side_edge_ptr[sd + 1]; t++) {
                    const int64_t e = m->side_edges[t], rr = e % d.L;
                    double leng;
                    if (rr >= d.Ns) { const int64_t iz = e / d.L; leng = m->h_zn[iz + 1] - m->h_zn[iz]; }
                    else if (rr >= d.Ny * (d.Nx + 1)) { const int64_t ix = (rr - d.Ny * (d.Nx + 1)) / (d.Ny + 1); leng = m->h_xn[ix + 1] - m->h_xn[ix]; }
                    else { const int64_t iy = rr % d.Ny; leng = m->h_yn[iy + 1] - m->h_yn[iy]; }
                    const double dir = m->side_dir[sd] * 1.0;
                    const int64_t r = map_edge_h[e];
                    re -= h_fx[2 * r] * leng * dir;
                    im -= h_fx[2 * r + 1] * leng * dir;
                }
                double *zz = z + 2 * ((int64_t)fi * P * P + q + (int64_t)P * p);
                zz[0] = re / cur;
                zz[1] = im / cur;
            }
        }
    }
    dfree(vhd, s); dfree(T, s); dfree(G, s); dfree(yr2, s); dfree(tmp4, s); dfree(yn, s); dfree(rhs, s);
    dfree(sol, s); dfree(fx, s); dfree(Jr, s);
    G2P_CUDA(cudaStreamSynchronize(s));
    return st;
}

}  // namespace g2p

using namespace g2p;

extern "C" g2p_status g2p_hessenberg_eig(int64_t n, const double *h, double *wr, double *wi) {
    if (n < 1 || !h || !wr || !wi) { set_last_message("g2p_hessenberg_eig: bad arguments"); return G2P_ERR_INVALID; }
    std::vector<double> a(h, h + n * n);
    for (int64_t j = 0; j < n; j++)
        for (int64_t i = j + 2; i < n; i++) a[(size_t)(i + j * n)] = 0;
    if (hqr_eigenvalues(n, a.data(), wr, wi) != 0) {
        set_last_message("g2p_hessenberg_eig: QR iteration did not converge");
        return G2P_ERR_NOT_CONVERGED;
    }
    return G2P_OK;
}

extern "C" g2p_status g2p_find_vh(g2p_mesh *m, int32_t k, int64_t *leng_vh) {
    if (!m || k < 2) { set_last_message("g2p_find_vh: need a mesh and k >= 2"); return G2P_ERR_INVALID; }
    if (!m->stiff_done) { set_last_message("g2p_find_vh: g2p_generate_stiff has not run"); return G2P_ERR_STATE; }
    cudaStream_t s = m->stream;
    const Dims &d = m->d;
    const auto t_start = std::chrono::steady_clock::now();
    if (!m->fw) m->fw = new FullWave();
    FullWave &F = *m->fw;
    F.release(s);
    const int64_t nr = m->S.n, n2 = 2 * nr;
    if ((int64_t)k > n2) { set_last_message("g2p_find_vh: k = %d exceeds the operator's order %lld", k, (long long)n2); return G2P_ERR_INVALID; }
    F.nr = nr;
    G2P_TRY(dalloc(&F.map_r, nr, s));
    (kbegin("k_fw_map_r", s), k_fw_map_r<<<grid_for(d.N_edge), kThreads, 0, s>>>(d.N_edge, m->map_edge, F.map_r), kend(s));
    double *V, *w, *Hd, *partial, *sv = nullptr;
    const int nb = kFwNb;
    // operators of at most 4 * 1024 rows (the register budget of 1024
    // threads): one launch per Gram-Schmidt step (G2P_FW_MGS_LAUNCHES=1 keeps
    // the launch per basis vector, comparison)
    int rounds = 1;
    while (rounds < 4 && (int64_t)rounds * 1024 < n2) rounds <<= 1;
    const bool one_launch = (int64_t)rounds * 1024 >= n2 && !getenv("G2P_FW_MGS_LAUNCHES");
    // S v by the assembled CSR rows, each summed in S's entry order as the
    // reference sums them; G2P_FW_STENCIL=1 applies the matrix-free stencil
    // instead (equal to rounding, and no S traffic, but at k = 1000 the
    // Arnoldi basis amplifies rounding: the count of eigenvalues past the
    // |Im| > 1e-6 filter can then differ from the reference's by a few)
    const bool csr = getenv("G2P_FW_STENCIL") == nullptr;
    if (!csr) {
        if (!m->stencil) G2P_TRY(stencil_build(m, &m->stencil));
        G2P_TRY(dalloc(&sv, nr, s));
    }
    G2P_TRY(dalloc(&V, (int64_t)(k + 1) * n2, s));
    G2P_TRY(dalloc(&w, n2, s));
    G2P_TRY(dalloc(&Hd, (int64_t)k * k + k, s));
    G2P_TRY(dalloc(&partial, nb, s));
    G2P_CUDA(cudaMemsetAsync(Hd, 0, sizeof(double) * ((int64_t)k * k + k), s));
    const double scale = 1.e+14;
    (kbegin("k_fw_fill", s), k_fw_fill<<<fw_grid(n2), kFwThreads, 0, s>>>(n2, V, 1 / std::sqrt((double)(2 * nr))), kend(s));
    double *hnext = Hd + (int64_t)k * k;       // the norm after the last step (not part of H)
    for (int j = 1; j <= k; j++) {
        const double *vp = V + (int64_t)(j - 1) * n2;
        if (csr) {
            (kbegin("k_fw_apply", s), k_fw_apply<<<fw_grid(nr), kFwThreads, 0, s>>>(nr, m->S.ptr, m->S.col, m->S.val, F.map_r, m->mark_edge, m->epsn, m->sign, d.L, m->k.eps0, scale, vp, w), kend(s));
        } else {
            G2P_TRY(stencil_apply(m, m->stencil, vp, sv, s));
            (kbegin("k_fw_apply_sv", s), k_fw_apply_sv<<<fw_grid(nr), kFwThreads, 0, s>>>(nr, sv, F.map_r, m->mark_edge, m->epsn, m->sign, d.L, m->k.eps0, scale, vp, w), kend(s));
        }
        double *hcol = Hd + (int64_t)(j - 1) * k;
        double *hn = j < k ? hcol + j : hnext;
        if (one_launch) {
            // the whole step in one launch (bit-identical to the loop below)
            kbegin("k_fw_mgs_step", s);
            switch (rounds) {
                case 1: k_fw_mgs_step<1><<<1, 1024, 0, s>>>(n2, j, V, w, hcol, hn, V + (int64_t)j * n2); break;
                case 2: k_fw_mgs_step<2><<<1, 1024, 0, s>>>(n2, j, V, w, hcol, hn, V + (int64_t)j * n2); break;
                default: k_fw_mgs_step<4><<<1, 1024, 0, s>>>(n2, j, V, w, hcol, hn, V + (int64_t)j * n2); break;
            }
            kend(s);
            G2P_CUDA(cudaGetLastError());
            continue;
        }
        // modified Gram-Schmidt: h_i = V_i . w, w -= h_i V_i, in order; the
        // last update also gives the partials of |w|^2
        (kbegin("k_fw_dot", s), k_fw_dot<<<nb, kFwThreads, 0, s>>>(n2, V, w, partial), kend(s));
        for (int i = 0; i < j; i++) {
            (kbegin("k_fw_finish", s), k_fw_finish<<<1, 32, 0, s>>>(partial, nb, hcol + i, 0), kend(s));
            const double *next = i + 1 < j ? V + (int64_t)(i + 1) * n2 : w;
            (kbegin("k_fw_axpy_dot", s), k_fw_axpy_dot<<<nb, kFwThreads, 0, s>>>(n2, hcol + i, V + (int64_t)i * n2, w, next, partial), kend(s));
        }
        (kbegin("k_fw_finish", s), k_fw_finish<<<1, 32, 0, s>>>(partial, nb, hn, 1), kend(s));
        (kbegin("k_fw_scale", s), k_fw_scale<<<fw_grid(n2), kFwThreads, 0, s>>>(n2, w, hn, V + (int64_t)j * n2), kend(s));
        G2P_CUDA(cudaGetLastError());
    }
    std::vector<double> H((size_t)k * k);
    G2P_CUDA(cudaMemcpyAsync(H.data(), Hd, sizeof(double) * k * k, cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    dfree(sv, s);
    if (!csr) {
        const g2p_status sc = stencil_check(m->stencil, s);
        if (sc != G2P_OK) { dfree(V, s); dfree(w, s); dfree(Hd, s); dfree(partial, s); return sc; }
    }
    // eigenvalues, and the right eigenvectors of those with |Im| > 1e-6
    std::vector<double> H1((size_t)k * k, 0.0), wr(k), wi(k);
    for (int i = 0; i < k; i++)
        for (int c = 0; c < k; c++)
            if (i <= c + 1) H1[(size_t)c * k + i] = H[(size_t)c * k + i];
    const bool dbg = getenv("G2P_DEBUG") != nullptr;
    auto tq = std::chrono::steady_clock::now();
    std::vector<double> Hq = H1;
    if (hqr_eigenvalues(k, Hq.data(), wr.data(), wi.data()) != 0) {
        set_last_message("g2p_find_vh: QR iteration on the %d x %d Hessenberg matrix did not converge", k);
        dfree(V, s); dfree(w, s); dfree(Hd, s); dfree(partial, s);
        return G2P_ERR_NOT_CONVERGED;
    }
    double hnorm = 0;
    for (int c = 0; c < k; c++)
        for (int i = 0; i <= std::min(c + 1, k - 1); i++) hnorm += std::fabs(H1[(size_t)c * k + i]);
    auto te = std::chrono::steady_clock::now();
    // the eigenvalues kept (|Im| > 1e-6, positive imaginary part of each
    // pair), in order; their eigenvectors are independent, so host threads
    // share them out and each result lands in its own slot
    std::vector<int> keep;
    for (int j = 0; j < k; j++) {
        if (!(std::fabs(wi[j]) > 1e-6)) continue;
        if (wi[j] > 0 && j + 1 < k) {
            keep.push_back(j);
            j++;
        }
    }
    std::vector<std::vector<cd>> xs(keep.size());
    std::atomic<bool> no_mem(false);     // an allocation failed in a worker
    {
        const unsigned hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        const size_t nt = std::min<size_t>(hw, keep.size());
        std::vector<std::thread> pool;
        auto one = [&](size_t q) {
            try {
                xs[q] = hessenberg_eigvec(k, H1.data(), cd(wr[keep[q]], wi[keep[q]]), hnorm);
            } catch (const std::exception &) {
                no_mem = true;
            }
        };
        auto work = [&](size_t t0) {
            for (size_t q = t0; q < keep.size(); q += std::max<size_t>(nt, 1)) one(q);
        };
        try {
            for (size_t t = 1; t < nt; t++) pool.emplace_back(work, t);
        } catch (const std::exception &) {
            // fewer threads: the remaining strides are done below
        }
        const size_t started = pool.size() + 1;
        if (started == nt || nt <= 1) {
            work(0);
        } else {
            for (size_t q = 0; q < keep.size(); q++)
                if (q % nt == 0 || q % nt >= started) one(q);
        }
        for (auto &th : pool) th.join();
    }
    if (no_mem) {
        set_last_message("g2p_find_vh: out of host memory for the %d x %d eigenvector solves", k, k);
        dfree(V, s); dfree(w, s); dfree(Hd, s); dfree(partial, s);
        return G2P_ERR_NOMEM;
    }
    std::vector<double> vcols;       // [mm][k] complex, interleaved
    int64_t mm = 0;
    for (const std::vector<cd> &x : xs) {
        for (int t = 0; t < 2; t++)
            for (int i = 0; i < k; i++) {
                vcols.push_back(x[(size_t)i].real());
                vcols.push_back(t == 0 ? x[(size_t)i].imag() : -x[(size_t)i].imag());
            }
        mm += 2;
    }
    if (dbg) {
        auto tv = std::chrono::steady_clock::now();
        fprintf(stderr, "[g2p find_vh] k=%d: Arnoldi %.1f ms, Hessenberg eigenvalues %.1f ms, %zu eigenvectors %.1f ms\n",
                k, std::chrono::duration<double, std::milli>(tq - t_start).count(),
                std::chrono::duration<double, std::milli>(te - tq).count(), keep.size(),
                std::chrono::duration<double, std::milli>(tv - te).count());
    }
    F.mm = mm;
    if (mm > 0) {
        double *vd;
        G2P_TRY(dalloc(&vd, 2 * mm * k, s));
        G2P_CUDA(cudaMemcpyAsync(vd, vcols.data(), sizeof(double) * 2 * mm * k, cudaMemcpyHostToDevice, s));
        G2P_TRY(dalloc(&F.vh, 2 * nr * mm, s));
        (kbegin("k_fw_vh", s), k_fw_vh<<<fw_grid(nr * mm), kFwThreads, 0, s>>>(nr, n2, k, mm, V, vd, F.vh), kend(s));
        G2P_CUDA(cudaStreamSynchronize(s));
        dfree(vd, s);
    }
    dfree(V, s); dfree(w, s); dfree(Hd, s); dfree(partial, s);
    G2P_CUDA(cudaStreamSynchronize(s));
    if (leng_vh) *leng_vh = mm;
    return G2P_OK;
}

extern "C" g2p_status g2p_export_vh(g2p_mesh *m, double *vh) {
    if (!m || !m->fw || !vh) { set_last_message("g2p_export_vh: g2p_find_vh has not run"); return G2P_ERR_STATE; }
    if (m->fw->mm > 0)
        G2P_CUDA(cudaMemcpyAsync(vh, m->fw->vh, sizeof(double) * 2 * m->fw->nr * m->fw->mm, cudaMemcpyDefault, m->stream));
    G2P_CUDA(cudaStreamSynchronize(m->stream));
    return G2P_OK;
}

extern "C" g2p_status g2p_set_vh(g2p_mesh *m, const double *vh, int64_t leng_vh) {
    if (!m || leng_vh < 0 || (leng_vh > 0 && !vh)) { set_last_message("g2p_set_vh: bad arguments"); return G2P_ERR_INVALID; }
    if (!m->stiff_done) { set_last_message("g2p_set_vh: g2p_generate_stiff has not run"); return G2P_ERR_STATE; }
    cudaStream_t s = m->stream;
    if (!m->fw) m->fw = new FullWave();
    FullWave &F = *m->fw;
    F.release(s);
    F.nr = m->S.n;
    G2P_TRY(dalloc(&F.map_r, F.nr, s));
    (kbegin("k_fw_map_r", s), k_fw_map_r<<<grid_for(m->d.N_edge), kThreads, 0, s>>>(m->d.N_edge, m->map_edge, F.map_r), kend(s));
    F.mm = leng_vh;
    if (leng_vh > 0) {
        G2P_TRY(dalloc(&F.vh, 2 * F.nr * leng_vh, s));
        G2P_CUDA(cudaMemcpyAsync(F.vh, vh, sizeof(double) * 2 * F.nr * leng_vh, cudaMemcpyDefault, s));
    }
    G2P_CUDA(cudaStreamSynchronize(s));
    return G2P_OK;
}

// Frequency of point id as the reference's freqNo2freq (fdtd.hpp:4319-4334)
// and print_z_V0's last point (fdtd.hpp:4280-4283).
static double fw_freq(const g2p_mesh *m, int id) {
    if (m->nfreq == 1) return m->freq_start * m->freq_unit;
    if (id == m->nfreq - 1) return m->freq_end * m->freq_unit;
    if (m->freq_scale == 1) return (m->freq_start + id * (m->freq_end - m->freq_start) / (m->nfreq - 1)) * m->freq_unit;
    return m->freq_start * m->freq_unit * pow(m->freq_end / m->freq_start, (id * 1.0 / (m->nfreq - 1)));
}

extern "C" g2p_status g2p_para_generator_vh(g2p_mesh *m, const g2p_solver_params *p, int32_t k, double *z_vh,
                                            double *z_v0, g2p_extract_stats *st) {
    if (!m || !z_vh) { set_last_message("g2p_para_generator_vh: null argument"); return G2P_ERR_INVALID; }
    if (m->num_ports < 1) { set_last_message("g2p_para_generator_vh: the mesh has no ports"); return G2P_ERR_INVALID; }
    if (!m->stiff_done) {
        int64_t leng = 0;
        G2P_TRY(g2p_generate_stiff(m, &leng));
    }
    int64_t mm = 0;
    if (!m->fw || m->fw->nr != m->S.n || !m->fw->map_r) G2P_TRY(g2p_find_vh(m, k, &mm));
    FullWave &F = *m->fw;
    F.release_ports(m->stream);
    std::vector<double> zv0((size_t)2 * m->nfreq * m->num_ports * m->num_ports);
    F.active = true;
    g2p_status rc = g2p_para_generator(m, p, z_v0 ? z_v0 : zv0.data(), st);
    F.active = false;
    if (rc != G2P_OK && rc != G2P_ERR_NOT_CONVERGED) { F.release_ports(m->stream); return rc; }
    std::vector<double> freqs(m->nfreq);
    for (int f = 0; f < m->nfreq; f++) freqs[f] = fw_freq(m, f);
    g2p_status rz = fullwave_z(m, freqs, z_vh);
    F.release_ports(m->stream);
    return rz != G2P_OK ? rz : rc;
}
