// paraGenerator on the device (matrixCon.cpp:11-907, default SKIP_VH path).
//
// Per port the reference forms J on the port edges, solves Ad, Ac, Ad with
// HYPRE and back-projects with MKL sparse mat-vecs (matrixCon.cpp:363-603),
// then assembles Z with Construct_Z_V0 (fdtd.hpp:4173-4215) and rescales
// Im Z by f0/f in print_z_V0 (fdtd.hpp:4249-4316).  Here all ports of a
// block are right-hand sides of one batched solve per system, the V0
// products use the per-edge view (V y) and the column lists (V^T x) built at
// assembly, and the operations keep the reference's order per entry.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

#include "primitives.cuh"
#include "solver.h"

g2p_status g2p_run_v0(g2p_mesh *m);
g2p_status g2p_run_v0_ex(g2p_mesh *m, bool defer_ad);
g2p_status g2p_v0_finish(g2p_mesh *m, bool *repatterned = nullptr);
g2p_status g2p_v0_provisional(g2p_mesh *m);
g2p_status g2p_solver_build(const g2p::Csr<double> &A, const g2p_solver_params *p, cudaStream_t stream,
                            g2p_solver **out);
g2p_status g2p_solver_set_operator(g2p_solver *S, const g2p::Csr<double> &A, bool same_pattern);
g2p_status g2p_solver_solve_dev(g2p_solver *S, const double *b, double *x, int k, g2p_solve_stats *st);

namespace g2p {

// B[c, r] += aval * J over the port edges of the block (matrixCon.cpp:384,
// 436).  One thread per port adds its edges in their fixed order, so the
// sums are the same on every run; ports write disjoint entries of B.
__global__ void k_rhs_ports(int kk, const int64_t *pptr, const int32_t *pe_edge, const double *pe_J,
                            const int32_t *ecol, const double *eaval, int k, double *B) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= kk) return;
    for (int64_t t = pptr[r]; t < pptr[r + 1]; t++) {
        const int64_t e = pe_edge[t];
        const double J = pe_J[t];
        for (int s = 0; s < 2; s++) {
            const int32_t c = ecol[2 * e + s];
            if (c >= 0) B[(int64_t)c * k + r] += eaval[2 * e + s] * J;
        }
    }
}

__global__ void k_scale(int64_t n, double *x, double a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] *= a;
}

__global__ void k_div(int64_t n, double *x, double a) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) x[i] /= a;
}

// y[e, r] = V x over the (<= 2) entries of edge e in ascending column order
__global__ void k_v0_apply(int64_t nedge, int k, const int32_t *ecol, const double *eval, const double *X, double *Y) {
    const int r = threadIdx.x;
    if (r >= k) return;
    G2P_FOR_ROWS(e, nedge) {
        int64_t t = e * k + r;
        int32_t c0 = ecol[2 * e], c1 = ecol[2 * e + 1];
        // (0.0 + a0 x0) + a1 x1: the first addition only turns -0.0 into +0.0,
        // so it is a bit test here (the FP64 pipe is this kernel's limit)
        double acc = 0.0;
        if (c0 >= 0) {
            const double p = eval[2 * e] * X[(int64_t)c0 * k + r];
            acc = __double_as_longlong(p) == (long long)0x8000000000000000ULL ? 0.0 : p;
        }
        if (c1 >= 0) acc += eval[2 * e + 1] * X[(int64_t)c1 * k + r];
        Y[t] = acc;
    }
}

// Edge-side factor applied before a V^T product:
//   mode 0 (crhs, matrixCon.cpp:445): src * (-1.0 * omega * stackEpsn * eps0)
//   mode 1 (yccp, matrixCon.cpp:534): -src * stackEpsn * eps0
struct EdgeFactor {
    Dims d;
    const double *epsn;
    double omega, eps0;
    int mode;
    __device__ __forceinline__ double operator()(int64_t e, double v) const {
        double ep = epsn[e / d.L];
        if (mode == 0) return v * (-1.0 * omega * ep * eps0);
        return -v * ep * eps0;
    }
};

// out[c, r] = sum over column c's entries (in order) of aval * f(src[e, r])
__global__ void k_v0t_short(int64_t ncol, int k, const int64_t *cptr, const int32_t *cedge, const double *caval,
                            const double *src, EdgeFactor f, double *out) {
    const int r = threadIdx.x;
    if (r >= k) return;
    G2P_FOR_ROWS(c, ncol) {
        int64_t t = c * k + r;
        int64_t s0 = cptr[c], s1 = cptr[c + 1];
        if (s1 - s0 > kLongRow) continue;
        double acc = 0.0;
        for (int64_t q = s0; q < s1; q++) {
            int64_t e = cedge[q];
            acc += caval[q] * f(e, src[e * k + r]);
        }
        out[t] = acc;
    }
}

__global__ void __launch_bounds__(256) k_v0t_long(const int32_t *cols, int k, const int64_t *cptr, const int32_t *cedge,
                                                  const double *caval, const double *src, EdgeFactor f, double *out) {
    __shared__ double red[256];
    int64_t c = cols[blockIdx.x];
    int64_t s0 = cptr[c], s1 = cptr[c + 1];
    for (int r = 0; r < k; r++) {
        double acc = 0.0;
        for (int64_t q = s0 + threadIdx.x; q < s1; q += blockDim.x) {
            int64_t e = cedge[q];
            acc += caval[q] * f(e, src[e * k + r]);
        }
        red[threadIdx.x] = acc;
        __syncthreads();
        for (int o = 128; o > 0; o >>= 1) {
            if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[c * k + r] = red[0];
        __syncthreads();
    }
}

// Columns longer than kHugeRow: one block per chunk of kLongChunk entries
// (threadIdx.x = right-hand side, threadIdx.y strides over the entries);
// the block that finishes a column's last chunk adds the column's partials
// in chunk order and writes out.
__global__ void __launch_bounds__(256) k_v0t_chunk(const int32_t *cols, const int32_t *crow, const int64_t *cbeg,
                                                   const int64_t *rcp, int k, const int64_t *cptr,
                                                   const int32_t *cedge, const double *caval, const double *src,
                                                   EdgeFactor f, double *partial, int32_t *done, double *out) {
    __shared__ double sm[256];
    __shared__ int last;
    const int r = threadIdx.x, ty = threadIdx.y, ny = blockDim.y;
    const int l = crow[blockIdx.x];
    const int64_t c = cols[l];
    const int64_t q0 = cbeg[blockIdx.x], q1 = min(q0 + (int64_t)kLongChunk, cptr[c + 1]);
    double acc = 0.0;
    if (r < k)
        for (int64_t q = q0 + ty; q < q1; q += ny) {
            const int64_t e = cedge[q];
            acc += caval[q] * f(e, src[e * k + r]);
        }
    sm[ty * blockDim.x + r] = acc;
    __syncthreads();
    if (ty == 0 && r < k) {
        double t = 0;
        for (int q = 0; q < ny; q++) t += sm[q * blockDim.x + r];
        partial[(int64_t)blockIdx.x * kMaxRhs + r] = t;
    }
    __threadfence();
    __syncthreads();
    if (r == 0 && ty == 0) {
        const int nch = (int)(rcp[l + 1] - rcp[l]);
        last = atomicAdd(&done[l], 1) == nch - 1;
        if (last) done[l] = 0;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double t = 0;
    if (r < k)
        for (int64_t ch = rcp[l] + ty; ch < rcp[l + 1]; ch += ny) t += __ldcg(partial + ch * kMaxRhs + r);
    sm[ty * blockDim.x + r] = t;
    __syncthreads();
    if (ty != 0 || r >= k) return;
    double u = 0;
    for (int q = 0; q < ny; q++) u += sm[q * blockDim.x + r];
    out[c * k + r] = u;
}

__global__ void k_add(int64_t n, double *a, const double *b) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] += b[i];
}

// Construct_Z_V0 for the block: Z[q + P*p] over side-0 edges of port q.
__global__ void k_construct_z(int P, int p0, int kb, const int64_t *rptr, const int32_t *redge, const int32_t *rdir,
                              Dims d, const double *xn, const double *yn, const double *zn, const double *yd1,
                              const double *yc, const double *yd2, const double *cur, double *zre, double *zim) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= P * kb) return;
    int q = t % P, r = t / P;
    int p = p0 + r;
    double re = 0.0, im = 0.0;
    for (int64_t j = rptr[q]; j < rptr[q + 1]; j++) {
        int64_t e = redge[j];
        int64_t n1, n2, inz, inx, iny;
        int kind = d.edge_nodes(e, n1, n2, inz, inx, iny);
        double leng = kind == 2 ? zn[inz + 1] - zn[inz] : (kind == 1 ? xn[inx + 1] - xn[inx] : yn[iny + 1] - yn[iny]);
        double dir = rdir[q] * 1.0;
        double yre = (yd2[e * kb + r] - 0.0) + yc[e * kb + r];
        double yim = 0.0 - yd1[e * kb + r];
        re -= yre * leng * dir;
        im -= yim * leng * dir;
    }
    zre[q + (int64_t)P * p] = re / cur[p];
    zim[q + (int64_t)P * p] = im / cur[p];
}

// print_z_V0 layout: frequency 0 as assembled, later ones transposed with
// Im Z scaled by f0/f (fdtd.hpp:4270-4300).
__global__ void k_z_layout(int P, int nfreq, const double *fr, double f0, const double *zre, const double *zim,
                           double *out) {
    int64_t total = (int64_t)nfreq * P * P;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int f = (int)(t / ((int64_t)P * P));
        int64_t w = t - (int64_t)f * P * P;
        int i = (int)(w / P), j = (int)(w % P);   // w = j + i*P for the source entry
        int64_t src = j + (int64_t)i * P;
        int64_t o0 = (int64_t)f * P * P;
        if (f == 0) {
            out[2 * (o0 + src)] = zre[src];
            out[2 * (o0 + src) + 1] = zim[src];
        } else {
            int64_t dst = o0 + i + (int64_t)j * P;
            out[2 * dst] = zre[src] + 0.0;
            out[2 * dst + 1] = zim[src] * f0 / fr[f];
        }
    }
}

static double ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace g2p

using namespace g2p;

static double freq_of(const g2p_mesh *m, int id) {
    if (m->nfreq == 1) return m->freq_start * m->freq_unit;
    if (id == m->nfreq - 1) return m->freq_end * m->freq_unit;
    if (m->freq_scale == 1)
        return (m->freq_start + id * (m->freq_end - m->freq_start) / (m->nfreq - 1)) * m->freq_unit;
    return m->freq_start * m->freq_unit * pow(m->freq_end / m->freq_start, (id * 1.0 / (m->nfreq - 1)));
}

// Block width of the port right-hand sides and Chebyshev degree of the Ad
// solves, per grid shape, port count and precision: the first choice made in
// the process is kept, so every later job of that shape runs the same way.
struct TuneKey {
    int64_t nx, ny, nz, nnz;
    int P, precision;
    bool operator<(const TuneKey &o) const {
        return std::tie(nx, ny, nz, nnz, P, precision) < std::tie(o.nx, o.ny, o.nz, o.nnz, o.P, o.precision);
    }
};
static std::mutex g_tune_mu;
static std::map<TuneKey, std::pair<int, int>> g_tuned;   // -> (block width, degree)
// Aggregation strength of Ac's AMG, keyed by Ac's entry count in nnz.  Ac's
// iteration count is far from monotonic in it (c3: 24 iterations at 0.02, 54
// at 0.04, 76 at 0.08; c2: 45, 37 and 33), so it is measured per shape.
// Ac's tuned solver: aggregation strength and precision mode
struct AcChoice {
    double strength;
    int precision;
    int restart;
    bool operator!=(const AcChoice &o) const {
        return strength != o.strength || precision != o.precision || restart != o.restart;
    }
};
static std::map<TuneKey, AcChoice> g_ac_tuned;

static bool ac_tuned(const TuneKey &key, AcChoice *c) {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_ac_tuned.find(key);
    if (it == g_ac_tuned.end()) return false;
    *c = it->second;
    return true;
}

// Times Ac's solve of the first block with the strength thresholds st0 / 2,
// st0 and 2 st0 (at most 0.1), st0 being Ad's, and, when modes lists more
// than one precision mode, with each of them (and, for FP64 Krylov with the
// FP32 V-cycle, with each restart length in restarts: its Gram-Schmidt is
// bound by the FP64 pipe, so a shorter restart pays where the iteration
// count does not grow much); *Sc (built with pc) is one of the candidates.  Each candidate: one untimed solve, then the better of two
// timed ones.  *Sc is replaced by the solver of the recorded choice: the
// fastest candidate, unless another job of the shape recorded its choice
// first.  (Ac in the mixed mode's FP32 refinement is faster where its sweeps
// converge, e.g. c3's 256 x 256 x 16 layout, and stalls into the FP64
// fallback where they do not, e.g. c2's; only timing tells them apart.)
static g2p_status tune_ac(g2p_mesh *m, const TuneKey &key, const g2p_solver_params &pc, double st0,
                          const std::vector<int> &modes, const std::vector<int> &restarts, g2p_solver **Sc,
                          const double *Bc, double *Yc, int kk, cudaStream_t s) {
    std::vector<AcChoice> cands;
    for (int mode : modes)
        for (int rs : mode == G2P_PREC_FP64_PC32 ? restarts : std::vector<int>{pc.restart})
            for (double st : {st0 / 2, st0, std::min(2 * st0, 0.1)}) cands.push_back({st, mode, rs});
    const AcChoice cur{pc.strength, pc.precision, pc.restart};
    double best_ms = 1e300;
    AcChoice best_c = cur;
    g2p_solver *best = nullptr;
    for (const AcChoice &c : cands) {
        g2p_solver *S = nullptr;
        if (!(c != cur)) {
            S = *Sc;
        } else {
            g2p_solver_params q = pc;
            q.strength = c.strength;
            q.precision = c.precision;
            q.restart = c.restart;
            if (g2p_solver_build(m->Ac, &q, s, &S) != G2P_OK) { cudaGetLastError(); continue; }
        }
        g2p_solve_stats ss;
        g2p_status rc = g2p_solver_solve_dev(S, Bc, Yc, kk, &ss);
        double ms = 1e300;
        for (int rep = 0; rep < 2 && rc == G2P_OK; rep++) {
            auto t = std::chrono::steady_clock::now();
            rc = g2p_solver_solve_dev(S, Bc, Yc, kk, &ss);
            ms = std::min(ms, ms_since(t));
        }
        if (getenv("G2P_DEBUG"))
            fprintf(stderr, "[g2p tune] Ac strength %.3g precision %d restart %d: %.3f ms%s\n", c.strength, c.precision,
                    c.restart, ms, rc == G2P_OK ? "" : " (not converged)");
        if (rc == G2P_OK && ms < best_ms) {
            if (best && best != *Sc) g2p_solver_destroy(best);
            best = S; best_ms = ms; best_c = c;
        } else if (S != *Sc) {
            cudaGetLastError();
            g2p_solver_destroy(S);
        }
    }
    if (best && best != *Sc) {
        g2p_solver_destroy(*Sc);
        *Sc = best;
    }
    AcChoice kept = best ? best_c : cur;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        kept = g_ac_tuned.emplace(key, kept).first->second;   // an earlier entry wins
    }
    if (best && kept != best_c) {
        // another job of this shape recorded its choice first: follow it, so
        // every job of the shape runs the same way
        g2p_solver_params q = pc;
        q.strength = kept.strength;
        q.precision = kept.precision;
        q.restart = kept.restart;
        g2p_solver *S = nullptr;
        G2P_TRY(g2p_solver_build(m->Ac, &q, s, &S));
        g2p_solver_destroy(*Sc);
        *Sc = S;
    }
    return G2P_OK;
}

// Times the Ad solve of the first block of ports with each candidate (after
// an untimed solve, best of two) and keeps the one with the least estimated
// time for all blocks.
template <class F>
static g2p_status tune_blocks(g2p_mesh *m, g2p_solver *Sd, int P, int precision, F &rhs_d, double *Bd, double *Yd,
                              int *kb) {
    const TuneKey key{m->d.nx, m->d.ny, m->d.nz, m->Ad.nnz, P, precision};
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tuned.find(key);
        if (it != g_tuned.end()) {
            *kb = it->second.first;
            Sd->cfg.degree = it->second.second;
            return G2P_OK;
        }
    }
    std::vector<int> widths = {*kb};
    for (int w : {64, 32, 16, 8})
        if (w < *kb) widths.push_back(w);
    const int degree0 = Sd->cfg.degree;
    int best_w = *kb, best_d = degree0;
    double best = 1e300;
    for (int w : widths) {
        G2P_TRY(rhs_d(0, w));
        for (int deg : {2, 3, 4}) {
            Sd->cfg.degree = deg;
            g2p_solve_stats ss;
            // one untimed solve (work vectors, graph captures), then the
            // better of two timed ones
            g2p_status rc = g2p_solver_solve_dev(Sd, Bd, Yd, w, &ss);
            double ms = 1e300;
            for (int rep = 0; rep < 2 && rc == G2P_OK; rep++) {
                auto t = std::chrono::steady_clock::now();
                rc = g2p_solver_solve_dev(Sd, Bd, Yd, w, &ss);
                ms = std::min(ms, ms_since(t));
            }
            if (rc != G2P_OK) continue;
            const double total = ms * ((P + w - 1) / w);
            if (total < best) { best = total; best_w = w; best_d = deg; }
        }
    }
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto ins = g_tuned.emplace(key, std::make_pair(best_w, best_d)).first;   // an earlier entry wins
    *kb = ins->second.first;
    Sd->cfg.degree = ins->second.second;
    return G2P_OK;
}

extern "C" g2p_status g2p_para_generator(g2p_mesh *m, const g2p_solver_params *pin, double *z_out,
                                         g2p_extract_stats *st) {
    if (!m || !z_out) { set_last_message("null argument"); return G2P_ERR_INVALID; }
    if (m->num_ports < 1) { set_last_message("mesh has no ports"); return G2P_ERR_INVALID; }
    g2p_solver_params p;
    if (pin) p = *pin; else g2p_default_params(&p, 0);
    auto t_all = std::chrono::steady_clock::now();
    cudaStream_t s = m->stream;
    const Dims &d = m->d;
    const int P = m->num_ports;
    g2p_extract_stats local;
    memset(&local, 0, sizeof(local));
    auto t0 = std::chrono::steady_clock::now();
    // Ad's ordered conductor sums keep running on the mesh's side stream
    // while the ports are prepared and the solvers are set up
    G2P_TRY(g2p_run_v0_ex(m, true));
    local.assembly_ms = ms_since(t0);
    // ---- port data: J entries (last side wins, matrixCon.cpp:367-374),
    //      response edges (side 0) and source currents
    std::vector<int32_t> pe_edge;
    std::vector<double> pe_J, cur(P, 0.0);
    std::vector<int64_t> pptr(P + 1, 0), rptr(P + 1, 0);
    std::vector<int32_t> redge, rdir(P);
    for (int q = 0; q < P; q++) {
        std::map<int64_t, int> J;
        for (int sd = m->port_side_ptr[q]; sd < m->port_side_ptr[q + 1]; sd++) {
            for (int64_t j = m->side_edge_ptr[sd]; j < m->side_edge_ptr[sd + 1]; j++) J[m->side_edges[j]] = m->side_dir[sd];
            cur[q] += m->side_area[sd];
        }
        for (auto &kv : J) { pe_edge.push_back((int32_t)kv.first); pe_J.push_back((double)kv.second); }
        pptr[q + 1] = (int64_t)pe_edge.size();
        int s0 = m->port_side_ptr[q];
        for (int64_t j = m->side_edge_ptr[s0]; j < m->side_edge_ptr[s0 + 1]; j++) redge.push_back((int32_t)m->side_edges[j]);
        rptr[q + 1] = (int64_t)redge.size();
        rdir[q] = m->side_dir[s0];
    }
    int32_t *d_pe_edge, *d_redge, *d_rdir;
    double *d_pe_J, *d_cur;
    int64_t *d_rptr, *d_pptr;
    int64_t npe = (int64_t)pe_edge.size();
    G2P_TRY(dalloc(&d_pe_edge, npe, s)); G2P_TRY(dalloc(&d_pe_J, npe, s)); G2P_TRY(dalloc(&d_pptr, P + 1, s));
    G2P_CUDA(cudaMemcpyAsync(d_pptr, pptr.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, s));
    G2P_TRY(dalloc(&d_redge, (int64_t)redge.size(), s)); G2P_TRY(dalloc(&d_rdir, P, s));
    G2P_TRY(dalloc(&d_rptr, P + 1, s)); G2P_TRY(dalloc(&d_cur, P, s));
    G2P_CUDA(cudaMemcpyAsync(d_pe_edge, pe_edge.data(), sizeof(int32_t) * npe, cudaMemcpyHostToDevice, s));
    G2P_CUDA(cudaMemcpyAsync(d_pe_J, pe_J.data(), sizeof(double) * npe, cudaMemcpyHostToDevice, s));
    G2P_CUDA(cudaMemcpyAsync(d_redge, redge.data(), sizeof(int32_t) * redge.size(), cudaMemcpyHostToDevice, s));
    G2P_CUDA(cudaMemcpyAsync(d_rdir, rdir.data(), sizeof(int32_t) * P, cudaMemcpyHostToDevice, s));
    G2P_CUDA(cudaMemcpyAsync(d_rptr, rptr.data(), sizeof(int64_t) * (P + 1), cudaMemcpyHostToDevice, s));
    G2P_CUDA(cudaMemcpyAsync(d_cur, cur.data(), sizeof(double) * P, cudaMemcpyHostToDevice, s));
    // ---- solvers (setup once per operator; the reference rebuilds per call)
    t0 = std::chrono::steady_clock::now();
    g2p_solver *Sd = nullptr, *Sc = nullptr;
    // Ac first: its setup overlaps Ad's ordered sums on the side stream.
    // Ac, the conductor Laplacian, keeps its Krylov iteration in FP64 by
    // default: a floating wire grounded at one node gives it a condition
    // number near (length/h)^2, beyond what an FP32 refinement sweep
    // resolves.  In the mixed method its V-cycle preconditioner runs in
    // FP32; with autotune the first job of a grid shape also times Ac in the
    // mixed method's FP32 refinement and keeps it where that is faster.
    // G2P_AC_PRECISION overrides the mode (comparisons).
    g2p_solver_params pc = p;
    const double st0 = p.strength > 0 ? p.strength : 0.04;
    const TuneKey ac_key{m->d.nx, m->d.ny, m->d.nz, m->Ac.nnz, P, p.precision};
    const bool ac_fixed = getenv("G2P_AC_STRENGTH") != nullptr;
    AcChoice ac_c{0.0, 0, 0};
    const bool ac_known = ac_tuned(ac_key, &ac_c);
    const bool ac_prec_fixed = getenv("G2P_AC_PRECISION") != nullptr;
    {
        if (p.precision == G2P_PREC_MIXED) pc.precision = G2P_PREC_FP64_PC32;
        if (ac_prec_fixed) pc.precision = atoi(getenv("G2P_AC_PRECISION"));
        else if (ac_known) pc.precision = ac_c.precision;
        // Ac's aggregation wants a stronger threshold than Ad's: twice Ad's,
        // at most 0.1 (c2 sweep: 0.04 -> 37 iterations, 0.08 -> 33, >= 0.15
        // stalls).  G2P_AC_STRENGTH / G2P_AC_DEGREE / G2P_AC_RESTART
        // override (comparisons).
        pc.strength = std::min(2 * st0, 0.1);
        if (ac_fixed) pc.strength = atof(getenv("G2P_AC_STRENGTH"));
        else if (ac_known) pc.strength = ac_c.strength;
        if (const char *t = getenv("G2P_AC_DEGREE")) pc.smoother_degree = atoi(t);
        if (const char *t = getenv("G2P_AC_RESTART")) pc.restart = atoi(t);
        else if (ac_known) pc.restart = ac_c.restart;
    }
    // Ac's solver is built by a second host thread on its own stream (after
    // Ac's assembly, an event on the job's stream) while this thread
    // finishes Ad and builds its solver: both setups are partly latency-bound
    // (per-level size read-backs).  Sequential while kernels are being timed
    // one by one (the timing collectors are single-threaded).
    g2p_status rs_c = G2P_OK, rs = G2P_OK;
    std::string err_c;
    cudaStream_t s2 = nullptr;
    cudaEvent_t ac_ready = nullptr;
    std::thread tc;
    if (!kprof_on() && cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking) == cudaSuccess &&
        cudaEventCreateWithFlags(&ac_ready, cudaEventDisableTiming) == cudaSuccess) {
        G2P_CUDA(cudaEventRecord(ac_ready, s));
        G2P_CUDA(cudaStreamWaitEvent(s2, ac_ready, 0));
        int dev = 0;
        G2P_CUDA(cudaGetDevice(&dev));
        try {
            tc = std::thread([&, dev] {
                cudaSetDevice(dev);
                rs_c = g2p_solver_build(m->Ac, &pc, s2, &Sc);
                if (rs_c != G2P_OK) err_c = g2p_last_error();
            });
        } catch (const std::exception &) {
            // no thread to be had: build Ac's solver here, after Ad's
        }
    } else {
        cudaGetLastError();
    }
    const bool ac_here = !tc.joinable();
    // Ad's preconditioner is built from Ad with stand-in sums for its
    // longest segments while their ordered sums finish on the side stream;
    // the solver's operator then gets the exact Ad
    rs = g2p_v0_provisional(m);
    if (rs == G2P_OK) rs = g2p_solver_build(m->Ad, &p, s, &Sd);
    if (rs == G2P_OK) {
        bool repatterned = false;
        rs = g2p_v0_finish(m, &repatterned);
        if (rs == G2P_OK) rs = g2p_solver_set_operator(Sd, m->Ad, !repatterned);
    }
    if (tc.joinable()) tc.join();
    if (ac_here && rs == G2P_OK) {
        rs_c = g2p_solver_build(m->Ac, &pc, s, &Sc);
        if (rs_c != G2P_OK) err_c = g2p_last_error();
    }
    if (Sc) Sc->stream = s;           // the solves run on the job's stream
    if (s2) { cudaStreamSynchronize(s2); cudaStreamDestroy(s2); }
    if (ac_ready) cudaEventDestroy(ac_ready);
    if (rs_c != G2P_OK || rs != G2P_OK) {
        if (rs == G2P_OK) set_last_message("%s", err_c.c_str());
        g2p_solver_destroy(Sc);
        g2p_solver_destroy(Sd);
        return rs != G2P_OK ? rs : rs_c;
    }
    local.setup_ms = ms_since(t0);
    local.ad_levels = Sd->levels;
    local.ac_levels = Sc->levels;
    local.ac_strength = pc.strength;
    local.ac_precision = pc.precision;
    LongRows lcol;   // long columns of V0d (conductor columns)
    {
        Csr<double> tmp;
        tmp.n = m->v0d.ncol; tmp.ptr = m->v0d.cptr;
        G2P_TRY(find_long_rows<double>(tmp, lcol, s));
    }
    // long V0d columns: up to kHugeRow entries one block each, longer ones in chunks
    const int32_t *d_mid_d = lcol.mid;
    const int64_t nmid_d = lcol.nmid;
    int kb = p.batch == 0 ? 1 : std::min(p.batch >= 2 ? p.batch : P, std::min(P, kMaxRhs));
    const int64_t nd = m->v0d.ncol, nc = m->v0c.ncol, ne = d.N_edge;
    double *Bd, *Yd, *Bc, *Yc, *crhs, *yd1, *yc, *yd2, *zre, *zim;
    G2P_TRY(dalloc(&Bd, nd * kb, s)); G2P_TRY(dalloc(&Yd, nd * kb, s));
    G2P_TRY(dalloc(&Bc, nc * kb, s)); G2P_TRY(dalloc(&Yc, nc * kb, s)); G2P_TRY(dalloc(&crhs, nc * kb, s));
    G2P_TRY(dalloc(&yd1, ne * kb, s)); G2P_TRY(dalloc(&yc, ne * kb, s)); G2P_TRY(dalloc(&yd2, ne * kb, s));
    G2P_TRY(dalloc(&zre, (int64_t)P * P, s)); G2P_TRY(dalloc(&zim, (int64_t)P * P, s));
    // full-wave mode keeps each port's V0 fields: the a-value products too
    const bool fw = fullwave_active(m->fw);
    double *ydat = nullptr, *yd2a = nullptr, *yca = nullptr;
    if (fw) { G2P_TRY(dalloc(&ydat, ne * kb, s)); G2P_TRY(dalloc(&yd2a, ne * kb, s)); G2P_TRY(dalloc(&yca, ne * kb, s)); }
    const double omega = (2 * 3.14159265358979323846 * m->freq_start * m->freq_unit);
    EdgeFactor f0{d, m->epsn, omega, m->k.eps0, 0};
    EdgeFactor f1{d, m->epsn, omega, m->k.eps0, 1};
    // (1) b_d = -V0da^T J for ports p0 .. p0 + kk - 1
    auto rhs_d = [&](int p0, int kk) -> g2p_status {
        const int64_t *d_pp = d_pptr + p0;     // entries of port p0 + r: [d_pp[r], d_pp[r + 1])
        const unsigned rg = (unsigned)((kk + 127) / 128);
        G2P_CUDA(cudaMemsetAsync(Bd, 0, sizeof(double) * nd * kk, s));
        (g2p::kbegin("k_rhs_ports", s), k_rhs_ports<<<rg, 128, 0, s>>>(kk, d_pp, d_pe_edge, d_pe_J, m->v0d.ecol, m->v0d.eaval, kk, Bd), g2p::kend(s));
        (g2p::kbegin("k_scale", s), k_scale<<<grid_for(nd * kk), kThreads, 0, s>>>(nd * kk, Bd, -1.0), g2p::kend(s));
        return G2P_OK;
    };
    if (p.autotune && p.batch) G2P_TRY(tune_blocks(m, Sd, P, p.precision, rhs_d, Bd, Yd, &kb));
    local.rhs_block = kb;
    local.ad_degree = Sd->cfg.degree;
    t0 = std::chrono::steady_clock::now();
    g2p_status worst_rc = G2P_OK;
    for (int p0 = 0; p0 < P; p0 += kb) {
        int kk = std::min(kb, P - p0);
        // entries of this block's ports, renumbered 0..kk-1
        const int64_t *d_pp = d_pptr + p0;     // entries of port p0 + r: [d_pp[r], d_pp[r + 1])
        const unsigned rg = (unsigned)((kk + 127) / 128);
        G2P_TRY(rhs_d(p0, kk));
        g2p_solve_stats ss;
        g2p_status rc = g2p_solver_solve_dev(Sd, Bd, Yd, kk, &ss);
        if (rc != G2P_OK && rc != G2P_ERR_NOT_CONVERGED) { worst_rc = rc; break; }
        if (rc == G2P_ERR_NOT_CONVERGED) worst_rc = rc;
        local.solves += kk; local.total_iterations += ss.iterations;
        local.max_rel_residual = std::max(local.max_rel_residual, ss.rel_residual);
        // (2) y0d /= omega ; yd1 = V0d y0d
        (g2p::kbegin("k_div", s), k_div<<<grid_for(nd * kk), kThreads, 0, s>>>(nd * kk, Yd, omega), g2p::kend(s));
        (g2p::kbegin("k_v0_apply", s), k_v0_apply<<<row_grid(ne, kk), row_block(kk), 0, s>>>(ne, kk, m->v0d.ecol, m->v0d.eval, Yd, yd1), g2p::kend(s));
        if (fw)
            (g2p::kbegin("k_v0_apply", s), k_v0_apply<<<row_grid(ne, kk), row_block(kk), 0, s>>>(ne, kk, m->v0d.ecol, m->v0d.eaval, Yd, ydat), g2p::kend(s));
        // (3) b_c = -V0ca^T J + V0ca^T(-omega D_eps yd1)
        G2P_CUDA(cudaMemsetAsync(Bc, 0, sizeof(double) * nc * kk, s));
        (g2p::kbegin("k_rhs_ports", s), k_rhs_ports<<<rg, 128, 0, s>>>(kk, d_pp, d_pe_edge, d_pe_J, m->v0c.ecol, m->v0c.eaval, kk, Bc), g2p::kend(s));
        (g2p::kbegin("k_scale", s), k_scale<<<grid_for(nc * kk), kThreads, 0, s>>>(nc * kk, Bc, -1.0), g2p::kend(s));
        (g2p::kbegin("k_v0t_short", s), k_v0t_short<<<row_grid(nc, kk), row_block(kk), 0, s>>>(nc, kk, m->v0c.cptr, m->v0c.cedge, m->v0c.caval, yd1, f0, crhs), g2p::kend(s));
        (g2p::kbegin("k_add", s), k_add<<<grid_for(nc * kk), kThreads, 0, s>>>(nc * kk, Bc, crhs), g2p::kend(s));
        // (4) Ac y0c = b_c
        if (p0 == 0 && p.autotune && !ac_fixed && !ac_known) {
            std::vector<int> modes = {pc.precision};
            if (p.precision == G2P_PREC_MIXED && !ac_prec_fixed && pc.precision != G2P_PREC_MIXED)
                modes.push_back(G2P_PREC_MIXED);
            std::vector<int> restarts = {pc.restart};
            if (!getenv("G2P_AC_RESTART") && pc.restart > 10) restarts.push_back(10);
            G2P_TRY(tune_ac(m, ac_key, pc, st0, modes, restarts, &Sc, Bc, Yc, kk, s));
            AcChoice tuned{0.0, 0, 0};
            if (ac_tuned(ac_key, &tuned)) {
                local.ac_strength = tuned.strength;
                local.ac_precision = tuned.precision;
            }
            local.ac_levels = Sc->levels;
        }
        rc = g2p_solver_solve_dev(Sc, Bc, Yc, kk, &ss);
        if (rc != G2P_OK && rc != G2P_ERR_NOT_CONVERGED) { worst_rc = rc; break; }
        if (rc == G2P_ERR_NOT_CONVERGED) worst_rc = rc;
        local.ac_iterations += ss.iterations;
        local.solves += kk; local.total_iterations += ss.iterations;
        local.max_rel_residual = std::max(local.max_rel_residual, ss.rel_residual);
        // (5) yc = V0c y0c ; b_d2 = V0da^T(-D_eps yc)
        (g2p::kbegin("k_v0_apply", s), k_v0_apply<<<row_grid(ne, kk), row_block(kk), 0, s>>>(ne, kk, m->v0c.ecol, m->v0c.eval, Yc, yc), g2p::kend(s));
        if (fw)
            (g2p::kbegin("k_v0_apply", s), k_v0_apply<<<row_grid(ne, kk), row_block(kk), 0, s>>>(ne, kk, m->v0c.ecol, m->v0c.eaval, Yc, yca), g2p::kend(s));
        (g2p::kbegin("k_v0t_short", s), k_v0t_short<<<row_grid(nd, kk), row_block(kk), 0, s>>>(nd, kk, m->v0d.cptr, m->v0d.cedge, m->v0d.caval, yc, f1, Bd), g2p::kend(s));
        if (nmid_d > 0)
            (g2p::kbegin("k_v0t_long", s), k_v0t_long<<<(unsigned)nmid_d, 256, 0, s>>>(d_mid_d, kk, m->v0d.cptr, m->v0d.cedge, m->v0d.caval, yc, f1, Bd), g2p::kend(s));
        if (lcol.nchunk > 0)
            (g2p::kbegin("k_v0t_chunk", s), k_v0t_chunk<<<(unsigned)lcol.nchunk, row_block(kk), 0, s>>>(lcol.rows, lcol.crow, lcol.cbeg, lcol.rcp, kk, m->v0d.cptr, m->v0d.cedge, m->v0d.caval, yc, f1, lcol.partial, lcol.done, Bd), g2p::kend(s));
        // (6) Ad y0d2 = b_d2 ; yd2 = V0d y0d2
        rc = g2p_solver_solve_dev(Sd, Bd, Yd, kk, &ss);
        if (rc != G2P_OK && rc != G2P_ERR_NOT_CONVERGED) { worst_rc = rc; break; }
        if (rc == G2P_ERR_NOT_CONVERGED) worst_rc = rc;
        local.solves += kk; local.total_iterations += ss.iterations;
        local.max_rel_residual = std::max(local.max_rel_residual, ss.rel_residual);
        (g2p::kbegin("k_v0_apply", s), k_v0_apply<<<row_grid(ne, kk), row_block(kk), 0, s>>>(ne, kk, m->v0d.ecol, m->v0d.eval, Yd, yd2), g2p::kend(s));
        if (fw) {
            (g2p::kbegin("k_v0_apply", s), k_v0_apply<<<row_grid(ne, kk), row_block(kk), 0, s>>>(ne, kk, m->v0d.ecol, m->v0d.eaval, Yd, yd2a), g2p::kend(s));
            G2P_TRY(fullwave_keep_ports(m, p0, kk, yd1, ydat, yd2, yc, yd2a, yca));
        }
        // (7) Construct_Z_V0
        (g2p::kbegin("k_construct_z", s), k_construct_z<<<(P * kk + 127) / 128, 128, 0, s>>>(P, p0, kk, d_rptr, d_redge, d_rdir, d, m->xn, m->yn, m->zn, yd1,
                                                          yc, yd2, d_cur, zre, zim), g2p::kend(s));
    }
    // ---- print_z_V0 layout
    std::vector<double> fr(m->nfreq);
    for (int f = 0; f < m->nfreq; f++) fr[f] = freq_of(m, f);
    double *d_fr, *d_out;
    G2P_TRY(dalloc(&d_fr, m->nfreq, s));
    G2P_TRY(dalloc(&d_out, 2LL * m->nfreq * P * P, s));
    G2P_CUDA(cudaMemcpyAsync(d_fr, fr.data(), sizeof(double) * m->nfreq, cudaMemcpyHostToDevice, s));
    (g2p::kbegin("k_z_layout", s), k_z_layout<<<grid_for((int64_t)m->nfreq * P * P), kThreads, 0, s>>>(P, m->nfreq, d_fr, m->freq_start * m->freq_unit,
                                                                        zre, zim, d_out), g2p::kend(s));
    G2P_CUDA(cudaMemcpyAsync(z_out, d_out, sizeof(double) * 2 * m->nfreq * P * P, cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    local.solve_ms = ms_since(t0);
    dfree(d_fr, s); dfree(d_out, s);
    dfree(Bd, s); dfree(Yd, s); dfree(Bc, s); dfree(Yc, s); dfree(crhs, s);
    dfree(yd1, s); dfree(yc, s); dfree(yd2, s); dfree(zre, s); dfree(zim, s);
    dfree(ydat, s); dfree(yd2a, s); dfree(yca, s);
    dfree(d_pe_edge, s); dfree(d_pptr, s); dfree(d_pe_J, s); dfree(d_redge, s); dfree(d_rdir, s);
    dfree(d_rptr, s); dfree(d_cur, s); lcol.release(s);
    g2p_solver_destroy(Sd);
    g2p_solver_destroy(Sc);
    G2P_CUDA(cudaStreamSynchronize(s));
    local.total_ms = ms_since(t_all);
    g2p_mesh_sizes(m, &local.sizes);
    if (st) *st = local;
    return worst_rc;
}
