// V0 bases and the node Laplacians Ad, Ac (a10-a13).
//
// merge_v0d1 (fdtd.hpp:1823-2774) with the block sizes paraGenerator uses
// (0; matrixCon.cpp:35-40) gives one column per dielectric node off the PEC
// planes, in node order, with entries on its <= 6 incident edges (V0d1),
// then one column per non-reference conductor with entries on its dielectric
// boundary edges in node order (V0d2).  merge_v0c (fdtd.hpp:2866-3479) gives
// one column per conductor node, conductor by conductor, dropping the last
// node of every non-reference conductor and the PEC-plane nodes of reference
// and passive conductors.  generateAd / generateAc (fdtd.hpp:2778-2862,
// 3481-3574) accumulate each column's entries through the other endpoint's
// column; the Ad rows of conductor columns, which can hold 10^4-10^5 entries,
// go through a stable radix sort so every (row, column) sum still runs in
// the reference's entry order.
//
// Compiled without FMA contraction so values match the reference bit for bit.
#include <vector>

#include "internal.h"
#include "primitives.cuh"

g2p_status g2p_run_index_maps(g2p_mesh *m);
g2p_status g2p_build_rowptr(g2p_mesh *m, int64_t *rowlen, int64_t n, int64_t **ptr_out, int64_t *nnz_out);
g2p_status g2p_export_csr(g2p_mesh *m, const g2p::Csr<double> &A, int64_t *row, int64_t *col, double *val);
namespace g2p { g2p_status ensure_scan_work(g2p_mesh *m, int64_t n); }

namespace g2p {

struct V0Ctx {
    Dims d;
    const double *xn, *yn, *zn, *epsn, *sign;
    const int32_t *mark_node, *mark_edge, *mark_port;
    const uint8_t *pec_node;
    double LX, LY, LZ, eps0;
    // Values of the reference's entry expressions per grid line, computed
    // once by k_v0_lines/k_v0_areas with the same operations (bit-equal):
    // ivx[i] = 1 / (xn[i+1] - xn[i]), ilx[i] = 1 / lx(i) with lx the
    // avg_length of node line i (likewise y, z), and the V0d2 area weights
    // axy[ix][iy] = lx*ly / W, ayz[iy][iz] = ly*lz / W, axz[ix][iz] = lx*lz / W.
    const double *ivx, *ivy, *ivz, *ilx, *ily, *ilz, *axy, *ayz, *axz;
};

// One incident edge of a node, in the reference's order (lower z, upper z,
// left x, right x, front y, back y).
struct Inc {
    int64_t e, other;
    double val, aval, area;   // +-1/h, +-1/l_avg, +-area-weighted (V0d2)
};

__device__ __forceinline__ void node_ijk(const Dims &d, int64_t n, int64_t &iz, int64_t &ix, int64_t &iy) {
    iz = n / d.N_node_s;
    int64_t r = n - iz * d.N_node_s;
    ix = r / (d.Ny + 1);
    iy = r - ix * (d.Ny + 1);
}


__device__ __forceinline__ int incident(const V0Ctx &c, int64_t n, Inc *out) {
    const Dims &d = c.d;
    int64_t iz, ix, iy;
    node_ijk(d, n, iz, ix, iy);
    // -1 / h == -(1 / h) and -lx * ly / W == -(lx * ly / W) exactly
    const double azxy = c.axy[ix * d.ny + iy], axyz = c.ayz[iy * d.nz + iz], ayxz = c.axz[ix * d.nz + iz];
    int k = 0;
    if (iz != 0) out[k++] = {(iz - 1) * d.L + d.Ns + ix * (d.Ny + 1) + iy, n - d.N_node_s, -c.ivz[iz - 1], -c.ilz[iz],
                             -azxy};
    if (iz != d.nz - 1) out[k++] = {iz * d.L + d.Ns + ix * (d.Ny + 1) + iy, n + d.N_node_s, c.ivz[iz], c.ilz[iz], azxy};
    if (ix != 0) out[k++] = {iz * d.L + d.XO + (ix - 1) * (d.Ny + 1) + iy, n - (d.Ny + 1), -c.ivx[ix - 1], -c.ilx[ix],
                             -axyz};
    if (ix != d.nx - 1) out[k++] = {iz * d.L + d.XO + ix * (d.Ny + 1) + iy, n + (d.Ny + 1), c.ivx[ix], c.ilx[ix], axyz};
    if (iy != 0) out[k++] = {iz * d.L + ix * d.Ny + iy - 1, n - 1, -c.ivy[iy - 1], -c.ily[iy], -ayxz};
    if (iy != d.ny - 1) out[k++] = {iz * d.L + ix * d.Ny + iy, n + 1, c.ivy[iy], c.ily[iy], ayxz};
    return k;
}

// Per-line tables (see V0Ctx): blockIdx.y picks the axis.
__global__ void k_v0_lines(V0Ctx c, double *ivx, double *ivy, double *ivz, double *lx, double *ly, double *lz,
                           double *ilx, double *ily, double *ilz) {
    const Dims &d = c.d;
    const int ax = blockIdx.y;
    const int64_t nn = ax == 0 ? d.nx : ax == 1 ? d.ny : d.nz;
    const double *p = ax == 0 ? c.xn : ax == 1 ? c.yn : c.zn;
    double *iv = ax == 0 ? ivx : ax == 1 ? ivy : ivz;
    double *la = ax == 0 ? lx : ax == 1 ? ly : lz;
    double *il = ax == 0 ? ilx : ax == 1 ? ily : ilz;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nn; i += (int64_t)gridDim.x * blockDim.x) {
        if (i < nn - 1) iv[i] = 1 / (p[i + 1] - p[i]);
        // avg_length (fdtd.hpp:4074-4104)
        double l;
        if (i == 0) l = p[1] - p[0];
        else if (i == nn - 1) l = p[i] - p[i - 1];
        else l = (p[i + 1] - p[i - 1]) / 2;
        la[i] = l;
        il[i] = 1 / l;
    }
}

__global__ void k_v0_areas(V0Ctx c, const double *lx, const double *ly, const double *lz, double *axy, double *ayz,
                           double *axz) {
    const Dims &d = c.d;
    const double W = c.LX * c.LY * c.LZ;
    const int64_t n1 = d.nx * d.ny, n2 = d.ny * d.nz, n3 = d.nx * d.nz;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n1 + n2 + n3; t += (int64_t)gridDim.x * blockDim.x) {
        if (t < n1) { const int64_t ix = t / d.ny, iy = t - ix * d.ny; axy[t] = lx[ix] * ly[iy] / W; }
        else if (t < n1 + n2) { const int64_t u = t - n1, iy = u / d.nz, iz = u - iy * d.nz; ayz[u] = ly[iy] * lz[iz] / W; }
        else { const int64_t u = t - n1 - n2, ix = u / d.nz, iz = u - ix * d.nz; axz[u] = lx[ix] * lz[iz] / W; }
    }
}

__device__ __forceinline__ int node_degree(const Dims &d, int64_t n) {
    int64_t iz, ix, iy;
    node_ijk(d, n, iz, ix, iy);
    return (iz != 0) + (iz != d.nz - 1) + (ix != 0) + (ix != d.nx - 1) + (iy != 0) + (iy != d.ny - 1);
}

__device__ __forceinline__ bool is_d1(const V0Ctx &c, int64_t n) {
    if (c.mark_node[n] != 0) return false;
    int64_t iz = n / c.d.N_node_s;
    return !((iz == 0 || iz == c.d.nz - 1) && c.pec_node[n]);
}

// Entry of V0d2 on edge e of conductor node n (fdtd.hpp:2676-2757).
__device__ __forceinline__ bool d2_edge(const V0Ctx &c, const Inc &in, int32_t me) {
    return c.mark_edge[in.e] == 0 && c.mark_node[in.other] != me;
}

// Edge length and layer for the Laplacian terms (generateAd's h and inz).
__device__ __forceinline__ void edge_geom(const V0Ctx &c, int64_t e, int64_t &n1, int64_t &n2, int64_t &inz, double &h) {
    int64_t inx, iny;
    int k = c.d.edge_nodes(e, n1, n2, inz, inx, iny);
    if (k == 2) h = c.zn[inz + 1] - c.zn[inz];
    else if (k == 1) h = c.xn[inx + 1] - c.xn[inx];
    else h = c.yn[iny + 1] - c.yn[iny];
}

// One V0 entry's contribution to row `col` of Ad (coef = stackEpsn*eps0
// path, is_ac = 0) or Ac (stackSign, only conductor edges).  Returns the
// other column (-1 for none) with its value, and the diagonal increment.
__device__ __forceinline__ bool lap_term(const V0Ctx &c, const int32_t *map, bool is_ac, int64_t e, int64_t col,
                                         double a, int64_t &other, double &off, double &dg) {
    if (is_ac && c.mark_edge[e] == 0) return false;
    int64_t n1, n2, inz;
    double h;
    edge_geom(c, e, n1, n2, inz, h);
    int32_t m1 = map[n1], m2 = map[n2];
    other = -1;
    off = 0.0;
    // the reference's a * 1 / h * s and a * (-1) / h * s: (a * 1) / h == q and
    // (a * (-1)) / h == -q exactly, so one division serves both
    const double q = a / h;
    if (is_ac) {
        double s = c.sign[inz];
        if (m1 != col + 1 && m1 != 0) { other = m1 - 1; off = q * s; dg = -q * s; }
        else if (m2 != col + 1 && m2 != 0) { other = m2 - 1; off = -q * s; dg = q * s; }
        else dg = fabs(q * s);
    } else {
        double ep = c.epsn[inz];
        if (m1 != col + 1 && m1 != 0) { other = m1 - 1; off = q * ep * c.eps0; dg = -q * ep * c.eps0; }
        else if (m2 != col + 1 && m2 != 0) { other = m2 - 1; off = -q * ep * c.eps0; dg = q * ep * c.eps0; }
        else dg = fabs(q * ep * c.eps0);
    }
    return true;
}

// --------------------------------------------------------------- V0d kernels
// Per conductor: has_entries and entry count of its V0d2 column.
__global__ void k_d2_count(V0Ctx c, int64_t *cnt, int32_t *bcnt) {
    const Dims &d = c.d;
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < d.N_node; n += (int64_t)gridDim.x * blockDim.x) {
        int32_t me = c.mark_node[n];
        int b = 0;
        if (me != 0 && c.mark_port[me - 1] != -1) {
            Inc in[6];
            int k = incident(c, n, in);
            for (int t = 0; t < k; t++) b += d2_edge(c, in[t], me);
            if (b) atomicAdd((unsigned long long *)&cnt[me - 1], (unsigned long long)b);
        }
        bcnt[n] = b;
    }
}

__global__ void k_cond_flags(int64_t ncdt, const int64_t *cnt, const int32_t *mark_port, int32_t *flags /*[2]*/) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncdt; i += (int64_t)gridDim.x * blockDim.x) {
        if (mark_port[i] == -1) continue;
        if (cnt[i] > 0) atomicAdd(&flags[0], 1);
        else atomicAdd(&flags[1], 1);
    }
}

// map for V0d: dielectric nodes -> their column, conductor nodes of
// non-reference conductors -> the conductor's column.
__global__ void k_d_map(V0Ctx c, const int32_t *d1col, const int64_t *ccol, int32_t *map) {
    const Dims &d = c.d;
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < d.N_node; n += (int64_t)gridDim.x * blockDim.x) {
        int32_t me = c.mark_node[n];
        int32_t v = 0;
        if (me == 0) v = is_d1(c, n) ? d1col[n] + 1 : 0;
        else if (c.mark_port[me - 1] != -1) v = (int32_t)ccol[me - 1] + 1;
        map[n] = v;
    }
}

// V0d1 entries and column pointers.
__global__ void k_d1_fill(V0Ctx c, const int32_t *d1col, const int64_t *d1off, int64_t *cptr, int32_t *cedge,
                          double *cval, double *caval) {
    const Dims &d = c.d;
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < d.N_node; n += (int64_t)gridDim.x * blockDim.x) {
        if (!is_d1(c, n)) continue;
        Inc in[6];
        int k = incident(c, n, in);
        int64_t o = d1off[n];
        cptr[d1col[n]] = o;
        for (int t = 0; t < k; t++) { cedge[o + t] = (int32_t)in[t].e; cval[o + t] = in[t].val; caval[o + t] = in[t].aval; }
    }
}

// V0d2 entries: `list` holds conductor nodes grouped by conductor in node
// order; off[i] is the entry offset of list[i].
__global__ void k_d2_fill(V0Ctx c, const int32_t *list, int64_t nlist, const int64_t *off, int32_t *cedge,
                          double *cval, double *caval) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nlist; i += (int64_t)gridDim.x * blockDim.x) {
        int64_t n = list[i];
        int32_t me = c.mark_node[n];
        if (c.mark_port[me - 1] == -1) continue;
        Inc in[6];
        int k = incident(c, n, in);
        int64_t o = off[i];
        for (int t = 0; t < k; t++)
            if (d2_edge(c, in[t], me)) { cedge[o] = (int32_t)in[t].e; cval[o] = in[t].val; caval[o] = in[t].area; o++; }
    }
}

__global__ void k_cond_cptr(int64_t ncdt, const int32_t *mark_port, const int64_t *cnt, const int64_t *ccol,
                            const int64_t *coff, int64_t *cptr) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncdt; i += (int64_t)gridDim.x * blockDim.x)
        if (mark_port[i] != -1 && cnt[i] > 0) cptr[ccol[i]] = coff[i];
}

// --------------------------------------------------------------- V0c kernels
// list position -> keeps a V0c column? (fdtd.hpp:2900-2912,3106-3110)
__device__ __forceinline__ bool c_keep(const V0Ctx &c, const int32_t *list, int64_t nlist, int64_t i) {
    int64_t n = list[i];
    int32_t me = c.mark_node[n];
    int mp = c.mark_port[me - 1];
    bool last = (i + 1 == nlist) || c.mark_node[list[i + 1]] != me;
    if (mp >= 0 && last) return false;
    if (mp <= 0 && c.pec_node[n]) return false;
    return true;
}

__global__ void k_c_fill(V0Ctx c, const int32_t *list, int64_t nlist, const int32_t *ccolv, const int64_t *coff,
                         int32_t *map, int64_t *cptr, int32_t *cedge, double *cval, double *caval) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nlist; i += (int64_t)gridDim.x * blockDim.x) {
        if (!c_keep(c, list, nlist, i)) continue;
        int64_t n = list[i];
        Inc in[6];
        int k = incident(c, n, in);
        int64_t o = coff[i];
        int32_t col = ccolv[i];
        map[n] = col + 1;
        cptr[col] = o;
        for (int t = 0; t < k; t++) { cedge[o + t] = (int32_t)in[t].e; cval[o + t] = in[t].val; caval[o + t] = in[t].aval; }
    }
}

// ------------------------------------------------------- per-edge V0 views
// Up to two entries per edge, ascending column: the endpoint columns.
__global__ void k_edge_view(V0Ctx c, bool is_c, const int32_t *map, const int32_t *d1col, int32_t *ecol, double *eval,
                            double *eaval) {
    const Dims &d = c.d;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d.N_edge; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t n[2], inz, inx, iny;
        d.edge_nodes(e, n[0], n[1], inz, inx, iny);
        int32_t col[2] = {-1, -1};
        double v[2] = {0, 0}, a[2] = {0, 0};
        for (int s = 0; s < 2; s++) {
            int64_t nn = n[s];
            int32_t me = c.mark_node[nn];
            bool has = false;
            int32_t cc = -1;
            if (is_c) {
                if (me != 0 && map[nn] != 0) { has = true; cc = map[nn] - 1; }
            } else if (me == 0) {
                if (is_d1(c, nn)) { has = true; cc = d1col[nn]; }
            } else if (c.mark_port[me - 1] != -1 && map[nn] != 0) {
                int64_t other = n[1 - s];
                if (c.mark_edge[e] == 0 && c.mark_node[other] != me) { has = true; cc = map[nn] - 1; }
            }
            if (!has) continue;
            Inc in[6];
            int k = incident(c, nn, in);
            for (int t = 0; t < k; t++)
                if (in[t].e == e) {
                    col[s] = cc;
                    v[s] = in[t].val;
                    a[s] = (is_c || me == 0) ? in[t].aval : in[t].area;
                }
        }
        int lo = 0, hi = 1;
        if (col[0] < 0 || (col[1] >= 0 && col[1] < col[0])) { lo = 1; hi = 0; }
        ecol[2 * e] = col[lo]; eval[2 * e] = v[lo]; eaval[2 * e] = a[lo];
        ecol[2 * e + 1] = col[hi]; eval[2 * e + 1] = v[hi]; eaval[2 * e + 1] = a[hi];
    }
}

// ----------------------------------------------------------- Laplacian rows
constexpr int kRowMax = 8;

// Row of a single-node column (V0d1 or V0c): <= 6 entries + diagonal,
// accumulated in entry order, sorted, optionally filtered |v| > 1e-8.
__device__ __forceinline__ int short_row(const V0Ctx &c, const int32_t *map, bool is_ac, const int64_t *cptr,
                                         const int32_t *cedge, const double *caval, int64_t col, int64_t *cols,
                                         double *vals) {
    int nr = 0;
    for (int64_t k = cptr[col]; k < cptr[col + 1]; k++) {
        int64_t other;
        double off, dg;
        if (!lap_term(c, map, is_ac, cedge[k], col, caval[k], other, off, dg)) continue;
        if (other >= 0) {
            int q = 0;
            while (q < nr && cols[q] != other) q++;
            if (q == nr) { cols[nr] = other; vals[nr] = 0.0; nr++; }
            vals[q] += off;
        }
        int q = 0;
        while (q < nr && cols[q] != col) q++;
        if (q == nr) { cols[nr] = col; vals[nr] = 0.0; nr++; }
        vals[q] += dg;
    }
    for (int i = 1; i < nr; i++) {
        int64_t cc = cols[i]; double v = vals[i];
        int j = i - 1;
        while (j >= 0 && cols[j] > cc) { cols[j + 1] = cols[j]; vals[j + 1] = vals[j]; j--; }
        cols[j + 1] = cc; vals[j + 1] = v;
    }
    if (!is_ac) {
        int w = 0;
        for (int i = 0; i < nr; i++)
            if (fabs(vals[i]) > 1e-8) { cols[w] = cols[i]; vals[w] = vals[i]; w++; }
        nr = w;
    }
    return nr;
}

__global__ void k_short_rows_count(V0Ctx c, const int32_t *map, bool is_ac, const int64_t *cptr, const int32_t *cedge,
                                   const double *caval, int64_t nrows, int64_t *rowlen) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
        int64_t cols[kRowMax];
        double vals[kRowMax];
        rowlen[r] = short_row(c, map, is_ac, cptr, cedge, caval, r, cols, vals);
    }
}

__global__ void k_short_rows_fill(V0Ctx c, const int32_t *map, bool is_ac, const int64_t *cptr, const int32_t *cedge,
                                  const double *caval, int64_t nrows, const int64_t *rowptr, int32_t *col, double *val) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
        int64_t cols[kRowMax];
        double vals[kRowMax];
        int nr = short_row(c, map, is_ac, cptr, cedge, caval, r, cols, vals);
        int64_t o = rowptr[r];
        for (int q = 0; q < nr; q++) { col[o + q] = (int32_t)cols[q]; val[o + q] = vals[q]; }
    }
}

// Long (conductor) rows of Ad: every entry emits (row, col) keys with values
// in entry order; a stable sort by key and an ordered per-key sum follow.
__global__ void k_long_terms(V0Ctx c, const int32_t *map, const int64_t *cptr, const int32_t *cedge,
                             const double *caval, int64_t row0, int64_t nrows, int64_t ncolall, const int64_t *toff,
                             uint64_t *keys, double *vals) {
    int64_t k0 = cptr[row0];
    int64_t nent = cptr[row0 + nrows] - k0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nent; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t k = k0 + t;
        // row of entry k: binary search in cptr[row0 .. row0+nrows]
        int64_t lo = row0, hi = row0 + nrows - 1;
        while (lo < hi) {
            int64_t mid = (lo + hi + 1) >> 1;
            if (cptr[mid] <= k) lo = mid; else hi = mid - 1;
        }
        int64_t row = lo;
        int64_t other;
        double off, dg;
        lap_term(c, map, false, cedge[k], row, caval[k], other, off, dg);
        int64_t o = toff[t];
        if (other >= 0) { keys[o] = (uint64_t)(row - row0) * (uint64_t)ncolall + (uint64_t)other; vals[o] = off; o++; }
        keys[o] = (uint64_t)(row - row0) * (uint64_t)ncolall + (uint64_t)row;
        vals[o] = dg;
    }
}

__global__ void k_long_nterms(V0Ctx c, const int32_t *map, const int64_t *cptr, const int32_t *cedge,
                              const double *caval, int64_t row0, int64_t nrows, int64_t *nt) {
    int64_t k0 = cptr[row0];
    int64_t nent = cptr[row0 + nrows] - k0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nent; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t k = k0 + t;
        int64_t lo = row0, hi = row0 + nrows - 1;
        while (lo < hi) {
            int64_t mid = (lo + hi + 1) >> 1;
            if (cptr[mid] <= k) lo = mid; else hi = mid - 1;
        }
        int64_t other;
        double off, dg;
        lap_term(c, map, false, cedge[k], lo, caval[k], other, off, dg);
        nt[t] = other >= 0 ? 2 : 1;
    }
}

// Segment heads of sorted keys: head[i] = 1 when keys[i] starts a new key.
__global__ void k_heads(const uint64_t *keys, int64_t n, int64_t *head) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        head[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1 : 0;
}

__global__ void k_seg_bounds(const int64_t *head, const int64_t *segid, int64_t n, int64_t nseg, int64_t *sstart) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (head[i]) sstart[segid[i]] = i;
    if (blockIdx.x == 0 && threadIdx.x == 0) sstart[nseg] = n;
}

// Ordered sum of each key's values (left to right, from 0.0, so bit-equal
// to the reference's accumulation); keeps |v| > 1e-8 (fdtd.hpp:2852).  The
// loads run eight ahead of the dependent additions.
constexpr int64_t kSegWarp = 256;   // segments longer than this are summed by a warp

__global__ void k_seg_sum(const uint64_t *keys, const double *vals, int64_t nseg, const int64_t *sstart,
                          uint64_t *okey, double *oval, int64_t *keep) {
    for (int64_t sg = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; sg < nseg; sg += (int64_t)gridDim.x * blockDim.x) {
        const int64_t b = sstart[sg], e = sstart[sg + 1];
        if (e - b > kSegWarp) continue;
        double s = 0.0;
        int64_t j = b;
        for (; j + 8 <= e; j += 8) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; u++) v[u] = vals[j + u];
#pragma unroll
            for (int u = 0; u < 8; u++) s += v[u];
        }
        for (; j < e; j++) s += vals[j];
        okey[sg] = keys[b];
        oval[sg] = s;
        keep[sg] = fabs(s) > 1e-8 ? 1 : 0;
    }
}

// The same ordered sum for segments longer than kSegWarp, one warp per
// segment: the lanes stage 256 consecutive values in shared memory with
// coalesced loads, then lane 0 adds them left to right, so the result is the
// sequential sum and the dependent chain holds only the additions.
__global__ void __launch_bounds__(256) k_seg_sum_long(const uint64_t *keys, const double *vals, int64_t nseg,
                                                      const int64_t *sstart, uint64_t *okey, double *oval,
                                                      int64_t *keep) {
    __shared__ double stage[8][256];
    const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
    double *st = stage[wi];
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t sg = warp; sg < nseg; sg += nwarp) {
        const int64_t b = sstart[sg], e = sstart[sg + 1];
        if (e - b <= kSegWarp) continue;
        double s = 0.0;
        for (int64_t j0 = b; j0 < e; j0 += 256) {
            const int cnt = e - j0 >= 256 ? 256 : (int)(e - j0);
#pragma unroll
            for (int u = 0; u < 8; u++) {
                const int t = 32 * u + lane;
                if (t < cnt) st[t] = vals[j0 + t];
            }
            __syncwarp();
            if (lane == 0) {
                if (cnt == 256) {
#pragma unroll 16
                    for (int t = 0; t < 256; t++) s += st[t];
                } else {
                    for (int t = 0; t < cnt; t++) s += st[t];
                }
            }
            __syncwarp();
        }
        if (lane == 0) {
            if (okey) okey[sg] = keys[b];
            oval[sg] = s;
            keep[sg] = fabs(s) > 1e-8 ? 1 : 0;
        }
    }
}

// Stand-in for k_seg_sum_long while it runs: each lane adds a strided share
// of the segment and a shuffle tree adds the 32 partials.  Deterministic but
// not the left-to-right sum; these values only build the preconditioner's
// copy of the Laplacian, and k_long_patch later writes the ordered sums.
__global__ void __launch_bounds__(256) k_seg_sum_tree(const uint64_t *keys, const double *vals, int64_t nseg,
                                                      const int64_t *sstart, uint64_t *okey, double *oval,
                                                      int64_t *keep) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarp = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t sg = warp; sg < nseg; sg += nwarp) {
        const int64_t b = sstart[sg], e = sstart[sg + 1];
        if (e - b <= kSegWarp) continue;
        double s = 0.0;
        for (int64_t j = b + lane; j < e; j += 32) s += vals[j];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) {
            okey[sg] = keys[b];
            oval[sg] = s;
            keep[sg] = fabs(s) > 1e-8 ? 1 : 0;
        }
    }
}

// Writes the ordered sums (xval, xkeep from k_seg_sum_long) of the segments
// longer than kSegWarp into a Laplacian assembled from k_seg_sum_tree's
// values.  A segment kept by one and dropped by the other changes the
// pattern: it sets *changed and the caller reassembles.
__global__ void k_long_patch(const int64_t *sstart, const int64_t *keep, const int64_t *kpos, const double *xval,
                             const int64_t *xkeep, int64_t nseg, const int64_t *rowptr, int64_t row0, double *val,
                             int *changed) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nseg; i += (int64_t)gridDim.x * blockDim.x) {
        if (sstart[i + 1] - sstart[i] <= kSegWarp) continue;
        if (xkeep[i] != keep[i]) { *changed = 1; continue; }
        if (keep[i]) val[rowptr[row0] + kpos[i]] = xval[i];
    }
}

__global__ void k_long_rowlen(const uint64_t *okey, const int64_t *keep, int64_t nseg, int64_t ncolall, int64_t *rowlen) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nseg; i += (int64_t)gridDim.x * blockDim.x)
        if (keep[i]) atomicAdd((unsigned long long *)&rowlen[okey[i] / (uint64_t)ncolall], 1ull);
}

__global__ void k_long_scatter(const uint64_t *okey, const double *oval, const int64_t *keep, const int64_t *kpos,
                               int64_t nseg, int64_t ncolall, int64_t row0, const int64_t *rowptr, int64_t rowbase,
                               int32_t *col, double *val) {
    // kept segments are in (row, col) order, so position = rowptr[row0] + rank
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nseg; i += (int64_t)gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        int64_t o = rowptr[row0] - rowbase + kpos[i];
        col[o] = (int32_t)(okey[i] % (uint64_t)ncolall);
        val[o] = oval[i];
    }
}

__global__ void k_add_i64(int64_t *a, int64_t n, int64_t v) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) a[i] += v;
}

}  // namespace g2p

using namespace g2p;

static V0Ctx make_ctx(g2p_mesh *m) {
    V0Ctx c;
    c.d = m->d;
    c.xn = m->xn; c.yn = m->yn; c.zn = m->zn; c.epsn = m->epsn; c.sign = m->sign;
    c.mark_node = m->mark_node; c.mark_edge = m->mark_edge; c.mark_port = m->mark_port;
    c.pec_node = m->pec_node;
    const Dims &d = m->d;
    c.LX = (m->h_xn[d.nx - 1] - m->h_xn[0]) / (d.nx - 1);
    c.LY = (m->h_yn[d.ny - 1] - m->h_yn[0]) / (d.ny - 1);
    c.LZ = (m->h_zn[d.nz - 1] - m->h_zn[0]) / (d.nz - 1);
    c.eps0 = m->k.eps0;
    return c;
}

static int bits_for(uint64_t v) {
    int b = 0;
    while (b < 64 && (v >> b) != 0) b++;
    return b < 8 ? 8 : ((b + 7) / 8) * 8;
}

// State of a Laplacian between lap_begin and lap_finish.
struct g2p::LapPending {
    V0Ctx c;
    V0Basis *B = nullptr;
    Csr<double> *A = nullptr;
    bool is_ac = false;
    int64_t ncol = 0, nshort = 0, nlong = 0, nseg = 0;
    int64_t *rowlen = nullptr, *keep = nullptr, *kpos = nullptr, *head = nullptr, *segid = nullptr, *sstart = nullptr;
    uint64_t *okey = nullptr, *k0 = nullptr, *k1 = nullptr;
    double *oval = nullptr, *v0 = nullptr, *v1 = nullptr;
    cudaEvent_t done = nullptr;     // recorded on the side stream after the ordered sums
    // split: the long segments' ordered sums go to xval/xkeep on the side
    // stream, k_seg_sum_tree's stand-ins to oval/keep on the job's stream;
    // provisional: A is assembled from the stand-ins, k_long_patch pending
    bool split = false, provisional = false;
    double *xval = nullptr;
    int64_t *xkeep = nullptr;
};

// Builds one Laplacian (Ad when is_ac false) from a V0 basis; rows [0, nshort)
// are single-node columns, rows [nshort, ncol) conductor columns.  Part one:
// everything up to the ordered per-key sums of the long rows.  With
// `on_side` the sums of segments longer than kSegWarp (the largest
// conductor's is a dependent chain of FP64 additions) run on m->side, and the
// job's stream gets tree-summed stand-ins for them at once, so a
// provisional Laplacian can be assembled (lap_finish) and the exact one
// completed later (lap_exact).
static g2p_status lap_begin(g2p_mesh *m, const V0Ctx &c, V0Basis &B, bool is_ac, int64_t nshort, Csr<double> &A,
                            LapPending &P, bool on_side) {
    cudaStream_t s = m->stream;
    P.c = c; P.B = &B; P.A = &A; P.is_ac = is_ac;
    const int64_t ncol = B.ncol, nlong = ncol - nshort;
    P.ncol = ncol; P.nshort = nshort; P.nlong = nlong;
    G2P_TRY(dalloc(&P.rowlen, ncol + 1, s));
    G2P_CUDA(cudaMemsetAsync(P.rowlen, 0, sizeof(int64_t) * (ncol + 1), s));
    if (nshort > 0)
        (g2p::kbegin("k_short_rows_count", s), k_short_rows_count<<<grid_for(nshort), kThreads, 0, s>>>(c, B.map, is_ac, B.cptr, B.cedge, B.caval, nshort, P.rowlen), g2p::kend(s));
    if (nlong == 0) return G2P_OK;
    // long rows through sort + ordered reduce
    int64_t h_ent[2];
    G2P_CUDA(cudaMemcpyAsync(h_ent, B.cptr + nshort, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaMemcpyAsync(h_ent + 1, B.cptr + ncol, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    const int64_t nent = h_ent[1] - h_ent[0];
    int64_t *nt, *toff;
    G2P_TRY(dalloc(&nt, nent + 1, s));
    G2P_TRY(dalloc(&toff, nent + 1, s));
    if (nent > 0)
        (g2p::kbegin("k_long_nterms", s), k_long_nterms<<<grid_for(nent), kThreads, 0, s>>>(c, B.map, B.cptr, B.cedge, B.caval, nshort, nlong, nt), g2p::kend(s));
    G2P_TRY(ensure_scan_work(m, nent + 1));
    const int64_t *ntp = nt;
    auto op = [ntp, nent] __device__(int64_t i) -> int64_t { return i < nent ? ntp[i] : 0; };
    G2P_TRY(exclusive_scan(op, nent + 1, toff, m->scan_work, s));
    int64_t nterm = 0;
    G2P_CUDA(cudaMemcpyAsync(&nterm, toff + nent, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    G2P_TRY(dalloc(&P.k0, nterm, s)); G2P_TRY(dalloc(&P.k1, nterm, s));
    G2P_TRY(dalloc(&P.v0, nterm, s)); G2P_TRY(dalloc(&P.v1, nterm, s));
    if (nent > 0)
        (g2p::kbegin("k_long_terms", s), k_long_terms<<<grid_for(nent), kThreads, 0, s>>>(c, B.map, B.cptr, B.cedge, B.caval, nshort, nlong, ncol, toff,
                                                         P.k0, P.v0), g2p::kend(s));
    dfree(nt, s); dfree(toff, s);
    int64_t *counts;
    G2P_TRY(dalloc(&counts, sort_counts_size(nterm), s));
    G2P_TRY(ensure_scan_work(m, sort_counts_size(nterm)));
    bool in1 = false;
    G2P_TRY(radix_sort_pairs(P.k0, P.v0, P.k1, P.v1, nterm, bits_for((uint64_t)nlong * (uint64_t)ncol), counts,
                             m->scan_work, &in1, s));
    dfree(counts, s);
    uint64_t *sk = in1 ? P.k1 : P.k0;
    double *sv = in1 ? P.v1 : P.v0;
    G2P_TRY(dalloc(&P.head, nterm + 1, s));
    G2P_TRY(dalloc(&P.segid, nterm + 1, s));
    (g2p::kbegin("k_heads", s), k_heads<<<grid_for(nterm), kThreads, 0, s>>>(sk, nterm, P.head), g2p::kend(s));
    G2P_TRY(ensure_scan_work(m, nterm + 1));
    const int64_t *hp = P.head;
    auto hop = [hp, nterm] __device__(int64_t i) -> int64_t { return i < nterm ? hp[i] : 0; };
    G2P_TRY(exclusive_scan(hop, nterm + 1, P.segid, m->scan_work, s));
    G2P_CUDA(cudaMemcpyAsync(&P.nseg, P.segid + nterm, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    const int64_t nseg = P.nseg;
    G2P_TRY(dalloc(&P.okey, nseg, s)); G2P_TRY(dalloc(&P.oval, nseg, s));
    G2P_TRY(dalloc(&P.keep, nseg + 1, s)); G2P_TRY(dalloc(&P.kpos, nseg + 1, s));
    G2P_TRY(dalloc(&P.sstart, nseg + 1, s));
    (g2p::kbegin("k_seg_bounds", s), k_seg_bounds<<<grid_for(nterm), kThreads, 0, s>>>(P.head, P.segid, nterm, nseg, P.sstart), g2p::kend(s));
    if (on_side) {
        if (!m->side) G2P_CUDA(cudaStreamCreateWithFlags(&m->side, cudaStreamNonBlocking));
        G2P_TRY(dalloc(&P.xval, nseg, s));
        G2P_TRY(dalloc(&P.xkeep, nseg, s));
        cudaEvent_t fork;
        G2P_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
        G2P_CUDA(cudaEventRecord(fork, s));
        G2P_CUDA(cudaStreamWaitEvent(m->side, fork, 0));
        cudaEventDestroy(fork);
        cudaStream_t ss = m->side;
        (g2p::kbegin("k_seg_sum_long", ss), k_seg_sum_long<<<grid_for(32 * nseg), kThreads, 0, ss>>>(sk, sv, nseg, P.sstart, nullptr, P.xval, P.xkeep), g2p::kend(ss));
        G2P_CUDA(cudaEventCreateWithFlags(&P.done, cudaEventDisableTiming));
        G2P_CUDA(cudaEventRecord(P.done, ss));
        P.split = true;
    }
    (g2p::kbegin("k_seg_sum", s), k_seg_sum<<<grid_for(nseg), kThreads, 0, s>>>(sk, sv, nseg, P.sstart, P.okey, P.oval, P.keep), g2p::kend(s));
    if (on_side)
        (g2p::kbegin("k_seg_sum_tree", s), k_seg_sum_tree<<<grid_for(32 * nseg), kThreads, 0, s>>>(sk, sv, nseg, P.sstart, P.okey, P.oval, P.keep), g2p::kend(s));
    else
        (g2p::kbegin("k_seg_sum_long", s), k_seg_sum_long<<<grid_for(32 * nseg), kThreads, 0, s>>>(sk, sv, nseg, P.sstart, P.okey, P.oval, P.keep), g2p::kend(s));
    return G2P_OK;
}

static g2p_status build_laplacian(g2p_mesh *m, const V0Ctx &c, V0Basis &B, bool is_ac, int64_t nshort, Csr<double> &A);

// Part two: row offsets and entries.  When split, from the stand-in sums
// and without waiting for the side stream: the buffers it reads (sorted
// terms, segment starts) and those lap_exact needs stay allocated.
static g2p_status lap_finish(g2p_mesh *m, LapPending &P) {
    cudaStream_t s = m->stream;
    const V0Ctx &c = P.c;
    V0Basis &B = *P.B;
    Csr<double> &A = *P.A;
    const int64_t ncol = P.ncol, nshort = P.nshort, nseg = P.nseg;
    if (P.nlong > 0) {
        (g2p::kbegin("k_long_rowlen", s), k_long_rowlen<<<grid_for(nseg), kThreads, 0, s>>>(P.okey, P.keep, nseg, ncol, P.rowlen + nshort), g2p::kend(s));
        const int64_t *kp = P.keep;
        auto kop = [kp, nseg] __device__(int64_t i) -> int64_t { return i < nseg ? kp[i] : 0; };
        G2P_TRY(ensure_scan_work(m, nseg + 1));
        G2P_TRY(exclusive_scan(kop, nseg + 1, P.kpos, m->scan_work, s));
        dfree(P.head, s); dfree(P.segid, s);
        if (!P.split) {
            dfree(P.sstart, s);
            dfree(P.k0, s); dfree(P.k1, s); dfree(P.v0, s); dfree(P.v1, s);
        }
    }
    int64_t nnz = 0;
    G2P_TRY(g2p_build_rowptr(m, P.rowlen, ncol, &A.ptr, &nnz));
    dfree(P.rowlen, s);
    A.n = A.m = ncol;
    A.nnz = nnz;
    G2P_TRY(dalloc(&A.col, nnz, s));
    G2P_TRY(dalloc(&A.val, nnz, s));
    if (nshort > 0)
        (g2p::kbegin("k_short_rows_fill", s), k_short_rows_fill<<<grid_for(nshort), kThreads, 0, s>>>(c, B.map, P.is_ac, B.cptr, B.cedge, B.caval, nshort, A.ptr,
                                                                A.col, A.val), g2p::kend(s));
    if (P.nlong > 0) {
        (g2p::kbegin("k_long_scatter", s), k_long_scatter<<<grid_for(nseg), kThreads, 0, s>>>(P.okey, P.oval, P.keep, P.kpos, nseg, ncol, nshort, A.ptr, 0, A.col,
                                                           A.val), g2p::kend(s));
        dfree(P.okey, s); dfree(P.oval, s);
        if (!P.split) { dfree(P.keep, s); dfree(P.kpos, s); }
    }
    G2P_CUDA(cudaGetLastError());
    G2P_CUDA(cudaStreamSynchronize(s));
    P.provisional = P.split;
    return G2P_OK;
}

// Part three of a split Laplacian: waits for the ordered sums and writes them
// over the stand-ins.  Every buffer the side stream reads is freed here,
// after the wait.  If a long segment's kept/dropped status differs from its
// stand-in's, the Laplacian is assembled again in one pass and *repatterned
// is set (G2P_AD_REPATTERN=1 takes that path always, for comparisons).
static g2p_status lap_exact(g2p_mesh *m, LapPending &P, bool *repatterned) {
    cudaStream_t s = m->stream;
    G2P_CUDA(cudaStreamWaitEvent(s, P.done, 0));
    cudaEventDestroy(P.done);
    P.done = nullptr;
    Csr<double> &A = *P.A;
    int *changed;
    G2P_TRY(dalloc(&changed, 1, s));
    G2P_CUDA(cudaMemsetAsync(changed, 0, sizeof(int), s));
    (g2p::kbegin("k_long_patch", s), k_long_patch<<<grid_for(P.nseg), kThreads, 0, s>>>(P.sstart, P.keep, P.kpos, P.xval, P.xkeep, P.nseg, A.ptr, P.nshort, A.val, changed), g2p::kend(s));
    int h = 0;
    G2P_CUDA(cudaMemcpyAsync(&h, changed, sizeof(int), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    dfree(changed, s);
    if (getenv("G2P_AD_REPATTERN")) h = 1;
    dfree(P.sstart, s); dfree(P.keep, s); dfree(P.kpos, s); dfree(P.xval, s); dfree(P.xkeep, s);
    dfree(P.k0, s); dfree(P.k1, s); dfree(P.v0, s); dfree(P.v1, s);
    P.provisional = false;
    if (repatterned) *repatterned = h != 0;
    if (h) {
        A.release(s);
        G2P_TRY(build_laplacian(m, P.c, *P.B, P.is_ac, P.nshort, A));
    }
    return G2P_OK;
}

static g2p_status build_laplacian(g2p_mesh *m, const V0Ctx &c, V0Basis &B, bool is_ac, int64_t nshort, Csr<double> &A) {
    LapPending P;
    G2P_TRY(lap_begin(m, c, B, is_ac, nshort, A, P, false));
    return lap_finish(m, P);
}

__global__ void k_is_cond_node(const int32_t *mark_node, int64_t n, int64_t *flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        flag[i] = mark_node[i] != 0;
}

__global__ void k_compact_cond(const int32_t *mark_node, int64_t n, const int64_t *pos, uint32_t *key, int32_t *node) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (mark_node[i] != 0) { key[pos[i]] = (uint32_t)mark_node[i]; node[pos[i]] = (int32_t)i; }
}

g2p_status g2p_v0_finish(g2p_mesh *m, bool *repatterned = nullptr);

// V0 bases and Laplacians.  With defer_ad, Ad's ordered conductor sums are
// left running on the side stream and g2p_v0_finish completes Ad; Ac and
// everything else is complete on return.
g2p_status g2p_run_v0_ex(g2p_mesh *m, bool defer_ad) {
    if (m->v0_done) return G2P_OK;
    if (m->ad_pending) return defer_ad ? G2P_OK : g2p_v0_finish(m);
    G2P_TRY(g2p_run_index_maps(m));
    const Dims &d = m->d;
    cudaStream_t s = m->stream;
    V0Ctx c = make_ctx(m);
    {
        // per-line tables, kept with the mesh
        const int64_t nl = 3 * (d.nx + d.ny + d.nz), na = d.nx * d.ny + d.ny * d.nz + d.nx * d.nz;
        dfree(m->v0_tab, s);
        G2P_TRY(dalloc(&m->v0_tab, 3 * nl + na, s));
        double *t = m->v0_tab;
        double *ivx = t, *ivy = ivx + d.nx, *ivz = ivy + d.ny;
        double *lx = ivz + d.nz, *ly = lx + d.nx, *lz = ly + d.ny;
        double *ilx = lz + d.nz, *ily = ilx + d.nx, *ilz = ily + d.ny;
        double *axy = ilz + d.nz, *ayz = axy + d.nx * d.ny, *axz = ayz + d.ny * d.nz;
        const int64_t nmax = std::max(d.nx, std::max(d.ny, d.nz));
        (g2p::kbegin("k_v0_lines", s), k_v0_lines<<<dim3(grid_for(nmax), 3), kThreads, 0, s>>>(c, ivx, ivy, ivz, lx, ly, lz, ilx, ily, ilz), g2p::kend(s));
        (g2p::kbegin("k_v0_areas", s), k_v0_areas<<<grid_for(na), kThreads, 0, s>>>(c, lx, ly, lz, axy, ayz, axz), g2p::kend(s));
        c.ivx = ivx; c.ivy = ivy; c.ivz = ivz; c.ilx = ilx; c.ily = ily; c.ilz = ilz;
        c.axy = axy; c.ayz = ayz; c.axz = axz;
    }
    const int64_t ncdt = m->num_cdt;
    // ---- conductor node lists grouped by conductor, node order kept
    int64_t *pos;
    G2P_TRY(dalloc(&pos, d.N_node + 1, s));
    G2P_TRY(ensure_scan_work(m, d.N_node + 1));
    const int32_t *mn = m->mark_node;
    int64_t NN = d.N_node;
    auto cop = [mn, NN] __device__(int64_t i) -> int64_t { return i < NN ? (mn[i] != 0) : 0; };
    G2P_TRY(exclusive_scan(cop, NN + 1, pos, m->scan_work, s));
    int64_t ncn = 0;
    G2P_CUDA(cudaMemcpyAsync(&ncn, pos + NN, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    uint32_t *ck0, *ck1;
    int32_t *cn0, *cn1;
    G2P_TRY(dalloc(&ck0, ncn, s)); G2P_TRY(dalloc(&ck1, ncn, s));
    G2P_TRY(dalloc(&cn0, ncn, s)); G2P_TRY(dalloc(&cn1, ncn, s));
    (g2p::kbegin("k_compact_cond", s), k_compact_cond<<<grid_for(NN), kThreads, 0, s>>>(mn, NN, pos, ck0, cn0), g2p::kend(s));
    dfree(pos, s);
    int64_t *counts;
    G2P_TRY(dalloc(&counts, sort_counts_size(ncn), s));
    G2P_TRY(ensure_scan_work(m, sort_counts_size(ncn)));
    bool in1 = false;
    G2P_TRY(radix_sort_pairs(ck0, cn0, ck1, cn1, ncn, bits_for((uint64_t)ncdt + 1), counts, m->scan_work, &in1, s));
    dfree(counts, s);
    int32_t *list = in1 ? cn1 : cn0;
    dfree(ck0, s); dfree(ck1, s);
    if (in1) dfree(cn0, s); else dfree(cn1, s);

    // ---- V0d numbering
    int64_t *cnt, *ccol, *coff;
    int32_t *bcnt, *flags, *d1col;
    int64_t *d1off;
    G2P_TRY(dalloc(&cnt, ncdt + 1, s));
    G2P_TRY(dalloc(&ccol, ncdt + 1, s));
    G2P_TRY(dalloc(&coff, ncdt + 1, s));
    G2P_TRY(dalloc(&bcnt, NN, s));
    G2P_TRY(dalloc(&flags, 2, s));
    G2P_TRY(dalloc(&d1col, NN + 1, s));
    G2P_TRY(dalloc(&d1off, NN + 1, s));
    G2P_CUDA(cudaMemsetAsync(cnt, 0, sizeof(int64_t) * (ncdt + 1), s));
    G2P_CUDA(cudaMemsetAsync(flags, 0, sizeof(int32_t) * 2, s));
    (g2p::kbegin("k_d2_count", s), k_d2_count<<<grid_for(NN), kThreads, 0, s>>>(c, cnt, bcnt), g2p::kend(s));
    (g2p::kbegin("k_cond_flags", s), k_cond_flags<<<grid_for(ncdt), kThreads, 0, s>>>(ncdt, cnt, m->mark_port, flags), g2p::kend(s));
    int32_t hflags[2];
    G2P_CUDA(cudaMemcpyAsync(hflags, flags, sizeof(hflags), cudaMemcpyDeviceToHost, s));
    // dielectric columns and their entry offsets
    V0Ctx cc = c;
    auto d1op = [cc, NN] __device__(int64_t i) -> int64_t { return i < NN ? (is_d1(cc, i) ? 1 : 0) : 0; };
    G2P_TRY(exclusive_scan(d1op, NN + 1, d1col, m->scan_work, s));
    auto degop = [cc, NN] __device__(int64_t i) -> int64_t { return i < NN ? (is_d1(cc, i) ? node_degree(cc.d, i) : 0) : 0; };
    G2P_TRY(exclusive_scan(degop, NN + 1, d1off, m->scan_work, s));
    int32_t nd1 = 0;
    int64_t nnz_d1 = 0;
    G2P_CUDA(cudaMemcpyAsync(&nd1, d1col + NN, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaMemcpyAsync(&nnz_d1, d1off + NN, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    if (hflags[1] > 0) {
        set_last_message("%d non-reference conductor(s) have no dielectric boundary edge; the reference's V0d2 "
                         "numbering (fdtd.hpp:2424-2759) is inconsistent for such layouts", hflags[1]);
        return G2P_ERR_UNSUPPORTED;
    }
    // conductor columns: nd1 + rank among conductors with entries
    const int64_t *cntp = cnt;
    const int32_t *mpp = m->mark_port;
    auto ccop = [cntp, mpp, ncdt] __device__(int64_t i) -> int64_t {
        return i < ncdt ? ((mpp[i] != -1 && cntp[i] > 0) ? 1 : 0) : 0;
    };
    G2P_TRY(exclusive_scan(ccop, ncdt + 1, ccol, m->scan_work, s));
    auto cnop = [cntp, mpp, ncdt] __device__(int64_t i) -> int64_t {
        return i < ncdt ? ((mpp[i] != -1) ? cntp[i] : 0) : 0;
    };
    G2P_TRY(exclusive_scan(cnop, ncdt + 1, coff, m->scan_work, s));
    int64_t nd2 = 0, nnz_d2 = 0;
    G2P_CUDA(cudaMemcpyAsync(&nd2, ccol + ncdt, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaMemcpyAsync(&nnz_d2, coff + ncdt, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    (g2p::kbegin("k_add_i64", s), k_add_i64<<<grid_for(ncdt), kThreads, 0, s>>>(ccol, ncdt, nd1), g2p::kend(s));
    V0Basis &Vd = m->v0d;
    Vd.ncol = nd1 + nd2;
    Vd.nnz = nnz_d1 + nnz_d2;
    G2P_TRY(dalloc(&Vd.cptr, Vd.ncol + 1, s));
    G2P_TRY(dalloc(&Vd.cedge, Vd.nnz, s));
    G2P_TRY(dalloc(&Vd.cval, Vd.nnz, s));
    G2P_TRY(dalloc(&Vd.caval, Vd.nnz, s));
    G2P_TRY(dalloc(&Vd.map, NN, s));
    (g2p::kbegin("k_d_map", s), k_d_map<<<grid_for(NN), kThreads, 0, s>>>(c, d1col, ccol, Vd.map), g2p::kend(s));
    (g2p::kbegin("k_d1_fill", s), k_d1_fill<<<grid_for(NN), kThreads, 0, s>>>(c, d1col, d1off, Vd.cptr, Vd.cedge, Vd.cval, Vd.caval), g2p::kend(s));
    (g2p::kbegin("k_add_i64", s), k_add_i64<<<grid_for(ncdt), kThreads, 0, s>>>(coff, ncdt, nnz_d1), g2p::kend(s));
    (g2p::kbegin("k_cond_cptr", s), k_cond_cptr<<<grid_for(ncdt), kThreads, 0, s>>>(ncdt, m->mark_port, cnt, ccol, coff, Vd.cptr), g2p::kend(s));
    G2P_CUDA(cudaMemcpyAsync(Vd.cptr + Vd.ncol, &Vd.nnz, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    int64_t *loff;
    G2P_TRY(dalloc(&loff, ncn + 1, s));
    G2P_TRY(ensure_scan_work(m, ncn + 1));
    {
        const int32_t *lp = list, *bp = bcnt;
        auto bop = [lp, bp, ncn] __device__(int64_t i) -> int64_t { return i < ncn ? bp[lp[i]] : 0; };
        G2P_TRY(exclusive_scan(bop, ncn + 1, loff, m->scan_work, s));
    }
    (g2p::kbegin("k_add_i64", s), k_add_i64<<<grid_for(ncn), kThreads, 0, s>>>(loff, ncn, nnz_d1), g2p::kend(s));
    (g2p::kbegin("k_d2_fill", s), k_d2_fill<<<grid_for(ncn), kThreads, 0, s>>>(c, list, ncn, loff, Vd.cedge, Vd.cval, Vd.caval), g2p::kend(s));
    dfree(cnt, s); dfree(ccol, s); dfree(coff, s); dfree(bcnt, s); dfree(flags, s); dfree(d1off, s);

    // ---- V0c
    V0Basis &Vc = m->v0c;
    int32_t *ccolv;
    int64_t *coffv;
    G2P_TRY(dalloc(&ccolv, ncn + 1, s));
    G2P_TRY(dalloc(&coffv, ncn + 1, s));
    {
        V0Ctx c2 = c;
        const int32_t *lp = list;
        auto kop = [c2, lp, ncn] __device__(int64_t i) -> int64_t { return i < ncn ? (c_keep(c2, lp, ncn, i) ? 1 : 0) : 0; };
        G2P_TRY(exclusive_scan(kop, ncn + 1, ccolv, m->scan_work, s));
        auto dop = [c2, lp, ncn] __device__(int64_t i) -> int64_t {
            return i < ncn ? (c_keep(c2, lp, ncn, i) ? node_degree(c2.d, lp[i]) : 0) : 0;
        };
        G2P_TRY(exclusive_scan(dop, ncn + 1, coffv, m->scan_work, s));
    }
    int32_t ncc = 0;
    int64_t nnz_c = 0;
    G2P_CUDA(cudaMemcpyAsync(&ncc, ccolv + ncn, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaMemcpyAsync(&nnz_c, coffv + ncn, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    Vc.ncol = ncc;
    Vc.nnz = nnz_c;
    G2P_TRY(dalloc(&Vc.cptr, Vc.ncol + 1, s));
    G2P_TRY(dalloc(&Vc.cedge, Vc.nnz, s));
    G2P_TRY(dalloc(&Vc.cval, Vc.nnz, s));
    G2P_TRY(dalloc(&Vc.caval, Vc.nnz, s));
    G2P_TRY(dalloc(&Vc.map, NN, s));
    G2P_CUDA(cudaMemsetAsync(Vc.map, 0, sizeof(int32_t) * NN, s));
    (g2p::kbegin("k_c_fill", s), k_c_fill<<<grid_for(ncn), kThreads, 0, s>>>(c, list, ncn, ccolv, coffv, Vc.map, Vc.cptr, Vc.cedge, Vc.cval, Vc.caval), g2p::kend(s));
    G2P_CUDA(cudaMemcpyAsync(Vc.cptr + Vc.ncol, &Vc.nnz, sizeof(int64_t), cudaMemcpyHostToDevice, s));
    dfree(ccolv, s); dfree(coffv, s); dfree(list, s); dfree(loff, s);

    // ---- per-edge views
    for (int which = 0; which < 2; which++) {
        V0Basis &B = which ? Vc : Vd;
        G2P_TRY(dalloc(&B.ecol, 2 * d.N_edge, s));
        G2P_TRY(dalloc(&B.eval, 2 * d.N_edge, s));
        G2P_TRY(dalloc(&B.eaval, 2 * d.N_edge, s));
        (g2p::kbegin("k_edge_view", s), k_edge_view<<<grid_for(d.N_edge), kThreads, 0, s>>>(c, which == 1, B.map, d1col, B.ecol, B.eval, B.eaval), g2p::kend(s));
    }
    G2P_CUDA(cudaGetLastError());
    // ---- Laplacians: Ad's ordered conductor sums run on the side stream
    // while Ac is built
    auto *P = new LapPending();
    g2p_status st = lap_begin(m, c, Vd, false, nd1, m->Ad, *P, true);
    if (st != G2P_OK) { delete P; return st; }
    m->ad_pending = P;
    G2P_TRY(build_laplacian(m, c, Vc, true, Vc.ncol, m->Ac));
    dfree(d1col, s);
    G2P_CUDA(cudaStreamSynchronize(s));
    return defer_ad ? G2P_OK : g2p_v0_finish(m);
}

g2p_status g2p_v0_finish(g2p_mesh *m, bool *repatterned) {
    if (repatterned) *repatterned = false;
    if (m->v0_done) return G2P_OK;
    if (!m->ad_pending) return g2p_run_v0_ex(m, false);
    LapPending *P = m->ad_pending;
    m->ad_pending = nullptr;
    g2p_status st = P->provisional ? G2P_OK : lap_finish(m, *P);
    if (st == G2P_OK && P->split) st = lap_exact(m, *P, repatterned);
    delete P;
    if (st == G2P_OK) m->v0_done = true;
    return st;
}

// Ad assembled with the stand-in sums of its longest segments, for a
// preconditioner to be built while the ordered sums run on; g2p_v0_finish
// then writes the exact values (Ad stays pending until then).
g2p_status g2p_v0_provisional(g2p_mesh *m) {
    if (m->v0_done) return G2P_OK;
    if (!m->ad_pending) return g2p_run_v0_ex(m, false);
    LapPending *P = m->ad_pending;
    if (!P->split) return g2p_v0_finish(m);
    if (P->provisional) return G2P_OK;
    return lap_finish(m, *P);
}

g2p_status g2p_run_v0(g2p_mesh *m) { return g2p_run_v0_ex(m, false); }

extern "C" g2p_status g2p_assemble_v0(g2p_mesh *m, g2p_sizes *out) {
    if (!m) return G2P_ERR_INVALID;
    G2P_TRY(g2p_run_v0(m));
    if (out) G2P_TRY(g2p_mesh_sizes(m, out));
    return G2P_OK;
}

__global__ void k_v0_export(const int64_t *cptr, int64_t ncol, const int32_t *cedge, int64_t *row, int64_t *col) {
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncol; c += (int64_t)gridDim.x * blockDim.x)
        for (int64_t k = cptr[c]; k < cptr[c + 1]; k++) { row[k] = cedge[k]; col[k] = c; }
}

__global__ void k_map_export(const int32_t *map, int64_t n, int64_t *out) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = map[i];
}

extern "C" g2p_status g2p_export_v0(g2p_mesh *m, int32_t which, int64_t *row, int64_t *col, double *val, double *aval,
                                    int64_t *map) {
    if (!m || (which != 0 && which != 1)) return G2P_ERR_INVALID;
    if (!m->v0_done) { set_last_message("g2p_assemble_v0 has not run"); return G2P_ERR_STATE; }
    V0Basis &B = which ? m->v0c : m->v0d;
    cudaStream_t s = m->stream;
    int64_t *r, *c2;
    G2P_TRY(dalloc(&r, B.nnz, s));
    G2P_TRY(dalloc(&c2, B.nnz > m->d.N_node ? B.nnz : m->d.N_node, s));
    (g2p::kbegin("k_v0_export", s), k_v0_export<<<grid_for(B.ncol), kThreads, 0, s>>>(B.cptr, B.ncol, B.cedge, r, c2), g2p::kend(s));
    if (row) G2P_CUDA(cudaMemcpyAsync(row, r, sizeof(int64_t) * B.nnz, cudaMemcpyDeviceToHost, s));
    if (col) G2P_CUDA(cudaMemcpyAsync(col, c2, sizeof(int64_t) * B.nnz, cudaMemcpyDeviceToHost, s));
    if (val) G2P_CUDA(cudaMemcpyAsync(val, B.cval, sizeof(double) * B.nnz, cudaMemcpyDeviceToHost, s));
    if (aval) G2P_CUDA(cudaMemcpyAsync(aval, B.caval, sizeof(double) * B.nnz, cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    if (map) {
        (g2p::kbegin("k_map_export", s), k_map_export<<<grid_for(m->d.N_node), kThreads, 0, s>>>(B.map, m->d.N_node, c2), g2p::kend(s));
        G2P_CUDA(cudaMemcpyAsync(map, c2, sizeof(int64_t) * m->d.N_node, cudaMemcpyDeviceToHost, s));
    }
    G2P_CUDA(cudaStreamSynchronize(s));
    dfree(r, s); dfree(c2, s);
    G2P_CUDA(cudaStreamSynchronize(s));
    return G2P_OK;
}

extern "C" g2p_status g2p_export_laplacian(g2p_mesh *m, int32_t which, int64_t *row, int64_t *col, double *val) {
    if (!m || (which != 0 && which != 1)) return G2P_ERR_INVALID;
    if (!m->v0_done) { set_last_message("g2p_assemble_v0 has not run"); return G2P_ERR_STATE; }
    return g2p_export_csr(m, which ? m->Ac : m->Ad, row, col, val);
}
