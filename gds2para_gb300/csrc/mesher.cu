// Conductor marking and port edges on the device: the part of meshAndMark
// that rasterises conductor boxes onto the structured grid (findInsideCond,
// src/mesh.cpp:683-940), numbers the conductors as connected components in the
// order of their lowest node (the BFS of src/mesh.cpp:943-1020), recolours
// markEdge with those numbers, and portSet's port edges, areas and
// directions (src/mesh.cpp:1196-1594).
//
// Boxes are closed ranges of node indices.  A later box overwrites an
// earlier one where they overlap, and the z = 0 plane is the lower PEC
// boundary (LOWER_BOUNDARY_PEC, src/fdtd.hpp:63) marked after all boxes.
#include <algorithm>
#include <set>
#include <vector>

#include "common.cuh"
#include "primitives.cuh"

using namespace g2p;

namespace g2p {
namespace {

struct BoxD {
    int64_t x0, x1, y0, y1, z0, z1;
};

// Raw marks: every (box, element) pair writes the box's number + 1 with an
// atomic maximum, so the last box containing an element wins, as when the
// boxes are applied in order.  Element kinds per box: y-edges, x-edges,
// z-edges, nodes; off[4 * b + kind] is the start of that range in the flat
// index space.
__global__ void k_raster(Dims d, const BoxD *boxes, int64_t nbox, const int64_t *off, int64_t total,
                         unsigned long long *edge_raw, unsigned long long *node_raw) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        // box and kind of t: binary search in off
        int64_t lo = 0, hi = 4 * nbox - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (off[mid] <= t) lo = mid; else hi = mid - 1;
        }
        const int64_t b = lo >> 2;
        const int kind = (int)(lo & 3);
        const BoxD B = boxes[b];
        int64_t r = t - off[lo];
        int64_t ex, ey;                      // extents of the range along x and y
        if (kind == 0) { ex = B.x1 - B.x0 + 1; ey = B.y1 - B.y0; }
        else if (kind == 1) { ex = B.x1 - B.x0; ey = B.y1 - B.y0 + 1; }
        else { ex = B.x1 - B.x0 + 1; ey = B.y1 - B.y0 + 1; }
        const int64_t iy = B.y0 + r % ey;
        r /= ey;
        const int64_t ix = B.x0 + r % ex;
        const int64_t iz = B.z0 + r / ex;
        const unsigned long long v = (unsigned long long)(b + 1);
        if (kind == 0) atomicMax(&edge_raw[d.ye(iz, ix, iy)], v);
        else if (kind == 1) atomicMax(&edge_raw[d.xe(iz, ix, iy)], v);
        else if (kind == 2) atomicMax(&edge_raw[d.ze(iz, ix, iy)], v);
        else node_raw[iz * d.N_node_s + ix * d.ny + iy] = 1;
    }
}

// LOWER_BOUNDARY_PEC: the z = 0 plane's surface edges carry nbox + 1 and its
// nodes are conductor nodes.
__global__ void k_lower_pec(Dims d, int64_t nbox, unsigned long long *edge_raw, unsigned long long *node_raw) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < d.Ns + d.N_node_s;
         t += (int64_t)gridDim.x * blockDim.x) {
        if (t < d.Ns) edge_raw[t] = (unsigned long long)(nbox + 1);
        else node_raw[t - d.Ns] = 1;
    }
}

__device__ __forceinline__ int64_t uf_find(int64_t *parent, int64_t a) {
    // path halving; roots are fixed points
    for (int it = 0; it < (1 << 30); it++) {
        const int64_t p = parent[a];
        if (p == a) return a;
        const int64_t g = parent[p];
        if (g != p) atomicCAS((unsigned long long *)&parent[a], (unsigned long long)p, (unsigned long long)g);
        a = p;
    }
    return a;
}

// Union of the two nodes of every marked edge.  The root of a component is
// always its smallest node: a root is only ever hooked under a smaller one.
// Each retry of the compare-and-swap follows a hook made by another thread,
// so the loop ends; it is still bounded and reports through *err.
__global__ void k_union(Dims d, const unsigned long long *edge_raw, int64_t *parent, int *err) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d.N_edge; e += (int64_t)gridDim.x * blockDim.x) {
        if (!edge_raw[e]) continue;
        int64_t a, b, z, x, y;
        d.edge_nodes(e, a, b, z, x, y);
        int it = 0;
        for (; it < (1 << 20); it++) {
            a = uf_find(parent, a);
            b = uf_find(parent, b);
            if (a == b) break;
            if (a > b) { const int64_t t = a; a = b; b = t; }
            // hook the larger root b under a, if b is still a root
            if (atomicCAS((unsigned long long *)&parent[b], (unsigned long long)b, (unsigned long long)a) ==
                (unsigned long long)b)
                break;
        }
        if (it == (1 << 20)) atomicExch(err, 1);
    }
}

__global__ void k_flatten(int64_t n, const unsigned long long *node_raw, int64_t *parent, int64_t *is_root) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = node_raw[i] ? uf_find(parent, i) : -1;
        is_root[i] = (node_raw[i] && r == i) ? 1 : 0;
    }
}

// Conductor numbers by lowest node: the root's rank among the roots, plus 1.
__global__ void k_label(int64_t n, const unsigned long long *node_raw, int64_t *parent, const int64_t *rank,
                        int64_t *mark_node) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        mark_node[i] = node_raw[i] ? rank[uf_find(parent, i)] + 1 : 0;
}

// markEdge recoloured: a marked edge takes the conductor of its first node.
__global__ void k_recolour(Dims d, const unsigned long long *edge_raw, const int64_t *mark_node, int64_t *mark_edge) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d.N_edge; e += (int64_t)gridDim.x * blockDim.x) {
        int64_t a, b, z, x, y;
        d.edge_nodes(e, a, b, z, x, y);
        mark_edge[e] = edge_raw[e] ? mark_node[a] : 0;
    }
}

__global__ void k_iota(int64_t *p, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) p[i] = i;
}

// portSet's dual length of a port point (src/mesh.cpp:1257-1277).
double side_len(const std::vector<double> &c, int64_t i, double v, int64_t N) {
    if (i == 0) return c[i + 1] - v;
    if (i == N) return v - c[i - 1];
    return (c[i + 1] - v) / 2 + (v - c[i - 1]) / 2;
}

}  // namespace
}  // namespace g2p

extern "C" g2p_status g2p_mesh_mark(int64_t nx, int64_t ny, int64_t nz, const double *xn, const double *yn,
                                    const double *zn, const g2p_box *boxes, int64_t nbox, int32_t num_ports,
                                    const int32_t *port_side_ptr, const g2p_port_side *sides, int64_t *mark_node,
                                    int64_t *mark_edge, int64_t *num_cdt, int32_t *mark_port, uint8_t *cdt_return,
                                    int64_t max_cdt, int64_t *side_edge_ptr, int64_t *side_edges,
                                    int64_t max_side_edges, double *side_area, int32_t *side_dir) {
    if (nx < 3 || ny < 3 || nz < 3 || nbox < 0 || num_ports < 0 || !xn || !yn || !zn || !mark_node || !mark_edge ||
        !num_cdt || (nbox > 0 && !boxes) || (num_ports > 0 && (!port_side_ptr || !sides))) {
        set_last_message("g2p_mesh_mark: invalid argument");
        return G2P_ERR_INVALID;
    }
    Dims d;
    d.init(nx, ny, nz);
    std::vector<BoxD> hb((size_t)nbox);
    std::vector<int64_t> off((size_t)(4 * nbox + 1), 0);
    for (int64_t b = 0; b < nbox; b++) {
        const g2p_box &B = boxes[b];
        if (B.x0 < 0 || B.x1 >= nx || B.y0 < 0 || B.y1 >= ny || B.z0 < 0 || B.z1 >= nz || B.x0 > B.x1 ||
            B.y0 > B.y1 || B.z0 > B.z1) {
            set_last_message("g2p_mesh_mark: box %lld outside the grid or empty", (long long)b);
            return G2P_ERR_INVALID;
        }
        hb[b] = {B.x0, B.x1, B.y0, B.y1, B.z0, B.z1};
        const int64_t lx = B.x1 - B.x0, ly = B.y1 - B.y0, lz = B.z1 - B.z0;
        const int64_t cnt[4] = {(lz + 1) * (lx + 1) * ly, (lz + 1) * lx * (ly + 1), lz * (lx + 1) * (ly + 1),
                                (lz + 1) * (lx + 1) * (ly + 1)};
        for (int k = 0; k < 4; k++) off[4 * b + k + 1] = off[4 * b + k] + cnt[k];
    }
    const int64_t total = off[4 * nbox];
    cudaStream_t s;
    G2P_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    g2p_status st = G2P_OK;
    BoxD *d_boxes = nullptr;
    int64_t *d_off = nullptr, *parent = nullptr, *is_root = nullptr, *rank = nullptr, *work = nullptr;
    int64_t *d_mn = nullptr, *d_me = nullptr;
    unsigned long long *edge_raw = nullptr, *node_raw = nullptr;
    int *d_err = nullptr;
    int64_t ncdt = 0;
    auto run = [&]() -> g2p_status {
        G2P_TRY(dalloc(&d_boxes, std::max<int64_t>(nbox, 1), s));
        G2P_TRY(dalloc(&d_off, 4 * nbox + 1, s));
        G2P_TRY(dalloc(&edge_raw, d.N_edge, s));
        G2P_TRY(dalloc(&node_raw, d.N_node, s));
        G2P_TRY(dalloc(&parent, d.N_node, s));
        G2P_TRY(dalloc(&is_root, d.N_node + 1, s));
        G2P_TRY(dalloc(&rank, d.N_node + 1, s));
        G2P_TRY(dalloc(&work, scan_work_size(d.N_node + 1) + 4, s));
        G2P_TRY(dalloc(&d_mn, d.N_node, s));
        G2P_TRY(dalloc(&d_me, d.N_edge, s));
        G2P_TRY(dalloc(&d_err, 1, s));
        if (nbox > 0) {
            G2P_CUDA(cudaMemcpyAsync(d_boxes, hb.data(), sizeof(BoxD) * nbox, cudaMemcpyHostToDevice, s));
            G2P_CUDA(cudaMemcpyAsync(d_off, off.data(), sizeof(int64_t) * (4 * nbox + 1), cudaMemcpyHostToDevice, s));
        }
        G2P_CUDA(cudaMemsetAsync(edge_raw, 0, sizeof(unsigned long long) * d.N_edge, s));
        G2P_CUDA(cudaMemsetAsync(node_raw, 0, sizeof(unsigned long long) * d.N_node, s));
        G2P_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), s));
        if (total > 0)
            (kbegin("k_raster", s), k_raster<<<grid_for(total), kThreads, 0, s>>>(d, d_boxes, nbox, d_off, total, edge_raw, node_raw), kend(s));
        (kbegin("k_lower_pec", s), k_lower_pec<<<grid_for(d.Ns + d.N_node_s), kThreads, 0, s>>>(d, nbox, edge_raw, node_raw), kend(s));
        (kbegin("k_iota", s), k_iota<<<grid_for(d.N_node), kThreads, 0, s>>>(parent, d.N_node), kend(s));
        (kbegin("k_union", s), k_union<<<grid_for(d.N_edge), kThreads, 0, s>>>(d, edge_raw, parent, d_err), kend(s));
        (kbegin("k_flatten", s), k_flatten<<<grid_for(d.N_node), kThreads, 0, s>>>(d.N_node, node_raw, parent, is_root), kend(s));
        const int64_t *ir = is_root;
        const int64_t nn = d.N_node;
        auto op = [ir, nn] __device__(int64_t i) -> int64_t { return i < nn ? ir[i] : 0; };
        G2P_TRY(exclusive_scan(op, d.N_node + 1, rank, work, s));
        (kbegin("k_label", s), k_label<<<grid_for(d.N_node), kThreads, 0, s>>>(d.N_node, node_raw, parent, rank, d_mn), kend(s));
        (kbegin("k_recolour", s), k_recolour<<<grid_for(d.N_edge), kThreads, 0, s>>>(d, edge_raw, d_mn, d_me), kend(s));
        int herr = 0;
        G2P_CUDA(cudaMemcpyAsync(&ncdt, rank + d.N_node, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaMemcpyAsync(mark_node, d_mn, sizeof(int64_t) * d.N_node, cudaMemcpyDefault, s));
        G2P_CUDA(cudaMemcpyAsync(mark_edge, d_me, sizeof(int64_t) * d.N_edge, cudaMemcpyDefault, s));
        G2P_CUDA(cudaStreamSynchronize(s));
        G2P_CUDA(cudaGetLastError());
        if (herr) { set_last_message("g2p_mesh_mark: conductor labelling did not settle"); return G2P_ERR_CUDA; }
        return G2P_OK;
    };
    st = run();
    dfree(d_boxes, s); dfree(d_off, s); dfree(edge_raw, s); dfree(node_raw, s); dfree(parent, s);
    dfree(is_root, s); dfree(rank, s); dfree(work, s); dfree(d_mn, s); dfree(d_me, s); dfree(d_err, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (st != G2P_OK) return st;
    *num_cdt = ncdt;
    if (num_ports == 0) return G2P_OK;

    // ---- portSet (host: a few entries per port side)
    if (!mark_port || !cdt_return || !side_edge_ptr || !side_edges || !side_area || !side_dir) {
        set_last_message("g2p_mesh_mark: port outputs missing");
        return G2P_ERR_INVALID;
    }
    if (ncdt > max_cdt) {
        set_last_message("g2p_mesh_mark: %lld conductors, room for %lld", (long long)ncdt, (long long)max_cdt);
        return G2P_ERR_INVALID;
    }
    std::vector<double> X(nx), Y(ny), Z(nz);
    G2P_CUDA(cudaMemcpy(X.data(), xn, sizeof(double) * nx, cudaMemcpyDefault));
    G2P_CUDA(cudaMemcpy(Y.data(), yn, sizeof(double) * ny, cudaMemcpyDefault));
    G2P_CUDA(cudaMemcpy(Z.data(), zn, sizeof(double) * nz, cudaMemcpyDefault));
    std::fill(mark_port, mark_port + ncdt, 0);
    std::fill(cdt_return, cdt_return + ncdt, (uint8_t)0);
    auto node_of = [&](int64_t x, int64_t y, int64_t z) { return z * d.N_node_s + x * ny + y; };
    auto cond_at = [&](int64_t x, int64_t y, int64_t z, int64_t *c) -> g2p_status {
        if (x < 0 || x >= nx || y < 0 || y >= ny || z < 0 || z >= nz) {
            set_last_message("g2p_mesh_mark: port point outside the grid");
            return G2P_ERR_INVALID;
        }
        G2P_CUDA(cudaMemcpy(c, mark_node + node_of(x, y, z), sizeof(int64_t), cudaMemcpyDefault));
        return G2P_OK;
    };
    std::set<int64_t> seen;
    int64_t ne = 0;
    side_edge_ptr[0] = 0;
    for (int32_t p = 0; p < num_ports; p++) {
        const int32_t s0 = port_side_ptr[p], s1 = port_side_ptr[p + 1];
        if (s1 <= s0) { set_last_message("g2p_mesh_mark: port %d has no side", p); return G2P_ERR_INVALID; }
        for (int32_t k = s0; k < s1; k++) {
            int64_t c1 = 0, c2 = 0;
            G2P_TRY(cond_at(sides[k].sx, sides[k].sy, sides[k].sz, &c1));
            G2P_TRY(cond_at(sides[k].rx, sides[k].ry, sides[k].rz, &c2));
            if (c1 == 0 || c2 == 0) {
                set_last_message("g2p_mesh_mark: port %d end outside a conductor", p);
                return G2P_ERR_INVALID;
            }
        }
        // the last side's conductors are marked; a return conductor gets its
        // PEC-plane sets only when first met as a return (src/mesh.cpp:941-953)
        const g2p_port_side &ls = sides[s1 - 1];
        int64_t c1 = 0, c2 = 0;
        G2P_TRY(cond_at(ls.sx, ls.sy, ls.sz, &c1));
        G2P_TRY(cond_at(ls.rx, ls.ry, ls.rz, &c2));
        mark_port[c1 - 1] = p + 1;
        mark_port[c2 - 1] = -1;
        seen.insert(c1);
        if (seen.insert(c2).second) cdt_return[c2 - 1] = 1;
        for (int32_t k = s0; k < s1; k++) {
            const g2p_port_side &q = sides[k];
            const double sx = X[q.sx], sy = Y[q.sy], sz = Z[q.sz];
            int64_t lo, hi;
            double area;
            std::vector<int64_t> e;
            if (q.sx != q.rx) {
                lo = std::min(q.sx, q.rx); hi = std::max(q.sx, q.rx);
                for (int64_t j = lo; j < hi; j++) e.push_back(d.xe(q.sz, j, q.sy));
                area = side_len(Y, q.sy, sy, d.Ny) * side_len(Z, q.sz, sz, d.Nz);
            } else if (q.sy != q.ry) {
                lo = std::min(q.sy, q.ry); hi = std::max(q.sy, q.ry);
                for (int64_t j = lo; j < hi; j++) e.push_back(d.ye(q.sz, q.sx, j));
                area = side_len(X, q.sx, sx, d.Nx) * side_len(Z, q.sz, sz, d.Nz);
            } else {
                lo = std::min(q.sz, q.rz); hi = std::max(q.sz, q.rz);
                for (int64_t j = lo; j < hi; j++) e.push_back(d.ze(j, q.sx, q.sy));
                area = side_len(X, q.sx, sx, d.Nx) * side_len(Y, q.sy, sy, d.Ny);
            }
            if (ne + (int64_t)e.size() > max_side_edges) {
                set_last_message("g2p_mesh_mark: more port edges than max_side_edges");
                return G2P_ERR_INVALID;
            }
            for (int64_t v : e) side_edges[ne++] = v;
            side_edge_ptr[k + 1] = ne;
            side_area[k] = area;
            // positiveCoordFlow: +1 when any supply coordinate exceeds the return's
            side_dir[k] = (q.sx > q.rx || q.sy > q.ry || q.sz > q.rz) ? 1 : -1;
        }
    }
    return G2P_OK;
}
