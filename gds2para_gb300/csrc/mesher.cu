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
#include <functional>
#include <map>
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

namespace g2p {
// Labels the conductors of raw marks (edge_raw: nonzero on conductor edges;
// node_raw: nonzero on conductor nodes) and writes markNode (conductor
// number, 0 outside) and the recoloured markEdge to host or device arrays.
g2p_status label_conductors(const Dims &d, unsigned long long *edge_raw, unsigned long long *node_raw,
                            int64_t *mark_node, int64_t *mark_edge, int64_t *num_cdt, cudaStream_t s) {
    int64_t *parent = nullptr, *is_root = nullptr, *rank = nullptr, *work = nullptr;
    int64_t *d_mn = nullptr, *d_me = nullptr;
    int *d_err = nullptr;
    int64_t ncdt = 0;
    auto run = [&]() -> g2p_status {
        G2P_TRY(dalloc(&parent, d.N_node, s));
        G2P_TRY(dalloc(&is_root, d.N_node + 1, s));
        G2P_TRY(dalloc(&rank, d.N_node + 1, s));
        G2P_TRY(dalloc(&work, scan_work_size(d.N_node + 1) + 4, s));
        G2P_TRY(dalloc(&d_mn, d.N_node, s));
        G2P_TRY(dalloc(&d_me, d.N_edge, s));
        G2P_TRY(dalloc(&d_err, 1, s));
        G2P_CUDA(cudaMemsetAsync(d_err, 0, sizeof(int), s));
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
        if (herr) { set_last_message("conductor labelling did not settle"); return G2P_ERR_CUDA; }
        return G2P_OK;
    };
    const g2p_status st = run();
    dfree(parent, s); dfree(is_root, s); dfree(rank, s); dfree(work, s); dfree(d_mn, s); dfree(d_me, s);
    dfree(d_err, s);
    cudaStreamSynchronize(s);
    if (st == G2P_OK) *num_cdt = ncdt;
    return st;
}

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
    int64_t *d_off = nullptr;
    unsigned long long *edge_raw = nullptr, *node_raw = nullptr;
    int64_t ncdt = 0;
    auto run = [&]() -> g2p_status {
        G2P_TRY(dalloc(&d_boxes, std::max<int64_t>(nbox, 1), s));
        G2P_TRY(dalloc(&d_off, 4 * nbox + 1, s));
        G2P_TRY(dalloc(&edge_raw, d.N_edge, s));
        G2P_TRY(dalloc(&node_raw, d.N_node, s));
        if (nbox > 0) {
            G2P_CUDA(cudaMemcpyAsync(d_boxes, hb.data(), sizeof(BoxD) * nbox, cudaMemcpyHostToDevice, s));
            G2P_CUDA(cudaMemcpyAsync(d_off, off.data(), sizeof(int64_t) * (4 * nbox + 1), cudaMemcpyHostToDevice, s));
        }
        G2P_CUDA(cudaMemsetAsync(edge_raw, 0, sizeof(unsigned long long) * d.N_edge, s));
        G2P_CUDA(cudaMemsetAsync(node_raw, 0, sizeof(unsigned long long) * d.N_node, s));
        if (total > 0)
            (kbegin("k_raster", s), k_raster<<<grid_for(total), kThreads, 0, s>>>(d, d_boxes, nbox, d_off, total, edge_raw, node_raw), kend(s));
        (kbegin("k_lower_pec", s), k_lower_pec<<<grid_for(d.Ns + d.N_node_s), kThreads, 0, s>>>(d, nbox, edge_raw, node_raw), kend(s));
        return label_conductors(d, edge_raw, node_raw, mark_node, mark_edge, &ncdt, s);
    };
    st = run();
    dfree(d_boxes, s); dfree(d_off, s); dfree(edge_raw, s); dfree(node_raw, s);
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

// ---------------------------------------------------------------------------
// Polygon marking: findInsideCond (src/fdtd.hpp:534-826) on the grid that
// meshAndMark builds from the same polygons (g2p_mesh_grid), followed by the
// conductor numbering above and meshAndMark's port placement (findPortNode,
// src/fdtd.hpp:1204-1384; markPort and the return conductors,
// src/mesh.cpp:884-953) and portSet (src/mesh.cpp:1196-1356) on the side
// coordinates in metres.
//
// findInsideCond cuts each polygon's x extent into windows between
// consecutive grid lines and, per window, keeps the y range the polygon's
// edges span there.  Every grid node of the window inside that y range (with
// the grid line just below it) is tested with the polygon point test, and so
// are the midpoints of the window's x- and y-edges: an inside node marks the
// z-edges through it over the polygon's layers, an inside midpoint the x- or
// y-edges on every grid plane of the layer, and both ends of every marked
// edge become conductor nodes.  The windows and their y ranges are a few per
// polygon edge and are made on the host; the point tests run on the device,
// one thread per (window, node), each edge marked with the polygon number +
// 1 by an atomic maximum (the last polygon wins, as when they are applied in
// order).
namespace g2p {
namespace {

struct PolyWin {
    int64_t poly;
    int64_t x1, x2, y1in, y2in, zlo, zhi;
    int64_t single;             // the polygon spans one x line: no x-edges
};

// The polygon point test (polyIn, src/fdtd.hpp:501-530): on an x- or y-
// directed polygon edge within 1e-10 is inside; otherwise crossings of the
// ray towards +x are counted, an edge counting for y in [low end, high end).
__device__ bool poly_in(double x, double y, const double *px, const double *py, int64_t n) {
    const double dm = 1.e-10;
    bool in = false;
    for (int64_t i = 0, j = n - 1; i < n; j = i++) {
        const double xi = px[i], yi = py[i], xj = px[j], yj = py[j];
        if (fabs(y - yj) < dm && fabs(y - yi) < dm && ((x >= xj && x <= xi) || (x >= xi && x <= xj))) return true;
        if (fabs(x - xj) < dm && fabs(x - xi) < dm && ((y >= yj && y <= yi) || (y >= yi && y <= yj))) return true;
        if (fabs(yi - yj) > dm && ((yi <= y && y < yj) || (yj <= y && y < yi)) && (x < (xj - xi) * (y - yi) / (yj - yi) + xi))
            in = !in;
    }
    return in;
}

__global__ void k_poly_mark(Dims d, const double *xn, const double *yn, const PolyWin *wins, const int64_t *woff,
                            int64_t nwin, int64_t total, const int64_t *vptr, const double *vx, const double *vy,
                            unsigned long long *edge_raw, unsigned long long *node_raw) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = nwin - 1;
        while (lo < hi) {
            const int64_t mid = (lo + hi + 1) >> 1;
            if (woff[mid] <= t) lo = mid; else hi = mid - 1;
        }
        const PolyWin W = wins[lo];
        const int64_t r = t - woff[lo], nyw = W.y2in - W.y1in + 1;
        const int64_t iy = W.y1in + r % nyw, ix = W.x1 + r / nyw;
        const double *px = vx + vptr[W.poly], *py = vy + vptr[W.poly];
        const int64_t n = vptr[W.poly + 1] - vptr[W.poly];
        const unsigned long long v = (unsigned long long)(W.poly + 1);
        if (poly_in(xn[ix], yn[iy], px, py, n)) {
            for (int64_t l = W.zlo; l < W.zhi; l++) {
                atomicMax(&edge_raw[d.ze(l, ix, iy)], v);
                node_raw[l * d.N_node_s + ix * d.ny + iy] = 1;
                node_raw[(l + 1) * d.N_node_s + ix * d.ny + iy] = 1;
            }
        }
        if (!W.single && ix < W.x2 && poly_in((xn[ix] + xn[ix + 1]) / 2, yn[iy], px, py, n)) {
            for (int64_t l = W.zlo; l <= W.zhi; l++) {
                atomicMax(&edge_raw[d.xe(l, ix, iy)], v);
                node_raw[l * d.N_node_s + ix * d.ny + iy] = 1;
                node_raw[l * d.N_node_s + (ix + 1) * d.ny + iy] = 1;
            }
        }
        if (iy < W.y2in && poly_in(xn[ix], (yn[iy] + yn[iy + 1]) / 2, px, py, n)) {
            for (int64_t l = W.zlo; l <= W.zhi; l++) {
                atomicMax(&edge_raw[d.ye(l, ix, iy)], v);
                node_raw[l * d.N_node_s + ix * d.ny + iy] = 1;
                node_raw[l * d.N_node_s + ix * d.ny + iy + 1] = 1;
            }
        }
    }
}

// Index of a coordinate on grid lines c[0..n): the line it was merged into
// when the lines were made (the last line at or below it), as meshAndMark's
// xi/yi/zi maps give it for the coordinates the grid was built from.
int64_t line_of(const std::vector<double> &c, double v) {
    const int64_t i = (int64_t)(std::upper_bound(c.begin(), c.end(), v) - c.begin()) - 1;
    return i < 0 ? 0 : i;
}

// The windows of one polygon (findInsideCond's xcoor / xrange / xcoory).
void polygon_windows(int64_t poly, const double *x, const double *y, int64_t n, int64_t zlo, int64_t zhi,
                     const std::vector<double> &X, const std::vector<double> &Y, std::vector<PolyWin> &out) {
    const int64_t ny = (int64_t)Y.size();
    int64_t ymax = 0, ymin = ny - 1;
    std::set<int64_t> xcoor;
    auto edge_span = [&](int64_t a, int64_t b) {
        ymax = std::max(ymax, std::max(line_of(Y, y[a]), line_of(Y, y[b])));
        ymin = std::min(ymin, std::min(line_of(Y, y[a]), line_of(Y, y[b])));
        int64_t x1, x2;
        if (x[a] < x[b]) { x1 = line_of(X, x[a]); x2 = line_of(X, x[b]); }
        else { x1 = line_of(X, x[b]); x2 = line_of(X, x[a]); }
        for (int64_t l = x1; l <= x2; l++) xcoor.insert(l);
    };
    for (int64_t j = 0; j + 1 < n; j++) edge_span(j, j + 1);
    edge_span(n - 1, 0);
    std::vector<int64_t> xv(xcoor.begin(), xcoor.end());
    std::map<int64_t, int64_t> xrange;
    const bool multi = xv.size() > 1;
    for (size_t j = 0; j + 1 < xv.size(); j++) xrange[xv[j]] = xv[j + 1];
    if (xv.size() == 1) xrange[xv[0]] = xv[0];
    std::map<int64_t, std::pair<double, double>> xcy;     // window -> (y low, y high)
    auto cross = [&](int64_t a, int64_t b) {
        int64_t ss, ee;
        if (x[a] < x[b]) { ss = line_of(X, x[a]); ee = line_of(X, x[b]); }
        else if (x[a] > x[b]) { ss = line_of(X, x[b]); ee = line_of(X, x[a]); }
        else return;
        if (ss == ee && multi) return;
        for (auto it = xrange.find(ss); it != xrange.end() && it->second <= ee; it = xrange.find(ss)) {
            auto w = xcy.emplace(ss, std::make_pair(1.e+30, -1.e+30)).first;
            const double dx = x[b] - x[a];
            const double y1 = (x[b] - X[ss]) / dx * y[a] + (X[ss] - x[a]) / dx * y[b];
            const double y2 = (x[b] - X[it->second]) / dx * y[a] + (X[it->second] - x[a]) / dx * y[b];
            w->second.first = std::min(w->second.first, std::min(y1, y2));
            w->second.second = std::max(w->second.second, std::max(y1, y2));
            if (!multi) break;
            ss = it->second;
        }
    };
    for (int64_t j = 0; j + 1 < n; j++) cross(j, j + 1);
    cross(n - 1, 0);
    for (const auto &w : xcy) {
        const double ylo = w.second.first, yhi = w.second.second;
        int64_t y1in = ymin, y2in = ymax;
        for (int64_t j = ymin; j <= ymax; j++) {
            if (Y[j] >= yhi) { y2in = j; break; }
            if (Y[j] < ylo) y1in = j;
        }
        if (y2in < y1in) continue;
        PolyWin pw;
        pw.poly = poly;
        pw.x1 = w.first;
        pw.x2 = multi ? xrange[w.first] : w.first;
        pw.y1in = y1in;
        pw.y2in = y2in;
        pw.zlo = zlo;
        pw.zhi = zhi;
        pw.single = multi ? 0 : 1;
        out.push_back(pw);
    }
}

}  // namespace
}  // namespace g2p

extern "C" g2p_status g2p_mesh_mark_polygons(int64_t nx, int64_t ny, int64_t nz, const double *xn, const double *yn,
                                             const double *zn, int64_t npoly, const int64_t *vert_ptr,
                                             const double *vx, const double *vy, const double *poly_z,
                                             int32_t num_ports, const int32_t *port_side_ptr, double *side_coords,
                                             const int32_t *side_dir_in, int64_t *mark_node, int64_t *mark_edge,
                                             int64_t *num_cdt, int32_t *mark_port, uint8_t *cdt_return,
                                             int64_t max_cdt, int64_t *side_edge_ptr, int64_t *side_edges,
                                             int64_t max_side_edges, double *side_area, int32_t *side_dir) {
    if (nx < 3 || ny < 3 || nz < 3 || npoly < 0 || num_ports < 0 || !xn || !yn || !zn || !mark_node || !mark_edge ||
        !num_cdt || (npoly > 0 && (!vert_ptr || !vx || !vy || !poly_z)) ||
        (num_ports > 0 && (!port_side_ptr || !side_coords || !side_dir_in))) {
        set_last_message("g2p_mesh_mark_polygons: invalid argument");
        return G2P_ERR_INVALID;
    }
    Dims d;
    d.init(nx, ny, nz);
    std::vector<double> X(nx), Y(ny), Z(nz);
    G2P_CUDA(cudaMemcpy(X.data(), xn, sizeof(double) * nx, cudaMemcpyDefault));
    G2P_CUDA(cudaMemcpy(Y.data(), yn, sizeof(double) * ny, cudaMemcpyDefault));
    G2P_CUDA(cudaMemcpy(Z.data(), zn, sizeof(double) * nz, cudaMemcpyDefault));
    std::vector<PolyWin> wins;
    for (int64_t p = 0; p < npoly; p++) {
        const int64_t n = vert_ptr[p + 1] - vert_ptr[p];
        if (n < 1) { set_last_message("g2p_mesh_mark_polygons: polygon %lld has no vertex", (long long)p); return G2P_ERR_INVALID; }
        if (poly_z[2 * p + 1] == poly_z[2 * p]) continue;          // on no stack layer
        polygon_windows(p, vx + vert_ptr[p], vy + vert_ptr[p], n, line_of(Z, poly_z[2 * p]), line_of(Z, poly_z[2 * p + 1]),
                        X, Y, wins);
    }
    std::vector<int64_t> woff(wins.size() + 1, 0);
    for (size_t w = 0; w < wins.size(); w++)
        woff[w + 1] = woff[w] + (wins[w].x2 - wins[w].x1 + 1) * (wins[w].y2in - wins[w].y1in + 1);
    const int64_t total = woff.back(), nvert = npoly > 0 ? vert_ptr[npoly] : 0;
    cudaStream_t s;
    G2P_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    PolyWin *d_w = nullptr;
    int64_t *d_woff = nullptr, *d_vptr = nullptr, ncdt = 0;
    double *d_x = nullptr, *d_y = nullptr, *d_vx = nullptr, *d_vy = nullptr;
    unsigned long long *edge_raw = nullptr, *node_raw = nullptr;
    auto run = [&]() -> g2p_status {
        G2P_TRY(dalloc(&d_w, std::max<int64_t>((int64_t)wins.size(), 1), s));
        G2P_TRY(dalloc(&d_woff, (int64_t)woff.size(), s));
        G2P_TRY(dalloc(&d_vptr, npoly + 1, s));
        G2P_TRY(dalloc(&d_vx, std::max<int64_t>(nvert, 1), s));
        G2P_TRY(dalloc(&d_vy, std::max<int64_t>(nvert, 1), s));
        G2P_TRY(dalloc(&d_x, nx, s));
        G2P_TRY(dalloc(&d_y, ny, s));
        G2P_TRY(dalloc(&edge_raw, d.N_edge, s));
        G2P_TRY(dalloc(&node_raw, d.N_node, s));
        if (!wins.empty()) {
            G2P_CUDA(cudaMemcpyAsync(d_w, wins.data(), sizeof(PolyWin) * wins.size(), cudaMemcpyHostToDevice, s));
            G2P_CUDA(cudaMemcpyAsync(d_woff, woff.data(), sizeof(int64_t) * woff.size(), cudaMemcpyHostToDevice, s));
        }
        if (npoly > 0) {
            G2P_CUDA(cudaMemcpyAsync(d_vptr, vert_ptr, sizeof(int64_t) * (npoly + 1), cudaMemcpyDefault, s));
            G2P_CUDA(cudaMemcpyAsync(d_vx, vx, sizeof(double) * nvert, cudaMemcpyDefault, s));
            G2P_CUDA(cudaMemcpyAsync(d_vy, vy, sizeof(double) * nvert, cudaMemcpyDefault, s));
        }
        G2P_CUDA(cudaMemcpyAsync(d_x, X.data(), sizeof(double) * nx, cudaMemcpyHostToDevice, s));
        G2P_CUDA(cudaMemcpyAsync(d_y, Y.data(), sizeof(double) * ny, cudaMemcpyHostToDevice, s));
        G2P_CUDA(cudaMemsetAsync(edge_raw, 0, sizeof(unsigned long long) * d.N_edge, s));
        G2P_CUDA(cudaMemsetAsync(node_raw, 0, sizeof(unsigned long long) * d.N_node, s));
        if (total > 0)
            (kbegin("k_poly_mark", s), k_poly_mark<<<grid_for(total), kThreads, 0, s>>>(d, d_x, d_y, d_w, d_woff, (int64_t)wins.size(), total, d_vptr, d_vx, d_vy, edge_raw, node_raw), kend(s));
        // LOWER_BOUNDARY_PEC: after the polygons, numCdtRow + 1 on the plane
        (kbegin("k_lower_pec", s), k_lower_pec<<<grid_for(d.Ns + d.N_node_s), kThreads, 0, s>>>(d, npoly, edge_raw, node_raw), kend(s));
        return label_conductors(d, edge_raw, node_raw, mark_node, mark_edge, &ncdt, s);
    };
    g2p_status st = run();
    dfree(d_w, s); dfree(d_woff, s); dfree(d_vptr, s); dfree(d_vx, s); dfree(d_vy, s); dfree(d_x, s); dfree(d_y, s);
    dfree(edge_raw, s); dfree(node_raw, s);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    if (st != G2P_OK) return st;
    *num_cdt = ncdt;
    if (num_ports == 0) return G2P_OK;
    if (!mark_port || !cdt_return || !side_edge_ptr || !side_edges || !side_area || !side_dir) {
        set_last_message("g2p_mesh_mark_polygons: port outputs missing");
        return G2P_ERR_INVALID;
    }
    if (ncdt > max_cdt) {
        set_last_message("g2p_mesh_mark_polygons: %lld conductors, room for %lld", (long long)ncdt, (long long)max_cdt);
        return G2P_ERR_INVALID;
    }
    std::vector<int64_t> MN((size_t)d.N_node);
    G2P_CUDA(cudaMemcpy(MN.data(), mark_node, sizeof(int64_t) * d.N_node, cudaMemcpyDefault));
    auto node = [&](int64_t x, int64_t y, int64_t z) -> int64_t & { return MN[(size_t)(z * d.N_node_s + x * ny + y)]; };
    std::fill(mark_port, mark_port + ncdt, 0);
    std::fill(cdt_return, cdt_return + ncdt, (uint8_t)0);
    // ---- meshAndMark's port section: findPortNode per side, then the last
    // side's two conductors are marked
    std::set<int64_t> seen;
    const int step = 50;
    for (int32_t p = 0; p < num_ports; p++) {
        const int32_t s0 = port_side_ptr[p], s1 = port_side_ptr[p + 1];
        if (s1 <= s0) { set_last_message("g2p_mesh_mark_polygons: port %d has no side", p); return G2P_ERR_INVALID; }
        int64_t c1 = 0, c2 = 0;
        for (int32_t k = s0; k < s1; k++) {
            double *c = side_coords + 6 * (int64_t)k;
            int64_t x1 = line_of(X, c[0]), y1 = line_of(Y, c[1]), z1 = line_of(Z, c[2]);
            int64_t x2 = line_of(X, c[3]), y2 = line_of(Y, c[4]), z2 = line_of(Z, c[5]);
            bool found = true;
            // a port end outside every conductor walks away from the other
            // end (or, for a z-directed port's supply, along -y then +y), up
            // to 50 lines, to the first conductor node
            auto walk = [&](int64_t &v, int dirv, int64_t lim_lo, int64_t lim_hi, std::function<int64_t &()> at,
                            double *coord, const std::vector<double> &lines) {
                int i = 0;
                while (i < step && (dirv < 0 ? v > lim_lo : v < lim_hi)) {
                    v += dirv;
                    if (at()) { *coord = lines[(size_t)v]; break; }
                    i++;
                }
                if (i == step || v == (dirv < 0 ? lim_lo : lim_hi)) found = false;
            };
            if (node(x1, y1, z1) == 0) {
                if (x1 < x2) walk(x1, -1, 0, nx - 1, [&]() -> int64_t & { return node(x1, y1, z1); }, &c[0], X);
                else if (y1 < y2) walk(y1, -1, 0, ny - 1, [&]() -> int64_t & { return node(x1, y1, z1); }, &c[1], Y);
                else if (z1 < z2) walk(z1, -1, 0, nz - 1, [&]() -> int64_t & { return node(x1, y1, z1); }, &c[2], Z);
                else if (x1 > x2) walk(x1, +1, 0, nx - 1, [&]() -> int64_t & { return node(x1, y1, z1); }, &c[0], X);
                else if (y1 > y2) walk(y1, +1, 0, ny - 1, [&]() -> int64_t & { return node(x1, y1, z1); }, &c[1], Y);
                else if (z1 > z2) {
                    int i = 0;
                    bool got = false;
                    while (i < step && y1 > 0) {
                        y1 -= 1;
                        if (node(x1, y1, z1)) { c[1] = Y[(size_t)y1]; got = true; break; }
                        i++;
                    }
                    if (!got)
                        while (i < step && y1 < ny - 1) {
                            y1 += 1;
                            if (node(x1, y1, z1)) { c[1] = Y[(size_t)y1]; got = true; break; }
                            i++;
                        }
                    if (!got) found = false;
                }
            }
            if (found && node(x2, y2, z2) == 0) {
                if (x1 < x2) walk(x2, +1, 0, nx - 1, [&]() -> int64_t & { return node(x2, y2, z2); }, &c[3], X);
                else if (y1 < y2) walk(y2, +1, 0, ny - 1, [&]() -> int64_t & { return node(x2, y2, z2); }, &c[4], Y);
                else if (z1 < z2) walk(z2, +1, 0, nz - 1, [&]() -> int64_t & { return node(x2, y2, z2); }, &c[5], Z);
                else if (x1 > x2) walk(x2, -1, 0, nx - 1, [&]() -> int64_t & { return node(x2, y2, z2); }, &c[3], X);
                else if (y1 > y2) walk(y2, -1, 0, ny - 1, [&]() -> int64_t & { return node(x2, y2, z2); }, &c[4], Y);
                else if (z1 > z2) walk(z2, -1, 0, nz - 1, [&]() -> int64_t & { return node(x2, y2, z2); }, &c[5], Z);
            }
            if (!found) {
                set_last_message("g2p_mesh_mark_polygons: port %d side %d could not be located within a conductor", p,
                                 k - s0);
                return G2P_ERR_INVALID;
            }
            if (z1 != z2) { c[4] = c[1]; c[3] = c[0]; }
            c1 = node(line_of(X, c[0]), line_of(Y, c[1]), line_of(Z, c[2]));
            c2 = node(line_of(X, c[3]), line_of(Y, c[4]), line_of(Z, c[5]));
        }
        if (c1 == 0 || c2 == 0) {
            set_last_message("g2p_mesh_mark_polygons: port %d end outside a conductor", p);
            return G2P_ERR_INVALID;
        }
        mark_port[c1 - 1] = p + 1;
        mark_port[c2 - 1] = -1;
        seen.insert(c1);
        if (seen.insert(c2).second) cdt_return[c2 - 1] = 1;
    }
    // ---- portSet: edges between the two ends, cross-section area at the
    // supply point (its dual lengths about the actual coordinate)
    auto dual = [](const std::vector<double> &c, int64_t i, double v, int64_t N) {
        if (i == 0) return c[(size_t)i + 1] - v;
        if (i == N) return v - c[(size_t)i - 1];
        return (c[(size_t)i + 1] - v) / 2 + (v - c[(size_t)i - 1]) / 2;
    };
    int64_t ne = 0;
    side_edge_ptr[0] = 0;
    for (int32_t p = 0; p < num_ports; p++)
        for (int32_t k = port_side_ptr[p]; k < port_side_ptr[p + 1]; k++) {
            const double *c = side_coords + 6 * (int64_t)k;
            const int64_t x1 = line_of(X, c[0]), y1 = line_of(Y, c[1]), z1 = line_of(Z, c[2]);
            const int64_t x2 = line_of(X, c[3]), y2 = line_of(Y, c[4]), z2 = line_of(Z, c[5]);
            const int64_t m1 = node(x1, y1, z1), m2 = node(x2, y2, z2);
            if (!((m1 != 0 && mark_port[m1 - 1] > -1) || (m2 != 0 && mark_port[m2 - 1] > -1))) {
                set_last_message("g2p_mesh_mark_polygons: port %d side %d has both ends on return conductors", p, k);
                return G2P_ERR_INVALID;
            }
            std::vector<int64_t> e;
            double area = 1.;
            if (c[0] != c[3]) {
                for (int64_t j = std::min(x1, x2); j < std::max(x1, x2); j++) e.push_back(d.xe(z1, j, y1));
                area *= dual(Y, y1, c[1], d.Ny);
                area *= dual(Z, z1, c[2], d.Nz);
            } else if (c[1] != c[4]) {
                for (int64_t j = std::min(y1, y2); j < std::max(y1, y2); j++) e.push_back(d.ye(z1, x1, j));
                area *= dual(X, x1, c[0], d.Nx);
                area *= dual(Z, z1, c[2], d.Nz);
            } else if (c[2] != c[5]) {
                for (int64_t j = std::min(z1, z2); j < std::max(z1, z2); j++) e.push_back(d.ze(j, x1, y1));
                area *= dual(X, x1, c[0], d.Nx);
                area *= dual(Y, y1, c[1], d.Ny);
            }
            if (ne + (int64_t)e.size() > max_side_edges) {
                set_last_message("g2p_mesh_mark_polygons: more port edges than max_side_edges");
                return G2P_ERR_INVALID;
            }
            for (int64_t v : e) side_edges[ne++] = v;
            side_edge_ptr[k + 1] = ne;
            side_area[k] = area;
            side_dir[k] = side_dir_in[k];
        }
    return G2P_OK;
}
