// fdtdMesh upload, PEC index maps (a2-a4) and the curl-curl stiffness S (a7-a9).
//
// Index maps restate setMapEdge/findBoundNodeEdge (fdtd.hpp:1444-1529) and
// the LOWER_BOUNDARY_PEC sets (mesh.cpp:963-987) as one flag pass plus an
// exclusive scan.  S restates generateStiff (generateStiff.cpp:6-565): the
// reference forms face-by-edge matrices Se (curl, +-1/h) and Sh (dual
// lengths over dual areas) and multiplies S = Sh*Se^T/mu with MKL, dropping
// PEC rows/columns.  Here each output row is generated directly from the
// (at most four) faces that contain its edge, visited in increasing face
// number so the sums run in the same order as the sparse product; at most 13
// distinct columns per row are accumulated in registers and sorted.
#include <atomic>
#include <cstdarg>
#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"
#include "primitives.cuh"

namespace g2p {

static thread_local std::string g_err;

void set_last_error(cudaError_t e, const char *what, const char *file, int line) {
    char buf[512];
    snprintf(buf, sizeof buf, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
    g_err = buf;
}

void set_last_message(const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
}

const char *last_error() { return g_err.c_str(); }

static std::atomic<int64_t> g_launches{0};
void launch_tick() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void launch_add(int64_t n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

struct NamedProfile {
    bool on = false;
    std::vector<cudaEvent_t> ev;
    size_t used = 0;
    std::vector<const char *> names;
    std::map<std::string, std::pair<int64_t, double>> totals;   // name -> (launches, ms)
};
static NamedProfile g_np;

static void np_record(cudaStream_t s) {
    if (g_np.used == g_np.ev.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        g_np.ev.push_back(e);
    }
    cudaEventRecord(g_np.ev[g_np.used++], s);
}
void (*kbracket_begin)(cudaStream_t) = nullptr;
void (*kbracket_end)(cudaStream_t) = nullptr;
void kbegin(const char *name, cudaStream_t s) {
    launch_tick();
    if (g_np.on) {
        g_np.names.push_back(name);
        np_record(s);
    }
    if (kbracket_begin) kbracket_begin(s);
}
void kend(cudaStream_t s) {
    if (kbracket_end) kbracket_end(s);
    if (g_np.on) np_record(s);
}
bool kprof_on() { return g_np.on; }
void kprof_set(bool on) {
    if (on) { g_np.used = 0; g_np.names.clear(); g_np.totals.clear(); }
    g_np.on = on;
}
g2p_status kprof_collect() {
    G2P_CUDA(cudaDeviceSynchronize());
    for (size_t i = 0; i < g_np.names.size() && 2 * i + 1 < g_np.used; i++) {
        float t = 0;
        G2P_CUDA(cudaEventElapsedTime(&t, g_np.ev[2 * i], g_np.ev[2 * i + 1]));
        auto &tot = g_np.totals[g_np.names[i]];
        tot.first += 1;
        tot.second += t;
    }
    g_np.used = 0;
    g_np.names.clear();
    return G2P_OK;
}

// Keeps freed stream-ordered allocations in the device pool instead of
// returning them to the driver at every synchronization (the default
// threshold of 0 makes each large allocation re-map its pages).
void retain_pool_memory(int device) {
    static std::once_flag once;
    std::call_once(once, [device]() {
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
            uint64_t thr = UINT64_MAX;
            cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
        }
    });
}

g2p_status ensure_scan_work(g2p_mesh *m, int64_t n) {
    int64_t need = scan_work_size(n) + 16;
    if (need <= m->scan_work_n) return G2P_OK;
    dfree(m->scan_work, m->stream);
    G2P_TRY(dalloc(&m->scan_work, need, m->stream));
    m->scan_work_n = need;
    return G2P_OK;
}

// ------------------------------------------------------------------ upload
__global__ void k_narrow(const int64_t *__restrict__ in, int32_t *__restrict__ out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = (int32_t)in[i];
}

// Conductor ids must lie in [0, num_cdt]; flag[0] is set otherwise.
__global__ void k_check_marks(const int32_t *a, int64_t n, int64_t ncdt, int *flag) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        if (a[i] < 0 || a[i] > ncdt) atomicExch(flag, 1);
}

// Dual lengths dxa/dya/dza (generateStiff.cpp:250-267).
__global__ void k_dual_lengths(const double *c, int64_t N, double *d) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= N; i += (int64_t)gridDim.x * blockDim.x) {
        if (i == 0) d[0] = c[1] - c[0];
        else if (i == N) d[N] = c[N] - c[N - 1];
        else d[i] = (c[i + 1] - c[i - 1]) / 2;
    }
}

}  // namespace g2p

using namespace g2p;

extern "C" const char *g2p_last_error(void) { return g2p::last_error(); }
extern "C" const char *g2p_version(void) { return "gds2para_gb300 0.1 (sm_103a)"; }
extern "C" int64_t g2p_launch_count(void) { return g2p::launch_count(); }

// One line per kernel, "name<TAB>launches<TAB>total_ms", by decreasing time.
namespace g2p {
void kprof_add_total(const char *name, int64_t launches, double ms) {
    auto &t = g_np.totals[name];
    t.first += launches;
    t.second += ms;
}
}  // namespace g2p

extern "C" int64_t g2p_profile_report(char *buf, int64_t cap) {
    std::vector<std::pair<double, std::string>> rows;
    for (auto &kv : g2p::g_np.totals) {
        char line[256];
        snprintf(line, sizeof line, "%s\t%lld\t%.6f\n", kv.first.c_str(), (long long)kv.second.first, kv.second.second);
        rows.push_back({kv.second.second, line});
    }
    std::sort(rows.begin(), rows.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
    std::string out;
    for (auto &r : rows) out += r.second;
    if (buf && cap > 0) {
        int64_t n = std::min<int64_t>(cap - 1, (int64_t)out.size());
        memcpy(buf, out.data(), (size_t)n);
        buf[n] = 0;
    }
    return (int64_t)out.size();
}

extern "C" g2p_status g2p_mesh_create(const g2p_mesh_desc *in, g2p_mesh **out) {
    if (!in || !out) { set_last_message("null argument"); return G2P_ERR_INVALID; }
    *out = nullptr;
    if (in->nx < 3 || in->ny < 3 || in->nz < 3) { set_last_message("grid must have at least 3 nodes per axis"); return G2P_ERR_INVALID; }
    if (!in->xn || !in->yn || !in->zn || !in->stack_epsn || !in->stack_sign || !in->mark_node || !in->mark_edge) {
        set_last_message("missing mesh array"); return G2P_ERR_INVALID;
    }
    if (in->num_cdt < 1 || !in->mark_port || !in->cdt_return) { set_last_message("mesh has no conductors"); return G2P_ERR_INVALID; }
    if (in->num_ports < 0 || (in->num_ports > 0 && (!in->port_side_ptr || !in->side_edge_ptr || !in->side_edges || !in->side_area || !in->side_dir))) {
        set_last_message("missing port arrays"); return G2P_ERR_INVALID;
    }
    if (in->nfreq < 1) { set_last_message("nfreq must be >= 1"); return G2P_ERR_INVALID; }
    g2p_mesh *m = new g2p_mesh();
    m->d.init(in->nx, in->ny, in->nz);
    if (m->d.N_edge >= (int64_t)INT32_MAX || m->d.N_node >= (int64_t)INT32_MAX) {
        delete m; set_last_message("grid exceeds 2^31 edges"); return G2P_ERR_UNSUPPORTED;
    }
    cudaGetDevice(&m->device);
    retain_pool_memory(m->device);
    cudaError_t e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { set_last_error(e, "cudaStreamCreate", __FILE__, __LINE__); delete m; return G2P_ERR_CUDA; }
    m->k.mu = G2P_MU;
    m->k.eps0 = G2P_EPSILON0;
    const Dims &d = m->d;
    cudaStream_t s = m->stream;
    // small arrays the host reads: copied with unified addressing so the
    // descriptor may point to host or device memory
    auto fetch = [&](auto &vec, const auto *src, int64_t n) -> bool {
        vec.resize((size_t)n);
        if (n == 0) return true;
        return cudaMemcpy(vec.data(), src, sizeof(vec[0]) * (size_t)n, cudaMemcpyDefault) == cudaSuccess;
    };
    bool ok = fetch(m->h_xn, in->xn, d.nx) && fetch(m->h_yn, in->yn, d.ny) && fetch(m->h_zn, in->zn, d.nz) &&
              fetch(m->h_epsn, in->stack_epsn, d.nz) && fetch(m->h_sign, in->stack_sign, d.nz) &&
              fetch(m->h_mark_port, in->mark_port, in->num_cdt);
    m->num_cdt = in->num_cdt;
    m->num_ports = in->num_ports;
    if (ok && in->num_ports > 0) {
        ok = fetch(m->port_side_ptr, in->port_side_ptr, in->num_ports + 1);
        int64_t ns = ok ? m->port_side_ptr.back() : 0;
        ok = ok && ns >= in->num_ports && fetch(m->side_edge_ptr, in->side_edge_ptr, ns + 1);
        ok = ok && fetch(m->side_edges, in->side_edges, m->side_edge_ptr.back()) &&
             fetch(m->side_area, in->side_area, ns) && fetch(m->side_dir, in->side_dir, ns);
        if (ok) {
            for (int64_t e2 : m->side_edges)
                if (e2 < 0 || e2 >= d.N_edge) { set_last_message("port edge out of range"); g2p_mesh_destroy(m); return G2P_ERR_INVALID; }
            for (int p = 0; p < in->num_ports; p++)
                if (m->port_side_ptr[p + 1] <= m->port_side_ptr[p]) { set_last_message("port %d has no side", p); g2p_mesh_destroy(m); return G2P_ERR_INVALID; }
        }
    }
    if (!ok) { set_last_message("could not read the mesh description arrays"); g2p_mesh_destroy(m); return G2P_ERR_INVALID; }
    m->freq_start = in->freq_start; m->freq_end = in->freq_end; m->freq_unit = in->freq_unit;
    m->nfreq = in->nfreq; m->freq_scale = in->freq_scale;
    g2p_status st = G2P_OK;
#define CK(x) do { st = (x); if (st != G2P_OK) { g2p_mesh_destroy(m); return st; } } while (0)
    CK(dalloc(&m->xn, d.nx, s)); CK(dalloc(&m->yn, d.ny, s)); CK(dalloc(&m->zn, d.nz, s));
    CK(dalloc(&m->dxa, d.nx, s)); CK(dalloc(&m->dya, d.ny, s)); CK(dalloc(&m->dza, d.nz, s));
    CK(dalloc(&m->epsn, d.nz, s)); CK(dalloc(&m->sign, d.nz, s));
    CK(dalloc(&m->mark_node, d.N_node, s)); CK(dalloc(&m->mark_edge, d.N_edge, s));
    CK(dalloc(&m->mark_port, in->num_cdt, s)); CK(dalloc(&m->cdt_return, in->num_cdt, s));
    int64_t *tmp = nullptr;
    CK(dalloc(&tmp, d.N_edge > d.N_node ? d.N_edge : d.N_node, s));
#define CP(dst, src, n) do { cudaError_t _e = cudaMemcpyAsync(dst, src, n, cudaMemcpyDefault, s); \
        if (_e != cudaSuccess) { set_last_error(_e, "H2D copy", __FILE__, __LINE__); dfree(tmp, s); g2p_mesh_destroy(m); return G2P_ERR_CUDA; } } while (0)
    CP(m->xn, in->xn, sizeof(double) * d.nx);
    CP(m->yn, in->yn, sizeof(double) * d.ny);
    CP(m->zn, in->zn, sizeof(double) * d.nz);
    CP(m->epsn, in->stack_epsn, sizeof(double) * d.nz);
    CP(m->sign, in->stack_sign, sizeof(double) * d.nz);
    CP(m->mark_port, in->mark_port, sizeof(int32_t) * in->num_cdt);
    CP(m->cdt_return, in->cdt_return, in->num_cdt);
    CP(tmp, in->mark_node, sizeof(int64_t) * d.N_node);
    (g2p::kbegin("k_narrow", s), k_narrow<<<grid_for(d.N_node), kThreads, 0, s>>>(tmp, m->mark_node, d.N_node), g2p::kend(s));
    CP(tmp, in->mark_edge, sizeof(int64_t) * d.N_edge);
    (g2p::kbegin("k_narrow", s), k_narrow<<<grid_for(d.N_edge), kThreads, 0, s>>>(tmp, m->mark_edge, d.N_edge), g2p::kend(s));
    int *flag = nullptr;
    CK(dalloc(&flag, 1, s));
    cudaMemsetAsync(flag, 0, sizeof(int), s);
    (g2p::kbegin("k_check_marks", s), k_check_marks<<<grid_for(d.N_node), kThreads, 0, s>>>(m->mark_node, d.N_node, in->num_cdt, flag), g2p::kend(s));
    (g2p::kbegin("k_check_marks", s), k_check_marks<<<grid_for(d.N_edge), kThreads, 0, s>>>(m->mark_edge, d.N_edge, in->num_cdt, flag), g2p::kend(s));
    int hflag = 0;
    cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    dfree(flag, s);
    if (hflag) { dfree(tmp, s); g2p_mesh_destroy(m); set_last_message("mark_node/mark_edge hold ids outside [0, num_cdt]"); return G2P_ERR_INVALID; }
    (g2p::kbegin("k_dual_lengths", s), k_dual_lengths<<<1, 256, 0, s>>>(m->xn, d.Nx, m->dxa), g2p::kend(s));
    (g2p::kbegin("k_dual_lengths", s), k_dual_lengths<<<1, 256, 0, s>>>(m->yn, d.Ny, m->dya), g2p::kend(s));
    (g2p::kbegin("k_dual_lengths", s), k_dual_lengths<<<1, 256, 0, s>>>(m->zn, d.Nz, m->dza), g2p::kend(s));
    dfree(tmp, s);
#undef CP
#undef CK
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) { set_last_error(le, "mesh upload", __FILE__, __LINE__); g2p_mesh_destroy(m); return G2P_ERR_CUDA; }
    *out = m;
    return G2P_OK;
}

g2p_status g2p_v0_finish(g2p_mesh *m, bool *repatterned = nullptr);

extern "C" g2p_status g2p_mesh_destroy(g2p_mesh *m) {
    if (!m) return G2P_OK;
    if (m->ad_pending) g2p_v0_finish(m);     // joins the side stream and frees its buffers
    if (m->side) { cudaStreamSynchronize(m->side); cudaStreamDestroy(m->side); m->side = nullptr; }
    cudaStream_t s = m->stream;
    dfree(m->xn, s); dfree(m->yn, s); dfree(m->zn, s);
    dfree(m->dxa, s); dfree(m->dya, s); dfree(m->dza, s); dfree(m->v0_tab, s);
    dfree(m->epsn, s); dfree(m->sign, s);
    dfree(m->mark_node, s); dfree(m->mark_edge, s); dfree(m->mark_port, s); dfree(m->cdt_return, s);
    dfree(m->pec_edge, s); dfree(m->pec_node, s); dfree(m->map_edge, s);
    m->S.release(s);
    m->v0d.release(s); m->v0c.release(s);
    m->Ad.release(s); m->Ac.release(s);
    dfree(m->scan_work, s);
    g2p::fullwave_release(m->fw, s);
    m->fw = nullptr;
    g2p::stencil_release(m->stencil, s);
    m->stencil = nullptr;
    if (s) { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
    delete m;
    return G2P_OK;
}

extern "C" g2p_status g2p_mesh_sizes(const g2p_mesh *m, g2p_sizes *out) {
    if (!m || !out) return G2P_ERR_INVALID;
    memset(out, 0, sizeof(*out));
    out->bden = m->bden;
    out->leng_S = m->S.nnz;
    out->leng_v0d = m->v0d.ncol; out->leng_v0c = m->v0c.ncol;
    out->nnz_v0d = m->v0d.nnz; out->nnz_v0c = m->v0c.nnz;
    out->nnz_ad = m->Ad.nnz; out->nnz_ac = m->Ac.nnz;
    return G2P_OK;
}

// ---------------------------------------------------------------- index maps
namespace g2p {

// lbde = whole z = 0 plane; ubde = top-plane conductor edges of return
// conductors (after colouring markEdge holds the conductor of both ends).
__global__ void k_pec_flags(Dims d, const int32_t *__restrict__ mark_edge, const int32_t *__restrict__ mark_node,
                            const uint8_t *__restrict__ cdt_return, uint8_t *__restrict__ pec_edge,
                            uint8_t *__restrict__ pec_node) {
    int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d.N_edge; e += stride) {
        uint8_t f = 0;
        if (e < d.Ns) f = 1;
        else if (e >= d.N_edge - d.Ns) {
            int32_t c = mark_edge[e];
            f = (c != 0 && cdt_return[c - 1]) ? 1 : 0;
        }
        pec_edge[e] = f;
    }
    for (int64_t n = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; n < d.N_node; n += stride) {
        uint8_t f = 0;
        if (n < d.N_node_s) f = 1;
        else if (n >= d.N_node - d.N_node_s) {
            int32_t c = mark_node[n];
            f = (c != 0 && cdt_return[c - 1]) ? 1 : 0;
        }
        pec_node[n] = f;
    }
}

__global__ void k_finish_map(int64_t n, const uint8_t *__restrict__ pec, int32_t *__restrict__ map) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        map[e] = pec[e] ? -1 : (int32_t)(e - map[e]);
}

}  // namespace g2p

g2p_status g2p_run_index_maps(g2p_mesh *m) {
    if (m->maps_done) return G2P_OK;
    const Dims &d = m->d;
    cudaStream_t s = m->stream;
    G2P_TRY(dalloc(&m->pec_edge, d.N_edge, s));
    G2P_TRY(dalloc(&m->pec_node, d.N_node, s));
    G2P_TRY(dalloc(&m->map_edge, d.N_edge, s));
    G2P_TRY(ensure_scan_work(m, d.N_edge));
    (g2p::kbegin("k_pec_flags", s), k_pec_flags<<<grid_for(d.N_edge), kThreads, 0, s>>>(d, m->mark_edge, m->mark_node, m->cdt_return, m->pec_edge,
                                                         m->pec_node), g2p::kend(s));
    const uint8_t *pe = m->pec_edge;
    auto op = [pe] __device__(int64_t i) -> int64_t { return pe[i]; };
    G2P_TRY(exclusive_scan(op, d.N_edge, m->map_edge, m->scan_work, s));
    (g2p::kbegin("k_finish_map", s), k_finish_map<<<grid_for(d.N_edge), kThreads, 0, s>>>(d.N_edge, m->pec_edge, m->map_edge), g2p::kend(s));
    G2P_CUDA(cudaMemcpyAsync(&m->bden, m->scan_work + scan_total_index(d.N_edge), sizeof(int64_t),
                             cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    m->maps_done = true;
    return G2P_OK;
}

__global__ void k_widen_map(const int32_t *in, int64_t *out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = in[i];
}

extern "C" g2p_status g2p_index_maps(g2p_mesh *m, int64_t *bden, int64_t *map_edge) {
    if (!m) return G2P_ERR_INVALID;
    G2P_TRY(g2p_run_index_maps(m));
    if (bden) *bden = m->bden;
    if (map_edge) {
        int64_t *tmp;
        G2P_TRY(dalloc(&tmp, m->d.N_edge, m->stream));
        (g2p::kbegin("k_widen_map", m->stream), k_widen_map<<<grid_for(m->d.N_edge), kThreads, 0, m->stream>>>(m->map_edge, tmp, m->d.N_edge), g2p::kend(m->stream));
        G2P_CUDA(cudaMemcpyAsync(map_edge, tmp, sizeof(int64_t) * m->d.N_edge, cudaMemcpyDeviceToHost, m->stream));
        dfree(tmp, m->stream);
        G2P_CUDA(cudaStreamSynchronize(m->stream));
    }
    return G2P_OK;
}

// ----------------------------------------------------------------- stiffness
namespace g2p {

struct FaceEnt {
    int64_t e[4];
    double se[4], sh[4];
};

struct Geo {
    Dims d;
    const double *xn, *yn, *zn, *dxa, *dya, *dza;
    // Quotients of generateStiff's face expressions, one per grid line or
    // line pair, computed once with the same IEEE operations (so bit-equal):
    // ivx[c] = 1 / (xn[c+1] - xn[c]) (likewise y, z), and
    // qa_b[i][j] = a[i] / (a[i] * b[j]) for the dual-length pairs a, b.
    const double *ivx, *ivy, *ivz;
    const double *qz_x, *qz_y;    // [Nz][Nx+1], [Nz][Ny+1]: a = dza
    const double *qx_z, *qx_y;    // [Nx+1][Nz+1], [Nx+1][Ny+1]: a = dxa
    const double *qy_z, *qy_x;    // [Ny+1][Nz+1], [Ny+1][Nx+1]: a = dya
};

// Face numbering of generateStiff: per (z, x, y) cell below the top layer
// {xy-bottom, yz, xz}; top layer cells {xy-bottom, yz, xz, xy-top}; then the
// x = Nx yz plane; then the y = Ny xz plane (generateStiff.cpp:33-245).
__device__ __forceinline__ int64_t fid_cell(const Dims &d, int64_t cz, int64_t cx, int64_t cy, int k) {
    if (cz < d.Nz - 1) return 3 * (cz * d.Nx * d.Ny + cx * d.Ny + cy) + k;
    return 3 * (d.Nz - 1) * d.Nx * d.Ny + 4 * (cx * d.Ny + cy) + k;
}
__device__ __forceinline__ int64_t fid_xy(const Dims &d, int64_t p, int64_t cx, int64_t cy) {
    return p < d.Nz ? fid_cell(d, p, cx, cy, 0) : fid_cell(d, d.Nz - 1, cx, cy, 3);
}
__device__ __forceinline__ int64_t fid_yz(const Dims &d, int64_t i, int64_t cz, int64_t cy) {
    return i < d.Nx ? fid_cell(d, cz, i, cy, 1) : d.Nx * d.Ny * (3 * d.Nz + 1) + cz * d.Ny + cy;
}
__device__ __forceinline__ int64_t fid_xz(const Dims &d, int64_t j, int64_t cz, int64_t cx) {
    return j < d.Ny ? fid_cell(d, cz, cx, j, 2) : d.Nx * d.Ny * (3 * d.Nz + 1) + d.Nz * d.Ny + cz * d.Nx + cx;
}

// The four (edge, Se, Sh) entries of each face kind, with the reference's
// expressions (generateStiff.cpp:33-484; the top xy face keeps dza[Nz-1]).
// The reference's face expressions, e.g. se = -1 / dx and sh = -q / (dxa * q),
// read from the Geo tables: -1 / dx == -(1 / dx) and q / (dxa * q) ==
// q / (q * dxa) in IEEE arithmetic, so every value is bit-equal to the
// expression evaluated in place.
__device__ __forceinline__ void face_xy(const Geo &g, int64_t p, int64_t cx, int64_t cy, FaceEnt &f) {
    const Dims &d = g.d;
    const double ix = g.ivx[cx], iy = g.ivy[cy];
    const double *qx = g.qz_x + (p < d.Nz ? p : d.Nz - 1) * (d.Nx + 1);
    const double *qy = g.qz_y + (p < d.Nz ? p : d.Nz - 1) * (d.Ny + 1);
    f.e[0] = d.ye(p, cx, cy);     f.se[0] = -ix; f.sh[0] = -qx[cx];
    f.e[1] = d.ye(p, cx + 1, cy); f.se[1] = ix;  f.sh[1] = qx[cx + 1];
    f.e[2] = d.xe(p, cx, cy);     f.se[2] = iy;  f.sh[2] = qy[cy];
    f.e[3] = d.xe(p, cx, cy + 1); f.se[3] = -iy; f.sh[3] = -qy[cy + 1];
}
__device__ __forceinline__ void face_yz(const Geo &g, int64_t i, int64_t cz, int64_t cy, FaceEnt &f) {
    const Dims &d = g.d;
    const double iy = g.ivy[cy], iz = g.ivz[cz];
    const double *qz = g.qx_z + i * (d.Nz + 1), *qy = g.qx_y + i * (d.Ny + 1);
    f.e[0] = d.ye(cz, i, cy);     f.se[0] = iz;  f.sh[0] = qz[cz];
    f.e[1] = d.ze(cz, i, cy);     f.se[1] = -iy; f.sh[1] = -qy[cy];
    f.e[2] = d.ze(cz, i, cy + 1); f.se[2] = iy;  f.sh[2] = qy[cy + 1];
    f.e[3] = d.ye(cz + 1, i, cy); f.se[3] = -iz; f.sh[3] = -qz[cz + 1];
}
__device__ __forceinline__ void face_xz(const Geo &g, int64_t j, int64_t cz, int64_t cx, FaceEnt &f) {
    const Dims &d = g.d;
    const double ix = g.ivx[cx], iz = g.ivz[cz];
    const double *qz = g.qy_z + j * (d.Nz + 1), *qx = g.qy_x + j * (d.Nx + 1);
    f.e[0] = d.xe(cz, cx, j);     f.se[0] = -iz; f.sh[0] = -qz[cz];
    f.e[1] = d.ze(cz, cx, j);     f.se[1] = ix;  f.sh[1] = qx[cx];
    f.e[2] = d.ze(cz, cx + 1, j); f.se[2] = -ix; f.sh[2] = -qx[cx + 1];
    f.e[3] = d.xe(cz + 1, cx, j); f.se[3] = iz;  f.sh[3] = qz[cz + 1];
}

// Edges of a face (no values), for the row-length pass.
__device__ __forceinline__ void face_edges(const Dims &d, int kind, int64_t a, int64_t b, int64_t c, int64_t *e) {
    if (kind == 0) { e[0] = d.ye(a, b, c); e[1] = d.ye(a, b + 1, c); e[2] = d.xe(a, b, c); e[3] = d.xe(a, b, c + 1); }
    else if (kind == 1) { e[0] = d.ye(b, a, c); e[1] = d.ze(b, a, c); e[2] = d.ze(b, a, c + 1); e[3] = d.ye(b + 1, a, c); }
    else { e[0] = d.xe(b, c, a); e[1] = d.ze(b, c, a); e[2] = d.ze(b, c + 1, a); e[3] = d.xe(b + 1, c, a); }
}

__global__ void k_inv_len(const double *xn, int64_t n, double *inv) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double h = xn[i + 1] - xn[i];
        inv[i] = 1 / h;
    }
}

// q[i][j] = a[i] / (a[i] * b[j])
__global__ void k_quot(const double *a, int64_t na, const double *b, int64_t nb, double *q) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < na * nb; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / nb, j = t - i * nb;
        const double ai = a[i];
        q[t] = ai / (ai * b[j]);
    }
}

// Faces containing edge e: kind (0 xy, 1 yz, 2 xz) and (a, b, c) arguments.
struct FaceRef {
    int64_t id;
    int kind;
    int64_t a, b, c;
};

__device__ __forceinline__ void face_cx(FaceRef &a, FaceRef &b) {
    if (b.id < a.id) { const FaceRef t = a; a = b; b = t; }
}

// The candidate faces sit in fixed slots (absent ones keyed last) and a
// five-step compare-exchange network orders them, so fr stays in registers.
__device__ __forceinline__ int edge_faces(const Dims &d, int64_t e, FaceRef *fr) {
    constexpr int64_t kNone = INT64_MAX;
    int64_t n1, n2, z, x, y;
    int kind = d.edge_nodes(e, n1, n2, z, x, y);
    if (kind == 0) {  // y-edge: plane z, node x, cell y
        fr[0] = {x >= 1 ? fid_xy(d, z, x - 1, y) : kNone, 0, z, x - 1, y};
        fr[1] = {x < d.Nx ? fid_xy(d, z, x, y) : kNone, 0, z, x, y};
        fr[2] = {z >= 1 ? fid_yz(d, x, z - 1, y) : kNone, 1, x, z - 1, y};
        fr[3] = {z < d.Nz ? fid_yz(d, x, z, y) : kNone, 1, x, z, y};
    } else if (kind == 1) {  // x-edge: plane z, cell x, node y
        fr[0] = {y >= 1 ? fid_xy(d, z, x, y - 1) : kNone, 0, z, x, y - 1};
        fr[1] = {y < d.Ny ? fid_xy(d, z, x, y) : kNone, 0, z, x, y};
        fr[2] = {z >= 1 ? fid_xz(d, y, z - 1, x) : kNone, 2, y, z - 1, x};
        fr[3] = {z < d.Nz ? fid_xz(d, y, z, x) : kNone, 2, y, z, x};
    } else {  // z-edge: layer z, node (x, y)
        fr[0] = {y >= 1 ? fid_yz(d, x, z, y - 1) : kNone, 1, x, z, y - 1};
        fr[1] = {y < d.Ny ? fid_yz(d, x, z, y) : kNone, 1, x, z, y};
        fr[2] = {x >= 1 ? fid_xz(d, y, z, x - 1) : kNone, 2, y, z, x - 1};
        fr[3] = {x < d.Nx ? fid_xz(d, y, z, x) : kNone, 2, y, z, x};
    }
    // increasing face number
    face_cx(fr[0], fr[1]);
    face_cx(fr[2], fr[3]);
    face_cx(fr[0], fr[2]);
    face_cx(fr[1], fr[3]);
    face_cx(fr[1], fr[2]);
    return (fr[0].id != kNone) + (fr[1].id != kNone) + (fr[2].id != kNone) + (fr[3].id != kNone);
}

__global__ void __launch_bounds__(256) k_stiff_count(Geo g, const uint8_t *__restrict__ pec, const int32_t *__restrict__ map,
                                                     int64_t *__restrict__ rowlen) {
    const Dims &d = g.d;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d.N_edge; e += (int64_t)gridDim.x * blockDim.x) {
        if (pec[e]) continue;
        // the structural row: e and the other edges of its faces (two faces
        // of the grid share at most one edge, so none repeats)
        FaceRef fr[4];
        const int nf = edge_faces(d, e, fr);
        int cnt = 1;
        for (int t = 0; t < nf; t++) {
            int64_t fe[4];
            face_edges(d, fr[t].kind, fr[t].a, fr[t].b, fr[t].c, fe);
#pragma unroll
            for (int k = 0; k < 4; k++) cnt += (fe[k] != e && !pec[fe[k]]) ? 1 : 0;
        }
        rowlen[map[e]] = cnt;
    }
}

// v / d rounded to nearest, from y = RN(1 / d) with one product and two
// FMAs instead of a division (FP64 division is an iterative sequence on the
// FP64 pipe, the limit of this kernel).  Markstein's theorem (P. Markstein,
// IBM J. Res. Dev. 34(1), 1990; Muller et al., Handbook of Floating-Point
// Arithmetic, "division with a correction step"): q = RN(v y) is within one
// ulp of v / d, r = v - q d is exact by FMA, and RN(q + r y) = RN(v / d),
// barring underflow and overflow.  Operands outside [2^-900, 2^900] take the
// division; zero keeps its sign.  The range test reads the exponent bits
// (integer pipe), leaving three FP64 operations.
__device__ __forceinline__ double div_rn(double v, double d, double y) {
    const int ex = (int)((__double_as_longlong(v) >> 52) & 0x7ff);   // biased exponent
    if (ex < 1023 - 900 || ex > 1023 + 899) return v / d;
    const double q = v * y;
    const double r = fma(-q, d, v);
    return fma(r, y, q);
}

// The row of edge e in registers.  Slot 0 is the diagonal; slot 1 + 4t + k
// is the k-th edge of e's t-th face (faces in increasing number).  e's own
// slot in each face, the slots of absent faces and PEC columns are empty.
// Two faces of the grid share at most one edge, e, so every other column has
// exactly one slot.  As in the reference's row (Sh Se^T accumulated per
// face, then sorted by column), the diagonal sums its per-face products from
// 0.0 in face order and every other entry is 0.0 plus its one product.  Each
// entry is written at its rank among the row's columns, so nothing is sorted
// in memory and the row never leaves registers.
__global__ void __launch_bounds__(256) k_stiff_fill(Geo g, const uint8_t *__restrict__ pec, const int32_t *__restrict__ map,
                                                    const int64_t *__restrict__ rowptr, int32_t *__restrict__ col,
                                                    double *__restrict__ val, double mu, double inv_mu) {
    const Dims &d = g.d;
    constexpr int64_t kNone = INT64_MAX;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d.N_edge; e += (int64_t)gridDim.x * blockDim.x) {
        if (pec[e]) continue;
        FaceRef fr[4];
        const int nf = edge_faces(d, e, fr);
        int64_t c[17];
        double v[17];
        double diag = 0.0;
#pragma unroll
        for (int t = 0; t < 4; t++) {
            FaceEnt f = {};
            if (t < nf) {
                if (fr[t].kind == 0) face_xy(g, fr[t].a, fr[t].b, fr[t].c, f);
                else if (fr[t].kind == 1) face_yz(g, fr[t].a, fr[t].b, fr[t].c, f);
                else face_xz(g, fr[t].a, fr[t].b, fr[t].c, f);
            }
            double sh = 0.0;
#pragma unroll
            for (int k = 0; k < 4; k++) if (t < nf && f.e[k] == e) sh = f.sh[k];
#pragma unroll
            for (int k = 0; k < 4; k++) {
                const bool self = t < nf && f.e[k] == e;
                if (self) diag += sh * f.se[k];
                const bool keep = t < nf && !self && !pec[f.e[k]];
                c[1 + 4 * t + k] = keep ? f.e[k] : kNone;
                // 0.0 + p: p itself except that -0.0 becomes +0.0 (a bit test,
                // not an FP64 add)
                const double p = sh * f.se[k];
                v[1 + 4 * t + k] = keep && __double_as_longlong(p) != (long long)0x8000000000000000ULL ? p : 0.0;
            }
        }
        c[0] = e;
        v[0] = diag;
        const int64_t o = rowptr[map[e]];
#pragma unroll
        for (int i = 0; i < 17; i++) {
            if (c[i] == kNone) continue;
            int r = 0;
#pragma unroll
            for (int j = 0; j < 17; j++) r += c[j] < c[i] ? 1 : 0;
            col[o + r] = map[c[i]];
            val[o + r] = div_rn(v[i], mu, inv_mu);
        }
    }
}

__global__ void k_csr_rows_i64(const int64_t *ptr, int64_t n, int64_t *rows) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        for (int64_t k = ptr[i]; k < ptr[i + 1]; k++) rows[k] = i;
}

__global__ void k_i32_to_i64(const int32_t *in, int64_t *out, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        out[i] = in[i];
}

}  // namespace g2p

g2p_status g2p_build_rowptr(g2p_mesh *m, int64_t *rowlen, int64_t n, int64_t **ptr_out, int64_t *nnz_out) {
    // ptr = exclusive scan of rowlen with ptr[n] = total
    cudaStream_t s = m->stream;
    G2P_TRY(ensure_scan_work(m, n + 1));
    int64_t *ptr;
    G2P_TRY(dalloc(&ptr, n + 1, s));
    const int64_t *rl = rowlen;
    auto op = [rl, n] __device__(int64_t i) -> int64_t { return i < n ? rl[i] : 0; };
    G2P_TRY(exclusive_scan(op, n + 1, ptr, m->scan_work, s));
    G2P_CUDA(cudaMemcpyAsync(nnz_out, ptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    *ptr_out = ptr;
    return G2P_OK;
}

g2p_status g2p_run_stiff(g2p_mesh *m) {
    if (m->stiff_done) return G2P_OK;
    G2P_TRY(g2p_run_index_maps(m));
    const Dims &d = m->d;
    cudaStream_t s = m->stream;
    // per-line quotient tables (see Geo)
    const int64_t NX = d.Nx + 1, NY = d.Ny + 1, NZ = d.Nz + 1;
    double *tab;
    const int64_t ntab = d.Nx + d.Ny + d.Nz + d.Nz * NX + d.Nz * NY + NX * NZ + NX * NY + NY * NZ + NY * NX;
    G2P_TRY(dalloc(&tab, ntab, s));
    Geo g{d, m->xn, m->yn, m->zn, m->dxa, m->dya, m->dza};
    double *t = tab;
    g.ivx = t; (g2p::kbegin("k_inv_len", s), k_inv_len<<<grid_for(d.Nx), kThreads, 0, s>>>(m->xn, d.Nx, t), g2p::kend(s)); t += d.Nx;
    g.ivy = t; (g2p::kbegin("k_inv_len", s), k_inv_len<<<grid_for(d.Ny), kThreads, 0, s>>>(m->yn, d.Ny, t), g2p::kend(s)); t += d.Ny;
    g.ivz = t; (g2p::kbegin("k_inv_len", s), k_inv_len<<<grid_for(d.Nz), kThreads, 0, s>>>(m->zn, d.Nz, t), g2p::kend(s)); t += d.Nz;
    struct QT { const double **dst; const double *a; int64_t na; const double *b; int64_t nb; };
    const QT qts[6] = {{&g.qz_x, m->dza, d.Nz, m->dxa, NX}, {&g.qz_y, m->dza, d.Nz, m->dya, NY},
                       {&g.qx_z, m->dxa, NX, m->dza, NZ}, {&g.qx_y, m->dxa, NX, m->dya, NY},
                       {&g.qy_z, m->dya, NY, m->dza, NZ}, {&g.qy_x, m->dya, NY, m->dxa, NX}};
    for (const QT &q : qts) {
        *q.dst = t;
        (g2p::kbegin("k_quot", s), k_quot<<<grid_for(q.na * q.nb), kThreads, 0, s>>>(q.a, q.na, q.b, q.nb, t), g2p::kend(s));
        t += q.na * q.nb;
    }
    int64_t n = d.N_edge - m->bden;
    int64_t *rowlen;
    G2P_TRY(dalloc(&rowlen, n, s));
    (g2p::kbegin("k_stiff_count", s), k_stiff_count<<<grid_for(d.N_edge, 256, 152LL * 32), 256, 0, s>>>(g, m->pec_edge, m->map_edge, rowlen), g2p::kend(s));
    int64_t nnz = 0;
    g2p_status st = g2p_build_rowptr(m, rowlen, n, &m->S.ptr, &nnz);
    dfree(rowlen, s);
    if (st != G2P_OK) { dfree(tab, s); return st; }
    m->S.n = m->S.m = n;
    m->S.nnz = nnz;
    G2P_TRY(dalloc(&m->S.col, nnz, s));
    G2P_TRY(dalloc(&m->S.val, nnz, s));
    (g2p::kbegin("k_stiff_fill", s), k_stiff_fill<<<grid_for(d.N_edge, 256, 152LL * 32), 256, 0, s>>>(g, m->pec_edge, m->map_edge, m->S.ptr, m->S.col,
                                                                     m->S.val, m->k.mu, 1.0 / m->k.mu), g2p::kend(s));
    dfree(tab, s);
    G2P_CUDA(cudaGetLastError());
    G2P_CUDA(cudaStreamSynchronize(s));
    m->stiff_done = true;
    return G2P_OK;
}

extern "C" g2p_status g2p_generate_stiff(g2p_mesh *m, int64_t *leng_S) {
    if (!m) return G2P_ERR_INVALID;
    G2P_TRY(g2p_run_stiff(m));
    if (leng_S) *leng_S = m->S.nnz;
    return G2P_OK;
}

// COO export of a device CSR (rows, int64 cols, values) to host buffers.
g2p_status g2p_export_csr(g2p_mesh *m, const Csr<double> &A, int64_t *row, int64_t *col, double *val) {
    cudaStream_t s = m->stream;
    int64_t *tmp;
    G2P_TRY(dalloc(&tmp, A.nnz, s));
    if (row) {
        (g2p::kbegin("k_csr_rows_i64", s), k_csr_rows_i64<<<grid_for(A.n), kThreads, 0, s>>>(A.ptr, A.n, tmp), g2p::kend(s));
        G2P_CUDA(cudaMemcpyAsync(row, tmp, sizeof(int64_t) * A.nnz, cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaStreamSynchronize(s));
    }
    if (col) {
        (g2p::kbegin("k_i32_to_i64", s), k_i32_to_i64<<<grid_for(A.nnz), kThreads, 0, s>>>(A.col, tmp, A.nnz), g2p::kend(s));
        G2P_CUDA(cudaMemcpyAsync(col, tmp, sizeof(int64_t) * A.nnz, cudaMemcpyDeviceToHost, s));
        G2P_CUDA(cudaStreamSynchronize(s));
    }
    if (val) G2P_CUDA(cudaMemcpyAsync(val, A.val, sizeof(double) * A.nnz, cudaMemcpyDeviceToHost, s));
    dfree(tmp, s);
    G2P_CUDA(cudaStreamSynchronize(s));
    return G2P_OK;
}

extern "C" g2p_status g2p_export_stiff(g2p_mesh *m, int64_t *row, int64_t *col, double *val) {
    if (!m) return G2P_ERR_INVALID;
    if (!m->stiff_done) { set_last_message("g2p_generate_stiff has not run"); return G2P_ERR_STATE; }
    return g2p_export_csr(m, m->S, row, col, val);
}
