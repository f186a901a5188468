// setMapEdge (src/fdtd.hpp:1444-1529, with LOWER_BOUNDARY_PEC and the
// return conductors' top-plane edges of findBoundNodeEdge, src/mesh.cpp:943-987)
// as a device-pointer entry point that allocates nothing.
//
// Its only temporary, the per-tile partial sums of the edge scan, lives in a
// file-scope device array of fixed size.  The allocating entry point
// (g2p_index_maps) gets the same numbers through a mesh handle and the
// stream-ordered pool; this one is for callers that hand the library memory
// they already own and cannot let it take more: a host runtime whose own
// arena or caching allocator holds the device's memory, where a pool
// allocation by the library either fails or escapes its accounting, and a
// per-layout loop on a fixed latency budget, where growing a pool can block
// in the driver.
#include <mutex>

#include "common.cuh"
#include "primitives.cuh"

namespace g2p {
namespace {

// One partial per 2,048-edge scan tile, plus the total: 256 KiB.
constexpr int64_t kNoAllocPartials = 32768;
constexpr int64_t kNoAllocMaxEdges = (kNoAllocPartials - 1) * kScanTile;   // 67,106,816 edges

// No word of it has to start at zero: every call writes each partial it
// later reads (k_scan_reduce, then the in-place scan and the total) before
// reading it.
static __device__ __align__(256) int64_t g_noalloc_partials[kNoAllocPartials];

constexpr int kMaxDevices = 64;
std::mutex g_addr_mu;
int64_t *g_addr[kMaxDevices];

// Address of the buffer on the current device, looked up on the first call
// made with that device current and kept for the life of the process.  The
// cache does not survive cudaDeviceReset (which unloads the module): a
// process that resets a device must not call this entry point afterwards.
g2p_status partials_on_current_device(int64_t **out) {
    int dev = -1;
    G2P_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) {
        set_last_message("device ordinal %d outside the %d devices g2p_map_edge_noalloc tracks", dev, kMaxDevices);
        return G2P_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lock(g_addr_mu);
    if (!g_addr[dev]) {
        void *p = nullptr;
        G2P_CUDA(cudaGetSymbolAddress(&p, g_noalloc_partials));
        if (!p) {
            set_last_message("cudaGetSymbolAddress returned a null address for the scan partials");
            return G2P_ERR_CUDA;
        }
        g_addr[dev] = static_cast<int64_t *>(p);
    }
    *out = g_addr[dev];
    return G2P_OK;
}

// The kernels read the caller's arrays directly: device, managed or mapped
// pinned host memory.
bool device_accessible(const void *p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged ||
           (a.type == cudaMemoryTypeHost && a.devicePointer == p);
}

// PEC flag of edge e: the whole z = 0 plane, and top-plane edges whose
// conductor is a return conductor.  Ids outside 1..num_cdt count as
// dielectric here; g2p_mesh_create rejects them.
struct PecEdge {
    Dims d;
    const int64_t *mark_edge;
    const uint8_t *cdt_return;
    int64_t num_cdt;
    __device__ int64_t operator()(int64_t e) const {
        if (e < d.Ns) return 1;
        if (e >= d.N_edge - d.Ns) {
            int64_t c = mark_edge[e];
            return (c >= 1 && c <= num_cdt && cdt_return[c - 1]) ? 1 : 0;
        }
        return 0;
    }
};

// map[e] holds the PEC edges before e on entry; leaves the edge's index
// among non-PEC edges (or -1), and the PEC total in *bden.
__global__ void k_noalloc_finish(PecEdge pec, const int64_t *partials, int64_t total_at, int64_t *map,
                                 int64_t *bden) {
    const int64_t n = pec.d.N_edge;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        map[e] = pec(e) ? -1 : e - map[e];
    if (blockIdx.x == 0 && threadIdx.x == 0) *bden = partials[total_at];
}

}  // namespace
}  // namespace g2p

using namespace g2p;

extern "C" g2p_status g2p_map_edge_noalloc(int64_t nx, int64_t ny, int64_t nz, const int64_t *mark_edge,
                                           const uint8_t *cdt_return, int64_t num_cdt, int64_t *map_edge,
                                           int64_t *bden, void *stream) {
    if (nx < 3 || ny < 3 || nz < 3) {
        set_last_message("grid must have at least 3 nodes per axis");
        return G2P_ERR_INVALID;
    }
    if (nx > (int64_t)1 << 20 || ny > (int64_t)1 << 20 || nz > (int64_t)1 << 20) {
        set_last_message("g2p_map_edge_noalloc: grid %lld x %lld x %lld has more than 2^20 (1,048,576) nodes "
                         "along an axis",
                         (long long)nx, (long long)ny, (long long)nz);
        return G2P_ERR_INVALID;
    }
    Dims d;
    d.init(nx, ny, nz);
    if (d.N_edge > kNoAllocMaxEdges) {
        set_last_message("g2p_map_edge_noalloc: %lld edges exceed its static scratch limit of %lld edges "
                         "(%lld scan tiles of %d); use g2p_index_maps",
                         (long long)d.N_edge, (long long)kNoAllocMaxEdges, (long long)(kNoAllocPartials - 1),
                         kScanTile);
        return G2P_ERR_INVALID;
    }
    if (num_cdt < 0 || !mark_edge || !map_edge || !bden || (num_cdt > 0 && !cdt_return)) {
        set_last_message("g2p_map_edge_noalloc: null array or negative num_cdt");
        return G2P_ERR_INVALID;
    }
    if (!device_accessible(mark_edge) || !device_accessible(map_edge) || !device_accessible(bden) ||
        (num_cdt > 0 && !device_accessible(cdt_return))) {
        set_last_message("g2p_map_edge_noalloc: every array must be device, managed or mapped host memory");
        return G2P_ERR_INVALID;
    }
    int64_t *partials = nullptr;
    G2P_TRY(partials_on_current_device(&partials));

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    PecEdge pec{d, mark_edge, cdt_return, num_cdt};
    const int64_t n = d.N_edge;
    const int64_t nb = (n + kScanTile - 1) / kScanTile;
    launch_tick();
    k_scan_reduce<PecEdge><<<(unsigned)nb, kScanThreads, 0, s>>>(pec, n, partials);
    launch_tick();
    k_scan_partials<<<1, 1024, 0, s>>>(partials, nb);
    launch_tick();
    k_scan_down<PecEdge, int64_t><<<(unsigned)nb, kScanThreads, 0, s>>>(pec, n, partials, map_edge);
    launch_tick();
    k_noalloc_finish<<<grid_for(n), kThreads, 0, s>>>(pec, partials, nb, map_edge, bden);
    G2P_CUDA(cudaGetLastError());
    return G2P_OK;
}
