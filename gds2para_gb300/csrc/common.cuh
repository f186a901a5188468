// Shared device/host definitions for the GB300 extraction path.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cuda_runtime.h>

#include "../../include/gds2para_gb300.h"

namespace g2p {

// Status propagation: every CUDA call inside the library goes through this.
#define G2P_CUDA(call)                                                          \
    do {                                                                        \
        cudaError_t _e = (call);                                                \
        if (_e != cudaSuccess) {                                                \
            g2p::set_last_error(_e, #call, __FILE__, __LINE__);                 \
            return G2P_ERR_CUDA;                                                \
        }                                                                       \
    } while (0)

#define G2P_TRY(expr)                                                           \
    do {                                                                        \
        g2p_status _s = (expr);                                                 \
        if (_s != G2P_OK) return _s;                                            \
    } while (0)

void set_last_error(cudaError_t e, const char *what, const char *file, int line);
void set_last_message(const char *fmt, ...);
void retain_pool_memory(int device);

// Counts kernel launches issued by the library and, while profiling is on,
// brackets each launch with CUDA events keyed by the kernel's name.
void launch_tick();
void launch_add(int64_t n);
int64_t launch_count();
void kbegin(const char *name, cudaStream_t s);
void kend(cudaStream_t s);
// Called right after kbegin's own event and right before kend's (when set):
// an inner bracket around exactly one launch, for the sparse-product timing.
extern void (*kbracket_begin)(cudaStream_t);
extern void (*kbracket_end)(cudaStream_t);
bool kprof_on();
void kprof_set(bool on);
g2p_status kprof_collect();
void kprof_add_total(const char *name, int64_t launches, double ms);

constexpr int kSMs = 152;            // GB300: 2 dies x 76 SMs
constexpr int kThreads = 256;

inline unsigned grid_for(int64_t n, int threads = kThreads, int64_t cap = 152LL * 64) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (unsigned)b;
}

// Structured-grid dimensions and the reference's edge/node numbering
// (mesh.cpp:393-402, fdtd.hpp:4107-4130).
struct Dims {
    int64_t nx, ny, nz, Nx, Ny, Nz;
    int64_t Ns, Nv, L, N_edge, N_node_s, N_node, XO;
    __host__ __device__ void init(int64_t nx_, int64_t ny_, int64_t nz_) {
        nx = nx_; ny = ny_; nz = nz_;
        Nx = nx - 1; Ny = ny - 1; Nz = nz - 1;
        Ns = Ny * (Nx + 1) + Nx * (Ny + 1);
        Nv = (Nx + 1) * (Ny + 1);
        L = Ns + Nv;
        N_edge = Ns * (Nz + 1) + Nv * Nz;
        N_node_s = Nv;
        N_node = (Nz + 1) * N_node_s;
        XO = Ny * (Nx + 1);
    }
    // edge -> (kind 0 y / 1 x / 2 z, layer, ix, iy) and its two nodes
    __host__ __device__ inline int edge_nodes(int64_t e, int64_t &n1, int64_t &n2, int64_t &inz, int64_t &inx,
                                              int64_t &iny) const {
        inz = e / L;
        int64_t r = e - inz * L;
        if (r >= Ns) {
            r -= Ns;
            inx = r / (Ny + 1); iny = r - inx * (Ny + 1);
            n1 = inz * N_node_s + (Ny + 1) * inx + iny;
            n2 = n1 + N_node_s;
            return 2;
        } else if (r >= XO) {
            r -= XO;
            inx = r / (Ny + 1); iny = r - inx * (Ny + 1);
            n1 = inz * N_node_s + inx * (Ny + 1) + iny;
            n2 = n1 + (Ny + 1);
            return 1;
        } else {
            inx = r / Ny; iny = r - inx * Ny;
            n1 = inz * N_node_s + inx * (Ny + 1) + iny;
            n2 = n1 + 1;
            return 0;
        }
    }
    __host__ __device__ inline int64_t ye(int64_t z, int64_t x, int64_t y) const { return z * L + x * Ny + y; }
    __host__ __device__ inline int64_t xe(int64_t z, int64_t x, int64_t y) const { return z * L + XO + x * (Ny + 1) + y; }
    __host__ __device__ inline int64_t ze(int64_t z, int64_t x, int64_t y) const { return z * L + Ns + x * (Ny + 1) + y; }
};

// fdtd.hpp:45-47, evaluated with the same operation order.
#define G2P_MU (4 * 3.14159265358979323846 * 1.e-7)
#define G2P_CSPED (299792458.)
#define G2P_EPSILON0 (1. / (G2P_CSPED * G2P_CSPED * G2P_MU))

// Device allocation through the stream-ordered pool.
template <class T>
g2p_status dalloc(T **p, int64_t n, cudaStream_t s) {
    size_t bytes = sizeof(T) * (size_t)(n > 0 ? n : 1);
    cudaError_t e = cudaMallocAsync((void **)p, bytes, s);
    if (e != cudaSuccess) {
        set_last_error(e, "cudaMallocAsync", __FILE__, __LINE__);
        return e == cudaErrorMemoryAllocation ? G2P_ERR_NOMEM : G2P_ERR_CUDA;
    }
    return G2P_OK;
}
template <class T>
void dfree(T *&p, cudaStream_t s) {
    if (p) cudaFreeAsync((void *)p, s);
    p = nullptr;
}

}  // namespace g2p
