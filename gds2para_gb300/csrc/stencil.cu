// The curl-curl operator S = Sh Se^T / mu (generateStiff.cpp:6-565) applied
// matrix-free as a structured-grid stencil, in two TMA-tiled passes over
// full-grid edge arrays:
//
//   1. face circulations c_f = sum over the face's four edges of se(f, e) v_e
//      for every xy, yz and xz face (the Se^T v product);
//   2. (S v)_e = sum over the faces containing e of sh(f, e) c_f / mu (the
//      Sh product), written straight to e's index after PEC removal.
//
// se and sh are generateStiff's per-face coefficients (1 / edge length and
// dual-length quotients, the same tables the assembled S is built from), so
// S v equals the assembled product to rounding.  Each face is computed once,
// so a product costs about eight FP64 multiply-adds per edge against about
// thirteen (one per stored entry) for the assembled CSR, and reads and
// writes each edge value once instead of streaming S's 12 bytes per entry.
//
// Layout: each of the y-, x- and z-edge families, and each of the xy-, yz-
// and xz-face families, is a [nz][nx][Yp] FP64 array (Yp = ny rounded up to
// even, so every row starts on a 16-byte boundary), zero where the grid has
// no such edge or face and on PEC edges.  A CTA takes a tile of TY x TX x TZ
// positions; thread 0 loads the three input boxes of the tile (with a
// one-line halo above for pass 1, below for pass 2) by cp.async.bulk.tensor
// into shared memory, completing on one mbarrier; boxes that run off the
// grid read zeros.  The innermost box coordinate is always even (FP64 rows of
// 16 bytes), box widths are multiples of 16 bytes and each box starts on a
// 128-byte boundary of shared memory; the kernel checks these before it
// issues a copy.  The wait on the
// mbarrier is bounded: a CTA that gives up sets an error flag and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "internal.h"
#include "primitives.cuh"

namespace g2p {

namespace {

constexpr int kTY = 32, kTX = 8, kTZ = 4;             // output tile
constexpr int kBY = kTY + 2, kBX = kTX + 1, kBZ = kTZ + 1;   // input box
constexpr int kBox = kBY * kBX * kBZ;                 // doubles per box
// boxes start 128 bytes apart in shared memory (a bulk tensor copy's
// shared-memory destination must be 128-byte aligned)
constexpr int kBoxPad = (kBox * 8 + 127) / 128 * 128 / 8;
constexpr int kStencilThreads = 256;
constexpr long long kTmaSpin = 1LL << 24;

struct Tables {
    const double *ivx, *ivy, *ivz;            // 1 / cell length
    const double *qz_x, *qz_y;                // [Nz][Nx+1], [Nz][Ny+1]
    const double *qx_z, *qx_y;                // [Nx+1][Nz+1], [Nx+1][Ny+1]
    const double *qy_z, *qy_x;                // [Ny+1][Nz+1], [Ny+1][Nx+1]
};

__global__ void k_st_inv_len(const double *c, int64_t n, double *inv) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        inv[i] = 1 / (c[i + 1] - c[i]);
}

__global__ void k_st_quot(const double *a, int64_t na, const double *b, int64_t nb, double *q) {
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < na * nb; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = t / nb, j = t - i * nb;
        q[t] = a[i] / (a[i] * b[j]);
    }
}

// full-grid position of edge e: family (0 y, 1 x, 2 z) and offset in its
// [nz][nx][Yp] array
__device__ __forceinline__ void edge_slot(const Dims &d, int64_t Yp, int64_t e, int &fam, int64_t &off) {
    int64_t n1, n2, z, x, y;
    fam = d.edge_nodes(e, n1, n2, z, x, y);
    off = (z * d.nx + x) * Yp + y;
}

// v (reduced numbering, non-PEC edges) into the full-grid arrays
__global__ void k_st_scatter(Dims d, int64_t Yp, int64_t nr, const int32_t *map_r, const double *v, double *ey,
                             double *ex, double *ez) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        int fam;
        int64_t off;
        edge_slot(d, Yp, map_r[r], fam, off);
        (fam == 0 ? ey : fam == 1 ? ex : ez)[off] = v[r];
    }
}

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Loads three boxes at (y, x, z) into s[0..3) and waits for them (bounded).
__device__ __forceinline__ bool load_boxes(const CUtensorMap *m0, const CUtensorMap *m1, const CUtensorMap *m2,
                                           double *s, uint64_t *bar, int y, int x, int z, int *err) {
    const uint32_t b = smem_u32(bar);
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(b));
        asm volatile("fence.mbarrier_init.release.cluster;" ::);
        asm volatile("fence.proxy.async.shared::cta;" ::);
    }
    __syncthreads();
    // the copies' alignment rules, checked before any copy is issued:
    // 128-byte shared destinations, an even innermost coordinate (16 bytes
    // of FP64), 64-byte aligned tensor maps
    const bool aligned = (smem_u32(s) & 127) == 0 && (y & 1) == 0 && ((uintptr_t)m0 & 63) == 0 &&
                         ((uintptr_t)m1 & 63) == 0 && ((uintptr_t)m2 & 63) == 0;
    if (!aligned) {
        if (threadIdx.x == 0) atomicExch(err, 2);
        return false;
    }
    if (threadIdx.x == 0) {
        const uint32_t bytes = 3u * kBox * (uint32_t)sizeof(double);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
        const CUtensorMap *maps[3] = {m0, m1, m2};
#pragma unroll
        for (int q = 0; q < 3; q++)
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                ::"r"(smem_u32(s + q * kBoxPad)), "l"(maps[q]), "r"(y), "r"(x), "r"(z), "r"(b)
                : "memory");
    }
    uint32_t done = 0;
    for (long long it = 0; it < kTmaSpin && !done; it++)
        asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}"
                     : "=r"(done) : "r"(b) : "memory");
    if (!done) { atomicExch(err, 1); return false; }
    return true;
}

// s[q][(z * kBX + x) * kBY + y], box-local coordinates
__device__ __forceinline__ double at(const double *s, int q, int z, int x, int y) {
    return s[q * kBoxPad + (z * kBX + x) * kBY + y];
}

// pass 1: circulations of the faces at the tile's positions; box origin at
// the tile origin, halo one line above in y, x and z
__global__ void __launch_bounds__(kStencilThreads) k_st_faces(const __grid_constant__ CUtensorMap tm_y,
                                                              const __grid_constant__ CUtensorMap tm_x,
                                                              const __grid_constant__ CUtensorMap tm_z, Dims d,
                                                              int64_t Yp, Tables t, double *fxy, double *fyz,
                                                              double *fxz, int *err) {
    __shared__ alignas(128) double s[3 * kBoxPad];
    __shared__ alignas(8) uint64_t bar;
    const int y0 = blockIdx.x * kTY, x0 = blockIdx.y * kTX, z0 = blockIdx.z * kTZ;
    if (!load_boxes(&tm_y, &tm_x, &tm_z, s, &bar, y0, x0, z0, err)) return;
    for (int q = threadIdx.x; q < kTY * kTX * kTZ; q += blockDim.x) {
        const int ly = q % kTY, lx = (q / kTY) % kTX, lz = q / (kTY * kTX);
        const int64_t y = y0 + ly, x = x0 + lx, z = z0 + lz;
        if (y >= Yp || x >= d.nx || z >= d.nz) continue;
        const int64_t off = (z * d.nx + x) * Yp + y;
        double cxy = 0, cyz = 0, cxz = 0;
        if (x < d.Nx && y < d.Ny) {
            const double ix = t.ivx[x], iy = t.ivy[y];
            cxy = -ix * at(s, 0, lz, lx, ly) + ix * at(s, 0, lz, lx + 1, ly) + iy * at(s, 1, lz, lx, ly) -
                  iy * at(s, 1, lz, lx, ly + 1);
        }
        if (z < d.Nz && y < d.Ny) {
            const double iz = t.ivz[z], iy = t.ivy[y];
            cyz = iz * at(s, 0, lz, lx, ly) - iy * at(s, 2, lz, lx, ly) + iy * at(s, 2, lz, lx, ly + 1) -
                  iz * at(s, 0, lz + 1, lx, ly);
        }
        if (z < d.Nz && x < d.Nx) {
            const double iz = t.ivz[z], ix = t.ivx[x];
            cxz = -iz * at(s, 1, lz, lx, ly) + ix * at(s, 2, lz, lx, ly) - ix * at(s, 2, lz, lx + 1, ly) +
                  iz * at(s, 1, lz + 1, lx, ly);
        }
        fxy[off] = cxy;
        fyz[off] = cyz;
        fxz[off] = cxz;
    }
}

// pass 2: (S v) of the tile's edges from the faces around them; box origin
// one line below the tile in y (two: the innermost coordinate stays even),
// x and z.  Writes y[map_edge[e]] for the non-PEC edges.
__global__ void __launch_bounds__(kStencilThreads) k_st_edges(const __grid_constant__ CUtensorMap tm_xy,
                                                              const __grid_constant__ CUtensorMap tm_yz,
                                                              const __grid_constant__ CUtensorMap tm_xz, Dims d,
                                                              int64_t Yp, Tables t, double inv_mu,
                                                              const int32_t *map_edge, double *out, int *err) {
    __shared__ alignas(128) double s[3 * kBoxPad];
    __shared__ alignas(8) uint64_t bar;
    const int y0 = blockIdx.x * kTY, x0 = blockIdx.y * kTX, z0 = blockIdx.z * kTZ;
    if (!load_boxes(&tm_xy, &tm_yz, &tm_xz, s, &bar, y0 - 2, x0 - 1, z0 - 1, err)) return;
    // box-local index of grid position p: p - origin
    for (int q = threadIdx.x; q < kTY * kTX * kTZ; q += blockDim.x) {
        const int ly = q % kTY, lx = (q / kTY) % kTX, lz = q / (kTY * kTX);
        const int64_t y = y0 + ly, x = x0 + lx, z = z0 + lz;
        if (y >= d.ny || x >= d.nx || z >= d.nz) continue;
        const int by = ly + 2, bx = lx + 1, bz = lz + 1;      // this position in the box
        const int64_t zc = z < d.Nz ? z : d.Nz - 1;
        // y-edge (z, x, y): xy faces at cells x-1 and x; yz faces at z-1 and z
        if (y < d.Ny) {
            const double qzx = t.qz_x[zc * (d.Nx + 1) + x], qxz = t.qx_z[x * (d.Nz + 1) + z];
            const double v = qzx * (at(s, 0, bz, bx - 1, by) - at(s, 0, bz, bx, by)) +
                             qxz * (at(s, 1, bz, bx, by) - at(s, 1, bz - 1, bx, by));
            const int32_t r = map_edge[d.ye(z, x, y)];
            if (r >= 0) out[r] = v * inv_mu;
        }
        // x-edge (z, x, y): xy faces at cells y-1 and y; xz faces at z-1 and z
        if (x < d.Nx) {
            const double qzy = t.qz_y[zc * (d.Ny + 1) + y], qyz = t.qy_z[y * (d.Nz + 1) + z];
            const double v = qzy * (at(s, 0, bz, bx, by) - at(s, 0, bz, bx, by - 1)) +
                             qyz * (at(s, 2, bz - 1, bx, by) - at(s, 2, bz, bx, by));
            const int32_t r = map_edge[d.xe(z, x, y)];
            if (r >= 0) out[r] = v * inv_mu;
        }
        // z-edge (z, x, y): yz faces at cells y-1 and y; xz faces at x-1 and x
        if (z < d.Nz) {
            const double qxy = t.qx_y[x * (d.Ny + 1) + y], qyx = t.qy_x[y * (d.Nx + 1) + x];
            const double v = qxy * (at(s, 1, bz, bx, by - 1) - at(s, 1, bz, bx, by)) +
                             qyx * (at(s, 2, bz, bx, by) - at(s, 2, bz, bx - 1, by));
            const int32_t r = map_edge[d.ze(z, x, y)];
            if (r >= 0) out[r] = v * inv_mu;
        }
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess && q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
    }
    return fn;
}

}  // namespace

struct CurlStencil {
    int64_t Yp = 0, nfull = 0;
    double *tab = nullptr;
    Tables t{};
    double *e[3] = {nullptr, nullptr, nullptr};     // y-, x-, z-edge values
    double *f[3] = {nullptr, nullptr, nullptr};     // xy-, yz-, xz-face circulations
    CUtensorMap me[3], mf[3];
    int32_t *map_r = nullptr;
    int64_t nr = 0;
    int *err = nullptr;
    void release(cudaStream_t s) {
        dfree(tab, s);
        for (int q = 0; q < 3; q++) { dfree(e[q], s); dfree(f[q], s); }
        dfree(map_r, s);
        dfree(err, s);
    }
};

void stencil_release(CurlStencil *st, cudaStream_t s) {
    if (!st) return;
    st->release(s);
    delete st;
}

namespace {

__global__ void k_st_map_r(int64_t ne, const int32_t *map_edge, int32_t *map_r) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < ne; e += (int64_t)gridDim.x * blockDim.x)
        if (map_edge[e] >= 0) map_r[map_edge[e]] = (int32_t)e;
}

g2p_status make_map(CUtensorMap *m, double *base, const Dims &d, int64_t Yp) {
    auto enc = encode_fn();
    if (!enc) { set_last_message("cuTensorMapEncodeTiled is not available from the driver"); return G2P_ERR_CUDA; }
    const cuuint64_t dims[3] = {(cuuint64_t)Yp, (cuuint64_t)d.nx, (cuuint64_t)d.nz};
    const cuuint64_t strides[2] = {(cuuint64_t)(Yp * 8), (cuuint64_t)(Yp * d.nx * 8)};
    const cuuint32_t box[3] = {kBY, kBX, kBZ};
    const cuuint32_t es[3] = {1, 1, 1};
    const CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 3, base, dims, strides, box, es,
                           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) { set_last_message("cuTensorMapEncodeTiled failed (%d)", (int)r); return G2P_ERR_CUDA; }
    return G2P_OK;
}

}  // namespace

// Builds the stencil of the mesh's S (after g2p_generate_stiff: the edge map
// and the grid are in place).
g2p_status stencil_build(g2p_mesh *m, CurlStencil **out) {
    const Dims &d = m->d;
    cudaStream_t s = m->stream;
    if (d.nx > INT32_MAX / 2 || d.ny > INT32_MAX / 2 || d.nz > INT32_MAX / 2) {
        set_last_message("grid too large for the stencil's tensor maps");
        return G2P_ERR_UNSUPPORTED;
    }
    CurlStencil *st = new CurlStencil();
    auto fail = [&](g2p_status e) { st->release(s); delete st; return e; };
    st->Yp = (d.ny + 1) & ~(int64_t)1;
    st->nfull = d.nz * d.nx * st->Yp;
    const int64_t NX = d.Nx + 1, NY = d.Ny + 1, NZ = d.Nz + 1;
    const int64_t ntab = d.Nx + d.Ny + d.Nz + d.Nz * NX + d.Nz * NY + NX * NZ + NX * NY + NY * NZ + NY * NX;
    g2p_status r;
    if ((r = dalloc(&st->tab, ntab, s)) != G2P_OK) return fail(r);
    double *t = st->tab;
    st->t.ivx = t; (kbegin("k_st_inv_len", s), k_st_inv_len<<<grid_for(d.Nx), kThreads, 0, s>>>(m->xn, d.Nx, t), kend(s)); t += d.Nx;
    st->t.ivy = t; (kbegin("k_st_inv_len", s), k_st_inv_len<<<grid_for(d.Ny), kThreads, 0, s>>>(m->yn, d.Ny, t), kend(s)); t += d.Ny;
    st->t.ivz = t; (kbegin("k_st_inv_len", s), k_st_inv_len<<<grid_for(d.Nz), kThreads, 0, s>>>(m->zn, d.Nz, t), kend(s)); t += d.Nz;
    struct QT { const double **dst; const double *a; int64_t na; const double *b; int64_t nb; };
    const QT qts[6] = {{&st->t.qz_x, m->dza, d.Nz, m->dxa, NX}, {&st->t.qz_y, m->dza, d.Nz, m->dya, NY},
                       {&st->t.qx_z, m->dxa, NX, m->dza, NZ}, {&st->t.qx_y, m->dxa, NX, m->dya, NY},
                       {&st->t.qy_z, m->dya, NY, m->dza, NZ}, {&st->t.qy_x, m->dya, NY, m->dxa, NX}};
    for (const QT &q : qts) {
        *q.dst = t;
        (kbegin("k_st_quot", s), k_st_quot<<<grid_for(q.na * q.nb), kThreads, 0, s>>>(q.a, q.na, q.b, q.nb, t), kend(s));
        t += q.na * q.nb;
    }
    for (int q = 0; q < 3; q++) {
        if ((r = dalloc(&st->e[q], st->nfull, s)) != G2P_OK) return fail(r);
        if ((r = dalloc(&st->f[q], st->nfull, s)) != G2P_OK) return fail(r);
        if (cudaMemsetAsync(st->e[q], 0, sizeof(double) * st->nfull, s) != cudaSuccess) return fail(G2P_ERR_CUDA);
        if ((r = make_map(&st->me[q], st->e[q], d, st->Yp)) != G2P_OK) return fail(r);
        if ((r = make_map(&st->mf[q], st->f[q], d, st->Yp)) != G2P_OK) return fail(r);
    }
    st->nr = m->S.n;
    if ((r = dalloc(&st->map_r, st->nr, s)) != G2P_OK) return fail(r);
    if ((r = dalloc(&st->err, 1, s)) != G2P_OK) return fail(r);
    cudaMemsetAsync(st->err, 0, sizeof(int), s);
    (kbegin("k_st_map_r", s), k_st_map_r<<<grid_for(d.N_edge), kThreads, 0, s>>>(d.N_edge, m->map_edge, st->map_r), kend(s));
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
        set_last_message("stencil setup failed");
        return fail(G2P_ERR_CUDA);
    }
    *out = st;
    return G2P_OK;
}

// y = S x for x, y in the reduced (non-PEC) numbering, device pointers.
g2p_status stencil_apply(g2p_mesh *m, CurlStencil *st, const double *x, double *y, cudaStream_t s) {
    const Dims &d = m->d;
    (kbegin("k_st_scatter", s), k_st_scatter<<<grid_for(st->nr), kThreads, 0, s>>>(d, st->Yp, st->nr, st->map_r, x, st->e[0], st->e[1], st->e[2]), kend(s));
    const dim3 grid((unsigned)((st->Yp + kTY - 1) / kTY), (unsigned)((d.nx + kTX - 1) / kTX), (unsigned)((d.nz + kTZ - 1) / kTZ));
    (kbegin("k_st_faces", s), k_st_faces<<<grid, kStencilThreads, 0, s>>>(st->me[0], st->me[1], st->me[2], d, st->Yp, st->t, st->f[0], st->f[1], st->f[2], st->err), kend(s));
    (kbegin("k_st_edges", s), k_st_edges<<<grid, kStencilThreads, 0, s>>>(st->mf[0], st->mf[1], st->mf[2], d, st->Yp, st->t, 1.0 / m->k.mu, m->map_edge, y, st->err), kend(s));
    G2P_CUDA(cudaGetLastError());
    return G2P_OK;
}

g2p_status stencil_check(CurlStencil *st, cudaStream_t s) {
    int h = 0;
    G2P_CUDA(cudaMemcpyAsync(&h, st->err, sizeof(int), cudaMemcpyDeviceToHost, s));
    G2P_CUDA(cudaStreamSynchronize(s));
    if (h == 2) { set_last_message("stencil: a tile's copy arguments broke the alignment rules; nothing was copied"); return G2P_ERR_CUDA; }
    if (h) { set_last_message("stencil: a tile's TMA load did not complete"); return G2P_ERR_CUDA; }
    return G2P_OK;
}

}  // namespace g2p

using namespace g2p;

// y = S x through the C ABI (x, y: host or device, leng = rows of S): the
// assembled CSR product or the matrix-free stencil; *ms (nullable) receives
// the device time of one product, averaged over reps >= 1 repetitions on
// device-resident vectors.
__global__ void k_st_csr_apply(int64_t n, const int64_t *ptr, const int32_t *col, const double *val, const double *x,
                               double *y) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
        double acc = 0;
        for (int64_t q = ptr[r]; q < ptr[r + 1]; q++) acc += val[q] * x[col[q]];
        y[r] = acc;
    }
}

extern "C" g2p_status g2p_stiff_apply(g2p_mesh *m, int32_t matrix_free, int32_t reps, const double *x, double *y,
                                      double *ms) {
    if (!m || !x || !y || reps < 1) { set_last_message("g2p_stiff_apply: bad arguments"); return G2P_ERR_INVALID; }
    if (!m->stiff_done) { set_last_message("g2p_stiff_apply: g2p_generate_stiff has not run"); return G2P_ERR_STATE; }
    cudaStream_t s = m->stream;
    if (matrix_free && !m->stencil) G2P_TRY(stencil_build(m, &m->stencil));
    const int64_t n = m->S.n;
    double *dx, *dy;
    G2P_TRY(dalloc(&dx, n, s));
    G2P_TRY(dalloc(&dy, n, s));
    G2P_CUDA(cudaMemcpyAsync(dx, x, sizeof(double) * n, cudaMemcpyDefault, s));
    cudaEvent_t e0, e1;
    G2P_CUDA(cudaEventCreate(&e0));
    G2P_CUDA(cudaEventCreate(&e1));
    g2p_status st = G2P_OK;
    for (int it = 0; it <= reps && st == G2P_OK; it++) {
        if (it == 1) cudaEventRecord(e0, s);       // the first product warms up
        if (matrix_free) st = stencil_apply(m, m->stencil, dx, dy, s);
        else (kbegin("k_st_csr_apply", s), k_st_csr_apply<<<grid_for(n), kThreads, 0, s>>>(n, m->S.ptr, m->S.col, m->S.val, dx, dy), kend(s));
    }
    cudaEventRecord(e1, s);
    if (st == G2P_OK && matrix_free) st = stencil_check(m->stencil, s);
    float t = 0;
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms) *ms = t / reps;
    if (st == G2P_OK) {
        G2P_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDefault, s));
        G2P_CUDA(cudaStreamSynchronize(s));
    }
    dfree(dx, s);
    dfree(dy, s);
    return st;
}
