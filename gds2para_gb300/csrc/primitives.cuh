// Device-wide primitives used by assembly and AMG setup: warp-shuffle block
// scans, a three-phase exclusive scan, and a stable LSD radix sort of
// (key, value) pairs whose in-tile ranks come from __match_any_sync.
#pragma once
#include "common.cuh"

namespace g2p {

__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <class T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per-row kernels over k interleaved right-hand sides use blocks of shape
// (kx, 256 / kx): threadIdx.x is the right-hand side (kx the power of two
// >= k), threadIdx.y the row -- no integer division in the index math.
inline int pow2_ge(int k) {
    int p = 1;
    while (p < k) p <<= 1;
    return p;
}
inline dim3 row_block(int k) {
    int kx = pow2_ge(k);
    return dim3(kx, 256 / kx);
}
inline unsigned row_grid(int64_t n, int k, int64_t cap = 152LL * 32) {
    int64_t ny = 256 / pow2_ge(k);
    int64_t b = (n + ny - 1) / ny;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (unsigned)b;
}
#define G2P_FOR_ROWS(i, n) \
    for (int64_t i = blockIdx.x * (int64_t)blockDim.y + threadIdx.y; i < (n); i += (int64_t)gridDim.x * blockDim.y)

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class F>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(F op, int64_t n, int64_t *partial) {
    int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int64_t i = base + (int64_t)k * kScanThreads + threadIdx.x;
        if (i < n) s += op(i);
    }
    s = warp_sum(s);
    __shared__ int64_t ws[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < kScanThreads / 32; w++) t += ws[w];
        partial[blockIdx.x] = t;
    }
}

// In-place exclusive scan of partial[0..m) by one block; partial[m] = total.
__global__ void __launch_bounds__(1024) k_scan_partials(int64_t *partial, int64_t m);

template <class F, class OutT>
__global__ void __launch_bounds__(kScanThreads) k_scan_down(F op, int64_t n, const int64_t *partial, OutT *out) {
    int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
    int64_t v[kScanItems];
    int64_t s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int64_t i = base + k;
        v[k] = i < n ? op(i) : 0;
        s += v[k];
    }
    int64_t excl;
    // block-wide exclusive scan of per-thread sums
    __shared__ int64_t wsum[kScanThreads / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int64_t inc = warp_inclusive_scan(s);
    if (lane == 31) wsum[w] = inc;
    __syncthreads();
    if (w == 0) {
        int64_t t = lane < kScanThreads / 32 ? wsum[lane] : 0;
        int64_t ti = warp_inclusive_scan(t);
        if (lane < kScanThreads / 32) wsum[lane] = ti - t;
    }
    __syncthreads();
    excl = inc - s + wsum[w] + partial[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        int64_t i = base + k;
        if (i < n) out[i] = (OutT)excl;
        excl += v[k];
    }
}

// Exclusive scan out[i] = sum_{j<i} op(j); *total_dev (device) receives the
// sum.  `work` must hold at least scan_work_size(n) int64 values.
inline int64_t scan_work_size(int64_t n) { return (n + kScanTile - 1) / kScanTile + 2; }

template <class F, class OutT>
g2p_status exclusive_scan(F op, int64_t n, OutT *out, int64_t *work, cudaStream_t s) {
    int64_t nb = (n + kScanTile - 1) / kScanTile;
    if (nb == 0) nb = 1;
    (g2p::kbegin("k_scan_reduce", s), k_scan_reduce<F><<<(unsigned)nb, kScanThreads, 0, s>>>(op, n, work), g2p::kend(s));
    (g2p::kbegin("k_scan_partials", s), k_scan_partials<<<1, 1024, 0, s>>>(work, nb), g2p::kend(s));
    (g2p::kbegin("k_scan_down", s), k_scan_down<F, OutT><<<(unsigned)nb, kScanThreads, 0, s>>>(op, n, work, out), g2p::kend(s));
    G2P_CUDA(cudaGetLastError());
    return G2P_OK;
}
// After exclusive_scan, work[nb] holds the total.
inline int64_t scan_total_index(int64_t n) {
    int64_t nb = (n + kScanTile - 1) / kScanTile;
    return nb == 0 ? 1 : nb;
}

// ------------------------------------------------------------------ radix sort
constexpr int kSortThreads = 256;
constexpr int kSortWarps = kSortThreads / 32;
constexpr int kSortBatches = 16;                       // 32-key batches per warp
constexpr int kSortTile = kSortThreads * kSortBatches; // 4096 keys per block

template <class K>
__global__ void __launch_bounds__(kSortThreads) k_sort_hist(const K *keys, int64_t n, int shift, int64_t nblocks,
                                                            int64_t *counts) {
    __shared__ int hist[256];
    for (int d = threadIdx.x; d < 256; d += kSortThreads) hist[d] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * kSortTile;
    for (int k = 0; k < kSortBatches; k++) {
        int64_t i = base + (int64_t)k * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&hist[(int)((keys[i] >> shift) & 0xFF)], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += kSortThreads) counts[(int64_t)d * nblocks + blockIdx.x] = hist[d];
}

// Stable scatter: within a tile, warp w owns keys [w*512, (w+1)*512) in order;
// ranks inside a 32-key batch come from __match_any_sync peers.
template <class K, class V>
__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(const K *keys, const V *vals, int64_t n, int shift,
                                                               int64_t nblocks, const int64_t *offs, K *okeys,
                                                               V *ovals) {
    __shared__ int whist[kSortWarps][257];
    __shared__ int64_t run[kSortWarps][256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = lane; d < 256; d += 32) whist[w][d] = 0;
    __syncwarp();
    int64_t wbase = (int64_t)blockIdx.x * kSortTile + (int64_t)w * 32 * kSortBatches;
    for (int k = 0; k < kSortBatches; k++) {
        int64_t i = wbase + (int64_t)k * 32 + lane;
        if (i < n) atomicAdd(&whist[w][(int)((keys[i] >> shift) & 0xFF)], 1);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < 256; d += kSortThreads) {
        int64_t acc = offs[(int64_t)d * nblocks + blockIdx.x];
        for (int q = 0; q < kSortWarps; q++) {
            int c = whist[q][d];
            run[q][d] = acc;
            acc += c;
        }
    }
    __syncthreads();
    const unsigned lt = lanemask_lt();
    for (int k = 0; k < kSortBatches; k++) {
        int64_t i = wbase + (int64_t)k * 32 + lane;
        bool valid = i < n;
        K key = valid ? keys[i] : K(0);
        int d = valid ? (int)((key >> shift) & 0xFF) : 256;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank = __popc(peers & lt);
        int leader = __ffs(peers) - 1;
        int64_t b = valid ? run[w][d] : 0;
        __syncwarp();
        if (valid) {
            int64_t dst = b + rank;
            okeys[dst] = key;
            ovals[dst] = vals[i];
            if (lane == leader) run[w][d] = b + __popc(peers);
        }
        __syncwarp();
    }
}

// Stable LSD radix sort of n pairs over key bits [0, bits).  Buffers ping-pong
// between (k0,v0) and (k1,v1); *result_in_1 tells where the output ended.
template <class K, class V>
g2p_status radix_sort_pairs(K *k0, V *v0, K *k1, V *v1, int64_t n, int bits, int64_t *counts, int64_t *work,
                            bool *result_in_1, cudaStream_t s) {
    int64_t nb = (n + kSortTile - 1) / kSortTile;
    if (nb == 0) nb = 1;
    K *ks = k0, *kd = k1;
    V *vs = v0, *vd = v1;
    bool in1 = false;
    for (int shift = 0; shift < bits; shift += 8) {
        (g2p::kbegin("k_sort_hist", s), k_sort_hist<K><<<(unsigned)nb, kSortThreads, 0, s>>>(ks, n, shift, nb, counts), g2p::kend(s));
        const int64_t *c = counts;
        auto op = [c] __device__(int64_t i) { return c[i]; };
        G2P_TRY(exclusive_scan(op, 256 * nb, counts + 256 * nb, work, s));
        (g2p::kbegin("k_sort_scatter", s), k_sort_scatter<K, V><<<(unsigned)nb, kSortThreads, 0, s>>>(ks, vs, n, shift, nb, counts + 256 * nb, kd, vd), g2p::kend(s));
        G2P_CUDA(cudaGetLastError());
        K *tk = ks; ks = kd; kd = tk;
        V *tv = vs; vs = vd; vd = tv;
        in1 = !in1;
    }
    *result_in_1 = in1;
    return G2P_OK;
}
// counts must hold 2 * 256 * ceil(n / kSortTile) values; work scan_work_size(256 * that).
inline int64_t sort_counts_size(int64_t n) { return 2 * 256 * ((n + kSortTile - 1) / kSortTile + 1); }

}  // namespace g2p
