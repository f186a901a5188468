// Out-of-line parts of the device primitives.
#include "primitives.cuh"

namespace g2p {

__global__ void __launch_bounds__(1024) k_scan_partials(int64_t *partial, int64_t m) {
    __shared__ int64_t wsum[32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int64_t base = 0; base < m; base += 1024) {
        int64_t i = base + threadIdx.x;
        int64_t v = i < m ? partial[i] : 0;
        int64_t inc = warp_inclusive_scan(v);
        if (lane == 31) wsum[w] = inc;
        __syncthreads();
        if (w == 0) {
            int64_t t = wsum[lane];
            int64_t ti = warp_inclusive_scan(t);
            wsum[lane] = ti - t;
        }
        __syncthreads();
        int64_t c = carry;
        if (i < m) partial[i] = c + wsum[w] + inc - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c + wsum[w] + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[m] = carry;
}

}  // namespace g2p
