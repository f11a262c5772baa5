// Deterministic block/grid reductions (FP64 accumulation).
#pragma once
#include <cuda_runtime.h>

namespace eqc {

constexpr int RED_BLOCKS = 2 * 152;
constexpr int RED_THREADS = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the CTA; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    v = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (w == 0) v = warp_sum(v);
    __syncthreads();
    return v;
}

// Finishes a reduction: the last CTA sums the partials and calls fin(total) in thread 0.
template <class Fin>
__device__ __forceinline__ void finish_reduction(double s, double* part, unsigned* count, double* sh, Fin fin) {
    __shared__ bool last;
    if (threadIdx.x == 0) {
        part[blockIdx.x] = s;
        __threadfence();
        const unsigned prev = atomicAdd(count, 1u);
        last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double t = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += blockDim.x) t += __ldcg(part + k);
    t = block_sum(t, sh);
    if (threadIdx.x == 0) {
        fin(t);
        *count = 0u;
    }
}

}  // namespace eqc
