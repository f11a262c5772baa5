// Deterministic reductions and fused vector updates.
//
// Dot products accumulate in FP64 (also for FP32 vectors).  Each launch uses a fixed
// grid: every CTA reduces a fixed grid-stride slice with warp shuffles, writes one
// partial, and the last CTA to finish (atomic ticket in a scratch counter) sums the
// partials in CTA order.  The result is therefore bitwise reproducible.
#include "model.h"
#include "reduce.cuh"
#include "vec.cuh"

namespace eqc {

int64_t g_launches = 0;

int vec_blocks() { return VEC_BLOCKS; }

// x and y 16-byte aligned; 4-wide chunks on a fixed grid, the n % 4 tail in thread 0
template <class T>
__global__ void __launch_bounds__(VEC_THREADS) k_dot(const T* __restrict__ x, const T* __restrict__ y, int64_t n,
                                                     double* part, unsigned* count, double* out) {
    EQC_GRID_WAIT();
    __shared__ double sh[32];
    DotAcc<T> acc;
    const int64_t n4 = n & ~(int64_t)3;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (int64_t i = n4; i < n; ++i) acc.add(x[i], y[i]);
    for (int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n4; i += 4 * (int64_t)gridDim.x * blockDim.x) {
        T a[4], b[4];
        ld4(x + i, a);
        ld4(y + i, b);
#pragma unroll
        for (int k = 0; k < 4; ++k) acc.add(a[k], b[k]);
    }
    double s = acc.value();
    s = block_sum(s, sh);
    finish_reduction(s, part, count, sh, [&](double t) { *out = t; });
}

static void check_vec(const void* x, const void* y, int64_t) {
    if (!aligned16(x) || !aligned16(y)) throw Error(EQC_E_ARG, "dot: vectors must be 16-byte aligned");
}

void dot64(Handle& h, const double* x, const double* y, int64_t n, double* out_dev) {
    check_vec(x, y, n);
    k_dot<double><<<vec_blocks(), VEC_THREADS, 0, h.stream>>>(x, y, n, h.red_part.p, h.red_count.p, out_dev);
    EQC_CHECK_LAUNCH();
    count_launch();
}
void dot32(Handle& h, const float* x, const float* y, int64_t n, double* out_dev) {
    check_vec(x, y, n);
    k_dot<float><<<vec_blocks(), VEC_THREADS, 0, h.stream>>>(x, y, n, h.red_part.p, h.red_count.p, out_dev);
    EQC_CHECK_LAUNCH();
    count_launch();
}

}  // namespace eqc
