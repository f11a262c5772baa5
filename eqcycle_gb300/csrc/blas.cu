// Deterministic reductions and fused vector updates.
//
// Dot products accumulate in FP64 (also for FP32 vectors).  Each launch uses a fixed
// grid: every CTA reduces a fixed grid-stride slice with warp shuffles, writes one
// partial, and the last CTA to finish (atomic ticket in a scratch counter) sums the
// partials in CTA order.  The result is therefore bitwise reproducible.
#include "model.h"
#include "reduce.cuh"

namespace eqc {

int64_t g_launches = 0;

template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_dot(const T* __restrict__ x, const T* __restrict__ y, int64_t n,
                                                     double* part, unsigned* count, double* out) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += (double)x[i] * (double)y[i];
    s = block_sum(s, sh);
    finish_reduction(s, part, count, sh, [&](double t) { *out = t; });
}

void dot64(Handle& h, const double* x, const double* y, int64_t n, double* out_dev) {
    k_dot<double><<<RED_BLOCKS, RED_THREADS, 0, h.stream>>>(x, y, n, h.red_part.p, h.red_count.p, out_dev);
    EQC_CHECK_LAUNCH();
    count_launch();
}
void dot32(Handle& h, const float* x, const float* y, int64_t n, double* out_dev) {
    k_dot<float><<<RED_BLOCKS, RED_THREADS, 0, h.stream>>>(x, y, n, h.red_part.p, h.red_count.p, out_dev);
    EQC_CHECK_LAUNCH();
    count_launch();
}

}  // namespace eqc
