// Kernel timing with CUDA events on the handle's stream (used by bench.py for the
// roofline figure of the stiffness apply).
#include "model.h"

namespace eqc {

// L2 flush by reading a buffer larger than L2: afterwards L2 holds clean lines only, so the
// timed kernel pays no write-back of someone else's dirty data (a read-modify-write flush
// would leave L2 full of dirty lines and inflate the next kernel's DRAM traffic).
__global__ void k_flush(const float4* __restrict__ buf, int64_t n4, float* sink) {
    float s = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += (int64_t)gridDim.x * blockDim.x) {
        const float4 v = buf[i];
        s += v.x + v.y + v.z + v.w;
    }
    if (s == 1.2345f) *sink = s;   // keeps the loads; the buffer holds zeros, so never taken
}

}  // namespace eqc

using namespace eqc;

extern "C" eqc_status eqc_time_apply(eqc_handle* H, int32_t dtype, int32_t nrep, int32_t flush_l2, double* ms) {
    if (!H || !ms || nrep < 1 || (dtype != 0 && dtype != 1)) return EQC_E_ARG;
    Handle& h = H->h;
    try {
        cudaStream_t s = h.stream;
        const int64_t N = h.L.size();
        const size_t es = dtype == 0 ? sizeof(double) : sizeof(float);
        void *x = nullptr, *y = nullptr;
        float* fl = nullptr;
        const int64_t nfl = (int64_t)(512ull << 20) / 4;  // 512 MB > L2
        EQC_CUDA(cudaMalloc(&x, N * es));
        EQC_CUDA(cudaMalloc(&y, N * es));
        if (flush_l2) EQC_CUDA(cudaMalloc(&fl, nfl * 4));
        EQC_CUDA(cudaMemsetAsync(x, 0, N * es, s));
        if (fl) EQC_CUDA(cudaMemsetAsync(fl, 0, nfl * 4, s));
        cudaEvent_t e0, e1;
        EQC_CUDA(cudaEventCreate(&e0));
        EQC_CUDA(cudaEventCreate(&e1));
        double tot = 0;
        for (int r = -2; r < nrep; ++r) {
            if (fl) {
                k_flush<<<8 * 152, 256, 0, s>>>(reinterpret_cast<const float4*>(fl), nfl / 4, fl);
                count_launch();
            }
            EQC_CUDA(cudaEventRecord(e0, s));
            if (dtype == 0) apply_K<double>((const double*)x, (double*)y, args64(h), 1.0, 0, s);
            else apply_K<float>((const float*)x, (float*)y, args32(h), 1.0f, 0, s);
            EQC_CUDA(cudaEventRecord(e1, s));
            EQC_CUDA(cudaEventSynchronize(e1));
            float t = 0;
            EQC_CUDA(cudaEventElapsedTime(&t, e0, e1));
            if (r >= 0) tot += t;
        }
        *ms = tot / nrep;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(x);
        cudaFree(y);
        if (fl) cudaFree(fl);
        return EQC_OK;
    } catch (const Error& e) {
        h.err = e.what();
        return e.code;
    }
}
