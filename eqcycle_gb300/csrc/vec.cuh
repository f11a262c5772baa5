// Four-wide vector access for the HBM-bound vector kernels: one 16-byte access per four
// floats, two per four doubles.  Every node vector of the library starts on a 32-byte
// boundary (cudaMalloc alignment plus a row pitch that is a multiple of 8 entries), so
// interior slices [ld, size) are 16-byte aligned as well.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

namespace eqc {

// 3 CTAs of 256 threads per SM of a GB300: the reductions' last-CTA tickets and partials cost
// less than with 8 per SM, and 4-wide grid-stride loops keep enough loads in flight (dz480
// quasi-static steps: 73.0 ms for 20 with 8 per SM, 72.6 with 4, 71.9 with 3, 72.1 with 2)
constexpr int VEC_BLOCKS = 3 * 152;
constexpr int VEC_THREADS = 256;

__device__ __forceinline__ void ld4(const float* p, float (&a)[4]) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    a[0] = v.x; a[1] = v.y; a[2] = v.z; a[3] = v.w;
}
__device__ __forceinline__ void ld4(const double* p, double (&a)[4]) {
    const double2 u = reinterpret_cast<const double2*>(p)[0], w = reinterpret_cast<const double2*>(p)[1];
    a[0] = u.x; a[1] = u.y; a[2] = w.x; a[3] = w.y;
}
__device__ __forceinline__ void st4(float* p, const float (&a)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(a[0], a[1], a[2], a[3]);
}
__device__ __forceinline__ void st4(double* p, const double (&a)[4]) {
    reinterpret_cast<double2*>(p)[0] = make_double2(a[0], a[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(a[2], a[3]);
}

// Dot-product accumulator.  FP64 vectors accumulate in FP64.  FP32 vectors accumulate the
// exact products (a*b = p + e, e by FMA) in an unevaluated FP32 pair (hi + lo, Knuth's
// TwoSum), about 44 significant bits, then hand a double to the cross-thread reduction:
// FP64-class dot products of FP32 vectors without FP64 arithmetic per element (GB300's FP64
// and FP32<->FP64 conversion rates are a small fraction of its FP32 rate).
template <class T> struct DotAcc;
template <> struct DotAcc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
    __device__ __forceinline__ double value() const { return s; }
};
template <> struct DotAcc<float> {
    float hi = 0.f, lo = 0.f;
    __device__ __forceinline__ void add(float a, float b) {
        const float p = __fmul_rn(a, b);
        const float e = __fmaf_rn(a, b, -p);
        const float s = __fadd_rn(hi, p);
        const float bb = __fsub_rn(s, hi);
        const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
        hi = s;
        lo = __fadd_rn(lo, __fadd_rn(err, e));
    }
    __device__ __forceinline__ double value() const { return (double)hi + (double)lo; }
};

inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

}  // namespace eqc
