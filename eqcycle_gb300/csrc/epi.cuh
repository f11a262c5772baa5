// Pointwise work fused into the operator kernels of the V-cycle (the stiffness apply on the
// spectral-element level, the 9-point stencils on the vertex levels): instead of writing
// t = A x and launching a vector kernel that reads it back, the operator kernel finishes each
// owned node itself.  The arithmetic is spelled out with round-to-nearest intrinsics, so the
// fused and the separate forms give the same bits.
#pragma once
#include <cuda_runtime.h>

namespace eqc {

// What an operator kernel does with t = (A x)_i at the nodes it owns.
template <class T>
struct OpEpi {
    int mode = 0;              // 0: y = t;  1: r = b - t (residual);  2: Chebyshev step, x of the
                               //    kernel is the direction dold (r, x updated, d' into dnew)
    const T* b = nullptr;      // mode 1
    T* r = nullptr;            // modes 1, 2
    const T* dinv = nullptr;   // mode 2
    const T* dold = nullptr;
    T* dnew = nullptr;
    T* x = nullptr;
    T c1 = T(0), c2 = T(0);
};

#if defined(__CUDACC__)
template <class T> __device__ __forceinline__ T fma_rn(T a, T b, T c);
template <> __device__ __forceinline__ float fma_rn<float>(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <> __device__ __forceinline__ double fma_rn<double>(double a, double b, double c) { return __fma_rn(a, b, c); }
template <class T> __device__ __forceinline__ T mul_rn(T a, T b);
template <> __device__ __forceinline__ float mul_rn<float>(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double mul_rn<double>(double a, double b) { return __dmul_rn(a, b); }
template <class T> __device__ __forceinline__ T add_rn(T a, T b);
template <> __device__ __forceinline__ float add_rn<float>(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ double add_rn<double>(double a, double b) { return __dadd_rn(a, b); }
template <class T> __device__ __forceinline__ T sub_rn(T a, T b);
template <> __device__ __forceinline__ float sub_rn<float>(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ double sub_rn<double>(double a, double b) { return __dsub_rn(a, b); }

// Chebyshev step at one node, t = (A d)_i:  r -= Dinv t ; d = c1 d + c2 r ; x += d
template <class T>
__device__ __forceinline__ void cheb_step_pt(T& r, T& d, T& x, T t, T dinv, T c1, T c2) {
    r = fma_rn<T>(-dinv, t, r);
    d = fma_rn<T>(c1, d, mul_rn<T>(c2, r));
    x = add_rn<T>(x, d);
}

// Four consecutive owned nodes starting at offset off (16-byte aligned, FP32).
__device__ __forceinline__ void epi_store4(const OpEpi<float>& E, float* y, int64_t off, float4 t) {
    if (E.mode == 0) {
        *reinterpret_cast<float4*>(y + off) = t;
    } else if (E.mode == 1) {
        const float4 b = __ldg(reinterpret_cast<const float4*>(E.b + off));
        *reinterpret_cast<float4*>(E.r + off) =
            make_float4(sub_rn(b.x, t.x), sub_rn(b.y, t.y), sub_rn(b.z, t.z), sub_rn(b.w, t.w));
    } else {
        float4 r = *reinterpret_cast<const float4*>(E.r + off);
        float4 x = *reinterpret_cast<const float4*>(E.x + off);
        float4 d = __ldg(reinterpret_cast<const float4*>(E.dold + off));
        const float4 di = __ldg(reinterpret_cast<const float4*>(E.dinv + off));
        cheb_step_pt(r.x, d.x, x.x, t.x, di.x, E.c1, E.c2);
        cheb_step_pt(r.y, d.y, x.y, t.y, di.y, E.c1, E.c2);
        cheb_step_pt(r.z, d.z, x.z, t.z, di.z, E.c1, E.c2);
        cheb_step_pt(r.w, d.w, x.w, t.w, di.w, E.c1, E.c2);
        *reinterpret_cast<float4*>(E.r + off) = r;
        *reinterpret_cast<float4*>(E.x + off) = x;
        *reinterpret_cast<float4*>(E.dnew + off) = d;
    }
}

// One node (any precision).
template <class T>
__device__ __forceinline__ void epi_store1(const OpEpi<T>& E, T* y, int64_t i, T t) {
    if (E.mode == 0) {
        y[i] = t;
    } else if (E.mode == 1) {
        E.r[i] = sub_rn<T>(E.b[i], t);
    } else {
        T r = E.r[i], d = E.dold[i], x = E.x[i];
        cheb_step_pt<T>(r, d, x, t, E.dinv[i], E.c1, E.c2);
        E.r[i] = r;
        E.x[i] = x;
        E.dnew[i] = d;
    }
}

#endif  // __CUDACC__

}  // namespace eqc
