// Pointwise work fused into the operator kernels of the V-cycle (the stiffness apply on the
// spectral-element level, the 9-point stencils on the vertex levels): instead of writing
// t = A x and launching a vector kernel that reads it back, the operator kernel finishes each
// owned node itself.  The arithmetic is spelled out with round-to-nearest intrinsics, so the
// fused and the separate forms give the same bits.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#if defined(__CUDACC__)
#include "vec.cuh"
#include "df.cuh"
#endif

namespace eqc {

// The end of a mixed-precision Newmark step at one node off the fault row (main.jl:309-339),
// given t = (K dd)_i, the FP32 apply of the step's displacement increment: K d += t (FP64),
// a = -K d, the absorbing terms a -= C v of the nodes on the edge x = -LX (column ix = 0, list
// iBcL) and on the edge y = LY (row iy = ny - 1, list iBcT) in that order (v the half-step
// velocity), then a /= M (a multiply by 1/M).  The reference's v += dt/2 a and the next step's
// predictor v += dt/2 a are taken as one update v += dt a, stored in v: the next step starts from
// it (an FP64 operation and 24 bytes per node fewer), and nm_state_at recovers the step's end
// velocity and acceleration where an output needs them.  The fault row is ended by the dynamic
// step's fault kernel and keeps v and a.
struct NmEpi {
    double *Kd = nullptr, *v = nullptr, *a = nullptr;
    const double* invM = nullptr;
    const double *cL = nullptr, *cT = nullptr;     // [ny] / [nx] coefficients on the two edges
    const int *hasL = nullptr, *hasT = nullptr;    // ... and whether the node is in the list
    const double* hdt = nullptr;                    // dt / 2 (in the control block)
    const int* kd_full = nullptr;                   // nonzero: K d recomputed in FP64 this step
    int* v_half = nullptr;                          // set: v holds the next half-step velocity
    int ld = 0, nx = 0, ny = 0;
};

// What an operator kernel does with t = (A x)_i at the nodes it owns.
template <class T>
struct OpEpi {
    int mode = 0;              // 0: y = t;  1: r = b - t (residual);  2: Chebyshev step, x of the
                               //    kernel is the direction dold (r, x updated, d' into dnew);
                               // 3: first Chebyshev step from x, t = A x: r = Dinv (b - t) and
                               //    d = r / theta into dnew, x += d left pending (x is the
                               //    operand other CTAs are still reading): the next step adds it
                               //    (x_pend) or the next reader of x does
    const T* b = nullptr;      // modes 1, 3
    T* r = nullptr;            // modes 1-3
    const T* dinv = nullptr;   // modes 2, 3
    const T* dold = nullptr;
    T* dnew = nullptr;
    T* x = nullptr;
    T c1 = T(0), c2 = T(0);
    T inv_theta = T(0);        // mode 3
    bool x_pend = false;       // mode 2: x += dold (the first step's pending direction) first
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

// First Chebyshev step from x at one node, t = (A x)_i:  r = Dinv (b - t) ; d = r / theta (the
// operations of k_cheb_first with x, in its order; its x += d is add_rn(x, d) wherever it lands)
template <class T>
__device__ __forceinline__ void cheb_first_rd_pt(T& r, T& d, T b, T t, T dinv, T inv_theta) {
    r = mul_rn<T>(dinv, sub_rn<T>(b, t));
    d = mul_rn<T>(r, inv_theta);
}

// FP32 -> FP64, exact, by integer operations on the bit patterns (GB300 converts to FP64 on its
// FP64 unit, a small fraction of its integer and FP32 rate).  Zeros, subnormals, infinities
// and NaNs included.
__device__ __forceinline__ double f32_to_f64(float f) {
    const uint32_t b = __float_as_uint(f);
    const uint64_t sign = (uint64_t)(b >> 31) << 63;
    const uint32_t e = (b >> 23) & 0xffu, m = b & 0x7fffffu;
    if (e == 0xffu) return __longlong_as_double((long long)(sign | (0x7ffull << 52) | ((uint64_t)m << 29)));
    if (e != 0) return __longlong_as_double((long long)(sign | ((uint64_t)(e + 896u) << 52) | ((uint64_t)m << 29)));
    if (m == 0) return __longlong_as_double((long long)sign);
    const int p = 31 - __clz((int)m);                 // leading one of a subnormal: m * 2^-149
    const uint64_t frac = ((uint64_t)m - (1ull << p)) << (52 - p);
    return __longlong_as_double((long long)(sign | ((uint64_t)(p + 874) << 52) | frac));
}

// The FP32 increment dt vh of a dynamic step from the half-step velocity vh: vh rounded to FP32
// (integer operations), times dt given as hi + lo in FP32, so the product is rounded once
// without the systematic error of a rounded dt, which K d would accumulate step after step.
__device__ __forceinline__ float nm_incr32(double vh, float dt_hi, float dt_lo) {
    const df vd = df_from_double(vh);
    const float v32 = __fadd_rn(vd.hi, vd.lo);
    return __fmaf_rn(dt_hi, v32, __fmul_rn(dt_lo, v32));
}

// One node (ix, iy >= 1) of the Newmark end (NmEpi).  add: t is added to K d (else K d was just
// recomputed in FP64).
__device__ __forceinline__ void newmark_node(const NmEpi& N, int64_t i, int ix, int iy, float t, bool add,
                                             double hdt) {
    double kd = N.Kd[i];
    if (add) {
        kd = __dadd_rn(kd, f32_to_f64(t));
        N.Kd[i] = kd;
    }
    double ai = -kd;
    const double vi = N.v[i];
    if (ix == 0 && N.hasL[iy]) ai = __dsub_rn(ai, __dmul_rn(N.cL[iy], vi));
    if (iy == N.ny - 1 && N.hasT[ix]) ai = __dsub_rn(ai, __dmul_rn(N.cT[ix], vi));
    ai = __dmul_rn(ai, N.invM[i]);
    N.v[i] = __fma_rn(2.0 * hdt, ai, vi);
}

// The step's end velocity and acceleration at node i off the fault row while v holds the next
// half-step velocity V = vh + dt a (newmark_node): a = (-K d - c vh) / M with c the node's
// absorbing coefficients, so a = (-K d - c V) / M / (1 - c dt / M), exactly the stored formula
// where c = 0; then v = V - dt/2 a.
__device__ __forceinline__ void nm_state_at(const NmEpi& N, int64_t i, double hdt, double* v_end, double* a_end) {
    const int iy = (int)(i / N.ld), ix = (int)(i - (int64_t)iy * N.ld);
    const double V = N.v[i], im = N.invM[i];
    double c = 0.0;
    if (ix == 0 && N.hasL[iy]) c += N.cL[iy];
    if (iy == N.ny - 1 && N.hasT[ix]) c += N.cT[ix];
    double a = __dmul_rn(-N.Kd[i], im);
    if (c != 0.0) a = ((-N.Kd[i] - c * V) * im) / (1.0 - c * 2.0 * hdt * im);
    *a_end = a;
    *v_end = __fma_rn(-hdt, a, V);
}

// Four consecutive nodes ix0 .. ix0 + 3 of row iy >= 1 (offset off, 32-byte aligned): 4-wide
// accesses off the edges, node by node on them and at the row's end.
__device__ __forceinline__ void newmark4(const NmEpi& N, int64_t off, int ix0, int iy, const float (&t)[4], bool add,
                                         double hdt) {
    if (ix0 + 3 >= N.nx || ix0 == 0 || iy == N.ny - 1) {
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (ix0 + q < N.nx) newmark_node(N, off + q, ix0 + q, iy, t[q], add, hdt);
        return;
    }
    double kd[4], vv[4], im[4];
    ld4(N.Kd + off, kd);
    ld4(N.v + off, vv);
    ld4(N.invM + off, im);
    const double dt = 2.0 * hdt;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (add) kd[q] = __dadd_rn(kd[q], f32_to_f64(t[q]));
        vv[q] = __fma_rn(dt, __dmul_rn(-kd[q], im[q]), vv[q]);
    }
    if (add) st4(N.Kd + off, kd);
    st4(N.v + off, vv);
}

// Four consecutive owned nodes starting at offset off (16-byte aligned, FP32).
__device__ __forceinline__ void epi_store4(const OpEpi<float>& E, float* y, int64_t off, float4 t) {
    if (E.mode == 0) {
        *reinterpret_cast<float4*>(y + off) = t;
    } else if (E.mode == 1) {
        const float4 b = __ldg(reinterpret_cast<const float4*>(E.b + off));
        *reinterpret_cast<float4*>(E.r + off) =
            make_float4(sub_rn(b.x, t.x), sub_rn(b.y, t.y), sub_rn(b.z, t.z), sub_rn(b.w, t.w));
    } else if (E.mode == 3) {
        const float4 b = __ldg(reinterpret_cast<const float4*>(E.b + off));
        const float4 di = __ldg(reinterpret_cast<const float4*>(E.dinv + off));
        float4 r, d;
        cheb_first_rd_pt(r.x, d.x, b.x, t.x, di.x, E.inv_theta);
        cheb_first_rd_pt(r.y, d.y, b.y, t.y, di.y, E.inv_theta);
        cheb_first_rd_pt(r.z, d.z, b.z, t.z, di.z, E.inv_theta);
        cheb_first_rd_pt(r.w, d.w, b.w, t.w, di.w, E.inv_theta);
        *reinterpret_cast<float4*>(E.r + off) = r;
        *reinterpret_cast<float4*>(E.dnew + off) = d;
    } else {
        float4 r = *reinterpret_cast<const float4*>(E.r + off);
        float4 x = *reinterpret_cast<const float4*>(E.x + off);
        float4 d = __ldg(reinterpret_cast<const float4*>(E.dold + off));
        const float4 di = __ldg(reinterpret_cast<const float4*>(E.dinv + off));
        if (E.x_pend) {
            x.x = add_rn(x.x, d.x);
            x.y = add_rn(x.y, d.y);
            x.z = add_rn(x.z, d.z);
            x.w = add_rn(x.w, d.w);
        }
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
    } else if (E.mode == 3) {
        T r, d;
        cheb_first_rd_pt<T>(r, d, E.b[i], t, E.dinv[i], E.inv_theta);
        E.r[i] = r;
        E.dnew[i] = d;
    } else {
        T r = E.r[i], d = E.dold[i], x = E.x[i];
        if (E.x_pend) x = add_rn<T>(x, d);
        cheb_step_pt<T>(r, d, x, t, E.dinv[i], E.c1, E.c2);
        E.r[i] = r;
        E.x[i] = x;
        E.dnew[i] = d;
    }
}

#endif  // __CUDACC__

}  // namespace eqc
