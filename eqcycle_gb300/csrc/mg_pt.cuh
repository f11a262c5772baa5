// Point operations of the vertex levels of the multigrid V-cycle (mg.cu): the 9-point stencil,
// the restriction and prolongation between levels, the Chebyshev steps and the dense coarse
// solve's rows.  Every multiply-add is an explicit round-to-nearest FMA, so any kernel built from
// these functions gives the same bits as the V-cycle's own.  Ld is the load of the vectors the
// V-cycle writes: plain (LdPlain) or with a pending Chebyshev direction added (LdPend).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include "epi.cuh"

namespace eqc {

struct LdPlain {
    template <class T> __device__ __forceinline__ T operator()(const T* p) const { return *p; }
};

// A coarse level's correction x read with its post-smoothing's pending first-step direction
// added (OpEpi mode 3): x + pend at the same offset from base, rounded as k_cheb_first rounds it.
struct LdPend {
    const void* base = nullptr;
    const void* pend = nullptr;   // null: plain loads
    template <class T> __device__ __forceinline__ T operator()(const T* p) const {
        const T v = *p;
        if (!pend) return v;
        return add_rn<T>(v, static_cast<const T*>(pend)[p - static_cast<const T*>(base)]);
    }
};

// The coarse level's first Chebyshev step from x = 0, fused into the restriction that produces
// its right-hand side (k_cheb_first with with_x = 0): r = Dinv b ; d = r / theta ; x = d.
template <class T>
struct ChebFirst {
    const T* dinv = nullptr;   // null: not fused
    T *x = nullptr, *r = nullptr, *d = nullptr;
    T inv_theta = T(0);
};
template <class T>
__device__ __forceinline__ void cheb_first_pt(const ChebFirst<T>& F, int64_t i, T b) {
    if (!F.dinv) return;
    const T ri = mul_rn<T>(F.dinv[i], b);
    const T di = mul_rn<T>(ri, F.inv_theta);
    F.r[i] = ri;
    F.d[i] = di;
    F.x[i] = di;
}

// (A x)_i of a 9-point stencil level (A[k N + i], offsets (k % 3 - 1, k / 3 - 1)); row 0 is the
// fault row and gives 0, as do neighbours in it.
template <class T, class Ld>
__device__ __forceinline__ T stencil_pt(const T* __restrict__ A, const T* x, int cx, int cy, int64_t N, int64_t i,
                                        Ld ld) {
    const int ix = (int)(i % cx), iy = (int)(i / cx);
    T s = T(0);
    if (iy >= 1) {
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const int gx = ix + (k % 3) - 1, gy = iy + (k / 3) - 1;
            if (gx >= 0 && gx < cx && gy >= 1 && gy < cy) s = fma_rn<T>(A[k * N + i], ld(x + (int64_t)gy * cx + gx), s);
        }
    }
    return s;
}

// (P^T rf) at coarse point (cxi, cyi >= 1) through the restriction lists of a level transfer.
template <class T, class Ld>
__device__ __forceinline__ T restrict_pt(const T* rf, int ldf, const int* __restrict__ rpx, const int* __restrict__ rix,
                                         const T* __restrict__ rwx, const int* __restrict__ rpy,
                                         const int* __restrict__ riy, const T* __restrict__ rwy, int cxi, int cyi,
                                         Ld ld) {
    T s = T(0);
    if (cyi >= 1) {
        for (int q = rpy[cyi]; q < rpy[cyi + 1]; ++q) {
            const int fy = riy[q];
            if (fy == 0) continue;
            const T wq = rwy[q];
            T sx = T(0);
            for (int p = rpx[cxi]; p < rpx[cxi + 1]; ++p) sx = fma_rn<T>(rwx[p], ld(rf + (int64_t)fy * ldf + rix[p]), sx);
            s = fma_rn<T>(wq, sx, s);
        }
    }
    return s;
}

// (P xc) at fine point (ix, iy >= 1): the two-by-two bilinear interpolation.
template <class T, class Ld>
__device__ __forceinline__ T prolong_pt(const T* xc, int ldc, const int* __restrict__ px, const int* __restrict__ py,
                                        const T* __restrict__ wx, const T* __restrict__ wy, int ix, int iy, Ld ld) {
    T s = T(0);
#pragma unroll
    for (int b = 0; b < 2; ++b) {
        const T wb = wy[2 * iy + b];
        if (wb == T(0)) continue;
        const int cyi = py[2 * iy + b];
#pragma unroll
        for (int a = 0; a < 2; ++a) {
            const T wa = wx[2 * ix + a];
            if (wa != T(0)) s = fma_rn<T>(mul_rn<T>(wa, wb), ld(xc + (int64_t)cyi * ldc + px[2 * ix + a]), s);
        }
    }
    return s;
}

// Chebyshev, first step at one point.  with_x: r = Dinv (b - t), else r = Dinv b and x = 0;
// d = r / theta ; x += d.
template <class T, class Ld>
__device__ __forceinline__ void cheb_first_step_pt(T* x, T* r, T* d, const T* b, const T* t, const T* __restrict__ Dinv,
                                                   int64_t i, T inv_theta, bool with_x, Ld ld) {
    const T ri = with_x ? mul_rn<T>(Dinv[i], sub_rn<T>(ld(b + i), ld(t + i))) : mul_rn<T>(Dinv[i], ld(b + i));
    const T di = mul_rn<T>(ri, inv_theta);
    r[i] = ri;
    d[i] = di;
    x[i] = with_x ? add_rn<T>(ld(x + i), di) : di;
}

// One row of the coarsest level's dense inverse times b, by one warp: the lanes' partial sums
// in two interleaved accumulators, then a shuffle tree; lane 0 holds the result.
template <class T, class Ld>
__device__ __forceinline__ T dense_row(const T* __restrict__ Cinv, const T* b, int n, int off, int row, int lane, Ld ld) {
    const T* rw = Cinv + (int64_t)row * n;
    T s0 = T(0), s1 = T(0);
    int j = lane;
    for (; j + 32 < n; j += 64) {
        s0 = fma_rn<T>(rw[j], ld(b + off + j), s0);
        s1 = fma_rn<T>(rw[j + 32], ld(b + off + j + 32), s1);
    }
    if (j < n) s0 = fma_rn<T>(rw[j], ld(b + off + j), s0);
    T v = add_rn<T>(s0, s1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = add_rn<T>(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

}  // namespace eqc
