// The coarse end of the multigrid V-cycle in one launch: a thread-block cluster of up to 16
// CTAs runs every level from `first` down to the dense coarsest solve, phase by phase, with a
// hardware cluster barrier (barrier.cluster, release/acquire) between phases.
//
// Why: below ~40K unknowns a level's kernels (stencil, Chebyshev update, residual, transfers)
// are latency-bound launches of 2-4 us each, ~40 per V-cycle.  Inside one cluster a phase
// costs one barrier plus an L2 round trip.  The level data (stencils, vectors; < 2 MB) stay
// L2-resident; values written inside the kernel are read with ld.global.cg (L2), so no L1
// line can be stale across CTAs.
//
// The arithmetic is the V-cycle of mg.cu (same smoother, transfers and dense coarse solve),
// with the Chebyshev step fused into the stencil pass: the direction vector is
// double-buffered (d <-> t), so one phase computes t = A d_old, r -= Dinv t,
// d_new = c1 d_old + c2 r and x += d_new.
#include "mg.h"
#include "epi.cuh"
#include "reduce.cuh"

namespace eqc {

__device__ __forceinline__ void cluster_sync_all() {
    // non-.aligned forms: threads of a warp may arrive after divergent point loops
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}
__device__ __forceinline__ unsigned cluster_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

template <class T> __device__ __forceinline__ T ldc(const T* p) { return __ldcg(p); }

// 9-point stencil (A_l x)_i at point (ix, iy), iy >= 1; x read through L2.
template <class T>
__device__ __forceinline__ T stencil_at(const T* __restrict__ A, const T* x, int ix, int iy, int cx, int cy, int64_t N) {
    const int64_t i = (int64_t)iy * cx + ix;
    T s = T(0);
#pragma unroll
    for (int k = 0; k < 9; ++k) {
        const int gx = ix + (k % 3) - 1, gy = iy + (k / 3) - 1;
        if (gx >= 0 && gx < cx && gy >= 1 && gy < cy) s += __ldg(A + k * N + i) * ldc(x + (int64_t)gy * cx + gx);
    }
    return s;
}

template <class T>
__global__ void __launch_bounds__(1024, 1) k_coarse_cycle(ClusterArgs<T> P) {
    EQC_GRID_WAIT();
    const int nthr = (int)(cluster_size() * blockDim.x);
    const int tid = (int)(cluster_rank() * blockDim.x + threadIdx.x);

    // ---------------- descent: pre-smooth, residual, restrict
    for (int l = 0; l < P.nlev; ++l) {
        const ClusterLevel<T>& L = P.lev[l];
        const int cx = L.cx, cy = L.cy;
        const int64_t N = (int64_t)cx * cy;
        T* x = L.x;
        T* r = L.r;
        T* d = L.d;
        T* dn = L.t;
        const T* b = L.b;
        // Chebyshev with x = 0: r = Dinv b, d = r / theta, x = d
        for (int64_t i = tid; i < N; i += nthr) {
            const T ri = L.Dinv[i] * ldc(b + i);
            const T di = ri * L.inv_theta;
            r[i] = ri;
            d[i] = di;
            x[i] = di;
        }
        cluster_sync_all();
        for (int k = 1; k < P.deg; ++k) {
            for (int64_t i = tid; i < N; i += nthr) {
                const int ix = (int)(i % cx), iy = (int)(i / cx);
                const T ti = iy >= 1 ? stencil_at(L.A, d, ix, iy, cx, cy, N) : T(0);
                T ri = ldc(r + i), di = ldc(d + i), xi = ldc(x + i);
                cheb_step_pt<T>(ri, di, xi, ti, L.Dinv[i], L.c1[k], L.c2[k]);
                r[i] = ri;
                dn[i] = di;
                x[i] = xi;
            }
            T* tmp = d; d = dn; dn = tmp;
            cluster_sync_all();
        }
        // residual r = b - A x
        for (int64_t i = tid; i < N; i += nthr) {
            const int ix = (int)(i % cx), iy = (int)(i / cx);
            const T ti = iy >= 1 ? stencil_at(L.A, x, ix, iy, cx, cy, N) : T(0);
            r[i] = ldc(b + i) - ti;
        }
        cluster_sync_all();
        // restrict to the next level's right-hand side (row 0 = 0)
        const int ncx = L.ncx, ncy = L.ncy;
        T* bc = (l + 1 < P.nlev) ? P.lev[l + 1].b : P.bd;
        for (int64_t c = tid; c < (int64_t)ncx * ncy; c += nthr) {
            const int cxi = (int)(c % ncx), cyi = (int)(c / ncx);
            T s = T(0);
            if (cyi >= 1) {
                for (int q = L.rpy[cyi]; q < L.rpy[cyi + 1]; ++q) {
                    const int fy = L.riy[q];
                    if (fy == 0) continue;
                    T sx = T(0);
                    for (int p = L.rpx[cxi]; p < L.rpx[cxi + 1]; ++p) sx += L.rwx[p] * ldc(r + (int64_t)fy * cx + L.rix[p]);
                    s += L.rwy[q] * sx;
                }
            }
            bc[c] = s;
        }
        cluster_sync_all();
    }

    // ---------------- coarsest: dense inverse on rows >= 1, one warp per row
    {
        const int warp = tid >> 5, lane = tid & 31, nwarp = nthr >> 5;
        for (int k = tid; k < P.dcx; k += nthr) P.xd[k] = T(0);
        for (int row = warp; row < P.nc; row += nwarp) {
            double s = 0.0;
            for (int j = lane; j < P.nc; j += 32) s += (double)__ldg(P.Cinv + (int64_t)row * P.nc + j) * (double)ldc(P.bd + P.dcx + j);
            s = warp_sum(s);
            if (lane == 0) P.xd[P.dcx + row] = (T)s;
        }
        cluster_sync_all();
    }

    // ---------------- ascent: prolong, post-smooth
    for (int l = P.nlev - 1; l >= 0; --l) {
        const ClusterLevel<T>& L = P.lev[l];
        const int cx = L.cx, cy = L.cy;
        const int64_t N = (int64_t)cx * cy;
        T* x = L.x;
        T* r = L.r;
        T* d = L.d;
        T* dn = L.t;
        const T* b = L.b;
        const T* xc = (l + 1 < P.nlev) ? P.lev[l + 1].x : P.xd;
        const int ldcx = L.ncx;
        // x += P xc (fine rows >= 1)
        for (int64_t i = tid; i < N; i += nthr) {
            const int ix = (int)(i % cx), iy = (int)(i / cx);
            if (iy == 0) continue;
            T s = T(0);
#pragma unroll
            for (int bb = 0; bb < 2; ++bb) {
                const T wb = L.wy[2 * iy + bb];
                if (wb == T(0)) continue;
                const int cyi = L.py[2 * iy + bb];
#pragma unroll
                for (int a = 0; a < 2; ++a) {
                    const T wa = L.wx[2 * ix + a];
                    if (wa != T(0)) s += wa * wb * ldc(xc + (int64_t)cyi * ldcx + L.px[2 * ix + a]);
                }
            }
            x[i] = ldc(x + i) + s;
        }
        cluster_sync_all();
        // Chebyshev with x: r = Dinv (b - A x), d = r / theta; x += d is applied by the next
        // phase (x is still being read by this one)
        for (int64_t i = tid; i < N; i += nthr) {
            const int ix = (int)(i % cx), iy = (int)(i / cx);
            const T ti = iy >= 1 ? stencil_at(L.A, x, ix, iy, cx, cy, N) : T(0);
            const T ri = L.Dinv[i] * (ldc(b + i) - ti);
            r[i] = ri;
            d[i] = ri * L.inv_theta;
        }
        cluster_sync_all();
        if (P.deg == 1) {
            for (int64_t i = tid; i < N; i += nthr) x[i] = ldc(x + i) + ldc(d + i);
            cluster_sync_all();
        }
        for (int k = 1; k < P.deg; ++k) {
            for (int64_t i = tid; i < N; i += nthr) {
                const int ix = (int)(i % cx), iy = (int)(i / cx);
                const T ti = iy >= 1 ? stencil_at(L.A, d, ix, iy, cx, cy, N) : T(0);
                const T dold = ldc(d + i);
                T ri = ldc(r + i), di = dold, xi = (k == 1) ? add_rn<T>(ldc(x + i), dold) : ldc(x + i);
                cheb_step_pt<T>(ri, di, xi, ti, L.Dinv[i], L.c1[k], L.c2[k]);
                r[i] = ri;
                dn[i] = di;
                x[i] = xi;
            }
            T* tmp = d; d = dn; dn = tmp;
            cluster_sync_all();
        }
    }
}

// Largest cluster size (16 non-portable, else 8, ...) the device co-schedules with 1024-thread CTAs.
static int pick_cluster(const void* fn) {
    for (int cs : {16, 8, 4, 2}) {
        cudaLaunchConfig_t cfg = {};
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cs;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.gridDim = dim3(cs);
        cfg.blockDim = dim3(1024);
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, fn, &cfg) == cudaSuccess && n > 0) return cs;
        cudaGetLastError();
    }
    return 0;
}

template <class T>
int cluster_setup() {
    const void* fn = (const void*)k_coarse_cycle<T>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return pick_cluster(fn);
}

template <class T>
void cluster_cycle(const ClusterArgs<T>& P, int cluster, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = cluster;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3(cluster);
    cfg.blockDim = dim3(1024);
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    EQC_CUDA(cudaLaunchKernelEx(&cfg, k_coarse_cycle<T>, P));
    count_launch();
}

template int cluster_setup<float>();
template int cluster_setup<double>();
template void cluster_cycle<float>(const ClusterArgs<float>&, int, cudaStream_t);
template void cluster_cycle<double>(const ClusterArgs<double>&, int, cudaStream_t);

}  // namespace eqc
