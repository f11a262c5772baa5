// K1: matrix-free spectral-element stiffness apply  y = sign * K x.
//
// Replaces the assembled SpMV Ksparse*x of src/main.jl:246,267,311 with the element
// form of src/PCG.jl:82 (element_computation!):
//     a_e = c1 * H * (W_e .* (H' u_e)) + c2 * (W_e .* (u_e H)) * H'
// scattered through the connectivity (the Conn product of src/PCG.jl:266).
//
// GB300 design.  The mesh is structured, so node indices are computed, not loaded; every
// node sums its element contributions in a fixed order (deterministic, no atomics, bitwise
// reproducible).  Per element the work is 5 x-lines and 5 y-lines (sum factorisation: two
// 5-point contractions per line).  Kernels, by apply_variant:
//   k_apply_rows   FP32, one lane per element, one warp per element row, ROWS rows per CTA
//                  plus a halo warp (variants 0, 4-7; the FP32 default);
//   k_apply_walk   the same arithmetic fed by TMA, one wave of CTAs each walking up a strip
//                  (variant 8; the autotuner's usual choice);
//   k_apply_pipe   persistent tiles with a TMA pipeline, node-line form (the FP64 default,
//                  FP32 variant 3); k_apply_tma / k_apply_lines: one tile per CTA (1, 2);
//   k_apply        the strip modes 2 and 3 (first element row only).
// The FP32 element kernels take an epilogue (epi.cuh) that finishes the V-cycle's residual or
// Chebyshev step at each owned node.
#include "model.h"
#include "vec.cuh"
#include "epi.cuh"
#include <cstdlib>
#include <cmath>
#include <type_traits>
#include <algorithm>

namespace eqc {

__constant__ double cH64[25];  // H[i + 5*j] = h'_i(x_j)
__constant__ float cH32[25];

template <class T> __device__ __forceinline__ T Hc(int i, int j);
template <> __device__ __forceinline__ double Hc<double>(int i, int j) { return cH64[i + 5 * j]; }
template <> __device__ __forceinline__ float Hc<float>(int i, int j) { return cH32[i + 5 * j]; }


// mode 0: full apply, every owned node written
// mode 1: full apply, fault row (iy = 0) written as zero (interior operator K_II)
// mode 2: fault strip: only element row 0, x rows > 0 read as zero, rows 1..4 written
//         (y_I = K_IF x_F, the right-hand side of the quasi-static solve)
// mode 3: fault strip: only element row 0, row 0 written (fault traction (K d)[iFlt])
template <class T, int TEX, int TEY>
__global__ void __launch_bounds__(256) k_apply(const T* __restrict__ x, T* __restrict__ y, ApplyArgs<T> A,
                                               T sign, int mode) {
    EQC_GRID_WAIT();
    if (A.gate && *A.gate != A.gate_val) return;
    const Layout L = A.L;
    const bool strip = mode >= 2;
    const int ex0 = blockIdx.x * TEX;
    const int ey0 = strip ? 0 : blockIdx.y * TEY;
    const int exs = max(ex0 - 1, 0), exe = min(ex0 + TEX, L.NelX);
    const int eys = strip ? 0 : max(ey0 - 1, 0);
    const int eye = strip ? 1 : min(ey0 + TEY, L.NelY);
    const int nex = exe - exs, ney = eye - eys, nE = nex * ney;
    const int tnx = 4 * nex + 1, tny = 4 * ney + 1;
    const int ix0 = 4 * exs, iy0 = 4 * eys;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* us = reinterpret_cast<T*>(smem_raw);
    constexpr int USZ = (4 * (TEX + 1) + 1) * (4 * (TEY + 1) + 1);
    constexpr int ESZ = (TEX + 1) * (TEY + 1) * 25;
    T* Ws = us + USZ;
    T* yl = Ws + ESZ;

    for (int k = threadIdx.x; k < tnx * tny; k += blockDim.x) {
        const int a = k % tnx, b = k / tnx;
        T v = x[(int64_t)(iy0 + b) * L.ld + ix0 + a];
        if (mode == 2 && (iy0 + b) > 0) v = T(0);
        us[k] = v;
    }
    for (int k = threadIdx.x; k < nE * 25; k += blockDim.x) {
        const int le = k / 25, q = k - 25 * le;
        const int lex = le % nex, ley = le / nex;
        Ws[k] = A.W[((int64_t)(eys + ley) * L.NelX + exs + lex) * 25 + q];
    }
    __syncthreads();

    // x-lines: for element le and GLL row j, contract along xi.
    for (int t = threadIdx.x; t < nE * 5; t += blockDim.x) {
        const int le = t / 5, j = t - 5 * le;
        const int lex = le % nex, ley = le / nex;
        const T* ul = us + (4 * ley + j) * tnx + 4 * lex;
        const T* w = Ws + le * 25;
        T u[5], s[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) u[k] = ul[k];
#pragma unroll
        for (int p = 0; p < 5; ++p) {
            T acc = T(0);
#pragma unroll
            for (int k = 0; k < 5; ++k) acc += Hc<T>(k, p) * u[k];
            s[p] = w[p + 5 * j] * acc;
        }
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            T acc = T(0);
#pragma unroll
            for (int p = 0; p < 5; ++p) acc += Hc<T>(i, p) * s[p];
            yl[le * 25 + i + 5 * j] = A.c1 * acc;
        }
    }
    __syncthreads();
    // y-lines: for element le and GLL column i, contract along eta.
    for (int t = threadIdx.x; t < nE * 5; t += blockDim.x) {
        const int le = t / 5, i = t - 5 * le;
        const int lex = le % nex, ley = le / nex;
        const T* ul = us + (4 * ley) * tnx + 4 * lex + i;
        const T* w = Ws + le * 25;
        T u[5], s[5];
#pragma unroll
        for (int l = 0; l < 5; ++l) u[l] = ul[l * tnx];
#pragma unroll
        for (int p = 0; p < 5; ++p) {
            T acc = T(0);
#pragma unroll
            for (int l = 0; l < 5; ++l) acc += u[l] * Hc<T>(l, p);
            s[p] = w[i + 5 * p] * acc;
        }
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            T acc = T(0);
#pragma unroll
            for (int p = 0; p < 5; ++p) acc += s[p] * Hc<T>(j, p);
            yl[le * 25 + i + 5 * j] += A.c2 * acc;
        }
    }
    __syncthreads();

    // Gather for owned nodes.
    const int ixb = 4 * ex0;
    const int ixe = (ex0 + TEX >= L.NelX) ? L.nx : 4 * (ex0 + TEX);
    int iyb, iye;
    if (mode == 2) { iyb = 1; iye = 5; }
    else if (mode == 3) { iyb = 0; iye = 1; }
    else { iyb = 4 * ey0; iye = (ey0 + TEY >= L.NelY) ? L.ny : 4 * (ey0 + TEY); }
    const int ownx = ixe - ixb, nown = ownx * (iye - iyb);
    for (int k = threadIdx.x; k < nown; k += blockDim.x) {
        const int ix = ixb + k % ownx, iy = iyb + k / ownx;
        int exA, iA, exB = -1, iB = 0;
        if (ix == 0) { exA = 0; iA = 0; }
        else if (ix == L.nx - 1) { exA = L.NelX - 1; iA = 4; }
        else if ((ix & 3) == 0) { exA = (ix >> 2) - 1; iA = 4; exB = ix >> 2; iB = 0; }
        else { exA = ix >> 2; iA = ix & 3; }
        int eyA, jA, eyB = -1, jB = 0;
        if (iy == 0) { eyA = 0; jA = 0; }
        else if (iy == L.ny - 1) { eyA = L.NelY - 1; jA = 4; }
        else if ((iy & 3) == 0) { eyA = (iy >> 2) - 1; jA = 4; eyB = iy >> 2; jB = 0; }
        else { eyA = iy >> 2; jA = iy & 3; }
        if (strip && eyB >= 1) eyB = -1;   // strip modes: element row 0 only
        T acc = T(0);
        acc += yl[((eyA - eys) * nex + exA - exs) * 25 + iA + 5 * jA];
        if (exB >= 0) acc += yl[((eyA - eys) * nex + exB - exs) * 25 + iB + 5 * jA];
        if (eyB >= 0) {
            acc += yl[((eyB - eys) * nex + exA - exs) * 25 + iA + 5 * jB];
            if (exB >= 0) acc += yl[((eyB - eys) * nex + exB - exs) * 25 + iB + 5 * jB];
        }
        T out = sign * acc;
        if (mode == 1 && iy == 0) out = T(0);
        y[(int64_t)iy * L.ld + ix] = out;
    }
}

// ---------------------------------------------------------------------------------------
// Full apply (modes 0 and 1), node-line formulation.
//
// For a node row iy the x-derivative part of K x is, element column by element column,
//   y1 = c1 * H * (Wrow .* (H' u_row))   with Wrow[p] = sum over the element rows holding iy
// of W_e[p, j_e] (one row inside an element, two on an element boundary: the operator is
// linear in W, so the two element rows collapse into one line).  Likewise every node column
// gives one y-line with the summed W column.  A CTA owns nodes [4ex0, 4ex0+4TEX) x
// [4ey0, 4ey0+4TEY) and runs one x-line item per (owned node row, element column incl. the
// left halo element) and one y-line item per (owned node column, element row incl. the
// bottom halo element).  An item writes its 4 owned outputs and hands the 5th (the shared
// endpoint, owned by the neighbour item) through a small shared array; the final pass adds
// those carries in a fixed order (deterministic, no atomics).  Elements outside the mesh
// act as W = 0, so the one extra CTA row/column that owns the last node line needs no
// special case.
// Even-odd form of the 5-point line contractions (the GLL derivative matrix is centro-
// antisymmetric, D(4-p, 4-k) = -D(p, k)): with e_m = v_m + v_(4-m), o_m = v_m - v_(4-m),
//   s_p, s_(4-p) = P +- Q,  P = sum_m a_pm o_m,  Q = sum_m b_pm e_m + g_p v_2   (p = 0, 1)
//   s_2 = sum_m d_m o_m,    a = (D(p,m) - D(p,4-m)) / 2, b = (D(p,m) + D(p,4-m)) / 2, g = D(p,2),
// 20 operations instead of 25 multiply-adds (Solomonoff's even-odd decomposition of spectral
// differentiation).  EO[0] holds the coefficients of s_p = sum_k H(k,p) v_k (the first
// contraction of a line), EO[1] those of o_i = sum_p H(i,p) s_p (the second).
struct EOCoef {
    float a[2][2], b[2][2], g[2], d[2];
};
struct EOCoef64 {   // the same coefficients for the FP64 kernels
    double a[2][2], b[2][2], g[2], d[2];
};
__constant__ EOCoef cEO[2];
__constant__ EOCoef64 cEO64[2];
__constant__ int cEO_ok;   // H is centro-antisymmetric (else the full contractions are used)

__device__ __forceinline__ void eo5(const float (&v)[5], float (&s)[5], const EOCoef& c) {
    const float e0 = v[0] + v[4], e1 = v[1] + v[3], o0 = v[0] - v[4], o1 = v[1] - v[3];
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        const float P = fmaf(c.a[p][1], o1, c.a[p][0] * o0);
        const float Q = fmaf(c.g[p], v[2], fmaf(c.b[p][1], e1, c.b[p][0] * e0));
        s[p] = P + Q;
        s[4 - p] = P - Q;
    }
    s[2] = fmaf(c.d[1], o1, c.d[0] * o0);
}

__device__ __forceinline__ void eo5(const double (&v)[5], double (&s)[5], const EOCoef64& c) {
    const double e0 = v[0] + v[4], e1 = v[1] + v[3], o0 = v[0] - v[4], o1 = v[1] - v[3];
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        const double P = fma(c.a[p][1], o1, c.a[p][0] * o0);
        const double Q = fma(c.g[p], v[2], fma(c.b[p][1], e1, c.b[p][0] * e0));
        s[p] = P + Q;
        s[4 - p] = P - Q;
    }
    s[2] = fma(c.d[1], o1, c.d[0] * o0);
}

// The FP64 node-line kernels take the even-odd contractions where H allows (FP64 issue rate
// bounds them on GB300: 20 operations per contraction instead of 25); the FP32 ones keep the
// full form.
template <class T> __device__ __forceinline__ bool eo_lines() { return false; }
template <> __device__ __forceinline__ bool eo_lines<double>() { return cEO_ok != 0; }
template <class T> struct EOSel;
template <> struct EOSel<float> {
    static __device__ __forceinline__ const EOCoef& c(int k) { return cEO[k]; }
};
template <> struct EOSel<double> {
    static __device__ __forceinline__ const EOCoef64& c(int k) { return cEO64[k]; }
};

// Line items and output pass shared by both full-apply kernels.  us: node tile with row
// pitch UP; ws: element tile, element stride WP, EX elements per row.
template <class T, int TEX, int TEY, int NT, int UP, int WP>
__device__ __forceinline__ void lines_compute(const T* __restrict__ us, const T* __restrict__ ws, T* ys, T* cx,
                                              T* cy, T* __restrict__ y, const ApplyArgs<T>& A, int ex0, int ey0,
                                              T sign, int zero_row0) {
    const Layout& L = A.L;
    constexpr int OX = 4 * TEX, OY = 4 * TEY;
    constexpr int EX = TEX + 1, EY = TEY + 1;
    // x-lines: item = (owned node row r, element column c = 0..TEX, c = 0 the left halo)
    for (int t = threadIdx.x; t < OY * EX; t += NT) {
        const int r = t / EX, c = t - r * EX;
        const int er = (r >> 2) + 1, j = r & 3;
        const T* ul = us + (r + 4) * UP + 4 * c;
        const T* w1 = ws + (er * EX + c) * WP + 5 * j;
        const T* w0 = ws + ((er - 1) * EX + c) * WP + 20;
        T u[5], s[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) u[k] = ul[k];
        T o[5];
        if (eo_lines<T>()) {
            eo5(u, s, EOSel<T>::c(0));
#pragma unroll
            for (int p = 0; p < 5; ++p) s[p] *= (j == 0) ? w1[p] + w0[p] : w1[p];
            eo5(s, o, EOSel<T>::c(1));
#pragma unroll
            for (int i = 0; i < 5; ++i) o[i] = A.c1 * o[i];
        } else {
#pragma unroll
            for (int p = 0; p < 5; ++p) {
                T acc = T(0);
#pragma unroll
                for (int k = 0; k < 5; ++k) acc += Hc<T>(k, p) * u[k];
                const T wr = (j == 0) ? w1[p] + w0[p] : w1[p];
                s[p] = wr * acc;
            }
#pragma unroll
            for (int i = 0; i < 5; ++i) {
                T acc = T(0);
#pragma unroll
                for (int p = 0; p < 5; ++p) acc += Hc<T>(i, p) * s[p];
                o[i] = A.c1 * acc;
            }
        }
        if (c > 0) {
#pragma unroll
            for (int i = 0; i < 4; ++i) ys[r * OX + 4 * (c - 1) + i] = o[i];
        }
        cx[r * EX + c] = o[4];
    }
    __syncthreads();
    // y-lines: item = (owned node column q, element row er = 0..TEY, er = 0 the bottom halo)
    for (int t = threadIdx.x; t < EY * OX; t += NT) {
        const int er = t / OX, q = t - er * OX;
        const int ec = (q >> 2) + 1, i = q & 3;
        const T* ul = us + (4 * er) * UP + q + 4;
        const T* w1 = ws + (er * EX + ec) * WP + i;
        const T* w0 = ws + (er * EX + ec - 1) * WP + 4;
        T u[5], s[5];
#pragma unroll
        for (int l = 0; l < 5; ++l) u[l] = ul[l * UP];
        T o[5];
        if (eo_lines<T>()) {
            eo5(u, s, EOSel<T>::c(0));
#pragma unroll
            for (int p = 0; p < 5; ++p) s[p] *= (i == 0) ? w1[5 * p] + w0[5 * p] : w1[5 * p];
            eo5(s, o, EOSel<T>::c(1));
#pragma unroll
            for (int jj = 0; jj < 5; ++jj) o[jj] = A.c2 * o[jj];
        } else {
#pragma unroll
            for (int p = 0; p < 5; ++p) {
                T acc = T(0);
#pragma unroll
                for (int l = 0; l < 5; ++l) acc += u[l] * Hc<T>(l, p);
                const T wc = (i == 0) ? w1[5 * p] + w0[5 * p] : w1[5 * p];
                s[p] = wc * acc;
            }
#pragma unroll
            for (int jj = 0; jj < 5; ++jj) {
                T acc = T(0);
#pragma unroll
                for (int p = 0; p < 5; ++p) acc += s[p] * Hc<T>(jj, p);
                o[jj] = A.c2 * acc;
            }
        }
        if (er > 0) {
#pragma unroll
            for (int jj = 0; jj < 4; ++jj) ys[(4 * (er - 1) + jj) * OX + q] += o[jj];
        }
        cy[er * OX + q] = o[4];
    }
    __syncthreads();
    for (int k = threadIdx.x; k < OY * OX; k += NT) {
        const int r = k / OX, q = k - r * OX;
        const int ix = 4 * ex0 + q, iy = 4 * ey0 + r;
        if (ix >= L.nx || iy >= L.ny) continue;
        T v = ys[k];
        if ((q & 3) == 0) v += cx[r * EX + (q >> 2)];
        if ((r & 3) == 0) v += cy[(r >> 2) * OX + q];
        v = sign * v;
        if (zero_row0 && iy == 0) v = T(0);
        y[(int64_t)iy * L.ld + ix] = v;
    }
}

template <class T, int TEX, int TEY, int NT>
__global__ void __launch_bounds__(NT) k_apply_lines(const T* __restrict__ x, T* __restrict__ y, ApplyArgs<T> A,
                                                    T sign, int zero_row0) {
    EQC_GRID_WAIT();
    if (A.gate && *A.gate != A.gate_val) return;
    const Layout L = A.L;
    constexpr int UX = 4 * TEX + 5, UY = 4 * TEY + 5;   // node tile incl. one halo element
    constexpr int OX = 4 * TEX, OY = 4 * TEY;           // owned nodes
    constexpr int EX = TEX + 1, EY = TEY + 1;           // elements incl. halo
    __shared__ T us[UY * UX];
    __shared__ T ws[EY * EX * 25];
    __shared__ T ys[OY * OX];
    __shared__ T cx[OY * EX];   // x-line endpoint carries [row][element column]
    __shared__ T cy[EY * OX];   // y-line endpoint carries [element row][column]
    const int ex0 = blockIdx.x * TEX, ey0 = blockIdx.y * TEY;
    const int ix0 = 4 * ex0 - 4, iy0 = 4 * ey0 - 4;

    // Issue every tile load of this thread before the first shared-memory store, so that
    // all of them are in flight together (compile-time trip counts, predicated).
    constexpr int NU = (UY * UX + NT - 1) / NT, NWL = (EY * EX * 25 + NT - 1) / NT;
    T ur[NU], wr[NWL];
#pragma unroll
    for (int it = 0; it < NU; ++it) {
        const int k = threadIdx.x + it * NT;
        const int b = k / UX, a = k - b * UX;
        const int ix = ix0 + a, iy = iy0 + b;
        ur[it] = (k < UY * UX && ix >= 0 && ix < L.nx && iy >= 0 && iy < L.ny) ? __ldg(x + (int64_t)iy * L.ld + ix)
                                                                                : T(0);
    }
#pragma unroll
    for (int it = 0; it < NWL; ++it) {
        const int k = threadIdx.x + it * NT;
        const int le = k / 25, q = k - le * 25;
        const int er = le / EX, ec = le - er * EX;
        const int ex = ex0 - 1 + ec, ey = ey0 - 1 + er;
        wr[it] = (k < EY * EX * 25 && ex >= 0 && ex < L.NelX && ey >= 0 && ey < L.NelY)
                     ? __ldg(A.W + ((int64_t)ey * L.NelX + ex) * 25 + q)
                     : T(0);
    }
#pragma unroll
    for (int it = 0; it < NU; ++it) {
        const int k = threadIdx.x + it * NT;
        if (k < UY * UX) us[k] = ur[it];
    }
#pragma unroll
    for (int it = 0; it < NWL; ++it) {
        const int k = threadIdx.x + it * NT;
        if (k < EY * EX * 25) ws[k] = wr[it];
    }
    __syncthreads();

    lines_compute<T, TEX, TEY, NT, UX, 25>(us, ws, ys, cx, cy, y, A, ex0, ey0, sign, zero_row0);
}

// ---- TMA version -------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// 2-D tiled bulk tensor load global -> shared, completion counted on the mbarrier.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

constexpr int UPT = 40;                    // node-tile row pitch of the TMA box (16-byte multiple)

// Full apply with the node tile and the element tile fetched by TMA.  The node box starts at
// x = 4*ex0 - 4 (a multiple of 4 elements, hence 16-byte aligned) and the hardware fills
// coordinates outside the grid with zeros; the element box starts at element ex0 - 1 of a
// copy of W padded to WPad values per element.
template <class T, int TEX, int TEY, int NT>
__global__ void __launch_bounds__(NT) k_apply_tma(const __grid_constant__ CUtensorMap umap,
                                                  const __grid_constant__ CUtensorMap wmap, T* __restrict__ y,
                                                  ApplyArgs<T> A, T sign, int zero_row0) {
    EQC_GRID_WAIT();
    if (A.gate && *A.gate != A.gate_val) return;
    constexpr int UY = 4 * TEY + 5;
    constexpr int OX = 4 * TEX, OY = 4 * TEY;
    constexpr int EX = TEX + 1, EY = TEY + 1;
    constexpr int WP = WPad<T>::v;
    __shared__ __align__(128) T us[UY * UPT];
    __shared__ __align__(128) T ws[EY * EX * WP];
    __shared__ T ys[OY * OX];
    __shared__ T cx[OY * EX];
    __shared__ T cy[EY * OX];
    __shared__ __align__(8) uint64_t bar;
    const int ex0 = blockIdx.x * TEX, ey0 = blockIdx.y * TEY;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, (uint32_t)(sizeof(T) * (UY * UPT + EY * EX * WP)));
        tma_load_2d(us, &umap, &bar, 4 * ex0 - 4, 4 * ey0 - 4);
        tma_load_2d(ws, &wmap, &bar, (ex0 - 1) * WP, ey0 - 1);
    }
    bool done = false;
    for (int it = 0; it < A.wait_polls && !done; ++it) done = mbar_try_wait(&bar, 0);
    if (__syncthreads_or(!done)) {
        // give up (every thread of the CTA alike): flag it, wait (bounded) for the copies still
        // targeting this CTA, leave
        if (threadIdx.x == 0) {
            if (A.err) atomicExch(A.err, 1);
            for (int it = 0; it < MBAR_SPIN_LIMIT; ++it)
                if (mbar_try_wait(&bar, 0)) break;
        }
        return;
    }
    lines_compute<T, TEX, TEY, NT, UPT, WP>(us, ws, ys, cx, cy, y, A, ex0, ey0, sign, zero_row0);
}

// ---- persistent, pipelined version ---------------------------------------------------------
// A grid of a few CTAs per SM walks the tile list (tile t = blockIdx.x + k*gridDim.x); each CTA
// keeps PSTAGES tiles in flight: the node and element tiles of tile i+PSTAGES are fetched by
// TMA while tile i is computed, so HBM streams continuously instead of once per CTA lifetime.
constexpr int PSTAGES = 3;

template <class T, int TEX, int TEY>
struct PipeLayout {
    static constexpr int UY = 4 * TEY + 5, OX = 4 * TEX, OY = 4 * TEY, EX = TEX + 1, EY = TEY + 1;
    static constexpr int WP = WPad<T>::v;
    static constexpr int U_BYTES = UY * UPT * (int)sizeof(T);            // node tile
    static constexpr int W_BYTES = EY * EX * WP * (int)sizeof(T);        // element tile
    static constexpr int STAGE = ((U_BYTES + 127) / 128 + (W_BYTES + 127) / 128) * 128;
    static constexpr int WORK = (OY * OX + OY * EX + EY * OX) * (int)sizeof(T);
    static constexpr int BYTES = PSTAGES * STAGE + ((WORK + 127) / 128) * 128 + 8 * PSTAGES;
};

template <class T, int TEX, int TEY, int NT>
__global__ void __launch_bounds__(NT) k_apply_pipe(const __grid_constant__ CUtensorMap umap,
                                                   const __grid_constant__ CUtensorMap wmap, T* __restrict__ y,
                                                   ApplyArgs<T> A, T sign, int zero_row0, int ntx, int ntiles) {
    EQC_GRID_WAIT();
    if (A.gate && *A.gate != A.gate_val) return;
    using PL = PipeLayout<T, TEX, TEY>;
    extern __shared__ __align__(128) unsigned char smem[];
    T* ys = reinterpret_cast<T*>(smem + PSTAGES * PL::STAGE);
    T* cxs = ys + PL::OY * PL::OX;
    T* cys = cxs + PL::OY * PL::EX;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + PSTAGES * PL::STAGE + ((PL::WORK + 127) / 128) * 128);
    auto us_of = [&](int st) { return reinterpret_cast<T*>(smem + st * PL::STAGE); };
    auto ws_of = [&](int st) { return reinterpret_cast<T*>(smem + st * PL::STAGE + ((PL::U_BYTES + 127) / 128) * 128); };
    auto issue = [&](int t, int st) {
        const int ex0 = (t % ntx) * TEX, ey0 = (t / ntx) * TEY;
        mbar_expect_tx(&bar[st], (uint32_t)(PL::U_BYTES + PL::W_BYTES));
        tma_load_2d(us_of(st), &umap, &bar[st], 4 * ex0 - 4, 4 * ey0 - 4);
        tma_load_2d(ws_of(st), &wmap, &bar[st], (ex0 - 1) * PL::WP, ey0 - 1);
    };
    if (threadIdx.x == 0) {
        for (int st = 0; st < PSTAGES; ++st) mbar_init(&bar[st], 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int st = 0; st < PSTAGES; ++st) {
            const int t = blockIdx.x + st * gridDim.x;
            if (t < ntiles) issue(t, st);
        }
    int i = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
        const int st = i % PSTAGES;
        const uint32_t parity = (uint32_t)((i / PSTAGES) & 1);
        bool done = false;
        const int polls = i == 0 ? A.wait_polls : MBAR_SPIN_LIMIT;
        for (int it = 0; it < polls && !done; ++it) done = mbar_try_wait(&bar[st], parity);
        if (__syncthreads_or(!done)) {
            // give up: flag it, wait (bounded) for every copy still targeting this CTA, leave
            if (threadIdx.x == 0) {
                if (A.err) atomicExch(A.err, 1);
                int j = i;
                for (int tt = t; tt < ntiles && j < i + PSTAGES; tt += gridDim.x, ++j) {
                    const int sj = j % PSTAGES;
                    const uint32_t pj = (uint32_t)((j / PSTAGES) & 1);
                    for (int it = 0; it < MBAR_SPIN_LIMIT; ++it)
                        if (mbar_try_wait(&bar[sj], pj)) break;
                }
            }
            return;
        }
        const int ex0 = (t % ntx) * TEX, ey0 = (t / ntx) * TEY;
        lines_compute<T, TEX, TEY, NT, UPT, PL::WP>(us_of(st), ws_of(st), ys, cxs, cys, y, A, ex0, ey0, sign,
                                                    zero_row0);
        __syncthreads();   // every thread is done with this stage and with ys/cx/cy
        if (threadIdx.x == 0) {
            const int tn = t + PSTAGES * gridDim.x;
            if (tn < ntiles) issue(tn, st);
        }
    }
}

// ---- element-per-lane version (FP32) --------------------------------------------------------
// One lane per element, one warp per element row of 31 elements plus a halo lane (lane 0 = the
// element left of the strip), ROWS element rows per CTA plus a halo warp (warp 0 = the row
// below the group).  Every lane contracts its element's 5 x-lines and 5 y-lines in registers
// (no W merging across elements): the 4 x 4 nodes it owns (local i, j < 4) are complete once the
// right-column contributions of the left lane (shuffle) and the top-row contributions of the warp
// below (shared memory, one barrier) are added.  Node rows arrive as 16-byte loads (the 5th node
// of a row is the next lane's first), element data as seven 16-byte loads of the padded W copy.
// The last node row and column are owned by a virtual element row / column with W = 0.
constexpr unsigned FULLMASK = 0xffffffffu;

// The 5 x-lines and 5 y-lines of one element (u: its 5 x 5 nodes, W: its 25 weights): the owned
// outputs out[j][i] (i, j < 4), the right column R[j] (j < 4) and the top row T[i] (i <= 4).
// top_only: only T is needed (the halo row).
template <class WAcc>
__device__ __forceinline__ void rows_lines_t(const float (&u)[5][5], const WAcc& W, float c1, float c2,
                                           bool top_only, float (&out)[4][4], float (&R)[4], float (&T)[5]) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
        for (int i = 0; i < 4; ++i) out[j][i] = 0.f;
    // x-lines (the halo warp needs only the top one)
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        if (top_only && j < 4) continue;
        float sp[5];
#pragma unroll
        for (int p = 0; p < 5; ++p) {
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < 5; ++k) acc += Hc<float>(k, p) * u[j][k];
            sp[p] = W[p + 5 * j] * acc;
        }
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            float acc = 0.f;
#pragma unroll
            for (int p = 0; p < 5; ++p) acc += Hc<float>(i, p) * sp[p];
            const float o = c1 * acc;
            if (j < 4) {
                if (i < 4) out[j][i] = o;
                else R[j] = o;
            } else {
                T[i] = o;
            }
        }
    }
    // y-lines
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        float sp[5];
#pragma unroll
        for (int p = 0; p < 5; ++p) {
            float acc = 0.f;
#pragma unroll
            for (int l = 0; l < 5; ++l) acc += u[l][i] * Hc<float>(l, p);
            sp[p] = W[i + 5 * p] * acc;
        }
#pragma unroll
        for (int jj = 0; jj < 5; ++jj) {
            float acc = 0.f;
#pragma unroll
            for (int p = 0; p < 5; ++p) acc += sp[p] * Hc<float>(jj, p);
            const float o = c2 * acc;
            if (jj < 4) {
                if (i < 4) out[jj][i] += o;
                else R[jj] += o;
            } else {
                T[i] += o;
            }
        }
    }
}

__device__ __forceinline__ void rows_lines_eo(const float (&u)[5][5], const float (&W)[28], float c1, float c2,
                                              bool top_only, float (&out)[4][4], float (&R)[4], float (&T)[5]) {
    // x-lines
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        if (top_only && j < 4) {   // the halo row needs only its top row T
#pragma unroll
            for (int i = 0; i < 4; ++i) out[j][i] = 0.f;
            R[j] = 0.f;
            continue;
        }
        float s[5], o[5];
        eo5(u[j], s, cEO[0]);
#pragma unroll
        for (int p = 0; p < 5; ++p) s[p] *= W[p + 5 * j];
        eo5(s, o, cEO[1]);
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            const float v = c1 * o[i];
            if (j < 4) {
                if (i < 4) out[j][i] = v;
                else R[j] = v;
            } else {
                T[i] = v;
            }
        }
    }
    // y-lines
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        float v[5], s[5], o[5];
#pragma unroll
        for (int l = 0; l < 5; ++l) v[l] = u[l][i];
        eo5(v, s, cEO[0]);
#pragma unroll
        for (int p = 0; p < 5; ++p) s[p] *= W[i + 5 * p];
        eo5(s, o, cEO[1]);
#pragma unroll
        for (int jj = 0; jj < 5; ++jj) {
            if (top_only && jj < 4) continue;
            const float w = c2 * o[jj];
            if (jj < 4) {
                if (i < 4) out[jj][i] += w;
                else R[jj] += w;
            } else {
                T[i] += w;
            }
        }
    }
}

__device__ __forceinline__ void rows_lines(const float (&u)[5][5], const float (&W)[28], float c1, float c2,
                                           bool top_only, float (&out)[4][4], float (&R)[4], float (&T)[5]) {
    if (cEO_ok) rows_lines_eo(u, W, c1, c2, top_only, out, R, T);
    else rows_lines_t(u, W, c1, c2, top_only, out, R, T);
}

template <int ROWS, int MINB>
__global__ void __launch_bounds__(32 * (ROWS + 1), MINB) k_apply_rows(const float* __restrict__ x, float* __restrict__ y,
                                                                     ApplyArgs<float> A, float sign, int zero_row0,
                                                                     OpEpi<float> E) {
    const Layout L = A.L;
    __shared__ float Ts[ROWS + 1][5][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ex = (int)blockIdx.x * 31 - 1 + lane;
    const int ey = (int)blockIdx.y * ROWS - 1 + w;
    const bool real = ex >= 0 && ex < L.NelX && ey >= 0 && ey < L.NelY;
    // the element data are constant (written only between launches, by the host): their loads
    // are issued before the wait for the grids this launch depends on, so they overlap the
    // predecessor's tail when the launch is programmatic
    float4 wq[7];
    const float4* wp = reinterpret_cast<const float4*>(A.Wp + ((int64_t)(real ? ey : 0) * L.NelX + (real ? ex : 0)) * 28);
#pragma unroll
    for (int k = 0; k < 7; ++k) wq[k] = real ? __ldg(wp + k) : make_float4(0.f, 0.f, 0.f, 0.f);
    EQC_GRID_WAIT();
    if (A.gate && *A.gate != A.gate_val) return;

    // every load of the lane is issued before the first use (one memory latency, not twelve)
    float4 v[5];
    float n4s[5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        const int iy = 4 * ey + j;
        const bool rowok = iy >= 0 && iy < L.ny;
        v[j] = (rowok && ex >= 0 && 4 * ex < L.nx) ? __ldg(reinterpret_cast<const float4*>(x + (int64_t)iy * L.ld + 4 * ex))
                                                   : make_float4(0.f, 0.f, 0.f, 0.f);
        const int ix = 4 * ex + 4;
        n4s[j] = (lane == 31 && rowok && ix >= 0 && ix < L.nx) ? __ldg(x + (int64_t)iy * L.ld + ix) : 0.f;
    }
    float u[5][5];
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        u[j][0] = v[j].x;
        u[j][1] = v[j].y;
        u[j][2] = v[j].z;
        u[j][3] = v[j].w;
        const float n4 = __shfl_down_sync(FULLMASK, v[j].x, 1);
        u[j][4] = lane == 31 ? n4s[j] : n4;
    }
    float W[28];
#pragma unroll
    for (int k = 0; k < 7; ++k) {
        W[4 * k] = wq[k].x;
        W[4 * k + 1] = wq[k].y;
        W[4 * k + 2] = wq[k].z;
        W[4 * k + 3] = wq[k].w;
    }

    float out[4][4], R[4], T[5];
    rows_lines(u, W, A.c1, A.c2, w == 0, out, R, T);
#pragma unroll
    for (int i = 0; i < 5; ++i) Ts[w][i][lane] = T[i];
    float Rl[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) Rl[j] = __shfl_up_sync(FULLMASK, R[j], 1);
    __syncthreads();
    if (w == 0 || lane == 0 || ex > L.NelX || ey > L.NelY) return;
    // contributions of the left element (right column) and of the element row below (top row)
#pragma unroll
    for (int j = 0; j < 4; ++j) out[j][0] += Rl[j];
#pragma unroll
    for (int i = 0; i < 4; ++i) out[0][i] += Ts[w - 1][i][lane];
    out[0][0] += Ts[w - 1][4][lane - 1];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int iy = 4 * ey + j;
        if (iy >= L.ny) break;
        const float z = (zero_row0 && iy == 0) ? 0.f : sign;
        epi_store4(E, y, (int64_t)iy * L.ld + 4 * ex,
                   make_float4(z * out[j][0], z * out[j][1], z * out[j][2], z * out[j][3]));
    }
}

// ---- element-per-lane apply fed by TMA, walking up the strips (FP32) ------------------------
// The grid is one wave (every CTA resident at once).  CTA b walks strip b % nsx (31 element
// columns plus the halo lane) upward through element rows [r0, r0 + rw) in tiles of 8 element
// rows, one per warp (warps past the walk's last row sit the last tile out).  Each tile's node rows (one 132 x 33 box) and element
// records (one 28 x 32 x 8 box of the padded W copy) arrive by TMA into one of two stages while
// the other stage's tile is computed, so a CTA never waits on memory between its tiles.  In the
// first tile warp 0 computes the row below the walk (top row only: the halo); in later tiles the
// row below warp 0 is the previous tile's warp 7, whose top-row contributions are carried in
// shared memory.  Coordinates outside the mesh read as zero (virtual elements have W = 0).  The
// arithmetic and the order of the carries are those of k_apply_rows: both give the same bits.
constexpr int WK_ROWS = 8, WK_UX = 132, WK_UY = 4 * WK_ROWS + 1;
constexpr int WK_U_BYTES = WK_UX * WK_UY * 4;                     // 17,424
constexpr int WK_W_BYTES = 28 * 32 * WK_ROWS * 4;                 // 28,672
constexpr int WK_W_OFF = ((WK_U_BYTES + 127) / 128) * 128;
constexpr int WK_STAGE = WK_W_OFF + WK_W_BYTES;
constexpr int WK_TS_OFF = 2 * WK_STAGE;                           // [2][ROWS][5][32] floats
constexpr int WK_BAR_OFF = WK_TS_OFF + 2 * WK_ROWS * 5 * 32 * 4;
constexpr int WK_BYTES = WK_BAR_OFF + 16;

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}
// orders this thread's earlier generic-proxy shared-memory accesses before later TMA writes
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__global__ void __launch_bounds__(32 * WK_ROWS, 2) k_apply_walk(const __grid_constant__ CUtensorMap umap,
                                                                const __grid_constant__ CUtensorMap wmap,
                                                                float* __restrict__ y, ApplyArgs<float> A, float sign,
                                                                int zero_row0, int nsx, int rw, OpEpi<float> E) {
    extern __shared__ __align__(128) unsigned char smem[];
    const Layout L = A.L;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ex0 = 31 * ((int)blockIdx.x % nsx);   // element of lane 1
    const int r0 = ((int)blockIdx.x / nsx) * rw;
    const int r_end = min(r0 + rw, L.NelY + 1);     // element row NelY is the virtual top row
    const int nt = (r_end - r0 + WK_ROWS) / WK_ROWS;  // tiles cover rows r0 - 1 .. r_end - 1
    float* Ts = reinterpret_cast<float*>(smem + WK_TS_OFF);
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + WK_BAR_OFF);
    auto issue_w = [&](int k) {   // element records of tile k; the barrier expects the node rows too
        const int st = k & 1, base = r0 - 1 + WK_ROWS * k;
        mbar_expect_tx(&bar[st], (uint32_t)(WK_U_BYTES + WK_W_BYTES));
        tma_load_3d(smem + st * WK_STAGE + WK_W_OFF, &wmap, &bar[st], 0, ex0 - 1, base);
    };
    auto issue_u = [&](int k) {   // node rows of tile k
        const int st = k & 1, base = r0 - 1 + WK_ROWS * k;
        tma_load_2d(smem + st * WK_STAGE, &umap, &bar[st], 4 * (ex0 - 1), 4 * base);
    };
    auto issue = [&](int k) {
        issue_w(k);
        issue_u(k);
    };
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
    }
    __syncthreads();
    // the element data are constant (written only between launches, by the host): the first
    // tile's records are requested before the wait for the grids this launch depends on, so they
    // stream in during the predecessor's tail when the launch is programmatic; the node rows (the
    // predecessor's output) after it.  The first tile alone: it reaches every CTA before any
    // second one.
    // A gated launch (A.gate) requests nothing before the wait: it may have no work.
    const bool gated = A.gate != nullptr;
    if (threadIdx.x == 0 && !gated) issue_w(0);
    EQC_GRID_WAIT();
    if (gated && *A.gate != A.gate_val) return;
    if (threadIdx.x == 0) {
        if (gated) issue_w(0);
        issue_u(0);
    }
    const int ex = ex0 - 1 + lane;
    for (int k = 0; k < nt; ++k) {
        const int st = k & 1;
        const uint32_t parity = (uint32_t)((k >> 1) & 1);
        bool done = false;
        const int polls = k == 0 ? A.wait_polls : MBAR_SPIN_LIMIT;
        for (int it = 0; it < polls && !done; ++it) done = mbar_try_wait(&bar[st], parity);
        if (__syncthreads_or(!done)) {
            // give up: flag it, wait (bounded) for the copies still in flight (tile 0, or tiles
            // k and k + 1), leave
            if (threadIdx.x == 0) {
                if (A.err) atomicExch(A.err, 1);
                for (int j = k; j < nt && j < (k == 0 ? 1 : k + 2); ++j)
                    for (int it = 0; it < MBAR_SPIN_LIMIT; ++it)
                        if (mbar_try_wait(&bar[j & 1], (uint32_t)((j >> 1) & 1))) break;
            }
            return;
        }
        if (k == 0 && nt > 1 && threadIdx.x == 0) issue(1);   // overlaps the first tile's compute
        const int ey = r0 - 1 + WK_ROWS * k + w;
        if (ey >= r_end) {   // past the walk (warp-uniform): no row to compute, only the barrier
            __syncthreads();
            if (threadIdx.x == 0 && k + 2 < nt) {
                fence_proxy_async_smem();
                issue(k + 2);
            }
            continue;
        }
        const float* xs = reinterpret_cast<const float*>(smem + st * WK_STAGE) + 4 * w * WK_UX;
        const float* wsm = reinterpret_cast<const float*>(smem + st * WK_STAGE + WK_W_OFF) + (w * 32 + lane) * 28;
        float u[5][5];
#pragma unroll
        for (int j = 0; j < 5; ++j) {
            const float4 v = *reinterpret_cast<const float4*>(xs + j * WK_UX + 4 * lane);
            u[j][0] = v.x;
            u[j][1] = v.y;
            u[j][2] = v.z;
            u[j][3] = v.w;
            const float n4 = __shfl_down_sync(FULLMASK, v.x, 1);
            u[j][4] = lane == 31 ? xs[j * WK_UX + 128] : n4;
        }
        float W[28];
#pragma unroll
        for (int q = 0; q < 7; ++q) {
            const float4 c = *reinterpret_cast<const float4*>(wsm + 4 * q);
            W[4 * q] = c.x;
            W[4 * q + 1] = c.y;
            W[4 * q + 2] = c.z;
            W[4 * q + 3] = c.w;
        }
        const bool halo = k == 0 && w == 0;
        float out[4][4], R[4], T[5];
        rows_lines(u, W, A.c1, A.c2, halo, out, R, T);
        float* Tk = Ts + st * (WK_ROWS * 160);
#pragma unroll
        for (int i = 0; i < 5; ++i) Tk[(w * 5 + i) * 32 + lane] = T[i];
        float Rl[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) Rl[j] = __shfl_up_sync(FULLMASK, R[j], 1);
        // warp 0 after the first tile: the top row of the previous tile's warp 7 (written before
        // the previous tile's barrier, overwritten only after this tile's)
        float cb[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        if (w == 0 && k > 0) {
            const float* Tp = Ts + (st ^ 1) * (WK_ROWS * 160) + (WK_ROWS - 1) * 160;
#pragma unroll
            for (int i = 0; i < 4; ++i) cb[i] = Tp[i * 32 + lane];
            cb[4] = Tp[4 * 32 + (lane > 0 ? lane - 1 : 0)];
        }
        __syncthreads();   // T of every warp written; every read of this stage done
        if (threadIdx.x == 0 && k + 2 < nt) {
            fence_proxy_async_smem();
            issue(k + 2);
        }
        if (lane == 0 || halo || ex > L.NelX || ey > L.NelY || ey >= r_end) continue;
#pragma unroll
        for (int j = 0; j < 4; ++j) out[j][0] += Rl[j];
        if (w > 0) {
            const float* Tb = Tk + (w - 1) * 160;
#pragma unroll
            for (int i = 0; i < 4; ++i) out[0][i] += Tb[i * 32 + lane];
            out[0][0] += Tb[4 * 32 + lane - 1];
        } else {
#pragma unroll
            for (int i = 0; i < 4; ++i) out[0][i] += cb[i];
            out[0][0] += cb[4];
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int iy = 4 * ey + j;
            if (iy >= L.ny) break;
            const float z = (zero_row0 && iy == 0) ? 0.f : sign;
            epi_store4(E, y, (int64_t)iy * L.ld + 4 * ex,
                       make_float4(z * out[j][0], z * out[j][1], z * out[j][2], z * out[j][3]));
        }
    }
}

typedef CUresult (*PFN_encodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                     const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                     CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static PFN_encodeTiled encode_fn() {
    static PFN_encodeTiled fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_encodeTiled)p;
    }
    return fn;
}

static bool encode_2d(CUtensorMap* m, bool f64, const void* base, uint64_t d0, uint64_t d1, uint64_t stride_bytes,
                      uint32_t b0, uint32_t b1) {
    PFN_encodeTiled fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {d0, d1};
    const cuuint64_t strides[1] = {stride_bytes};
    const cuuint32_t box[2] = {b0, b1};
    const cuuint32_t es[2] = {1, 1};
    return fn(m, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base),
              dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
              CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// W of the walk apply as a 3-D tensor [NelY][NelX][28] with a 28 x 32 x WK_ROWS box.
static bool encode_w_walk(CUtensorMap* m, const float* base, int NelX, int NelY) {
    PFN_encodeTiled fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {28, (cuuint64_t)NelX, (cuuint64_t)NelY};
    const cuuint64_t strides[2] = {28 * sizeof(float), (cuuint64_t)NelX * 28 * sizeof(float)};
    const cuuint32_t box[3] = {28, 32, WK_ROWS};
    const cuuint32_t es[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, es,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

constexpr int TEX = 8, TEY = 8;

template <class T>
static size_t apply_smem() {
    return sizeof(T) * ((size_t)(4 * (TEX + 1) + 1) * (4 * (TEY + 1) + 1) + 2 * (size_t)(TEX + 1) * (TEY + 1) * 25);
}

constexpr int LTEX = 8, LTEY = 7, LNT = 256;

template <class T> static CUtensorMap& wmap_ref(TmaCache& c);
template <> CUtensorMap& wmap_ref<float>(TmaCache& c) { return c.w32; }
template <> CUtensorMap& wmap_ref<double>(TmaCache& c) { return c.w64; }
template <class T> static std::unordered_map<const void*, CUtensorMap>& umap_ref(TmaCache& c);
template <> std::unordered_map<const void*, CUtensorMap>& umap_ref<float>(TmaCache& c) { return c.u32; }
template <> std::unordered_map<const void*, CUtensorMap>& umap_ref<double>(TmaCache& c) { return c.u64; }

template <class T>
static const CUtensorMap& tma_wmap(TmaCache& c) { return wmap_ref<T>(c); }

// Tensor map of a node vector (cached by address): the nx x ny grid, row pitch ld, box
// UPT x (4*LTEY+5); coordinates outside the grid read as zero.
template <class T>
static const CUtensorMap* tma_umap(TmaCache& c, const T* x, const Layout& L) {
    if (!c.ok) return nullptr;
    auto& m = umap_ref<T>(c);
    auto it = m.find(x);
    if (it != m.end()) return &it->second;
    if ((reinterpret_cast<uintptr_t>(x) & 15) != 0) return nullptr;
    CUtensorMap tm;
    if (!encode_2d(&tm, sizeof(T) == 8, x, (uint64_t)L.nx, (uint64_t)L.ny, (uint64_t)L.ld * sizeof(T), UPT,
                   4 * LTEY + 5))
        return nullptr;
    return &(m[x] = tm);
}

// Node-vector map of the walk apply (cached by address): box WK_UX x WK_UY.
static const CUtensorMap* tma_umap_walk(TmaCache& c, const float* x, const Layout& L) {
    if (!c.walk_ok) return nullptr;
    auto it = c.u32walk.find(x);
    if (it != c.u32walk.end()) return &it->second;
    if ((reinterpret_cast<uintptr_t>(x) & 15) != 0) return nullptr;
    CUtensorMap tm;
    if (!encode_2d(&tm, false, x, (uint64_t)L.nx, (uint64_t)L.ny, (uint64_t)L.ld * sizeof(float), WK_UX, WK_UY))
        return nullptr;
    return &(c.u32walk[x] = tm);
}

// Encodes the element-data maps of the padded W copies W32p / W64p; leaves the cache disabled
// (plain loads) if TMA is unavailable.
void tma_init_for(TmaCache& c, const Layout& L, const float* W32p, const double* W64p) {
    c.ok = false;
    c.walk_ok = false;
    c.u32.clear();
    c.u64.clear();
    c.u32walk.clear();
    if (getenv("EQC_NO_TMA")) return;
    const int EX = LTEX + 1, EY = LTEY + 1;
    bool ok = encode_2d(&c.w32, false, W32p, (uint64_t)L.NelX * WPad<float>::v, (uint64_t)L.NelY,
                        (uint64_t)L.NelX * WPad<float>::v * sizeof(float), EX * WPad<float>::v, EY);
    ok = ok && encode_2d(&c.w64, true, W64p, (uint64_t)L.NelX * WPad<double>::v, (uint64_t)L.NelY,
                         (uint64_t)L.NelX * WPad<double>::v * sizeof(double), EX * WPad<double>::v, EY);
    c.ok = ok;
    c.walk_ok = ok && encode_w_walk(&c.w32walk, W32p, L.NelX, L.NelY);
}
void tma_init(Handle& h) { tma_init_for(h.tma, h.L, h.W32p.p, h.W64p.p); }

// CTAs of the pipelined apply: as many as fit on every SM at once.
static int g_pipe_blocks[2] = {0, 0};
template <class T>
static int pipe_blocks() { return g_pipe_blocks[sizeof(T) == 8 ? 1 : 0]; }

template <class T>
static void pipe_setup() {
    const int bytes = PipeLayout<T, LTEX, LTEY>::BYTES;
    EQC_CUDA(cudaFuncSetAttribute(k_apply_pipe<T, LTEX, LTEY, LNT>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    int per_sm = 0, dev = 0, nsm = 0;
    EQC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_apply_pipe<T, LTEX, LTEY, LNT>, LNT, bytes));
    EQC_CUDA(cudaGetDevice(&dev));
    EQC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    g_pipe_blocks[sizeof(T) == 8 ? 1 : 0] = std::max(1, per_sm) * nsm;
}

// CTAs of the walk apply that are resident at once (its grid never exceeds one wave).
static int g_walk_slots = 0;
static void walk_setup() {
    EQC_CUDA(cudaFuncSetAttribute(k_apply_walk, cudaFuncAttributeMaxDynamicSharedMemorySize, WK_BYTES));
    int per_sm = 0, dev = 0, nsm = 0;
    EQC_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_apply_walk, 32 * WK_ROWS, WK_BYTES));
    EQC_CUDA(cudaGetDevice(&dev));
    EQC_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    g_walk_slots = std::max(1, per_sm) * nsm;
}

// Walk length: the rows of every strip split evenly over the resident CTAs (one wave, every
// SM holding the same number of rows to within one walk).
static void walk_shape(const Layout& L, int* nsx, int* rw, int* nblk) {
    *nsx = (L.NelX + 1 + 30) / 31;
    const int64_t rows = L.NelY + 1;
    int64_t r = std::max<int64_t>(1, (rows * *nsx + g_walk_slots - 1) / g_walk_slots);
    while (r < rows && *nsx * ((rows + r - 1) / r) > g_walk_slots) ++r;
    *rw = (int)r;
    *nblk = *nsx * (int)((rows + r - 1) / r);
}

static bool launch_walk(const float* x, float* y, const ApplyArgs<float>& A, float sign, int zr, cudaStream_t s,
                        const OpEpi<float>& E = OpEpi<float>()) {
    if (!A.tma || !A.tma->walk_ok || g_walk_slots <= 0) return false;
    const CUtensorMap* um = tma_umap_walk(*A.tma, x, A.L);
    if (!um) return false;
    int nsx, rw, nblk;
    walk_shape(A.L, &nsx, &rw, &nblk);
    k_apply_walk<<<nblk, 32 * WK_ROWS, WK_BYTES, s>>>(*um, A.tma->w32walk, y, A, sign, zr, nsx, rw, E);
    EQC_CHECK_LAUNCH();
    count_launch();
    return true;
}

void set_H(const double* H, cudaStream_t s) {
    float hf[25];
    for (int k = 0; k < 25; ++k) hf[k] = (float)H[k];
    EQC_CUDA(cudaMemcpyToSymbolAsync(cH64, H, sizeof(double) * 25, 0, cudaMemcpyHostToDevice, s));
    EQC_CUDA(cudaMemcpyToSymbolAsync(cH32, hf, sizeof(float) * 25, 0, cudaMemcpyHostToDevice, s));
    {   // even-odd coefficients of the two line contractions (H[i + 5 j] = h'_i(x_j))
        auto D1 = [&](int p, int k) { return H[k + 5 * p]; };   // s_p = sum_k H(k,p) v_k
        auto D2 = [&](int i, int p) { return H[i + 5 * p]; };   // o_i = sum_p H(i,p) s_p
        double hmax = 0.0, asym = 0.0;
        for (int k = 0; k < 25; ++k) hmax = std::max(hmax, std::fabs(H[k]));
        for (int i = 0; i < 5; ++i)
            for (int j = 0; j < 5; ++j) asym = std::max(asym, std::fabs(H[i + 5 * j] + H[(4 - i) + 5 * (4 - j)]));
        EOCoef c[2];
        for (int t = 0; t < 2; ++t) {
            auto M = [&](int r, int q) { return t == 0 ? D1(r, q) : D2(r, q); };
            for (int p = 0; p < 2; ++p) {
                for (int m = 0; m < 2; ++m) {
                    c[t].a[p][m] = (float)(0.5 * (M(p, m) - M(p, 4 - m)));
                    c[t].b[p][m] = (float)(0.5 * (M(p, m) + M(p, 4 - m)));
                }
                c[t].g[p] = (float)M(p, 2);
                c[t].d[p] = (float)M(2, p);
            }
        }
        EOCoef64 c64[2];
        for (int t = 0; t < 2; ++t) {
            auto M = [&](int r, int q) { return t == 0 ? D1(r, q) : D2(r, q); };
            for (int p = 0; p < 2; ++p) {
                for (int m = 0; m < 2; ++m) {
                    c64[t].a[p][m] = 0.5 * (M(p, m) - M(p, 4 - m));
                    c64[t].b[p][m] = 0.5 * (M(p, m) + M(p, 4 - m));
                }
                c64[t].g[p] = M(p, 2);
                c64[t].d[p] = M(2, p);
            }
        }
        const int ok = asym <= 1e-12 * hmax ? 1 : 0;
        EQC_CUDA(cudaMemcpyToSymbolAsync(cEO, c, sizeof(c), 0, cudaMemcpyHostToDevice, s));
        EQC_CUDA(cudaMemcpyToSymbolAsync(cEO64, c64, sizeof(c64), 0, cudaMemcpyHostToDevice, s));
        EQC_CUDA(cudaMemcpyToSymbolAsync(cEO_ok, &ok, sizeof(int), 0, cudaMemcpyHostToDevice, s));
    }
    EQC_CUDA(cudaStreamSynchronize(s));
    // kernel attributes are set here, at handle creation, never during a stream capture
    EQC_CUDA(cudaFuncSetAttribute(k_apply<double, TEX, TEY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)apply_smem<double>()));
    EQC_CUDA(cudaFuncSetAttribute(k_apply<float, TEX, TEY>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)apply_smem<float>()));
    pipe_setup<float>();
    pipe_setup<double>();
    walk_setup();

}

// Element-per-lane apply: variant 0 -> 6 element rows per CTA (default), 4..7 -> 4, 6, 8, 12.
static void launch_rows(const float* x, float* y, const ApplyArgs<float>& A, float sign, int zr, cudaStream_t s,
                        const OpEpi<float>& E = OpEpi<float>()) {
    const int sx = (A.L.NelX + 1 + 30) / 31;
    auto go = [&](auto rows_tag, auto minb_tag) {
        constexpr int R = decltype(rows_tag)::value, M = decltype(minb_tag)::value;
        dim3 g(sx, (A.L.NelY + 1 + R - 1) / R);
        k_apply_rows<R, M><<<g, 32 * (R + 1), 0, s>>>(x, y, A, sign, zr, E);
    };
    using I = std::integral_constant<int, 0>;
    (void)sizeof(I);
    switch (A.variant) {
        case 4: go(std::integral_constant<int, 4>{}, std::integral_constant<int, 3>{}); break;
        case 5: go(std::integral_constant<int, 8>{}, std::integral_constant<int, 2>{}); break;
        case 6: go(std::integral_constant<int, 12>{}, std::integral_constant<int, 1>{}); break;
        case 7: go(std::integral_constant<int, 6>{}, std::integral_constant<int, 2>{}); break;
        default: go(std::integral_constant<int, 6>{}, std::integral_constant<int, 3>{}); break;
    }
    EQC_CHECK_LAUNCH();
    count_launch();
}

template <class T>
void apply_K(const T* x, T* y, const ApplyArgs<T>& A, T sign, int mode, cudaStream_t s) {
    if (mode <= 1) {
        dim3 grid(A.L.NelX / LTEX + 1, A.L.NelY / LTEY + 1);
        if constexpr (sizeof(T) == 4) {
            if (A.variant == 8 && A.Wp && aligned16(x) && aligned16(y) && launch_walk(x, y, A, sign, mode == 1 ? 1 : 0, s))
                return;
            if ((A.variant == 0 || A.variant >= 4) && A.Wp && aligned16(x) && aligned16(y)) {
                launch_rows(x, y, A, sign, mode == 1 ? 1 : 0, s);
                return;
            }
        }
        const CUtensorMap* um = (A.tma && A.variant != 2) ? tma_umap<T>(*A.tma, x, A.L) : nullptr;
        if (um && A.variant == 1) {
            k_apply_tma<T, LTEX, LTEY, LNT><<<grid, LNT, 0, s>>>(*um, tma_wmap<T>(*A.tma), y, A, sign, mode == 1 ? 1 : 0);
        } else if (um) {
            const int ntx = (int)grid.x, ntiles = (int)(grid.x * grid.y);
            const int nblk = std::min(ntiles, pipe_blocks<T>());
            k_apply_pipe<T, LTEX, LTEY, LNT><<<nblk, LNT, PipeLayout<T, LTEX, LTEY>::BYTES, s>>>(
                *um, tma_wmap<T>(*A.tma), y, A, sign, mode == 1 ? 1 : 0, ntx, ntiles);
        } else {
            k_apply_lines<T, LTEX, LTEY, LNT><<<grid, LNT, 0, s>>>(x, y, A, sign, mode == 1 ? 1 : 0);
        }
        EQC_CHECK_LAUNCH();
        count_launch();
        return;
    }
    const size_t sm = apply_smem<T>();
    dim3 grid((A.L.NelX + TEX - 1) / TEX, mode >= 2 ? 1 : (A.L.NelY + TEY - 1) / TEY);
    k_apply<T, TEX, TEY><<<grid, 256, sm, s>>>(x, y, A, sign, mode);
    EQC_CHECK_LAUNCH();
    count_launch();
}

bool apply_K_fault32(const float* x, float* y, const ApplyArgs<float>& A, cudaStream_t s) {
    if (!A.Wp || !aligned16(x) || !aligned16(y)) return false;
    // one element row per CTA (warp 0 the virtual row below the fault, W = 0), grid row 0 only
    const dim3 g((A.L.NelX + 1 + 30) / 31, 1);
    k_apply_rows<1, 8><<<g, 64, 0, s>>>(x, y, A, 1.0f, 0, OpEpi<float>());
    EQC_CHECK_LAUNCH();
    count_launch();
    return true;
}

bool apply_K_epi(const float* x, const ApplyArgs<float>& A, int mode, const OpEpi<float>& E, cudaStream_t s) {
    if (mode > 1 || !A.Wp || !aligned16(x)) return false;
    if (A.variant == 8 && launch_walk(x, nullptr, A, 1.0f, mode, s, E)) return true;
    if (A.variant == 0 || (A.variant >= 4 && A.variant <= 7)) {
        launch_rows(x, nullptr, A, 1.0f, mode, s, E);
        return true;
    }
    return false;
}

template void apply_K<double>(const double*, double*, const ApplyArgs<double>&, double, int, cudaStream_t);
template void apply_K<float>(const float*, float*, const ApplyArgs<float>&, float, int, cudaStream_t);

}  // namespace eqc
