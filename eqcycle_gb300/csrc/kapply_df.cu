// K1 in double-float: y = sign * K x for FP64 x and y, evaluated with FP32 operations on
// unevaluated hi + lo pairs (df.cuh), ~1e-14 relative per operation, for callers that need an
// FP64-class apply at the FP32 rate (eqc_apply_K_device dtype 2, and the mixed solver's
// intermediate reliable updates, r -= K dx with dx the correction since the previous update).
// The solver's full true residuals b - K_II x do not use it: late in a cycle the displacement
// grows until the 1e-14 error of K x floors the residual near 1e-5 of |b|, above the CG
// tolerance (measured), so those stay FP64; K dx has the size of the residual it corrects.
//
// Layout as k_apply_rows: one lane per element, one warp per element row of 31 elements plus a
// halo lane, ROWS element rows per CTA plus a halo warp; the line contractions in even-odd form.
// To keep registers for the 25 double-float outputs, each lane reads its element's nodes twice
// (rows for the x-lines, columns for the y-lines; L1 hits) instead of holding them.
#include "model.h"
#include "df.cuh"
#include <cmath>

namespace eqc {

struct EODF {
    df a[2][2], b[2][2], g[2], d[2];
};
__constant__ EODF cEOdf[2];   // [0]: s_p = sum_k H(k,p) v_k ; [1]: o_i = sum_p H(i,p) s_p

__device__ __forceinline__ void eo5_df(const df (&v)[5], df (&s)[5], const EODF& c) {
    const df e0 = df_add(v[0], v[4]), e1 = df_add(v[1], v[3]);
    const df o0 = df_sub(v[0], v[4]), o1 = df_sub(v[1], v[3]);
#pragma unroll
    for (int p = 0; p < 2; ++p) {
        const df P = df_add(df_mul(c.a[p][0], o0), df_mul(c.a[p][1], o1));
        const df Q = df_add(df_add(df_mul(c.b[p][0], e0), df_mul(c.b[p][1], e1)), df_mul(c.g[p], v[2]));
        s[p] = df_add(P, Q);
        s[4 - p] = df_sub(P, Q);
    }
    s[2] = df_add(df_mul(c.d[0], o0), df_mul(c.d[1], o1));
}

__device__ __forceinline__ df shfl_up_df(df v) {
    return df{__shfl_up_sync(0xffffffffu, v.hi, 1), __shfl_up_sync(0xffffffffu, v.lo, 1)};
}

template <int ROWS>
__global__ void __launch_bounds__(32 * (ROWS + 1), 2)
    k_apply_df(const double* __restrict__ x, double* __restrict__ y, const float* __restrict__ Whi,
               const float* __restrict__ Wlo, Layout L, df c1, df c2, double sign, int zero_row0,
               const int* gate, int gate_val) {
    EQC_GRID_WAIT();
    if (gate && *gate != gate_val) return;
    __shared__ float Th[ROWS + 1][5][32], Tl[ROWS + 1][5][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int ex = (int)blockIdx.x * 31 - 1 + lane;
    const int ey = (int)blockIdx.y * ROWS - 1 + w;
    const bool real = ex >= 0 && ex < L.NelX && ey >= 0 && ey < L.NelY;
    const bool halo = w == 0;
    const int64_t eo = real ? ((int64_t)ey * L.NelX + ex) * 28 : 0;
    auto Wd = [&](int q) { return real ? df{__ldg(Whi + eo + q), __ldg(Wlo + eo + q)} : df{0.f, 0.f}; };
    // node (4 ex + i, 4 ey + j) of the element, zero outside the grid
    auto node = [&](int i, int j) {
        const int ix = 4 * ex + i, iy = 4 * ey + j;
        return (ix >= 0 && ix < L.nx && iy >= 0 && iy < L.ny) ? df_from_double(__ldg(x + (int64_t)iy * L.ld + ix))
                                                             : df{0.f, 0.f};
    };
    df out[4][4], R[4], T[5];
    // x-lines (the halo warp needs only the top one, for T)
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        if (halo && j < 4) continue;
        df v[5], s[5], o[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) v[k] = node(k, j);
        eo5_df(v, s, cEOdf[0]);
#pragma unroll
        for (int p = 0; p < 5; ++p) s[p] = df_mul(s[p], Wd(p + 5 * j));
        eo5_df(s, o, cEOdf[1]);
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            const df r = df_mul(c1, o[i]);
            if (j < 4) {
                if (i < 4) out[j][i] = r;
                else R[j] = r;
            } else {
                T[i] = r;
            }
        }
    }
    if (halo) {
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#pragma unroll
            for (int i = 0; i < 4; ++i) out[j][i] = df{0.f, 0.f};
            R[j] = df{0.f, 0.f};
        }
    }
    // y-lines
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        df v[5], s[5], o[5];
#pragma unroll
        for (int l = 0; l < 5; ++l) v[l] = node(i, l);
        eo5_df(v, s, cEOdf[0]);
#pragma unroll
        for (int p = 0; p < 5; ++p) s[p] = df_mul(s[p], Wd(i + 5 * p));
        eo5_df(s, o, cEOdf[1]);
#pragma unroll
        for (int jj = 0; jj < 5; ++jj) {
            if (halo && jj < 4) continue;
            const df r = df_mul(c2, o[jj]);
            if (jj < 4) {
                if (i < 4) out[jj][i] = df_add(out[jj][i], r);
                else R[jj] = df_add(R[jj], r);
            } else {
                T[i] = df_add(T[i], r);
            }
        }
    }
#pragma unroll
    for (int i = 0; i < 5; ++i) {
        Th[w][i][lane] = T[i].hi;
        Tl[w][i][lane] = T[i].lo;
    }
    df Rl[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) Rl[j] = shfl_up_df(R[j]);
    __syncthreads();
    if (halo || lane == 0 || ex > L.NelX || ey > L.NelY) return;
#pragma unroll
    for (int j = 0; j < 4; ++j) out[j][0] = df_add(out[j][0], Rl[j]);
#pragma unroll
    for (int i = 0; i < 4; ++i) out[0][i] = df_add(out[0][i], df{Th[w - 1][i][lane], Tl[w - 1][i][lane]});
    out[0][0] = df_add(out[0][0], df{Th[w - 1][4][lane - 1], Tl[w - 1][4][lane - 1]});
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int iy = 4 * ey + j;
        if (iy >= L.ny) break;
        const double z = (zero_row0 && iy == 0) ? 0.0 : sign;
        double* row = y + (int64_t)iy * L.ld + 4 * ex;
        reinterpret_cast<double2*>(row)[0] = make_double2(z * df_to_double(out[j][0]), z * df_to_double(out[j][1]));
        reinterpret_cast<double2*>(row)[1] = make_double2(z * df_to_double(out[j][2]), z * df_to_double(out[j][3]));
    }
}

static df host_df(double v) {
    const float hi = (float)v;
    return df{hi, (float)(v - (double)hi)};
}

void set_H_df(const double* H, cudaStream_t s) {
    EODF c[2];
    for (int t = 0; t < 2; ++t) {
        auto M = [&](int r, int q) { return t == 0 ? H[q + 5 * r] : H[r + 5 * q]; };
        for (int p = 0; p < 2; ++p) {
            for (int m = 0; m < 2; ++m) {
                c[t].a[p][m] = host_df(0.5 * (M(p, m) - M(p, 4 - m)));
                c[t].b[p][m] = host_df(0.5 * (M(p, m) + M(p, 4 - m)));
            }
            c[t].g[p] = host_df(M(p, 2));
            c[t].d[p] = host_df(M(2, p));
        }
    }
    EQC_CUDA(cudaMemcpyToSymbolAsync(cEOdf, c, sizeof(c), 0, cudaMemcpyHostToDevice, s));
    EQC_CUDA(cudaStreamSynchronize(s));
}

bool apply_K_df(Handle& h, const double* x, double* y, double sign, int mode, cudaStream_t s, const int* gate,
                int gate_val) {
    if (!h.df_ok || mode > 1 || !h.W32lo.p || (reinterpret_cast<uintptr_t>(y) & 15)) return false;
    constexpr int R = 6;
    const Layout& L = h.L;
    dim3 g((L.NelX + 1 + 30) / 31, (L.NelY + 1 + R - 1) / R);
    k_apply_df<R><<<g, 32 * (R + 1), 0, s>>>(x, y, h.W32p.p, h.W32lo.p, L, host_df(h.c1), host_df(h.c2), sign,
                                             mode == 1 ? 1 : 0, gate, gate_val);
    EQC_CHECK_LAUNCH();
    count_launch();
    return true;
}

}  // namespace eqc
