// Learned initial guess: network kernels (forward, backward, Adam), the coarse-grid
// transfers and the time-loop hooks.  See learn.h for the network.
//
// All kernels are deterministic (fixed reduction orders), so training on the same pairs with
// the same seed gives bitwise the same weights.
#include "learn.h"
#include "reduce.cuh"
#include <cmath>
#include <random>
#include <algorithm>

namespace eqc {

__device__ __forceinline__ float tof(float v) { return v; }
__device__ __forceinline__ float tof(__nv_bfloat16 v) { return __bfloat162float(v); }

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.39894228040143268f * expf(-0.5f * x * x);
}

// ---- GEMM: C[m][n] = sum_k A(m,k) B(k,n) (+ bias[n]); optional GELU copy.  64x64 tiles,
// 16-deep k slices, 256 threads with 4x4 outputs each; operands BF16 or FP32, FP32 products.
template <class TA, class TB>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const TA* __restrict__ A, int64_t sam, int64_t sak,
                                              const TB* __restrict__ B, int64_t sbk, int64_t sbn, float* __restrict__ C,
                                              int64_t ldc, const float* __restrict__ bias, float* __restrict__ Cg) {
    EQC_GRID_WAIT();
    __shared__ float As[16][65];
    __shared__ float Bs[16][65];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
    for (int k0 = 0; k0 < K; k0 += 16) {
        for (int e = threadIdx.x; e < 16 * 64; e += 256) {
            int kk, mm;
            if (sak == 1) { mm = e >> 4; kk = e & 15; } else { kk = e >> 6; mm = e & 63; }
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = (m < M && k < K) ? tof(A[(int64_t)m * sam + (int64_t)k * sak]) : 0.f;
        }
        for (int e = threadIdx.x; e < 16 * 64; e += 256) {
            int kk, nn;
            if (sbn == 1) { kk = e >> 6; nn = e & 63; } else { nn = e >> 4; kk = e & 15; }
            const int n = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = (n < N && k < K) ? tof(B[(int64_t)k * sbk + (int64_t)n * sbn]) : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int m = m0 + ty + 16 * i, n = n0 + tx + 16 * j;
            if (m < M && n < N) {
                const float v = acc[i][j] + (bias ? bias[n] : 0.f);
                C[(int64_t)m * ldc + n] = v;
                if (Cg) Cg[(int64_t)m * ldc + n] = gelu(v);
            }
        }
}

template <class TA, class TB>
static void gemm(int M, int N, int K, const TA* A, int64_t sam, int64_t sak, const TB* B, int64_t sbk, int64_t sbn,
                 float* C, int64_t ldc, const float* bias, float* Cg, cudaStream_t s) {
    dim3 grid((N + 63) / 64, (M + 63) / 64);
    k_gemm<TA, TB><<<grid, 256, 0, s>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, bias, Cg);
    EQC_CHECK_LAUNCH();
    count_launch();
}

// ---- GEMV for small batches (inference): y[b][o] = sum_i x[b][i] W[o][i] + bias[o]; one warp
// per output row o, lanes striding over i in BF16 pairs; optional GELU copy.
template <int BMAX>
__global__ void __launch_bounds__(256) k_gemv(int B, int N, int K, const float* __restrict__ x,
                                              const __nv_bfloat16* __restrict__ W, const float* __restrict__ bias,
                                              float* __restrict__ y, float* __restrict__ yg) {
    EQC_GRID_WAIT();
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= N) return;
    const __nv_bfloat16* w = W + (int64_t)warp * K;
    float acc[BMAX];
#pragma unroll
    for (int b = 0; b < BMAX; ++b) acc[b] = 0.f;
    const bool pairs = ((K & 1) == 0) && ((reinterpret_cast<uintptr_t>(w) & 3) == 0);
    if (pairs) {
        const __nv_bfloat162* w2 = reinterpret_cast<const __nv_bfloat162*>(w);
        for (int i = lane; i < K / 2; i += 32) {
            const float2 wf = __bfloat1622float2(w2[i]);
#pragma unroll
            for (int b = 0; b < BMAX; ++b)
                if (b < B) acc[b] = fmaf(wf.y, x[(int64_t)b * K + 2 * i + 1], fmaf(wf.x, x[(int64_t)b * K + 2 * i], acc[b]));
        }
    } else {
        for (int i = lane; i < K; i += 32) {
            const float wf = __bfloat162float(w[i]);
#pragma unroll
            for (int b = 0; b < BMAX; ++b)
                if (b < B) acc[b] = fmaf(wf, x[(int64_t)b * K + i], acc[b]);
        }
    }
#pragma unroll
    for (int b = 0; b < BMAX; ++b) {
        float v = acc[b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0 && b < B) {
            v += bias ? bias[warp] : 0.f;
            y[(int64_t)b * N + warp] = v;
            if (yg) yg[(int64_t)b * N + warp] = gelu(v);
        }
    }
}

// y = x W^T + bias for x [B][K] (FP32), W [N][K] (BF16): GEMV below 5 rows, tiled GEMM above.
static void linear(int B, int N, int K, const float* x, const __nv_bfloat16* W, const float* bias, float* y, float* yg,
                   cudaStream_t s) {
    if (B <= 4) {
        k_gemv<4><<<(N * 32 + 255) / 256, 256, 0, s>>>(B, N, K, x, W, bias, y, yg);
        EQC_CHECK_LAUNCH();
        count_launch();
    } else {
        gemm(B, N, K, x, (int64_t)K, (int64_t)1, W, (int64_t)1, (int64_t)K, y, (int64_t)N, bias, yg, s);
    }
}

// ---- convolution (kernel 5, stride 2, padding 2) ----------------------------------------
// z[b][co][t] = bias[co] + sum_{ci,k} W[co][ci][k] in[b][ci][2t+k-2] ; a = GELU(z)
__global__ void k_conv_fwd(const float* __restrict__ in, int Cin, int Tin, const __nv_bfloat16* __restrict__ W,
                           const float* __restrict__ bias, float* __restrict__ z, float* __restrict__ a, int Tout,
                           int B) {
    EQC_GRID_WAIT();
    const int64_t n = (int64_t)B * GN_C * Tout;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
        const int t = (int)(idx % Tout);
        const int co = (int)((idx / Tout) % GN_C);
        const int b = (int)(idx / ((int64_t)Tout * GN_C));
        float acc = bias[co];
        const float* ib = in + (int64_t)b * Cin * Tin;
        const __nv_bfloat16* wc = W + (int64_t)co * Cin * GN_K;
        for (int ci = 0; ci < Cin; ++ci) {
#pragma unroll
            for (int k = 0; k < GN_K; ++k) {
                const int s = 2 * t + k - 2;
                if (s >= 0 && s < Tin) acc = fmaf(__bfloat162float(wc[ci * GN_K + k]), ib[(int64_t)ci * Tin + s], acc);
            }
        }
        z[idx] = acc;
        a[idx] = gelu(acc);
    }
}

// g_in[b][ci][s] = sum_{co,k : 2t+k-2 = s} W[co][ci][k] g_z[b][co][t]
__global__ void k_conv_dgrad(const float* __restrict__ gz, int Tout, const __nv_bfloat16* __restrict__ W, int Cin,
                             float* __restrict__ gin, int Tin, int B) {
    EQC_GRID_WAIT();
    const int64_t n = (int64_t)B * Cin * Tin;
    for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < n; idx += (int64_t)gridDim.x * blockDim.x) {
        const int s = (int)(idx % Tin);
        const int ci = (int)((idx / Tin) % Cin);
        const int b = (int)(idx / ((int64_t)Tin * Cin));
        float acc = 0.f;
        const float* gb = gz + (int64_t)b * GN_C * Tout;
        for (int co = 0; co < GN_C; ++co) {
#pragma unroll
            for (int k = 0; k < GN_K; ++k) {
                const int u = s + 2 - k;
                if (u >= 0 && (u & 1) == 0 && (u >> 1) < Tout)
                    acc = fmaf(__bfloat162float(W[((int64_t)co * Cin + ci) * GN_K + k]), gb[(int64_t)co * Tout + (u >> 1)], acc);
            }
        }
        gin[idx] = acc;
    }
}

// gW[co][ci][k] = sum_{b,t} g_z[b][co][t] in[b][ci][2t+k-2] ; one CTA per (co, ci)
__global__ void __launch_bounds__(256) k_conv_wgrad(const float* __restrict__ gz, const float* __restrict__ in, int Cin,
                                                    int Tin, int Tout, int B, float* __restrict__ gW) {
    EQC_GRID_WAIT();
    __shared__ double sh[32];
    const int co = blockIdx.x / Cin, ci = blockIdx.x % Cin;
    float acc[GN_K] = {0.f, 0.f, 0.f, 0.f, 0.f};
    for (int64_t e = threadIdx.x; e < (int64_t)B * Tout; e += blockDim.x) {
        const int b = (int)(e / Tout), t = (int)(e % Tout);
        const float g = gz[((int64_t)b * GN_C + co) * Tout + t];
        const float* ib = in + ((int64_t)b * Cin + ci) * Tin;
#pragma unroll
        for (int k = 0; k < GN_K; ++k) {
            const int s = 2 * t + k - 2;
            if (s >= 0 && s < Tin) acc[k] = fmaf(g, ib[s], acc[k]);
        }
    }
#pragma unroll
    for (int k = 0; k < GN_K; ++k) {
        const double v = block_sum((double)acc[k], sh);
        if (threadIdx.x == 0) gW[((int64_t)co * Cin + ci) * GN_K + k] = (float)v;
    }
}

// out[c] = sum over rows r and positions t of g[r][c][t]   (bias gradients; T = 1 for fc)
__global__ void __launch_bounds__(256) k_bias_grad(const float* __restrict__ g, int B, int Cn, int T, float* __restrict__ out) {
    EQC_GRID_WAIT();
    __shared__ double sh[32];
    const int c = blockIdx.x;
    double s = 0.0;
    for (int64_t e = threadIdx.x; e < (int64_t)B * T; e += blockDim.x) {
        const int b = (int)(e / T), t = (int)(e % T);
        s += g[((int64_t)b * Cn + c) * T + t];
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) out[c] = (float)s;
}

// g *= GELU'(z)
__global__ void k_gelu_bwd(float* __restrict__ g, const float* __restrict__ z, int64_t n) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        g[i] *= gelu_grad(z[i]);
}

// Mean squared error over B x nout: g = 2 (out - tgt) / (B nout); loss[b] = sum_j (out - tgt)^2
__global__ void __launch_bounds__(256) k_mse(const float* __restrict__ out, const float* __restrict__ tgt, int nout, int B,
                                             float* __restrict__ g, double* __restrict__ loss) {
    EQC_GRID_WAIT();
    __shared__ double sh[32];
    const int b = blockIdx.x;
    const float sc = 2.f / ((float)B * (float)nout);
    double s = 0.0;
    for (int j = threadIdx.x; j < nout; j += blockDim.x) {
        const float e = out[(int64_t)b * nout + j] - tgt[(int64_t)b * nout + j];
        g[(int64_t)b * nout + j] = sc * e;
        s += (double)e * (double)e;
    }
    s = block_sum(s, sh);
    if (threadIdx.x == 0) loss[b] = s;
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       int64_t n, float lr, float b1, float b2, float eps, float c1, float c2) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

__global__ void k_to_bf16(const float* __restrict__ x, __nv_bfloat16* __restrict__ y, int64_t n) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = __float2bfloat16_rn(x[i]);
}

static inline int nblk(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 8 * 152); }

// ---- network set-up -------------------------------------------------------------------
void gn_reserve(GuessNet& g, int batch) {
    if (batch <= g.cap) return;
    g.cap = batch;
    g.x0.alloc((size_t)batch * 2 * g.T[0]);
    for (int l = 0; l < GN_LAYERS; ++l) {
        const size_t n = (size_t)batch * GN_C * g.T[l + 1];
        g.z[l].alloc(n);
        g.a[l].alloc(n);
        g.g_a[l].alloc(n);
    }
    g.zf1.alloc((size_t)batch * GN_NH);
    g.af1.alloc((size_t)batch * GN_NH);
    g.g_af1.alloc((size_t)batch * GN_NH);
    g.out.alloc((size_t)batch * g.nout);
    g.g_out.alloc((size_t)batch * g.nout);
    g.loss.alloc(batch);
}

void gn_init(Handle& h, uint64_t seed) {
    GuessNet& g = *h.net;
    g.Nf = h.F.Nf;
    g.T[0] = g.Nf;
    for (int l = 0; l < GN_LAYERS; ++l) g.T[l + 1] = (g.T[l] - 1) / 2 + 1;
    g.flat = GN_C * g.T[GN_LAYERS];
    int64_t o = 0;
    for (int l = 0; l < GN_LAYERS; ++l) {
        const int cin = l == 0 ? 2 : GN_C;
        g.off_cw[l] = o; o += (int64_t)GN_C * cin * GN_K;
        g.off_cb[l] = o; o += GN_C;
    }
    g.off_f1w = o; o += (int64_t)GN_NH * g.flat;
    g.off_f1b = o; o += GN_NH;
    g.off_f2w = o; o += (int64_t)g.nout * GN_NH;
    g.off_f2b = o; o += g.nout;
    g.nparam = o;
    // He-uniform weights (fan-in), zero biases, from a seeded stream
    std::vector<float> p(o, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](int64_t off, int64_t n, int fan_in) {
        const float lim = std::sqrt(6.0f / (float)fan_in);
        std::uniform_real_distribution<float> U(-lim, lim);
        for (int64_t i = 0; i < n; ++i) p[off + i] = U(rng);
    };
    for (int l = 0; l < GN_LAYERS; ++l) {
        const int cin = l == 0 ? 2 : GN_C;
        fill(g.off_cw[l], (int64_t)GN_C * cin * GN_K, cin * GN_K);
    }
    fill(g.off_f1w, (int64_t)GN_NH * g.flat, g.flat);
    fill(g.off_f2w, (int64_t)g.nout * GN_NH, GN_NH);
    cudaStream_t s = h.stream;
    g.master.alloc(o);
    g.master.upload(p.data(), o, s);
    g.grad.alloc(o);
    g.m1.alloc(o);
    g.m2.alloc(o);
    g.wbf.alloc(o);
    g.adam_t = 0;
    g.trained = false;
    gn_refresh_bf16(g, s);
    g.feat.alloc(2 * g.Nf);
    g.scale.alloc(1);
    gn_reserve(g, 1);
    EQC_CUDA(cudaStreamSynchronize(s));
}

void gn_refresh_bf16(GuessNet& g, cudaStream_t s) {
    k_to_bf16<<<nblk(g.nparam), 256, 0, s>>>(g.master.p, g.wbf.p, g.nparam);
    EQC_CHECK_LAUNCH();
    count_launch();
}

// ---- forward / backward ----------------------------------------------------------------
void gn_forward(GuessNet& g, const float* x0, int B, cudaStream_t s) {
    const float* in = x0;
    int cin = 2;
    for (int l = 0; l < GN_LAYERS; ++l) {
        const int64_t n = (int64_t)B * GN_C * g.T[l + 1];
        k_conv_fwd<<<nblk(n), 256, 0, s>>>(in, cin, g.T[l], g.wbf.p + g.off_cw[l], g.master.p + g.off_cb[l], g.z[l].p,
                                           g.a[l].p, g.T[l + 1], B);
        EQC_CHECK_LAUNCH();
        count_launch();
        in = g.a[l].p;
        cin = GN_C;
    }
    // fc1: zf1 = a3 W1^T + b1, af1 = GELU(zf1) ; fc2: out = af1 W2^T + b2
    linear(B, GN_NH, g.flat, g.a[GN_LAYERS - 1].p, g.wbf.p + g.off_f1w, g.master.p + g.off_f1b, g.zf1.p, g.af1.p, s);
    linear(B, g.nout, GN_NH, g.af1.p, g.wbf.p + g.off_f2w, g.master.p + g.off_f2b, g.out.p, nullptr, s);
}

// Gradient of the mean squared error of g.out (after gn_forward on x0) against tgt.
void gn_backward(GuessNet& g, const float* x0, const float* tgt, int B, cudaStream_t s) {
    k_mse<<<B, 256, 0, s>>>(g.out.p, tgt, g.nout, B, g.g_out.p, g.loss.p);
    count_launch();
    // fc2
    gemm(g.nout, GN_NH, B, g.g_out.p, 1, g.nout, g.af1.p, GN_NH, 1, g.grad.p + g.off_f2w, GN_NH, (const float*)nullptr,
         (float*)nullptr, s);
    k_bias_grad<<<g.nout, 256, 0, s>>>(g.g_out.p, B, g.nout, 1, g.grad.p + g.off_f2b);
    count_launch();
    gemm(B, GN_NH, g.nout, g.g_out.p, g.nout, 1, g.wbf.p + g.off_f2w, GN_NH, 1, g.g_af1.p, GN_NH,
         (const float*)nullptr, (float*)nullptr, s);
    k_gelu_bwd<<<nblk((int64_t)B * GN_NH), 256, 0, s>>>(g.g_af1.p, g.zf1.p, (int64_t)B * GN_NH);
    count_launch();
    // fc1
    const float* a3 = g.a[GN_LAYERS - 1].p;
    gemm(GN_NH, g.flat, B, g.g_af1.p, 1, GN_NH, a3, g.flat, 1, g.grad.p + g.off_f1w, g.flat, (const float*)nullptr,
         (float*)nullptr, s);
    k_bias_grad<<<GN_NH, 256, 0, s>>>(g.g_af1.p, B, GN_NH, 1, g.grad.p + g.off_f1b);
    count_launch();
    gemm(B, g.flat, GN_NH, g.g_af1.p, GN_NH, 1, g.wbf.p + g.off_f1w, g.flat, 1, g.g_a[GN_LAYERS - 1].p, g.flat,
         (const float*)nullptr, (float*)nullptr, s);
    // convolutions, last to first
    for (int l = GN_LAYERS - 1; l >= 0; --l) {
        const int cin = l == 0 ? 2 : GN_C;
        const int64_t n = (int64_t)B * GN_C * g.T[l + 1];
        k_gelu_bwd<<<nblk(n), 256, 0, s>>>(g.g_a[l].p, g.z[l].p, n);
        const float* in = l == 0 ? x0 : g.a[l - 1].p;
        k_conv_wgrad<<<GN_C * cin, 256, 0, s>>>(g.g_a[l].p, in, cin, g.T[l], g.T[l + 1], B, g.grad.p + g.off_cw[l]);
        k_bias_grad<<<GN_C, 256, 0, s>>>(g.g_a[l].p, B, GN_C, g.T[l + 1], g.grad.p + g.off_cb[l]);
        count_launch(3);
        if (l > 0) {
            const int64_t ni = (int64_t)B * GN_C * g.T[l];
            k_conv_dgrad<<<nblk(ni), 256, 0, s>>>(g.g_a[l].p, g.T[l + 1], g.wbf.p + g.off_cw[l], GN_C, g.g_a[l - 1].p,
                                                  g.T[l], B);
            count_launch();
        }
        EQC_CHECK_LAUNCH();
    }
}

void gn_adam(GuessNet& g, double lr, cudaStream_t s) {
    g.adam_t += 1;
    const double b1 = 0.9, b2 = 0.999;
    const float c1 = (float)(1.0 - std::pow(b1, (double)g.adam_t)), c2 = (float)(1.0 - std::pow(b2, (double)g.adam_t));
    k_adam<<<nblk(g.nparam), 256, 0, s>>>(g.master.p, g.grad.p, g.m1.p, g.m2.p, g.nparam, (float)lr, (float)b1,
                                          (float)b2, 1e-8f, c1, c2);
    EQC_CHECK_LAUNCH();
    count_launch();
    gn_refresh_bf16(g, s);
}

// ---- coarse grid <-> GLL nodes ----------------------------------------------------------
// Position of lattice index i (4*nel+1 points) as a fraction of the axis.
__device__ __forceinline__ float node_frac(int i, int nel, const float* sk) {
    const int e = min(i >> 2, nel - 1);
    return ((float)e + sk[i - 4 * e]) / (float)nel;
}
// Lattice interval containing fraction f: lower index and weight of the upper one.
__device__ __forceinline__ void locate(float f, int nel, const float* sk, int& i0, float& w) {
    float u = f * (float)nel;
    int e = min(max((int)floorf(u), 0), nel - 1);
    const float loc = u - (float)e;
    int k = 0;
    while (k < 3 && loc > sk[k + 1]) ++k;
    i0 = 4 * e + k;
    w = (loc - sk[k]) / (sk[k + 1] - sk[k]);
    w = fminf(fmaxf(w, 0.f), 1.f);
}

struct GllFrac {
    float s[5];   // (1 + xi_k) / 2
};

// d[i] += s * P(out) and g32[i] = that increment, rows >= 1 (P bilinear from the coarse grid)
__global__ void k_guess_prolong(const float* __restrict__ out, const float* __restrict__ scale, double* __restrict__ d,
                                float* __restrict__ g32, Layout L, GllFrac f) {
    EQC_GRID_WAIT();
    const float sc = scale[0];
    const int64_t n = L.size();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % L.ld), iy = (int)(i / L.ld);
        float v = 0.f;
        if (iy >= 1 && ix < L.nx && sc > 0.f) {
            const float gx = node_frac(ix, L.NelX, f.s) * (GN_GX - 1), gy = node_frac(iy, L.NelY, f.s) * (GN_GY - 1);
            const int i0 = min((int)gx, GN_GX - 2), j0 = min((int)gy, GN_GY - 2);
            const float wx = gx - (float)i0, wy = gy - (float)j0;
            const float* o = out + (int64_t)j0 * GN_GX + i0;
            v = sc * ((1.f - wy) * ((1.f - wx) * o[0] + wx * o[1]) + wy * ((1.f - wx) * o[GN_GX] + wx * o[GN_GX + 1]));
            d[i] += (double)v;
        }
        g32[i] = v;
    }
}

// Features of the first solve of a step: dF = d - dPre on the fault row, s = max |dF|,
// feat = [dF / s, log10(V / Vpl) / 4] with V = Vf0 (slip rate at the start of the step).
__global__ void __launch_bounds__(1024) k_guess_features(const double* __restrict__ d, const double* __restrict__ dPre,
                                                         const double* __restrict__ Vf0, int Nf, double Vpl,
                                                         float* __restrict__ feat, float* __restrict__ scale) {
    EQC_GRID_WAIT();
    __shared__ double sh[32];
    __shared__ double smax;
    double m = 0.0;
    for (int k = threadIdx.x; k < Nf; k += blockDim.x) m = fmax(m, fabs(d[k] - dPre[k]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        double b = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) b = fmax(b, sh[q]);
        smax = b;
        scale[0] = (float)b;
    }
    __syncthreads();
    const double s = smax;
    for (int k = threadIdx.x; k < Nf; k += blockDim.x) {
        feat[k] = s > 0 ? (float)((d[k] - dPre[k]) / s) : 0.f;
        feat[Nf + k] = (float)(log10(fmax(Vf0[k], 1e-30) / Vpl) / 4.0);
    }
}

// Logged pair at slot *count: the features and the target (d - dPre) / s sampled at the
// coarse grid points (bilinear in the GLL lattice).
__global__ void k_guess_log(const float* __restrict__ feat, const float* __restrict__ scale, const double* __restrict__ d,
                            const double* __restrict__ dPre, Layout L, GllFrac f, int Nf, float* __restrict__ log_in,
                            float* __restrict__ log_tgt, const long long* __restrict__ count, long long cap) {
    EQC_GRID_WAIT();
    const long long c = *count;
    if (c >= cap) return;
    const float sc = scale[0];
    const int nin = 2 * Nf, nout = GN_GX * GN_GY;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < nin + nout; j += gridDim.x * blockDim.x) {
        if (j < nin) {
            log_in[c * nin + j] = feat[j];
            continue;
        }
        const int q = j - nin, gi = q % GN_GX, gj = q / GN_GX;
        int i0, j0;
        float wx, wy;
        locate((float)gi / (GN_GX - 1), L.NelX, f.s, i0, wx);
        locate((float)gj / (GN_GY - 1), L.NelY, f.s, j0, wy);
        const int i1 = min(i0 + 1, L.nx - 1), j1 = min(j0 + 1, L.ny - 1);
        auto at = [&](int ix, int iy) {
            const int64_t p = (int64_t)iy * L.ld + ix;
            return (float)(d[p] - dPre[p]);
        };
        const float v = (1.f - wy) * ((1.f - wx) * at(i0, j0) + wx * at(i1, j0)) +
                        wy * ((1.f - wx) * at(i0, j1) + wx * at(i1, j1));
        log_tgt[c * nout + q] = sc > 0.f ? v / sc : 0.f;
    }
}
__global__ void k_guess_log_commit(long long* count, long long cap) {
    EQC_GRID_WAIT();
    if (*count < cap) *count += 1;
}

static GllFrac gll_frac() {
    static const double xg[5] = {-1.0, -0.65465367070797714, 0.0, 0.65465367070797714, 1.0};
    GllFrac f;
    for (int k = 0; k < 5; ++k) f.s[k] = (float)(0.5 * (1.0 + xg[k]));
    return f;
}

void gn_enqueue_features(Handle& h) {
    GuessNet& g = *h.net;
    k_guess_features<<<1, 1024, 0, h.stream>>>(h.d.p, h.dPre.p, h.F.Vf0.p, h.F.Nf, h.Vpl, g.feat.p, g.scale.p);
    EQC_CHECK_LAUNCH();
    count_launch();
}

void gn_enqueue_guess(Handle& h) {
    GuessNet& g = *h.net;
    gn_forward(g, g.feat.p, 1, h.stream);
    k_guess_prolong<<<nblk(h.L.size()), 256, 0, h.stream>>>(g.out.p, g.scale.p, h.d.p, h.g32.p, h.L, gll_frac());
    EQC_CHECK_LAUNCH();
    count_launch();
}

void gn_enqueue_log(Handle& h) {
    GuessNet& g = *h.net;
    const int n = 2 * g.Nf + GN_GX * GN_GY;
    k_guess_log<<<(n + 255) / 256, 256, 0, h.stream>>>(g.feat.p, g.scale.p, h.d.p, h.dPre.p, h.L, gll_frac(), g.Nf,
                                                       g.log_in.p, g.log_tgt.p, g.log_count.p, g.log_cap);
    k_guess_log_commit<<<1, 1, 0, h.stream>>>(g.log_count.p, g.log_cap);
    EQC_CHECK_LAUNCH();
    count_launch(2);
}

// ---- training ---------------------------------------------------------------------------
// x0[b] = pin[idx[b]], tgt[b] = ptgt[idx[b]]
__global__ void k_gather_batch(const float* __restrict__ pin, const float* __restrict__ ptgt, const int* __restrict__ idx,
                               int B, int nin, int nout, float* __restrict__ x0, float* __restrict__ tgt) {
    EQC_GRID_WAIT();
    const int64_t n = (int64_t)B * (nin + nout);
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(e / (nin + nout)), j = (int)(e % (nin + nout));
        const int64_t src = idx[b];
        if (j < nin) x0[(int64_t)b * nin + j] = pin[src * nin + j];
        else tgt[(int64_t)b * nout + (j - nin)] = ptgt[src * nout + (j - nin)];
    }
}
__global__ void k_sum_loss(const double* __restrict__ loss, int B, double* acc) {
    EQC_GRID_WAIT();
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int b = 0; b < B; ++b) s += loss[b];
        *acc += s;
    }
}

struct TrainBufs {
    DBuf<int> idx;
    DBuf<float> tgt;
    DBuf<double> acc;
};

// Trains on the n pairs resident in g.pin / g.ptgt; epoch_loss[e] = mean squared error per output.
static void gn_train(Handle& h, int64_t n, int epochs, double lr, int batch, uint64_t seed, double* epoch_loss) {
    GuessNet& g = *h.net;
    cudaStream_t s = h.stream;
    const int nin = 2 * g.Nf, nout = g.nout;
    batch = (int)std::max<int64_t>(1, std::min<int64_t>(batch, n));
    gn_reserve(g, batch);
    TrainBufs tb;
    tb.idx.alloc(n);
    tb.tgt.alloc((size_t)batch * nout);
    tb.acc.alloc(1);
    std::vector<int> perm(n);
    std::mt19937_64 rng(seed ^ 0x9e3779b97f4a7c15ull);
    for (int e = 0; e < epochs; ++e) {
        for (int64_t i = 0; i < n; ++i) perm[i] = (int)i;
        std::shuffle(perm.begin(), perm.end(), rng);
        tb.idx.upload(perm.data(), n, s);
        tb.acc.zero(s);
        for (int64_t b0 = 0; b0 + batch <= n; b0 += batch) {   // whole batches only
            k_gather_batch<<<nblk((int64_t)batch * (nin + nout)), 256, 0, s>>>(g.pin.p, g.ptgt.p, tb.idx.p + b0, batch,
                                                                             nin, nout, g.x0.p, tb.tgt.p);
            count_launch();
            gn_forward(g, g.x0.p, batch, s);
            gn_backward(g, g.x0.p, tb.tgt.p, batch, s);
            k_sum_loss<<<1, 1, 0, s>>>(g.loss.p, batch, tb.acc.p);
            count_launch();
            gn_adam(g, lr, s);
        }
        double acc = 0;
        tb.acc.download(&acc, 1, s);
        EQC_CUDA(cudaStreamSynchronize(s));
        const int64_t used = (n / batch) * batch;
        if (epoch_loss) epoch_loss[e] = used ? acc / ((double)used * nout) : 0.0;
    }
    EQC_CUDA(cudaStreamSynchronize(s));
    g.trained = true;
}

// Mean squared error per output over n pairs (batched forward); out (optional) gets the outputs.
static double gn_eval(Handle& h, int64_t n, float* out_host) {
    GuessNet& g = *h.net;
    cudaStream_t s = h.stream;
    const int nin = 2 * g.Nf, nout = g.nout;
    const int batch = (int)std::min<int64_t>(std::max<int64_t>(n, 1), 256);
    gn_reserve(g, batch);
    TrainBufs tb;
    tb.idx.alloc(batch);
    tb.tgt.alloc((size_t)batch * nout);
    tb.acc.alloc(1);
    tb.acc.zero(s);
    std::vector<int> ids(batch);
    for (int64_t b0 = 0; b0 < n; b0 += batch) {
        const int B = (int)std::min<int64_t>(batch, n - b0);
        for (int b = 0; b < B; ++b) ids[b] = (int)(b0 + b);
        tb.idx.upload(ids.data(), B, s);
        k_gather_batch<<<nblk((int64_t)B * (nin + nout)), 256, 0, s>>>(g.pin.p, g.ptgt.p, tb.idx.p, B, nin, nout,
                                                                       g.x0.p, tb.tgt.p);
        gn_forward(g, g.x0.p, B, s);
        k_mse<<<B, 256, 0, s>>>(g.out.p, tb.tgt.p, nout, B, g.g_out.p, g.loss.p);
        k_sum_loss<<<1, 1, 0, s>>>(g.loss.p, B, tb.acc.p);
        count_launch(3);
        if (out_host) g.out.download(out_host + b0 * nout, (size_t)B * nout, s);
        EQC_CUDA(cudaStreamSynchronize(s));
    }
    double acc = 0;
    tb.acc.download(&acc, 1, s);
    EQC_CUDA(cudaStreamSynchronize(s));
    return n ? acc / ((double)n * nout) : 0.0;
}

static void upload_pairs(Handle& h, const float* in, const float* tgt, int64_t n) {
    GuessNet& g = *h.net;
    const int nin = 2 * g.Nf, nout = g.nout;
    if ((int64_t)g.pin.n < n * nin) g.pin.alloc((size_t)n * nin);
    if ((int64_t)g.ptgt.n < n * nout) g.ptgt.alloc((size_t)n * nout);
    if (in) {
        g.pin.upload(in, (size_t)n * nin, h.stream);
        g.ptgt.upload(tgt, (size_t)n * nout, h.stream);
    } else {   // the pairs logged by this handle's time loop
        long long c = 0;
        g.log_count.download(&c, 1, h.stream);
        EQC_CUDA(cudaStreamSynchronize(h.stream));
        if (c < n) throw Error(EQC_E_ARG, "fewer logged pairs than requested");
        EQC_CUDA(cudaMemcpyAsync(g.pin.p, g.log_in.p, sizeof(float) * n * nin, cudaMemcpyDeviceToDevice, h.stream));
        EQC_CUDA(cudaMemcpyAsync(g.ptgt.p, g.log_tgt.p, sizeof(float) * n * nout, cudaMemcpyDeviceToDevice, h.stream));
    }
    g.npairs = n;
}

static GuessNet& net_of(Handle& h) {
    if (!h.net) {
        h.net = new GuessNet();
        gn_init(h, 1234);
    }
    return *h.net;
}

}  // namespace eqc

using namespace eqc;

template <class F>
static eqc_status guarded_net(eqc_handle* H, F&& f) {
    if (!H) return EQC_E_ARG;
    try {
        f(H->h);
        return EQC_OK;
    } catch (const Error& e) {
        H->h.err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        H->h.err = e.what();
        return EQC_E_ARG;
    }
}

extern "C" {

eqc_status eqc_guess_shape(eqc_handle* H, int32_t* nin, int32_t* nout, int64_t* nparam) {
    return guarded_net(H, [&](Handle& h) {
        GuessNet& g = net_of(h);
        if (nin) *nin = 2 * g.Nf;
        if (nout) *nout = g.nout;
        if (nparam) *nparam = g.nparam;
    });
}

eqc_status eqc_guess_init(eqc_handle* H, uint64_t seed) {
    return guarded_net(H, [&](Handle& h) {
        net_of(h);
        gn_init(h, seed);
        destroy_graphs(h);
    });
}

eqc_status eqc_guess_get_params(eqc_handle* H, float* p) {
    if (!p) return EQC_E_ARG;
    return guarded_net(H, [&](Handle& h) {
        GuessNet& g = net_of(h);
        g.master.download(p, g.nparam, h.stream);
        EQC_CUDA(cudaStreamSynchronize(h.stream));
    });
}

eqc_status eqc_guess_set_params(eqc_handle* H, const float* p) {
    if (!p) return EQC_E_ARG;
    return guarded_net(H, [&](Handle& h) {
        GuessNet& g = net_of(h);
        g.master.upload(p, g.nparam, h.stream);
        gn_refresh_bf16(g, h.stream);
        g.m1.zero(h.stream);
        g.m2.zero(h.stream);
        g.adam_t = 0;
        g.trained = true;
        EQC_CUDA(cudaStreamSynchronize(h.stream));
        destroy_graphs(h);
    });
}

eqc_status eqc_guess_log(eqc_handle* H, int64_t capacity) {
    if (capacity < 0) return EQC_E_ARG;
    return guarded_net(H, [&](Handle& h) {
        GuessNet& g = net_of(h);
        g.log_cap = capacity;
        if (capacity > 0) {
            g.log_in.alloc((size_t)capacity * 2 * g.Nf);
            g.log_tgt.alloc((size_t)capacity * g.nout);
        } else {
            g.log_in.release();
            g.log_tgt.release();
        }
        g.log_count.alloc(1);
        destroy_graphs(h);
    });
}

eqc_status eqc_guess_pairs(eqc_handle* H, float* in, float* tgt, int64_t* n) {
    if (!n) return EQC_E_ARG;
    return guarded_net(H, [&](Handle& h) {
        GuessNet& g = net_of(h);
        long long c = 0;
        if (g.log_count.p) {
            g.log_count.download(&c, 1, h.stream);
            EQC_CUDA(cudaStreamSynchronize(h.stream));
        }
        *n = c;
        if (in && c) g.log_in.download(in, (size_t)c * 2 * g.Nf, h.stream);
        if (tgt && c) g.log_tgt.download(tgt, (size_t)c * g.nout, h.stream);
        EQC_CUDA(cudaStreamSynchronize(h.stream));
    });
}

eqc_status eqc_guess_train(eqc_handle* H, const float* in, const float* tgt, int64_t n, int32_t epochs, double lr,
                           int32_t batch, uint64_t seed, double* epoch_loss) {
    if (n < 1 || epochs < 1 || batch < 1 || !(lr > 0) || (in == nullptr) != (tgt == nullptr)) return EQC_E_ARG;
    return guarded_net(H, [&](Handle& h) {
        net_of(h);
        upload_pairs(h, in, tgt, n);
        gn_train(h, n, epochs, lr, batch, seed, epoch_loss);
        destroy_graphs(h);
    });
}

eqc_status eqc_guess_eval(eqc_handle* H, const float* in, const float* tgt, int64_t n, double* mse, float* out) {
    if (!in || !tgt || n < 1 || !mse) return EQC_E_ARG;
    return guarded_net(H, [&](Handle& h) {
        net_of(h);
        destroy_graphs(h);   // batch buffers may move
        upload_pairs(h, in, tgt, n);
        *mse = gn_eval(h, n, out);
    });
}

eqc_status eqc_guess_grad(eqc_handle* H, const float* in, const float* tgt, int64_t n, float* grad, double* loss) {
    if (!in || !tgt || n < 1 || !grad) return EQC_E_ARG;
    return guarded_net(H, [&](Handle& h) {
        GuessNet& g = net_of(h);
        destroy_graphs(h);   // batch buffers may move
        upload_pairs(h, in, tgt, n);
        gn_reserve(g, (int)n);
        EQC_CUDA(cudaMemcpyAsync(g.x0.p, g.pin.p, sizeof(float) * n * 2 * g.Nf, cudaMemcpyDeviceToDevice, h.stream));
        gn_forward(g, g.x0.p, (int)n, h.stream);
        gn_backward(g, g.x0.p, g.ptgt.p, (int)n, h.stream);
        g.grad.download(grad, g.nparam, h.stream);
        std::vector<double> l(n);
        g.loss.download(l.data(), n, h.stream);
        EQC_CUDA(cudaStreamSynchronize(h.stream));
        double t = 0;
        for (double v : l) t += v;
        if (loss) *loss = t / ((double)n * g.nout);
    });
}

}  // extern "C"
