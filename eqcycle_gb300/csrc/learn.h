// Learned initial guess for the quasi-static solve: a small network maps the fault slip
// increment and slip-rate profile of a solve to the displacement increment on a coarse
// GX x GY grid over the domain, prolonged bilinearly to the GLL nodes.
//
//   input  [2][Nf]: dF / s and log10(V / Vpl) / 4, s = max |dF| (dF = F - F_prev on the fault)
//   conv1..conv4: kernel 5, stride 2, padding 2, 64 channels, GELU  -> [64][T4]
//   fc1: 64*T4 -> NH, GELU ; fc2: NH -> GX*GY  (the increment / s on the coarse grid)
//
// Weights are stored in BF16 (FP32 master copies and Adam moments for training); every
// product accumulates in FP32.  Forward and backward kernels are in learn.cu.
#pragma once
#include "model.h"
#include <cuda_bf16.h>

namespace eqc {

constexpr int GN_C = 64, GN_K = 5, GN_LAYERS = 4, GN_NH = 512, GN_GX = 121, GN_GY = 61;

struct GuessNet {
    int Nf = 0;
    int T[GN_LAYERS + 1] = {};   // T[0] = Nf, T[l+1] = (T[l] - 1) / 2 + 1
    int flat = 0, nout = GN_GX * GN_GY;
    // parameter offsets (floats) in the flat parameter vector
    int64_t off_cw[GN_LAYERS], off_cb[GN_LAYERS], off_f1w, off_f1b, off_f2w, off_f2b, nparam = 0;
    DBuf<float> master, grad, m1, m2;     // FP32 master weights, gradient, Adam moments
    DBuf<__nv_bfloat16> wbf;              // BF16 copy used by every product
    int64_t adam_t = 0;
    bool trained = false;
    // activations for a batch of up to cap samples
    int cap = 0;
    DBuf<float> x0, z[GN_LAYERS], a[GN_LAYERS], zf1, af1, out, g_out, g_af1, g_a[GN_LAYERS], g_x;
    // training pairs resident on the device
    DBuf<float> pin, ptgt;
    int64_t npairs = 0;
    DBuf<double> loss;                     // per-sample squared error sums
    // logging in the time loop
    int64_t log_cap = 0;
    DBuf<float> log_in, log_tgt;
    DBuf<long long> log_count;
    // inference in the time loop (batch 1)
    DBuf<float> feat, scale;
};

void gn_init(Handle& h, uint64_t seed);                 // shapes, buffers, seeded weights
void gn_reserve(GuessNet& g, int batch);
void gn_forward(GuessNet& g, const float* x0, int B, cudaStream_t s);          // -> g.out
void gn_backward(GuessNet& g, const float* x0, const float* tgt, int B, cudaStream_t s);  // -> g.grad, g.loss
void gn_adam(GuessNet& g, double lr, cudaStream_t s);
void gn_refresh_bf16(GuessNet& g, cudaStream_t s);
// time-loop hooks (stepper.cu): features of the first solve of a step, guess increment, logging
void gn_enqueue_features(Handle& h);
void gn_enqueue_guess(Handle& h);      // d += g (rows >= 1), g32 = g
void gn_enqueue_log(Handle& h);        // after the first solve: (features, target) pair

}  // namespace eqc
