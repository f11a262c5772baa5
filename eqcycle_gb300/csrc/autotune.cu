// Solver autotuner: picks, by timing graph-replayed trial solves of the next quasi-static solve
// of the current model, (1) the Chebyshev smoothing degrees of the multigrid V-cycle (spectral-
// element level and vertex levels), then, in mixed precision, (2) the FP32 stiffness-apply
// kernel and its tile shape (element rows per CTA, or the TMA-fed walk with its one-wave grid)
// and (3) the residual-replacement factor of the reliable updates.  Which choice is fastest
// depends on the mesh (a cheaper coarse smoother can cost more CG iterations; a tile shape
// changes the number of waves; fewer FP64 updates can cost restarts), so it is measured, not
// fixed.
#include "model.h"
#include "mg.h"
#include <cstring>

namespace eqc {

// d0 = d with the fault row moved to the next step's first F = d + v dt (src/main.jl:231-238)
__global__ void k_trial_rhs(const double* __restrict__ d, const double* __restrict__ v, double* __restrict__ d0,
                            int64_t n, int Nf, const Ctrl* C) {
    EQC_GRID_WAIT();
    const double dt = C->dt;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        d0[i] = (i < Nf) ? d[i] + v[i] * dt : d[i];
}

static double trial(Handle& h, const double* d0, int reps, int* iters) {
    cudaStream_t s = h.stream;
    const int64_t n = h.L.size();
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    try {
        EQC_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        EQC_CUDA(cudaMemcpyAsync(h.d.p, d0, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        enqueue_solve(h, h.opt.cg_tol, h.opt.cg_maxit, true, false, nullptr);
        EQC_CUDA(cudaStreamEndCapture(s, &g));
        make_programmatic(g);
    } catch (...) {
        abort_capture(h);
        throw;
    }
    EQC_CUDA(cudaGraphInstantiate(&ge, g, 0));
    cudaEvent_t e0, e1;
    EQC_CUDA(cudaEventCreate(&e0));
    EQC_CUDA(cudaEventCreate(&e1));
    EQC_CUDA(cudaGraphLaunch(ge, s));   // warm-up
    EQC_CUDA(cudaEventRecord(e0, s));
    for (int r = 0; r < reps; ++r) EQC_CUDA(cudaGraphLaunch(ge, s));
    EQC_CUDA(cudaEventRecord(e1, s));
    EQC_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    EQC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    Ctrl c;
    EQC_CUDA(cudaMemcpy(&c, h.ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost));
    *iters = c.cg_last_it;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGraphExecDestroy(ge);
    cudaGraphDestroy(g);
    if (c.cg_fail) throw Error(EQC_E_CG, "autotune trial solve did not converge");
    return ms / reps;
}

}  // namespace eqc

using namespace eqc;

extern "C" eqc_status eqc_autotune(eqc_handle* H, int32_t reps, int32_t* deg_out, int32_t* degc_out,
                                   double* ms_out) {
    if (!H || reps < 1) return EQC_E_ARG;
    Handle& h = H->h;
    try {
        if (!h.initialized) throw Error(EQC_E_STATE, "eqc_autotune before eqc_init");
        if (!h.mg) throw Error(EQC_E_STATE, "eqc_autotune needs the multigrid preconditioner");
        cudaStream_t s = h.stream;
        const int64_t n = h.L.size();
        DBuf<double> dsave, d0;
        dsave.alloc(n);
        d0.alloc(n);
        DBuf<Ctrl> csave;
        csave.alloc(1);
        EQC_CUDA(cudaMemcpyAsync(dsave.p, h.d.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        EQC_CUDA(cudaMemcpyAsync(csave.p, h.ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToDevice, s));
        k_trial_rhs<<<(int)std::min<int64_t>((n + 255) / 256, 1216), 256, 0, s>>>(h.d.p, h.v.p, d0.p, n, h.F.Nf,
                                                                                   h.ctrl.p);
        EQC_CHECK_LAUNCH();
        count_launch();
        MGHier& m = *h.mg;
        const int deg0 = m.deg, degc0 = m.deg_coarse;
        int best_d = deg0, best_c = degc0;
        double best = 1e30;
        for (int dg : {3, 4, 5})
            for (int dc : {1, 3, 4}) {
                m.deg = dg;
                m.deg_coarse = dc;
                int it = 0;
                const double ms = trial(h, d0.p, reps, &it);
                if (ms < best) { best = ms; best_d = dg; best_c = dc; }
            }
        m.deg = best_d;
        m.deg_coarse = best_c;
        h.opt.mg_degree = best_d;
        h.opt.mg_degree_coarse = best_c;
        if (h.opt.precision == EQC_MIXED) {
            // FP32 apply: 6 element rows per CTA (3 or 2 CTAs per SM), 4 rows, or the walk
            const int v0 = h.opt.apply_variant;
            int best_v = v0;
            for (int v : {0, 7, 4, 8}) {
                if (v == v0) continue;
                h.opt.apply_variant = v;
                int it = 0;
                const double ms = trial(h, d0.p, reps, &it);
                if (ms < best) { best = ms; best_v = v; }
            }
            h.opt.apply_variant = best_v;
            // reliable-update factor
            const double r0 = h.opt.reliable_delta > 0 ? h.opt.reliable_delta : 1e-3;
            double best_r = r0;
            for (double r : {1e-2, 1e-4}) {
                h.opt.reliable_delta = r;
                int it = 0;
                const double ms = trial(h, d0.p, reps, &it);
                if (ms < best) { best = ms; best_r = r; }
            }
            h.opt.reliable_delta = best_r;
        }
        // the state and the counters as they were; the trial solves overwrote the residual
        EQC_CUDA(cudaMemcpyAsync(h.d.p, dsave.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
        EQC_CUDA(cudaMemcpyAsync(h.ctrl.p, csave.p, sizeof(Ctrl), cudaMemcpyDeviceToDevice, s));
        invalidate_residual(h);
        EQC_CUDA(cudaMemcpyAsync(h.h_ctrl, h.ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
        EQC_CUDA(cudaStreamSynchronize(s));
        destroy_graphs(h);
        if (deg_out) *deg_out = best_d;
        if (degc_out) *degc_out = best_c;
        if (ms_out) *ms_out = best;
        return EQC_OK;
    } catch (const Error& e) {
        h.err = e.what();
        return e.code;
    }
}
