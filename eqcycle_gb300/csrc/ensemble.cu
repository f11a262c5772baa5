// Ensemble of fault models advanced by one CUDA-graph launch per time step.
//
// Every member (an independent eqc_handle on the same GPU) is a branch of one graph: a selector
// kernel reads the member's regime from its device control block and sets two conditional IF
// nodes, one holding the member's quasi-static step (with its device-driven CG loops), the other
// its dynamic step.  Members therefore advance concurrently, each in its own regime, without the
// host choosing anything; after the launch the host reads every member's control block once and
// runs its output bookkeeping (main.jl:361-436), exactly as for a single model.
#include "model.h"
#include <chrono>

namespace eqc {

__global__ void k_regime_select(const Ctrl* C, cudaGraphConditionalHandle hq, cudaGraphConditionalHandle hd) {
    EQC_GRID_WAIT();
    const unsigned q = C->isolver == 1 ? 1u : 0u;
    cudaGraphSetConditional(hq, q);
    cudaGraphSetConditional(hd, 1u - q);
}

}  // namespace eqc

using namespace eqc;

struct eqc_ensemble {
    std::vector<Handle*> mem;
    std::vector<StepGraph> rec;      // [2 m + (regime - 1)]: kernels of the member's step bodies
    std::vector<PostBufs> pb;
    cudaStream_t stream = nullptr;
    std::vector<cudaEvent_t> ev;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<int64_t> gens;       // members' K generations at capture (damage evolution)
    std::string err;
    void drop_graph() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        exec = nullptr;
        graph = nullptr;
    }
    ~eqc_ensemble() {
        drop_graph();
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace eqc {

static void ensemble_capture(eqc_ensemble& E) {
    const size_t n = E.mem.size();
    E.rec.assign(2 * n, StepGraph());
    cudaStream_t s0 = E.stream;
    capture_counting(true);
    try {
        EQC_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
        EQC_CUDA(cudaEventRecord(E.ev[0], s0));
        for (size_t m = 0; m < n; ++m) {
            Handle& h = *E.mem[m];
            EQC_CUDA(cudaStreamWaitEvent(h.stream, E.ev[0], 0));   // the member's stream joins the capture
            const cudaGraphConditionalHandle hq = cond_handle(h), hd = cond_handle(h);
            k_regime_select<<<1, 1, 0, h.stream>>>(h.ctrl.p, hq, hd);
            EQC_CHECK_LAUNCH();
            count_launch();
            for (int reg = 1; reg <= 2; ++reg) {
                StepGraph& G = E.rec[2 * m + (reg - 1)];
                h.capturing = &G;
                const int64_t t0 = capture_tally();
                cond_begin(h, cudaGraphCondTypeIf, reg == 1 ? hq : hd);
                enqueue_step(h, reg, true);
                cond_end(h);
                h.pdl_off = false;
                G.k_fixed = (capture_tally() - t0) - G.k_bodies + G.k_fixed_extra + 1;   // + the selector
                h.capturing = nullptr;
            }
            EQC_CUDA(cudaEventRecord(E.ev[1 + m], h.stream));
            EQC_CUDA(cudaStreamWaitEvent(s0, E.ev[1 + m], 0));    // join
        }
        EQC_CUDA(cudaStreamEndCapture(s0, &E.graph));
        make_programmatic(E.graph);
    } catch (...) {
        for (Handle* hp : E.mem) {
            hp->capturing = nullptr;
            abort_capture(*hp);
        }
        cudaGraph_t g = nullptr;
        cudaStreamEndCapture(s0, &g);
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        capture_counting(false);
        throw;
    }
    capture_counting(false);
    EQC_CUDA(cudaGraphInstantiate(&E.exec, E.graph, 0));
    E.gens.resize(n);
    for (size_t m = 0; m < n; ++m) E.gens[m] = E.mem[m]->gen;
}

// A member whose K changed (damage evolution) invalidates the captured ensemble step.
static void check_gens(eqc_ensemble& E) {
    for (size_t m = 0; m < E.mem.size() && E.exec; ++m)
        if (m >= E.gens.size() || E.gens[m] != E.mem[m]->gen) E.drop_graph();
}

}  // namespace eqc

extern "C" {

eqc_status eqc_ensemble_create(eqc_handle* const* members, int32_t n, eqc_ensemble** out) {
    if (!members || n < 1 || !out) return EQC_E_ARG;
    *out = nullptr;
    eqc_ensemble* E = new eqc_ensemble();
    try {
        int dev = -1;
        for (int32_t m = 0; m < n; ++m) {
            if (!members[m]) throw Error(EQC_E_ARG, "null member handle");
            Handle& h = members[m]->h;
            if (m == 0) dev = h.opt.device;
            if (h.opt.device != dev) throw Error(EQC_E_ARG, "ensemble members must share one device");
            for (int32_t k = 0; k < m; ++k)
                if (members[k] == members[m]) throw Error(EQC_E_ARG, "a handle appears twice in the ensemble");
            E->mem.push_back(&h);
        }
        EQC_CUDA(cudaSetDevice(dev));
        EQC_CUDA(cudaStreamCreateWithFlags(&E->stream, cudaStreamNonBlocking));
        E->ev.resize(n + 1);
        for (cudaEvent_t& e : E->ev) EQC_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        E->pb.resize(n);
    } catch (const Error& e) {
        set_thread_error(e.what());
        eqc_status c = e.code;
        delete E;
        return c;
    }
    *out = E;
    return EQC_OK;
}

eqc_status eqc_ensemble_destroy(eqc_ensemble* E) {
    if (!E) return EQC_E_ARG;
    delete E;
    return EQC_OK;
}

const char* eqc_ensemble_last_error(const eqc_ensemble* E) { return E ? E->err.c_str() : ""; }

eqc_status eqc_ensemble_run(eqc_ensemble* E, int64_t steps, eqc_run_stats* stats, double* gpu_ms) {
    if (!E || steps < 0) return EQC_E_ARG;
    const size_t n = E->mem.size();
    try {
        for (Handle* h : E->mem)
            if (!h->initialized) throw Error(EQC_E_STATE, "ensemble member not initialised (eqc_init)");
        check_gens(*E);
        if (!E->exec) ensemble_capture(*E);
        cudaStream_t s0 = E->stream;
        auto t0 = std::chrono::steady_clock::now();
        std::vector<eqc_run_stats> st(n, eqc_run_stats{});
        std::vector<long long> cg0(n), qs0(n);
        for (size_t m = 0; m < n; ++m) {
            Handle& h = *E->mem[m];
            EQC_CUDA(cudaStreamSynchronize(h.stream));
            EQC_CUDA(cudaMemcpyAsync(h.h_ctrl, h.ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost, s0));
        }
        EQC_CUDA(cudaStreamSynchronize(s0));
        for (size_t m = 0; m < n; ++m) {
            cg0[m] = E->mem[m]->h_ctrl->cg_iters;
            qs0[m] = E->mem[m]->h_ctrl->cg_solves;
        }
        cudaEvent_t e0, e1;
        EQC_CUDA(cudaEventCreate(&e0));
        EQC_CUDA(cudaEventCreate(&e1));
        EQC_CUDA(cudaEventRecord(e0, s0));
        std::vector<int> iso(n);
        std::vector<Ctrl> before(n);
        for (int64_t k = 0; k < steps; ++k) {
            for (size_t m = 0; m < n; ++m) {
                before[m] = *E->mem[m]->h_ctrl;
                iso[m] = before[m].isolver;
            }
            check_gens(*E);
            if (!E->exec) ensemble_capture(*E);
            EQC_CUDA(cudaGraphLaunch(E->exec, s0));
            for (size_t m = 0; m < n; ++m)
                EQC_CUDA(cudaMemcpyAsync(E->mem[m]->h_ctrl, E->mem[m]->ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost, s0));
            EQC_CUDA(cudaStreamSynchronize(s0));
            for (size_t m = 0; m < n; ++m) {
                Handle& h = *E->mem[m];
                const Ctrl& C = *h.h_ctrl;
                const StepGraph& G = E->rec[2 * m + (iso[m] - 1)];
                const long long carried = C.cg_carried - before[m].cg_carried;
                g_launches += G.k_fixed + G.k_iter * (C.cg_iters - before[m].cg_iters) +
                              G.k_update * (C.cg_updates - before[m].cg_updates) + G.k_carry * carried +
                              G.k_full * (C.cg_solves - before[m].cg_solves - carried);
                post_step(h, iso[m], st[m], E->pb[m]);
            }
        }
        EQC_CUDA(cudaEventRecord(e1, s0));
        EQC_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        EQC_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (size_t m = 0; m < n; ++m) {
            Handle& h = *E->mem[m];
            const Ctrl& C = *h.h_ctrl;
            st[m].cg_iters = C.cg_iters - cg0[m];
            st[m].qs_solves = C.cg_solves - qs0[m];
            st[m].t = C.t;
            st[m].dt = C.dt;
            st[m].isolver = C.isolver;
            st[m].events = (int32_t)h.it_s;
            st[m].wall_s = wall;
            st[m].gpu_ms = ms;
            if (stats) stats[m] = st[m];
        }
        if (gpu_ms) *gpu_ms = ms;
        return EQC_OK;
    } catch (const Error& e) {
        E->err = e.what();
        return e.code;
    }
}

}  // extern "C"
