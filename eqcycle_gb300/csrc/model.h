// The handle: one fault model resident on one GPU.
#pragma once
#include "common.h"
#include "epi.cuh"
#include <memory>

namespace eqc {

// Fault-row parameters and state, [Nf] each, in fault order (= iFlt order = row 0 of the layout).
struct FaultDev {
    int Nf = 0;
    int NFBC0 = 0;  // first friction node (0-based), NFBC - 1 of src/main.jl:186
    DBuf<double> fo, Vo, xLf, cca, ccb, Seff, tauo, XiLf, FltB, FltZ, FltX, Mf;
    DBuf<double> psi, psi1, psi2, tau, tau1, tau2, Vf, Vf0, Vf1, Vf2, FltVfree, vPre;
    DBuf<double> Flast;   // fault displacement the carried CG residual belongs to
    DBuf<int> creep;   // 1 for fault nodes listed in iFBC (creeping), [Nf]
};

// Device-side control block of the time loop.
struct Ctrl {
    double t, dt, dtmin, half_dt, half_dt_sq, Vpl;
    double Vfmax;          // of the step just taken
    int isolver;           // regime of the next step
    int fail;              // 1 + node of a friction failure
    long long it;
    double vhypo;          // max of 2v+Vpl over the fault and
    int ihypo;             // its first index
    int apply_err;         // set by the stiffness apply when a bounded TMA wait gives up
    // quasi-static solve counters, accumulated on the device
    long long cg_iters;    // CG iterations over all solves
    long long cg_solves;   // solves
    long long cg_updates;  // reliable updates (mixed precision)
    long long cg_carried;  // solves that started from the carried residual
    long long cg_restarts; // reliable updates after which the search direction restarted
    long long guess_tried, guess_kept;   // initial-guess increments judged / kept
    int cg_fail;           // bit 0: a solve reached maxit; bit 1: non-finite residual
    int cg_last_it;        // iterations of the last solve
    double cg_last_relres; // ||r|| / ||b|| of the last solve
    int r_valid;           // r64 holds the FP64 true residual of d with fault row Flast
                           // (mixed precision: carried into the next solve)
    double dt_prev;        // dt of the step before the current one
    int qs_prev;           // the last step was quasi-static: dPre holds the solution before it
    // batched steps (several steps per graph launch): the host's output-trigger state, written
    // before each launch, and the device logs' fill counts (k_step_end)
    double tvsx, tevneb, tevne, t_end, Vthres, Vevne;
    int slipstart, idelevne, verbose, max_batch, rec_cap;
    int nlog, nrec;        // steps logged (time_, Vfmax) / receiver records in this launch
    // mixed-precision Newmark: Kd = K d kept in FP64, updated by the FP32 apply of each step's
    // increment and refreshed in FP64 at the start of a dynamic phase and every KD_REFRESH steps
    int kd_valid, kd_age, kd_full;
    int v_half;            // mixed method's dynamic phase: v off the fault row holds the next step's
                           // half-step velocity v + dt/2 a (a there is not kept); 0: v and a as is
    double dt_step;        // dt of the dynamic step in progress (the mixed method's split predictor)
};
constexpr int KD_REFRESH = 256;

// Device-resident scalars of one CG solve.
struct CGState {
    double rho, rho_prev, pq, rr, bb;
    double nb, reltol, res, rmax;
    int it, maxit;
    int done;          // 0 running, 1 converged, 2 maxit reached, 3 non-finite residual
    int need_update;   // mixed precision: a reliable update is due
    int upd_incr;      // ... and it is an intermediate one (the residual fell by the update factor,
                       // the loop goes on): r -= K dx in double-float; else b - K x in FP64
    int incr_ok;       // this solve's updates may take the double-float form
    int restart;       // the next direction update starts afresh (beta = 0)
    double sigma;      // mixed precision: the FP32 recurrence vectors hold sigma * (true value),
                       // sigma a power of two near 1 / ||b|| (keeps tiny residuals out of
                       // FP32 underflow); 1 in FP64.  rr is in those scaled units.
    double rr_guess;   // ||r||^2 with the initial-guess increment applied
    int guess_keep;    // the increment lowered the residual and is kept
};

// A captured time step (one per regime) and the kernels it launches.
struct StepGraph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t k_fixed = 0;     // kernels outside conditional bodies
    int64_t k_iter = 0;      // kernels of one CG iteration (while body, without the update)
    int64_t k_update = 0;    // kernels of one reliable update (if body)
    int64_t k_carry = 0;     // kernels of a carried residual set-up (if body)
    int64_t k_full = 0;      // kernels of a full residual set-up (if body)
    int64_t k_bodies = 0;    // capture tally of all conditional bodies
    int64_t k_fixed_extra = 0;   // kernels of if-bodies that run every step (one of a pair)
};

// Multigrid hierarchy (defined in mg.h), learned-guess network (learn.h).
struct MGHier;
struct GuessNet;

struct Handle {
    eqc_options opt{};
    std::string err;
    // damage evolution (damageEvol.jl): elements (0-based) whose W is scaled by damage_factor
    // at the end of every event; gen counts changes of K (graphs holding the old K are stale)
    std::vector<int64_t> damage_el;
    double damage_factor = 1.0;
    int64_t damage_count = 0;
    int64_t gen = 0;
    double setup_ms[5] = {0, 0, 0, 0, 0};
    int64_t pdl_edges = 0;   // programmatic kernel-to-kernel edges in the captured graphs
    int tma_wait_polls = MBAR_SPIN_LIMIT;   // first-tile wait bound of the TMA applies (testing)
    int64_t cap_time = 1900000;              // capacity of time_ / Vfmax (main.jl:154-163)
    // V-cycle pointwise work fused into the operator kernels (EQC_NO_FUSE set at creation: the
    // separate kernels, for comparisons)
    bool fuse = true;   // eqc_create phases: numbering, elements, nodes, other, hierarchy
    // Stream that work is enqueued on: the handle's own stream, or, while a conditional
    // body of a step graph is being captured, that body's capture stream.
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t cap_streams[4] = {nullptr, nullptr, nullptr, nullptr};
    std::vector<cudaStream_t> stream_stack;
    StepGraph graphs[2];       // [0] quasi-static step, [1] dynamic step
    StepGraph batched[2];      // the same, looping over steps on the device (k_step_end)
    DBuf<double> log_t, log_vf, log_seis;   // per-step device logs of a batched launch
    StepGraph* capturing = nullptr;   // graph whose capture is in progress
    int device = 0;
    Layout L{};
    int64_t nglob = 0, Nel = 0;
    double dxe = 0, dye = 0, c1 = 0, c2 = 0;
    double Vpl = 0, Vthres = 0, Vevne = 0, dt0 = 0, Total_time = 0, yr2sec = 0;
    // reference numbering <-> layout
    std::vector<int64_t> ref2lay;    // [nglob] reference node (0-based) -> layout index
    // the dynamic step's boundary operations per node of iCreep U iBcL U iBcT: bit 0 zero a,
    // bit 1 subtract the left term, bit 2 the top term (k_dyn_bc's order)
    DBuf<int64_t> bcNode;
    DBuf<int> bcOps;
    DBuf<double> bcL, bcT;
    int nBcNodes = 0;
    bool creep_prefix = false;   // iCreep lies in the fault row (its nodes: the prefix [0, NFBC0))
    // the mixed method's dynamic step in four kernels: absorbing-boundary coefficients by position
    // on the two edges the lists lie on (column ix = 0: iBcL; row iy = ny - 1: iBcT)
    DBuf<double> edgeL, edgeT;
    DBuf<int> edgeLhas, edgeThas;
    bool nm_fused = false;       // the lists lie on those edges, once each, and creep_prefix
    int edgeL0has = 0;           // the fault's bottom node (0, 0) is in iBcL, with coefficient
    double edgeL0 = 0.0;
    DBuf<unsigned> fault_count;  // CTAs of k_dyn_fault_nm done (its last one runs the control)
    DBuf<double> fault_part;     // their partial reductions (three doubles' room each)
    // the fault row of that step runs on a second stream beside the other rows, the FP64
    // recomputation of K d (refresh steps) on a third beside the FP32 apply of the increment
    cudaStream_t side_stream = nullptr, side_stream2 = nullptr;
    bool pdl_off = false;        // the graph being captured holds that step: no programmatic edges
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_fork2 = nullptr, ev_join2 = nullptr;
    DBuf<int> d_ref2lay;         // ref2lay on the device (eqc_get_state / eqc_set_state), and
    DBuf<double> ref_stage;      // the field in the reference numbering on its way in or out
    // element data
    DBuf<double> W64, W64p;
    DBuf<float> W32, W32p;
    DBuf<float> W32lo;   // W - W32p rounded to FP32 (padded like W32p): W as double-float
    bool df_ok = false;  // the double-float FP64-class apply is usable (EQC_NO_DF unset, H symmetric)
    TmaCache tma;
    double H[25];
    // node arrays [L.size()]
    DBuf<double> M, d, v, a, dPre, tmp64a, tmp64b, tmp64c;
    DBuf<double> dx64, kdx64;   // mixed CG: correction since the last reliable update, -K_II of it
    DBuf<double> Kd;          // K d of the mixed-precision dynamic step
    DBuf<double> invM;        // 1 / M (mixed-precision dynamic step)
    DBuf<double> diag64;   // diagonal of K (rows >= 1), Jacobi preconditioner
    DBuf<float> diag32;
    // boundary lists (layout indices) and coefficients
    DBuf<int64_t> iBcL, iBcT, iCreep, iSeis;
    DBuf<double> BcLC, BcTC;
    int nBcL = 0, nBcT = 0, nCreep = 0, nSeis = 0;
    FaultDev F;
    DBuf<int> bcflag;          // FltIglobBC membership per fault node
    DBuf<double> seis;         // receiver gather buffer [3*nSeis]
    std::vector<double> h_tauo, h_FltX;
    // control
    DBuf<Ctrl> ctrl;
    Ctrl* h_ctrl = nullptr;  // pinned mirror
    // reductions
    DBuf<double> red_part;        // partial sums
    DBuf<unsigned int> red_count; // last-block counters
    DBuf<double> scal;            // scratch scalars (power iterations, timing)
    double* h_scal = nullptr;     // pinned mirror
    DBuf<CGState> cg;             // CG scalars
    CGState* h_cg = nullptr;      // pinned mirror
    // CG work vectors
    DBuf<double> r64, z64, p64, q64;
    DBuf<float> r32, z32, p32, q32, x32;
    DBuf<float> g32;      // initial-guess increment added to d before the first solve of a step
    // multigrid
    MGHier* mg = nullptr;     // owned; released by mg_destroy
    GuessNet* net = nullptr;  // owned; created on first use of the learned-guess entry points
    bool initialized = false;
    // results (main.jl:154-163) gathered on the host
    struct Results {
        std::vector<double> seismic_stress, seismic_slipvel, seismic_slip;
        std::vector<double> is_stress, is_slipvel, is_slip;
        std::vector<double> dSeis, vSeis, aSeis;
        std::vector<double> tStart, tEnd, hypo, taubefore, tauafter, delfafter;
        std::vector<double> time_, Vfmax;
    } res;
    // output bookkeeping (main.jl:166-181)
    double tvsx = 0, tvsxinc = 0, tevneinc = 0.5, tevneb = 0, tevne = 0;
    int64_t idelevne = 0, ntvsx = 0, nevne = 0, slipstart = 0, idd = 0, it_s = 0, it_e = 0, rit = 0;
    std::vector<double> delfref;
    ~Handle();
};

// stepper.cu: v and a off the fault row as the reference keeps them, where the mixed method's
// dynamic phase holds the next half-step velocity in v (before a caller reads or sets them)
void materialize_dyn_state(Handle& h);

// kapply.cu
void set_H(const double* H, cudaStream_t s);
template <class T>
void apply_K(const T* x, T* y, const ApplyArgs<T>& A, T sign, int mode, cudaStream_t s);

inline ApplyArgs<double> args64(Handle& h) {
    return {h.W64.p, h.c1, h.c2, h.L, h.W64p.p, &h.ctrl.p->apply_err, &h.tma, h.opt.apply_variant, h.tma_wait_polls};
}
inline ApplyArgs<float> args32(Handle& h) {
    return {h.W32.p, (float)h.c1, (float)h.c2, h.L, h.W32p.p, &h.ctrl.p->apply_err, &h.tma, h.opt.apply_variant,
            h.tma_wait_polls};
}
void tma_init(Handle& h);
void set_H_df(const double* H, cudaStream_t s);
// y = sign K x (FP64 vectors, mode 0/1) in double-float arithmetic; false when unavailable.
bool apply_K_df(Handle& h, const double* x, double* y, double sign, int mode, cudaStream_t s,
                const int* gate = nullptr, int gate_val = 0);
void tma_init_for(TmaCache& c, const Layout& L, const float* W32p, const double* W64p);
// FP32 apply y = K x (mode 0/1 as apply_K) whose owned nodes are finished by the epilogue E
// (residual or Chebyshev step) instead of stored; false when the selected kernel has none.
bool apply_K_epi(const float* x, const ApplyArgs<float>& A, int mode, const OpEpi<float>& E, cudaStream_t s);
// y = K x (FP32) on the node rows 0..3 of the fault's element row, by the element-per-lane
// arithmetic of the full FP32 applies (variants 0 and 4-8): row 0 has the bits of their row 0.
// False when the padded element data or 16-byte aligned vectors are missing.
bool apply_K_fault32(const float* x, float* y, const ApplyArgs<float>& A, cudaStream_t s);

// blas.cu
int vec_blocks();   // grid of the vector and reduction kernels
void dot64(Handle& h, const double* x, const double* y, int64_t n, double* out_dev);
void dot32(Handle& h, const float* x, const float* y, int64_t n, double* out_dev);

// solver.cu
// Enqueues one CG solve on h.stream.  graph: inside a stream capture, the iteration loop
// becomes a conditional while node; otherwise the host drives it (one sync per iteration).
// carry: mixed precision in the time loop may start from the residual the previous solve
// left (r_valid), updated for the change of the fault row, instead of a full FP64 apply.
// guess: the FP32 increment g already added to d (rows >= 1); a carried residual is then
// corrected by -K_II g (FP32 apply: the first reliable update recomputes r in FP64).
void enqueue_solve(Handle& h, double tol, int maxit, bool graph, bool carry = false, const float* guess = nullptr);
// Marks the carried residual stale (after the state was changed from outside the loop).
void invalidate_residual(Handle& h);
int qs_solve_device(Handle& h, double tol, int maxit, double* relres);
// Throws EQC_E_TIMEOUT (and clears the device flag) when a TMA apply gave up a bounded wait.
void check_apply_err(Handle& h);

// graph.cu
// Handle of a conditional node of the graph h.stream is capturing (value 0 at each launch
// unless a kernel upstream of the node sets it).
cudaGraphConditionalHandle cond_handle(Handle& h, unsigned dflt = 0);
// Conditional node with handle c on the stream h.stream is capturing; until cond_end,
// h.stream is the capture stream of the node's body.
void cond_begin(Handle& h, cudaGraphConditionalNodeType type, cudaGraphConditionalHandle c);
void cond_end(Handle& h);
// Ends every capture in progress on the handle's streams and restores h.stream.
void abort_capture(Handle& h);
// Turns the edges of graph g between two of this library's kernels, where the second has no
// other dependency, into programmatic edges (the second kernel's CTAs may be scheduled once
// every CTA of the first has started; each kernel's EQC_GRID_WAIT holds them until the first
// has finished).  Returns the number of edges changed; 0 when EQC_NO_PDL is set.
int64_t make_programmatic(cudaGraph_t g);
// Kernel counting during capture (count_launch adds to the capture tally instead).
void capture_counting(bool on);
int64_t capture_tally();

// stepper.cu
void init_state(Handle& h, double V_init);
void destroy_graphs(Handle& h);
void damage_evolve(Handle& h);
void setup_element_data_device(Handle& h, const eqc_material& mat);
void setup_node_data_device(Handle& h, const eqc_material& mat, const std::vector<int64_t>& lBcL, const double* BcLC,
                            const std::vector<int64_t>& lBcT, const double* BcTC);
// One whole time step of regime iso (1 quasi-static, 2 dynamic) on h.stream; graph: inside a capture.
void enqueue_step(Handle& h, int iso, bool graph);
// Host side of a finished step (control block already in h.h_ctrl): checks and outputs.
struct PostBufs {
    std::vector<double> dF, vF, tauF, seis;
};
// logged: the step's time_, Vfmax and receiver records were already taken from the device logs.
void post_step(Handle& h, int iso, eqc_run_stats& stats, PostBufs& pb, bool logged = false);
void run_steps(Handle& h, int64_t max_steps, double t_end, eqc_run_stats* st);
void fault_slrFunc(Handle& h, const double* psi, double* psi1, const double* Vf, double* Vf1, const double* tau1,
                   double dt);
int fault_FBC(Handle& h, double* psi1, double* Vf1, double* tau1, double* psi2, double* Vf2, double* tau2,
              const double* psi, const double* Vf, const double* FltVfree, double dt);
double fault_dtevol(Handle& h, double dt, double dtmin, const double* Vf, int isolver);

// mg_setup.cpp / mg.cu
void mg_build(Handle& h);
void mg_destroy(Handle& h);
void mg_apply64(Handle& h, const double* r, double* z);
void mg_apply32(Handle& h, const float* r, float* z);

}  // namespace eqc

// The opaque handle of the C ABI.
struct eqc_handle {
    eqc::Handle h;
};
