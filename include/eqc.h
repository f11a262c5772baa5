/*
 * eqc.h -- C ABI of libeqc.so, the GB300 (sm_103a) implementation of the
 * eqcycle time-stepping hot path.
 *
 * The reference (thehalfspace/eqcycle, Julia) has no FFI: its hot path is the
 * Julia function main(P) (src/main.jl:67-477) with P built by setParameters
 * (par.jl:15-231).  These entry points are what a Julia `ccall` shim keeping
 * main(P)'s signature binds.  Every
 * entry point takes plain pointers and sizes; host arrays use the reference's
 * layouts (Julia column-major, node indices 1-based, reference node numbering
 * of src/MeshBox.jl:27-88).  The library copies what it needs and never keeps
 * a caller pointer after returning.  All functions return an eqc_status.
 *
 * One handle = one fault model on one GPU, driven from one host thread.
 */
#ifndef EQC_H
#define EQC_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    EQC_OK = 0,
    EQC_E_ARG = 1,       /* invalid argument or model arrays                          */
    EQC_E_CUDA = 2,      /* CUDA runtime error (message in eqc_last_error)            */
    EQC_E_NR = 3,        /* friction Newton failed: the reference's "NR SEARCH FAILED!"
                            (src/NRsearch_serial.jl:19-31)                            */
    EQC_E_CG = 4,        /* CG reached maxit without meeting its tolerance            */
    EQC_E_NAN = 5,       /* NaN/Inf detected in the state                             */
    EQC_E_CAPACITY = 6,  /* an output array of main.jl:154-163 would overflow         */
    EQC_E_TIMEOUT = 7,   /* a bounded device wait gave up                              */
    EQC_E_NOMEM = 8,     /* device allocation failed                                   */
    EQC_E_STATE = 9,     /* call out of order (e.g. run before init)                  */
    EQC_E_NOGPU = 10     /* no usable CUDA device                                      */
} eqc_status;

/* The model: exactly the tuple main(P) receives (par.jl:227-230), plus the
 * element data the matrix-free stiffness apply consumes (par.jl:99-152: the
 * mesh connectivity iglob, the GLL weights-times-rigidity W and the GLL
 * derivative matrix H), in place of the assembled Ksparse. */
typedef struct {
    /* params_int (par.jl:236-249) */
    int64_t Nel, FltNglob, yr2sec, IDstate, nglob;
    double Total_time;
    /* params_float (par.jl:251-266) */
    double ETA, Vpl, Vthres, Vevne, dt0;
    /* mesh (par.jl:17-36, 99-152) */
    int64_t NelX, NelY, NGLL;   /* NGLL must be 5 */
    double dxe, dye;
    const int64_t* iglob;       /* [NGLL,NGLL,Nel] column-major, 1-based        */
    const double* W;            /* [NGLL,NGLL,Nel] column-major                 */
    const double* H;            /* [NGLL,NGLL] column-major, H[i,j] = h'_i(x_j) */
    /* params_farray (par.jl:268-292) */
    const double *fo, *Vo, *xLf;            /* [FltNglob] */
    const double* M;                        /* [nglob]    */
    const double *BcLC, *BcTC;              /* [n_iBcL], [n_iBcT] */
    const double *FltB, *FltZ, *FltX, *cca, *ccb, *Seff, *tauo, *XiLf;  /* [FltNglob] */
    /* params_iarray (par.jl:294-301), 1-based */
    const int64_t *iFlt;                    /* [FltNglob] */
    const int64_t *iBcL, *iBcT, *FltIglobBC, *FltNI, *out_seis;
    int64_t n_iBcL, n_iBcT, n_FltIglobBC, n_FltNI, n_out_seis;
} eqc_model;

/* Solver choices. */
enum { EQC_FP64 = 0,      /* plain FP64: every kernel in double precision       */
       EQC_MIXED = 1 };   /* FP32 stiffness apply + preconditioner inside an FP64
                             reliable-update CG; FP64 friction, state, Newmark   */
enum { EQC_PC_AMG = 0, EQC_PC_JACOBI = 1 };
enum { EQC_GUESS_PREVIOUS = 0,   /* dnew .= d[FltNI] (src/main.jl:241)            */
       EQC_GUESS_LEARNED = 1,    /* learned initial guess, previous-step fallback  */
       EQC_GUESS_EXTRAPOLATE = 2 }; /* d_n + (dt_n / dt_{n-1}) (d_n - d_{n-1}) after a
                                      quasi-static step, previous-step otherwise  */
enum { EQC_TOL_RHS = 0,          /* stop when ||r|| <= tol*||b|| (IterativeSolvers 0.8 rule) */
       EQC_TOL_R0 = 1 };         /* stop when ||r|| <= tol*||r0||                  */

typedef struct {
    int32_t precision;   /* EQC_FP64 / EQC_MIXED                         */
    int32_t precond;     /* EQC_PC_AMG / EQC_PC_JACOBI                   */
    int32_t guess;       /* EQC_GUESS_PREVIOUS / _LEARNED / _EXTRAPOLATE  */
    int32_t tol_rule;    /* EQC_TOL_RHS / EQC_TOL_R0                     */
    double cg_tol;       /* main.jl:256 uses 1e-6; the workloads use 1e-8 */
    int32_t cg_maxit;    /* <= 0: size of the system (IterativeSolvers default) */
    int32_t device;      /* CUDA device ordinal                          */
    int32_t use_graphs;  /* capture the per-step work in CUDA graphs     */
    int32_t verbose;     /* print "Time (yr) = ..." every 500 steps (main.jl:425-427) */
    /* solver tuning (0 = default) */
    double reliable_delta;  /* mixed precision: a reliable update whenever the recurrence
                               residual fell by this factor (default 1e-3): r -= K dx with
                               a double-float apply, b - K x in FP64 for the update that
                               certifies convergence                                   */
    int32_t mg_degree;      /* Chebyshev smoothing steps on the spectral-element level, pre and
                               post (default 4)                                        */
    int32_t mg_coarse_max;  /* largest coarsest level, solved densely (default 2048 unknowns) */
    int32_t apply_variant;  /* stiffness apply kernel: 0 default (FP32: one element per lane,
                               6 element rows per CTA; FP64: persistent TMA pipeline),
                               1 one tile per CTA by TMA, 2 plain tile loads, 3 persistent
                               TMA pipeline, FP32 only: 4 / 5 / 6 / 7 one element per lane
                               with 4 / 8 / 12 / 6 (2 CTAs per SM) element rows per CTA,
                               8 one element per lane fed by TMA, one wave of CTAs each
                               walking up a strip of 31 element columns                 */
    int32_t mg_degree_coarse; /* Chebyshev steps on the vertex levels (default 3)          */
    int32_t step_batch;     /* with use_graphs: at most this many time steps per graph launch,
                               outputs logged on the device (default 0 = 512; 1 = one step per
                               launch).  A launch ends early at any step whose outputs need
                               the host (event start/end, snapshots) or on a regime switch. */
} eqc_options;

typedef struct eqc_handle eqc_handle;

/* Fill *opt with the defaults (FP64, AMG, previous-step guess, tol 1e-8). */
void eqc_default_options(eqc_options* opt);

/* Uploads the model, builds the device layout and the multigrid hierarchy
 * (src/main.jl:193-211 builds its AMG once per run as well). */
eqc_status eqc_create(const eqc_model* model, const eqc_options* opt, eqc_handle** out);

/* Material of a structured box model, for the setup on the device (no counterpart in the
 * reference, whose setParameters builds W and M on the host, par.jl:99-152). */
typedef struct {
    int32_t rule;                  /* 0 homogeneous (rho1, vs1); 1 rectangle per element
                                      (Assemble.jl:34-35: ex*dxe >= ThickX and dye <= ey*dye
                                      <= ThickY, 1-based ex, ey); 2 trapezoid per GLL node:
                                      depth z = -x <= trap_z1 and y <= trap_w0 + (trap_w1 -
                                      trap_w0) z / trap_z1                                 */
    double rho1, vs1, rho2, vs2;   /* host rock; damage zone                               */
    double ThickX, ThickY;         /* rule 1                                                */
    double trap_w0, trap_w1, trap_z1;   /* rule 2                                           */
    double LX;                     /* domain depth: x runs from -LX to 0                    */
    const double* xgll;            /* the 5 GLL nodes and weights (as the host setup uses)  */
    const double* wgll;
} eqc_material;

/* eqc_create for a structured box mesh whose element data are built on the device: the node
 * numbering is MeshBox.jl's (model->iglob is not read), W, the lumped mass M with the
 * absorbing-boundary terms M[iB] += dt0/2 * Bc of par.jl:173-174, 1/M and diag(K) are
 * computed by kernels from `mat` (model->W, model->M and model->FltNI are not read; every other
 * field is, as in eqc_create).  The result is bitwise the model eqc_create builds from the
 * host setup's arrays. */
eqc_status eqc_create_structured(const eqc_model* model, const eqc_material* mat, const eqc_options* opt,
                                 eqc_handle** out);
eqc_status eqc_destroy(eqc_handle* h);
const char* eqc_last_error(const eqc_handle* h);

/* ---- hot-path operators on host arrays (reference numbering) ---------------- */

/* y = K x  (replaces Ksparse*x, src/main.jl:246,267; element form src/PCG.jl:82). */
eqc_status eqc_apply_K(eqc_handle* h, const double* x, double* y);

/* Quasi-static displacement solve (src/main.jl:241-262): with F_fault [FltNglob]
 * the fault displacement F[iFlt], solve K[FltNI,FltNI] d = -(K F)[FltNI] by
 * preconditioned CG from the guess d_inout[FltNI]; on return d_inout[FltNI]
 * holds the solution and d_inout[iFlt] = F_fault.  Replaces
 * cg!(dnew, kni, rhs; Pl = aspreconditioner(ruge_stuben(kni)), tol = tol). */
eqc_status eqc_qs_solve(eqc_handle* h, const double* F_fault, double* d_inout,
                        double tol, int32_t maxit, int32_t* iters, double* relres);

/* slrFunc! (src/otherFunctions_serial.jl:62-83) on [FltNglob] arrays. */
eqc_status eqc_slrFunc(eqc_handle* h, const double* psi, double* psi1, const double* Vf,
                       double* Vf1, const double* tau1, double dt);

/* FBC! (src/NRsearch_serial.jl:6-43) on [FltNglob] arrays.  *fail_node gets 0,
 * or the 1-based node where the reference stops with "NR SEARCH FAILED!"
 * (status EQC_E_NR). */
eqc_status eqc_FBC(eqc_handle* h, double* psi1, double* Vf1, double* tau1, double* psi2,
                   double* Vf2, double* tau2, const double* psi, const double* Vf,
                   const double* FltVfree, double dt, int64_t* fail_node);

/* dtevol! (src/dtevol.jl:5-44). */
eqc_status eqc_dtevol(eqc_handle* h, double dt, double dtmin, const double* Vf,
                      int32_t isolver, double* dt_out);

/* Largest fault-node count eqc_dtevol_noalloc accepts. */
#define EQC_NOALLOC_MAX_NODES (1 << 22)

/* No counterpart in the reference.  The time step of eqc_dtevol, for callers that
 * cannot allocate device memory (a host code that owns a fixed device arena, an
 * allocator budget that forbids library cudaMalloc, a call site where allocation
 * would synchronise the device): it needs no handle and allocates nothing.  Vf and
 * XiLf are the caller's device arrays of n fault nodes, NFBC the 1-based first
 * friction node (src/main.jl:186), dt_out a device double written on `stream`
 * (a cudaStream_t, NULL for the default stream).  n may not exceed
 * EQC_NOALLOC_MAX_NODES (EQC_E_ARG otherwise; message in eqc_last_error(NULL)).
 * The reduction scratch is a fixed static device array shared by every call: calls
 * that overlap on the GPU race on it.  The first call on a device looks up that
 * array's device address; make it before any stream capture. */
eqc_status eqc_dtevol_noalloc(const double* Vf, const double* XiLf, int64_t n, int64_t NFBC,
                              double dt, double dtmin, int32_t isolver, double* dt_out,
                              void* stream);

/* ---- learned initial guess -------------------------------------------------------
 * No counterpart in the reference (src/main.jl:241 always starts CG from the previous
 * displacement).  A network maps the fault slip increment and slip-rate profile of the
 * first solve of a quasi-static step ([2][FltNglob] features) to the displacement
 * increment on a 121 x 61 grid over the domain ([61][121] outputs, depth fastest), which is
 * prolonged bilinearly to the nodes and added to the previous displacement.  It is used
 * when the handle was created with guess = EQC_GUESS_LEARNED and the network has been
 * trained (eqc_guess_train) or given weights (eqc_guess_set_params); CG always runs to the
 * same tolerance, so the guess changes iteration counts, never the converged result.
 * Pairs are logged by eqc_run when logging is on (eqc_guess_log). */

/* Feature count (2*FltNglob), output count (121*61) and parameter count of the network. */
eqc_status eqc_guess_shape(eqc_handle* h, int32_t* nin, int32_t* nout, int64_t* nparam);
/* Re-initialise the network with seeded He-uniform weights (untrained). */
eqc_status eqc_guess_init(eqc_handle* h, uint64_t seed);
/* FP32 master parameters [nparam]; set marks the network trained. */
eqc_status eqc_guess_get_params(eqc_handle* h, float* params);
eqc_status eqc_guess_set_params(eqc_handle* h, const float* params);
/* Log up to `capacity` training pairs during eqc_run (0 switches logging off). */
eqc_status eqc_guess_log(eqc_handle* h, int64_t capacity);
/* Logged pairs: *n gets their count; in [n][2][FltNglob] and tgt [n][61][121] (either may be NULL). */
eqc_status eqc_guess_pairs(eqc_handle* h, float* in, float* tgt, int64_t* n);
/* Adam training (FP32 master, BF16 weights in every product) on n pairs (in, tgt), or on the
 * first n pairs this handle logged when both are NULL; epoch_loss[epochs] (optional) gets the
 * mean squared error per output of every epoch. */
eqc_status eqc_guess_train(eqc_handle* h, const float* in, const float* tgt, int64_t n, int32_t epochs, double lr,
                           int32_t batch, uint64_t seed, double* epoch_loss);
/* Mean squared error per output on n pairs; out [n][61][121] (optional) gets the outputs. */
eqc_status eqc_guess_eval(eqc_handle* h, const float* in, const float* tgt, int64_t n, double* mse, float* out);
/* Gradient of that error over one batch of n pairs with respect to every parameter (no update). */
eqc_status eqc_guess_grad(eqc_handle* h, const float* in, const float* tgt, int64_t n, float* grad, double* loss);

/* ---- the time loop (src/main.jl:67-477) ------------------------------------- */

/* Initial state of main.jl:89-190 with v = V_init/2 (main.jl:102 uses
 * V_init = 1e-3 m/s): d = a = 0, psi from tauo (main.jl:125), t = 0. */
eqc_status eqc_init(eqc_handle* h, double V_init);

typedef struct {
    int64_t steps;         /* steps taken by this call          */
    int64_t qs_steps, dyn_steps;
    int64_t cg_iters;      /* CG iterations summed over QS solves */
    int64_t qs_solves;
    double t;              /* simulated time reached [s]         */
    double dt;             /* next time step [s]                 */
    int32_t isolver;       /* regime for the next step (1 QS, 2 dynamic) */
    int32_t events;        /* events started so far               */
    double wall_s;         /* wall time spent in this call        */
    double gpu_ms;         /* CUDA-event time on the handle's stream between the first
                              and the last kernel of this call     */
} eqc_run_stats;

/* Advance the time loop until t >= t_end or max_steps steps were taken.  The
 * results of main.jl:154-163 accumulate on the device between calls. */
eqc_status eqc_run(eqc_handle* h, int64_t max_steps, double t_end, eqc_run_stats* stats);

/* State on the host (reference numbering): name is one of "d", "v", "a"
 * [nglob], "psi", "tau" [FltNglob].  eqc_set_state writes it back.  The array
 * crosses to or from the device as it is (page-locked host memory, e.g. from
 * cudaHostAlloc, makes that one DMA) and is permuted on the device; both calls
 * return when the transfer is complete. */
eqc_status eqc_get_state(eqc_handle* h, const char* name, double* out);
eqc_status eqc_set_state(eqc_handle* h, const char* name, const double* in);
/* Scalars "t", "dt", "isolver", "it" (and, read-only, the solver counters "cg_iters",
 * "qs_solves", "cg_updates" (reliable updates), "cg_carried" (solves that started from
 * the residual the previous solve left), "guess_tried" / "guess_kept" (initial-guess
 * increments judged against the previous-step guess / kept because they lowered ||r||),
 * "cg_restarts" (mixed precision: reliable updates after which the CG direction restarted),
 * the solver settings "apply_variant" and "reliable_delta" (as chosen by eqc_autotune), and
 * "damage_events" (damage steps applied, eqc_set_damage), and the host time in ms of the
 * phases of eqc_create: "setup_ms_numbering", "setup_ms_elements", "setup_ms_nodes",
 * "setup_ms_other", "setup_ms_hierarchy" (the multigrid hierarchy), and "pdl_edges", the
 * kernel-to-kernel edges of the captured step graphs launched as programmatic dependent
 * launches (0 with the environment variable EQC_NO_PDL set at capture)).
 * eqc_set_scalar sets "t", "dt" or "isolver" of the state (main.jl's loop variables), after
 * eqc_init.  Two settings of the handle are read and set the same way, at any time:
 * "time_capacity", the length of the time_ / Vfmax records (default 1,900,000, the
 * reference's preallocation, main.jl:154-163; eqc_run returns EQC_E_CAPACITY when a step
 * would exceed it), and "tma_wait_polls", the bound, in polls, of the first tile wait of the
 * TMA-fed stiffness applies (default and maximum 4,194,304; every later wait keeps that bound).
 * A kernel whose wait runs out flags it, waits with the full bound for the copies it issued
 * and returns; the call reports EQC_E_TIMEOUT and the handle stays usable.  Setting it to 0
 * makes every TMA apply give up at once: that is how the failure path is tested. */
eqc_status eqc_get_scalar(eqc_handle* h, const char* name, double* out);
eqc_status eqc_set_scalar(eqc_handle* h, const char* name, double value);

/* Results of main.jl:479-498, trimmed as in main.jl:455-472.  eqc_result_size
 * gives the element count of a field (fault-major matrices are FltNglob x n,
 * receiver matrices n x nseis, both column-major); eqc_get_result copies it. */
int64_t    eqc_result_size(eqc_handle* h, const char* field);
eqc_status eqc_get_result(eqc_handle* h, const char* field, double* out);

/* ---- ensembles --------------------------------------------------------------------
 * No counterpart in the reference (it runs one model per process).  An ensemble advances
 * several independent models (handles created by eqc_create on the same device, initialised
 * by eqc_init, uneven sizes allowed) by one CUDA-graph launch per time step: each member is a
 * branch of the graph whose regime (quasi-static or dynamic) is chosen on the device from the
 * member's own state, and the members run concurrently.  Every member keeps its own results
 * (eqc_get_result on the member handle); the ensemble does not own the handles. */
typedef struct eqc_ensemble eqc_ensemble;
eqc_status eqc_ensemble_create(eqc_handle* const* members, int32_t n, eqc_ensemble** out);
/* Advance every member by `steps` time steps; stats[n] (optional) gets each member's
 * statistics, *gpu_ms (optional) the CUDA-event time of the whole call. */
eqc_status eqc_ensemble_run(eqc_ensemble* e, int64_t steps, eqc_run_stats* stats, double* gpu_ms);
eqc_status eqc_ensemble_destroy(eqc_ensemble* e);
const char* eqc_ensemble_last_error(const eqc_ensemble* e);

/* ---- damage evolution (damageEvol.jl:5-7; its call at the end of each event,
 * main.jl:377-378, is commented out in the reference, so it is off unless set here) */

/* Elements (1-based, the numbering of W: e = (ey-1)*NelX + ex) whose weights W[:, :, e] are
 * multiplied by `factor` at the end of every event of eqc_run (damageEvol.jl uses 0.95, on
 * the damage_idx that Assemble.jl:25-35 returns).  K changes with W, so the multigrid
 * hierarchy is rebuilt and the solver's carried state is dropped.  n = 0 turns it off. */
eqc_status eqc_set_damage(eqc_handle* h, const int64_t* damage_idx, int64_t n, double factor);

/* Apply one damage step now (the same scaling and rebuild as at an event end).  The scalar
 * "damage_events" counts the steps applied. */
eqc_status eqc_damage_evolve(eqc_handle* h);

/* ---- device-resident entry points (benchmarks, integration with device codes) */

/* Internal node layout: lexicographic grid, depth fastest, fault = row 0.
 * eqc_layout gives nx = 4*NelX+1, ny = 4*NelY+1 and the row pitch ld (elements). */
eqc_status eqc_layout(eqc_handle* h, int64_t* nx, int64_t* ny, int64_t* ld);

/* y = K x on device buffers in the internal layout, FP64 (dtype 0), FP32 (dtype 1, W held in
 * FP32) or FP64 vectors in double-float arithmetic (dtype 2: the mixed solver's true-residual
 * apply, ~1e-14 relative), on the handle's stream.  Asynchronous. */
eqc_status eqc_apply_K_device(eqc_handle* h, const void* x, void* y, int32_t dtype);

/* Time nrep launches of the stiffness apply (dtype as for eqc_apply_K_device) with CUDA
 * events on the handle's stream, flushing L2 between launches when flush_l2 != 0; *ms gets
 * the mean launch duration. */
eqc_status eqc_time_apply(eqc_handle* h, int32_t dtype, int32_t nrep, int32_t flush_l2, double* ms);

/* Time nrep back-to-back launches of the stiffness apply rotating over ncopies replicas of its
 * whole working set (x, y, W), so that with replicas larger than L2 together every launch
 * streams its data from HBM; *ms gets the mean launch duration (CUDA events around the
 * batch, on the handle's stream).  The batch is one CUDA graph whose consecutive launches are
 * programmatic dependent launches, as the library's step graphs run their kernels. */
eqc_status eqc_time_apply_stream(eqc_handle* h, int32_t dtype, int32_t nrep, int32_t ncopies, double* ms);

/* Solver autotuner (no counterpart in the reference): times `reps` graph-replayed trial
 * solves of the next quasi-static solve from the current state for a set of Chebyshev
 * degrees (spectral-element level x vertex levels) and keeps the fastest; in mixed precision
 * it then tries the FP32 apply kernels (apply_variant 0, 7, 4, 8) and the reliable-update
 * factors 1e-2, 1e-3, 1e-4 in turn.  The state and the counters are restored.  *mg_degree,
 * *mg_degree_coarse and *solve_ms (all optional) get the choice and its trial time; the
 * apply kernel and the factor chosen are the scalars "apply_variant" and "reliable_delta"
 * (eqc_get_scalar).  Call after eqc_init (or between eqc_run calls). */
eqc_status eqc_autotune(eqc_handle* h, int32_t reps, int32_t* mg_degree, int32_t* mg_degree_coarse, double* solve_ms);

/* Kernel launches of the library since the handle was created. */
int64_t eqc_launch_count(eqc_handle* h);

/* Block until the handle's stream is idle. */
eqc_status eqc_sync(eqc_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* EQC_H */
