/*
 * CPU oracle for the eqcycle time-stepping hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This library restates, in plain C++17 (+OpenMP), the algorithm of the Julia
 * reference thehalfspace/eqcycle (par.jl, src/main.jl and the src files they include).  It is the
 * checker for the GPU product (eqcycle_gb300/libeqc.so): only tests/,
 * __graft_entry__.smoke() and the cpu_baseline / --impl reference legs of
 * bench.py may load it.  Nothing in the product links or calls it.
 *
 * Parity pinning: the only data the reference ships for this path is the GLL
 * table src/gll_xwh/gll_05.tab; the oracle's GLL nodes, weights and derivative
 * matrix are checked against it (tests/golden/gll_05.json).  Julia is absent,
 * so everything downstream of GLL (assembly, friction, AMG-PCG, the time loop)
 * is a restatement whose parity with the reference is UNPINNED: no reference
 * test, golden vector or runnable reference exists for it.
 *
 * Numbering: the oracle works in the reference's own node numbering
 * (src/MeshBox.jl:27-88), 0-based internally; arrays returned through
 * orc_get() that hold node indices are 1-based like the Julia arrays.
 */
#ifndef EQC_ORACLE_API_H
#define EQC_ORACLE_API_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Model configuration.  Mirrors the inputs of par.jl:setParameters (par.jl:15-231)
 * generalised so that the workload presets (48x48 homogeneous, 480x240
 * damage zone, ...) and the reference's own defaults are all expressible. */
typedef struct {
    int32_t profile;   /* 0: reference depth profiles (defaultInitialConditions.jl:9-84)
                          1: uniform a, tapered b, uniform sigma, seeded theta noise */
    int32_t damage;    /* 0: homogeneous; 1: rectangle, per element (MaterialProperties.jl:3-21);
                          2: trapezoid, per GLL node (mat_trap style, MaterialProperties.jl:77-101) */
    int32_t NelX;      /* elements along depth  (x, par.jl:20) */
    int32_t NelY;      /* elements fault-normal (y, par.jl:21) */
    double LX, LY;     /* depth and fault-normal extent [m] */
    double rho1, vs1, rho2, vs2;
    double ThickX, ThickY;              /* rectangle rule of Assemble.jl:151 */
    double trap_w0, trap_w1, trap_z1;   /* trapezoid: width at surface, width at depth z1 */
    double fo, Vo, Dc;
    double a0, b0, b1, zb0, zb1;        /* profile 1: b = b0 above zb0, linear to b1 at zb1 */
    double sigma;                       /* profile 1 effective normal stress */
    double V_init;                      /* initial slip rate (main.jl:102 uses 2*0.5e-3) */
    double noise_amp;                   /* profile 1: theta *= 1 + amp*U(-1,1) */
    uint64_t seed;
    double Vpl;
    double creep_depth;                 /* fault nodes deeper than this creep at Vpl */
    int32_t creep_inclusive;            /* 1: depth >= creep_depth, 0: depth > creep_depth */
    int32_t nrec;
    double CFL;
    double total_years;
    double Vthres;
    double rec_x[8], rec_y[8];          /* receivers (par.jl:118-119) */
} orc_config;

typedef struct orc_model orc_model;

orc_model* orc_create(const orc_config* cfg);
void       orc_destroy(orc_model* m);

/* Sizes and arrays by name (see orc_api.cpp for the list). */
int64_t orc_size(const orc_model* m, const char* name);
int     orc_get(const orc_model* m, const char* name, void* out);
double  orc_scalar(const orc_model* m, const char* name);

/* GLL tables for any NGLL (GetGLL.jl:17-28 reads them from gll_NN.tab). */
int orc_gll(int ngll, double* x, double* w, double* H /* col-major H[i,j]=h'_i(x_j) */);

/* y = K x with the assembled CSR stiffness (Kassemble.jl:3-63), reference numbering. */
void orc_apply_K_csr(const orc_model* m, const double* x, double* y);
/* y = K x through the element form c1*H*(W.*(H'u)) + c2*(W.*(uH))*H' (PCG.jl:82). */
void orc_apply_K_elem(const orc_model* m, const double* x, double* y);

/* Quasi-static solve (main.jl:236-262): given fault displacement F on iFlt,
 * find d on FltNI with K[FltNI,FltNI] d = -K[FltNI,iFlt] F.
 *   mode 0: reference mode -- Ruge-Stueben AMG (AlgebraicMultigrid.jl defaults)
 *           as preconditioner of CG with the IterativeSolvers.jl 0.8 stopping rule.
 *   mode 1: tight mode -- Jacobi-PCG to the given tolerance (for 1e-12 checks).
 * d_full: [nglob] in/out, initial guess taken from d_full[FltNI]; on return
 * d_full[FltNI] holds the solution and d_full[iFlt] = F_fault.
 * Returns iterations (negative if maxit reached). */
int orc_qs_solve(orc_model* m, const double* F_fault, double* d_full,
                 double tol, int mode, int maxit, double* relres);

/* Friction (otherFunctions_serial.jl, NRsearch_serial.jl), FP64 and binary128. */
double orc_IDS(double xLf, double Vo, double psi, double dt, double Vf, double cnd);
double orc_IDS2(double xLf, double Vo, double psi, double psi1, double dt, double Vf, double Vf1);
int    orc_NR(double fo, double Vo, double cca, double ccb, double Seff, double tau,
              double tauo, double psi, double FltZ, double FltVfree,
              double* Vf_out, double* tau_out);
int    orc_NR_q(double fo, double Vo, double cca, double ccb, double Seff, double tau,
                double tauo, double psi, double FltZ, double FltVfree,
                double* Vf_out, double* tau_out);
void   orc_slrFunc(const orc_model* m, const double* psi, double* psi1, const double* Vf,
                   double* Vf1, const double* tau1, double dt);
int    orc_FBC(const orc_model* m, double* psi1, double* Vf1, double* tau1, double* psi2,
               double* Vf2, double* tau2, const double* psi, const double* Vf,
               const double* FltVfree, double dt);
double orc_dtevol(const orc_model* m, double dt, double dtmin, const double* Vf, int isolver);

/* Time loop (main.jl:67-477). Runs until t >= t_end_s or nsteps steps were
 * taken (whichever first), continuing from the state kept in the model.
 * qs_mode / qs_tol / qs_maxit select the QS solver as in orc_qs_solve.
 * Returns steps taken, or a negative status on NR failure. */
int64_t orc_run(orc_model* m, int64_t nsteps, double t_end_s, int qs_mode,
                double qs_tol, int qs_maxit);
/* Re-initialise the state to t = 0 (main.jl:89-190). */
void orc_reset(orc_model* m);
/* State access: d, v, a [nglob]; psi, tau [FltNglob]; scalars t, dt, it, isolver. */
int orc_state(const orc_model* m, const char* name, void* out);
int orc_set_state(orc_model* m, const char* name, const void* in);

/* Damage evolution (damageEvol.jl): elements (1-based) whose W is scaled by factor at every
 * event end of orc_run, or now by orc_damage_evolve; K is assembled again. */
int  orc_set_damage(orc_model* m, const int64_t* idx, int64_t n, double factor);
void orc_damage_evolve(orc_model* m);

void orc_set_threads(int n);
int  orc_get_threads(void);

#ifdef __cplusplus
}
#endif
#endif
