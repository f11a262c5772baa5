// The handle: one fault model resident on one GPU.
#pragma once
#include "common.h"
#include <memory>

namespace eqc {

// Fault-row parameters and state, [Nf] each, in fault order (= iFlt order = row 0 of the layout).
struct FaultDev {
    int Nf = 0;
    int NFBC0 = 0;  // first friction node (0-based), NFBC - 1 of src/main.jl:186
    DBuf<double> fo, Vo, xLf, cca, ccb, Seff, tauo, XiLf, FltB, FltZ, FltX, Mf;
    DBuf<double> psi, psi1, psi2, tau, tau1, tau2, Vf, Vf0, Vf1, Vf2, FltVfree, vPre;
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
};

// Multigrid hierarchy (defined in mg.h).
struct MGHier;

struct Handle {
    eqc_options opt{};
    std::string err;
    cudaStream_t stream = nullptr;
    int device = 0;
    Layout L{};
    int64_t nglob = 0, Nel = 0;
    double dxe = 0, dye = 0, c1 = 0, c2 = 0;
    double Vpl = 0, Vthres = 0, Vevne = 0, dt0 = 0, Total_time = 0, yr2sec = 0;
    // reference numbering <-> layout
    std::vector<int64_t> ref2lay;    // [nglob] reference node (0-based) -> layout index
    DBuf<int64_t> d_ref2lay;
    // element data
    DBuf<double> W64, W64p;
    DBuf<float> W32, W32p;
    TmaCache tma;
    double H[25];
    // node arrays [L.size()]
    DBuf<double> M, d, v, a, dPre, tmp64a, tmp64b;
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
    DBuf<double> scal;            // CG scalars
    double* h_scal = nullptr;     // pinned mirror
    // CG work vectors
    DBuf<double> r64, z64, p64, q64;
    DBuf<float> r32, z32, p32, q32, x32;
    // multigrid
    MGHier* mg = nullptr;     // owned; released by mg_destroy
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
    // statistics
    int64_t cg_iters_total = 0, qs_solves_total = 0;
    ~Handle();
};

// kapply.cu
void set_H(const double* H, cudaStream_t s);
template <class T>
void apply_K(const T* x, T* y, const ApplyArgs<T>& A, T sign, int mode, cudaStream_t s);

inline ApplyArgs<double> args64(Handle& h) {
    return {h.W64.p, h.c1, h.c2, h.L, h.W64p.p, &h.ctrl.p->apply_err, &h.tma};
}
inline ApplyArgs<float> args32(Handle& h) {
    return {h.W32.p, (float)h.c1, (float)h.c2, h.L, h.W32p.p, &h.ctrl.p->apply_err, &h.tma};
}
void tma_init(Handle& h);

// blas.cu
void dot64(Handle& h, const double* x, const double* y, int64_t n, double* out_dev);
void dot32(Handle& h, const float* x, const float* y, int64_t n, double* out_dev);

// solver.cu
int qs_solve_device(Handle& h, double tol, int maxit, double* relres);

// stepper.cu
void init_state(Handle& h, double V_init);
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
