// Internal data of the CPU oracle (test infrastructure; see orc_api.h).
#pragma once
#include "orc_api.h"
#include <cstdint>
#include <vector>
#include <string>

namespace orc {

using vec = std::vector<double>;
using ivec = std::vector<int64_t>;

struct CSR {
    int64_t n = 0, m = 0;          // rows, cols
    std::vector<int64_t> ptr;      // n+1
    std::vector<int64_t> col;
    vec val;
    int64_t nnz() const { return ptr.empty() ? 0 : ptr[n]; }
    void spmv(const double* x, double* y) const;   // y = A x
};

CSR transpose(const CSR& A);
CSR matmul(const CSR& A, const CSR& B);

// Ruge-Stueben hierarchy restating AlgebraicMultigrid.jl (ruge_stuben defaults).
struct AMGLevel {
    CSR A, P, R;
};
struct AMG {
    std::vector<AMGLevel> levels;  // levels[k].A is the operator of level k
    CSR Acoarse;                   // coarsest operator
    vec coarse_pinv;               // dense pseudo-inverse, row-major
    int64_t nc = 0;
    // workspace
    std::vector<vec> res, cb, cx;
    void build(const CSR& A, double theta = 0.25, int max_levels = 10, int max_coarse = 10);
    void vcycle(int lvl, double* x, const double* b);
    void precond(double* x, const double* b);      // x = M^{-1} b (one V-cycle from 0)
    double operator_complexity() const;
};

struct Results {
    // fixed-capacity output arrays of main.jl:154-163 (FltNglob-major, column per record)
    std::vector<vec> seismic_stress, seismic_slipvel, seismic_slip;
    std::vector<vec> is_stress, is_slipvel, is_slip;
    std::vector<vec> dSeis, vSeis, aSeis;   // per record: nseis values
    vec tStart, tEnd, hypo;
    std::vector<vec> taubefore, tauafter, delfafter;
    vec time_, Vfmax;
    std::vector<int> regime;                 // isolver used for each step
    std::vector<int> cg_iters;               // total CG iterations of each QS step
};

}  // namespace orc

struct orc_model {
    orc_config cfg;
    // params_int (par.jl:236-249)
    int64_t Nel, FltNglob, nglob, IDstate;
    double yr2sec, Total_time;
    // params_float (par.jl:251-266)
    double ETA, Vpl, Vthres, Vevne, dt0;
    // geometry
    int64_t NelX, NelY, NGLL;
    double dxe, dye, dx_dxi, dy_deta, jac, coefint1, coefint2, muMax;
    orc::vec xgll, wgll, H;   // H col-major: H[i + NGLL*j] = h'_i(x_j)
    orc::ivec iglob;          // [NGLL,NGLL,Nel] col-major, 0-based node ids
    orc::vec x, y;            // [nglob]
    orc::vec W;               // [NGLL,NGLL,Nel]
    orc::vec rho_node, mu_node;   // trapezoid per-node properties (damage 2)
    orc::CSR K;               // assembled stiffness, reference numbering
    orc::ivec damage_idx;     // 0-based elements of the damage zone (Assemble.jl:25-35)
    orc::ivec damage_el;      // elements whose W is scaled at every event end (damageEvol.jl)
    double damage_factor = 1.0;
    int64_t damage_count = 0;
    // params_farray (par.jl:268-292)
    orc::vec fo, Vo, xLf, M, BcLC, BcTC, FltB, FltZ, FltX, cca, ccb, Seff, tauo, XiLf, xout, yout;
    // params_iarray (par.jl:294-301), 0-based
    orc::ivec iFlt, iBcL, iBcT, FltIglobBC, FltNI, out_seis;
    // QS solver pieces built on first use
    bool qs_ready = false;
    orc::CSR Kni;             // -K[FltNI,FltNI] (main.jl:195)
    orc::CSR Knf;             //  K[FltNI,iFlt]
    orc::AMG amg;
    orc::vec diagKni;
    // time-loop state (main.jl:99-190)
    orc::vec d, v, a, psi, tau, Vf, Vf0, Vf1, Vf2, psi1, psi2, tau1, tau2, FltVfree;
    orc::vec F, dPre, vPre, dnew;
    orc::ivec iFBC;
    int64_t NFBC;
    double t, dt, dtmin, half_dt, half_dt_sq;
    int64_t it;
    int isolver;
    // output bookkeeping
    double tvsx, tvsxinc, tevneinc, tevneb, tevne;
    int64_t idelevne, ntvsx, nevne, slipstart, idd, it_s, it_e, rit;
    orc::vec delfref;
    orc::Results out;
};

namespace orc {
void setup_model(orc_model* m);
void assemble_K(orc_model* m);
void damage_evolve(orc_model* m);
void gll(int ngll, double* x, double* w, double* H);
void init_state(orc_model* m);
void qs_prepare(orc_model* m);
}  // namespace orc
