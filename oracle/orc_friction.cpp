// CPU oracle -- rate-and-state friction and time-step restatement (test infrastructure).
//
//   IDS!     src/otherFunctions_serial.jl:5-32   (aging law in log form, IDstate = 2)
//   IDS2!    src/otherFunctions_serial.jl:35-59
//   slrFunc! src/otherFunctions_serial.jl:62-83  (quasi-static slip rate)
//   NRsearch!src/NRsearch_serial.jl:47-98        (Newton on tau, tol 0.001*a*sigma, cap 1000)
//   FBC!     src/NRsearch_serial.jl:6-43
//   dtevol!  src/dtevol.jl:5-44
// Expressions keep the reference's left-to-right evaluation order.  The reference runs
// NRsearch! with BigFloat temporaries; orc_NR is the FP64 restatement and orc_NR_q the
// binary128 one used to bound the FP64-vs-extended-precision gap.
#include "orc_internal.h"
#include <cmath>
#if defined(__aarch64__)
// long double is IEEE binary128 on AArch64 Linux.
typedef long double quad_t_;
static inline quad_t_ qexp(quad_t_ x) { return expl(x); }
static inline quad_t_ qabs(quad_t_ x) { return fabsl(x); }
#else
#include <quadmath.h>
typedef __float128 quad_t_;
static inline quad_t_ qexp(quad_t_ x) { return expq(x); }
static inline quad_t_ qabs(quad_t_ x) { return fabsq(x); }
#endif

extern "C" double orc_IDS(double xLf, double Vo, double psi, double dt, double Vf, double cnd) {
    const double VdtL = std::fabs(Vf) * dt / xLf;
    if (VdtL < cnd)
        return std::log(std::exp(psi - VdtL) + Vo * dt / xLf - 0.5 * Vo * std::fabs(Vf) * dt * dt / (xLf * xLf));
    return std::log(std::exp(psi - VdtL) + (Vo / std::fabs(Vf)) * (1 - std::exp(-VdtL)));
}

extern "C" double orc_IDS2(double xLf, double Vo, double psi, double psi1, double dt, double Vf, double Vf1) {
    const double VdtL = 0.5 * std::fabs(Vf1 + Vf) * dt / xLf;
    if (VdtL < 1e-6)
        return std::log(std::exp(psi - VdtL) + Vo * dt / xLf - 0.5 * Vo * 0.5 * std::fabs(Vf1 + Vf) * dt * dt / (xLf * xLf));
    return std::log(std::exp(psi - VdtL) + (Vo / (0.5 * std::fabs(Vf + Vf1))) * (1 - std::exp(-VdtL)));
}

// Status: 0 converged, 1 iteration cap (k == 1000), 2 |delta| > 1e10.
extern "C" int orc_NR(double fo, double Vo, double cca, double ccb, double Seff, double tau, double tauo,
                      double psi, double FltZ, double FltVfree, double* Vf_out, double* tau_out) {
    const double Vw = 1e10;
    const double fact = 1. + (Vo / Vw) * std::exp(-psi);
    const double eps = 0.001 * cca * Seff;
    int k = 0;
    double delta = INFINITY, Vf = 0.0;
    while (std::fabs(delta) > eps) {
        const double fa = fact * tau / (Seff * cca);
        const double help = -(fo + ccb * psi) / cca;
        const double help1 = std::exp(help + fa);
        const double help2 = std::exp(help - fa);
        Vf = Vo * (help1 - help2);
        const double Vfprime = fact * (Vo / (cca * Seff)) * (help1 + help2);
        delta = (FltZ * FltVfree - FltZ * Vf + tauo - tau) / (1 + FltZ * Vfprime);
        tau = tau + delta;
        k = k + 1;
        if (std::fabs(delta) > 1e10 || k == 1000) {
            *Vf_out = Vf;
            *tau_out = tau;
            return std::fabs(delta) > 1e10 ? 2 : 1;
        }
    }
    const double fa = fact * tau / (Seff * cca);
    const double help = -(fo + ccb * psi) / cca;
    *Vf_out = Vo * (std::exp(help + fa) - std::exp(help - fa));
    *tau_out = tau;
    return 0;
}

extern "C" int orc_NR_q(double fo, double Vo, double cca, double ccb, double Seff, double tau0, double tauo,
                        double psi, double FltZ, double FltVfree, double* Vf_out, double* tau_out) {
    using q = quad_t_;
    const double Vw = 1e10;
    const double fact = 1. + (Vo / Vw) * std::exp(-psi);
    const double eps = 0.001 * cca * Seff;
    const double help = -(fo + ccb * psi) / cca;  // Float64 in the reference as well
    int k = 0;
    q delta = (q)INFINITY, Vf = 0, tau = tau0;
    bool first = true;
    while (qabs(delta) > (q)eps) {
        // first iterate: fact*tau/(Seff*cca) is evaluated in Float64 before promotion
        q fa = first ? (q)(fact * tau0 / (Seff * cca)) : ((q)fact * tau) / (q)(Seff * cca);
        first = false;
        q help1 = qexp((q)help + fa), help2 = qexp((q)help - fa);
        Vf = (q)Vo * (help1 - help2);
        q Vfprime = (q)(fact * (Vo / (cca * Seff))) * (help1 + help2);
        delta = ((q)(FltZ * FltVfree) - (q)FltZ * Vf + (q)tauo - tau) / ((q)1 + (q)FltZ * Vfprime);
        tau = tau + delta;
        k = k + 1;
        if (qabs(delta) > (q)1e10 || k == 1000) {
            *Vf_out = (double)Vf;
            *tau_out = (double)tau;
            return qabs(delta) > (q)1e10 ? 2 : 1;
        }
    }
    q fa = ((q)fact * tau) / (q)(Seff * cca);
    *Vf_out = (double)((q)Vo * (qexp((q)help + fa) - qexp((q)help - fa)));
    *tau_out = (double)tau;
    return 0;
}

extern "C" void orc_slrFunc(const orc_model* m, const double* psi, double* psi1, const double* Vf, double* Vf1,
                            const double* tau1, double dt) {
    for (int64_t j = m->NFBC; j < m->FltNglob; ++j) {
        psi1[j] = orc_IDS(m->xLf[j], m->Vo[j], psi[j], dt, Vf[j], 1e-6);
        const double tauAB = tau1[j] + m->tauo[j];
        const double fa = tauAB / (m->Seff[j] * m->cca[j]);
        const double help = -(m->fo[j] + m->ccb[j] * psi1[j]) / m->cca[j];
        const double help1 = std::exp(help + fa);
        const double help2 = std::exp(help - fa);
        Vf1[j] = m->Vo[j] * (help1 - help2);
    }
}

// Returns 0, or (1 + node index) of the first node where the reference would stop with
// "NR SEARCH FAILED!" (NRsearch_serial.jl:19-31).
extern "C" int orc_FBC(const orc_model* m, double* psi1, double* Vf1, double* tau1, double* psi2, double* Vf2,
                       double* tau2, const double* psi, const double* Vf, const double* FltVfree, double dt) {
    for (int64_t j = m->NFBC; j < m->FltNglob; ++j) {
        psi1[j] = orc_IDS(m->xLf[j], m->Vo[j], psi[j], dt, Vf[j], 1e-5);
        orc_NR(m->fo[j], m->Vo[j], m->cca[j], m->ccb[j], m->Seff[j], 0.0, m->tauo[j], psi1[j], m->FltZ[j],
               FltVfree[j], &Vf1[j], &tau1[j]);
        if (Vf[j] > 1e10 || std::isnan(Vf[j]) || std::isnan(tau1[j])) return (int)j + 1;
        psi2[j] = orc_IDS2(m->xLf[j], m->Vo[j], psi[j], psi1[j], dt, Vf[j], Vf1[j]);
        orc_NR(m->fo[j], m->Vo[j], m->cca[j], m->ccb[j], m->Seff[j], tau1[j], m->tauo[j], psi2[j], m->FltZ[j],
               FltVfree[j], &Vf2[j], &tau2[j]);
    }
    return 0;
}

extern "C" double orc_dtevol(const orc_model* m, double dt, double dtmin, const double* Vf, int isolver) {
    const double dtmax = 50.0 * 24 * 60 * 60;
    const double dtincf = 1.2;
    if (isolver == 1) {
        double dtnx = dtmax;
        for (int64_t i = m->NFBC; i < m->FltNglob; ++i) {
            if (std::fabs(Vf[i]) * dtmax > m->XiLf[i]) {
                const double dtcell = m->XiLf[i] / std::fabs(Vf[i]);
                if (dtcell < dtnx) dtnx = dtcell;
            }
        }
        if (dtmin > dtnx) dtnx = dtmin;
        if (dtnx > dtincf * dt) dtnx = dtincf * dt;
        return dtnx;
    }
    return dtmin;
}
