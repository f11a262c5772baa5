// Rate-and-state friction on the device (FP64).  Expressions keep the reference's
// evaluation order; this translation unit is compiled without FMA contraction so the
// arithmetic is the plain sequence of IEEE double operations the reference performs
// (exp/log are CUDA's double-precision functions).
#pragma once
#include <cuda_runtime.h>

namespace eqc {

// IDS! with IDstate = 2 (src/otherFunctions_serial.jl:5-32): aging law, log form.
__device__ __forceinline__ double dev_IDS(double xLf, double Vo, double psi, double dt, double Vf, double cnd) {
    const double VdtL = fabs(Vf) * dt / xLf;
    if (VdtL < cnd) return log(exp(psi - VdtL) + Vo * dt / xLf - 0.5 * Vo * fabs(Vf) * dt * dt / (xLf * xLf));
    return log(exp(psi - VdtL) + (Vo / fabs(Vf)) * (1 - exp(-VdtL)));
}

// IDS2! with IDstate = 2 (src/otherFunctions_serial.jl:35-59).
__device__ __forceinline__ double dev_IDS2(double xLf, double Vo, double psi, double psi1, double dt, double Vf,
                                           double Vf1) {
    const double VdtL = 0.5 * fabs(Vf1 + Vf) * dt / xLf;
    if (VdtL < 1e-6)
        return log(exp(psi - VdtL) + Vo * dt / xLf - 0.5 * Vo * 0.5 * fabs(Vf1 + Vf) * dt * dt / (xLf * xLf));
    return log(exp(psi - VdtL) + (Vo / (0.5 * fabs(Vf + Vf1))) * (1 - exp(-VdtL)));
}

// NRsearch! (src/NRsearch_serial.jl:47-98): Newton on the shear stress tau of
//   tau = tauo + FltZ*(FltVfree - Vf(tau)),  Vf = 2 Vo e^{-(fo+b psi)/a} sinh(fact tau/(a sigma)).
// Stops when |delta| <= 0.001 a sigma; gives up after 1000 iterations (status 1) or when
// |delta| > 1e10 (status 2), returning the last iterate like the reference.
__device__ __forceinline__ int dev_NR(double fo, double Vo, double cca, double ccb, double Seff, double tau,
                                      double tauo, double psi, double FltZ, double FltVfree, double* Vf_out,
                                      double* tau_out) {
    const double Vw = 1e10;
    const double fact = 1. + (Vo / Vw) * exp(-psi);
    const double eps = 0.001 * cca * Seff;
    const double help = -(fo + ccb * psi) / cca;
    int k = 0;
    double delta = __longlong_as_double(0x7ff0000000000000LL);  // +Inf
    double Vf = 0.0;
    while (fabs(delta) > eps) {
        const double fa = fact * tau / (Seff * cca);
        const double help1 = exp(help + fa);
        const double help2 = exp(help - fa);
        Vf = Vo * (help1 - help2);
        const double Vfprime = fact * (Vo / (cca * Seff)) * (help1 + help2);
        delta = (FltZ * FltVfree - FltZ * Vf + tauo - tau) / (1 + FltZ * Vfprime);
        tau = tau + delta;
        k = k + 1;
        if (fabs(delta) > 1e10 || k == 1000) {
            *Vf_out = Vf;
            *tau_out = tau;
            return fabs(delta) > 1e10 ? 2 : 1;
        }
    }
    const double fa = fact * tau / (Seff * cca);
    *Vf_out = Vo * (exp(help + fa) - exp(help - fa));
    *tau_out = tau;
    return 0;
}

// The mixed method's Newton search: NRsearch!'s iteration (src/NRsearch_serial.jl:47-98),
// stopping rule and failure statuses, with the loop's constants hoisted (fa = s tau,
// Vf' = vp (help1 + help2), the right-hand side FltZ FltVfree + tauo summed once) and explicit
// fused multiply-adds.  The caller starts it from
// the node's current shear stress instead of 0: the function tau -> tauo + FltZ (FltVfree - Vf(tau))
// - tau is concave and decreasing, so from a start left of the root the first step lands right of
// it by the curvature over the distance, and from the right the iterates decrease monotonically
// by about a sigma / fact per step while Vf is far above its root value.  From 0 the first step
// overshoots by about FltZ Vf (megapascals at seismic slip rates, several a sigma), from the
// current stress by the step's stress change: fewer iterations, the same root to within the
// stopping tolerance 0.001 a sigma.  (Evaluating the exponentials on the FP32 unit after an FP64
// range reduction took the dz480 fault kernel from 30.5 to 24.4 us, but that kernel runs beside
// the longer chain of the other rows, so the step did not get faster, and the slip rate's error
// against FP64 after 60 dynamic steps rose from below 1e-6 to 1.1e-6: not kept.)
__device__ __forceinline__ int dev_NR_warm(double fo, double Vo, double cca, double ccb, double Seff, double tau,
                                           double tauo, double psi, double FltZ, double FltVfree, double* Vf_out,
                                           double* tau_out) {
    const double Vw = 1e10;
    const double fact = 1. + (Vo / Vw) * exp(-psi);
    const double eps = 0.001 * cca * Seff;
    const double help = -(fo + ccb * psi) / cca;
    const double s = fact / (Seff * cca);
    const double vp = Vo * s;
    const double rhs = __fma_rn(FltZ, FltVfree, tauo);
    int k = 0;
    double delta = __longlong_as_double(0x7ff0000000000000LL);  // +Inf
    while (fabs(delta) > eps) {
        const double fa = s * tau;
        const double help1 = exp(help + fa);
        const double help2 = exp(help - fa);
        const double Vf = Vo * (help1 - help2);
        delta = (__fma_rn(-FltZ, Vf, rhs) - tau) / __fma_rn(FltZ, vp * (help1 + help2), 1.0);
        tau = tau + delta;
        k = k + 1;
        if (fabs(delta) > 1e10 || k == 1000) {
            *Vf_out = Vf;
            *tau_out = tau;
            return fabs(delta) > 1e10 ? 2 : 1;
        }
    }
    const double fa = s * tau;
    *Vf_out = Vo * (exp(help + fa) - exp(help - fa));
    *tau_out = tau;
    return 0;
}

// Closed-form quasi-static slip rate of slrFunc! (src/otherFunctions_serial.jl:74-78).
__device__ __forceinline__ double dev_slr_V(double fo, double Vo, double cca, double ccb, double Seff, double tauo,
                                            double tau1, double psi1) {
    const double tauAB = tau1 + tauo;
    const double fa = tauAB / (Seff * cca);
    const double help = -(fo + ccb * psi1) / cca;
    const double help1 = exp(help + fa);
    const double help2 = exp(help - fa);
    return Vo * (help1 - help2);
}

}  // namespace eqc
