// The time loop of src/main.jl:220-452 on the device.
//
// Node arrays live in the lexicographic layout (fault = row 0, so fault node k of iFlt is
// layout index k).  The quasi-static branch (main.jl:226-295) runs two predictor-corrector
// passes, each one CG solve (solver.cu) plus fault-row kernels; the dynamic branch
// (main.jl:297-345) is an explicit Newmark step with the friction Newton solve per fault
// node (K5).  After each step a single-CTA control kernel reduces the fault slip rate
// (Vfmax, main.jl:348), switches regime (main.jl:439-443) and computes the next dt
// (dtevol!, src/dtevol.jl:5-44).  Output triggers (main.jl:361-436) are evaluated on the
// host from the control block.
#include "model.h"
#include "learn.h"
#include "fault.cuh"
#include "reduce.cuh"
#include "vec.cuh"
#include "df.cuh"
#include <cmath>
#include <algorithm>
#include <chrono>

namespace eqc {

constexpr int FT = 1024;  // threads of the single-CTA fault-row reductions
constexpr int FNT = 32;   // threads per CTA of the per-node fault kernels (FP64 Newton: spread over SMs)
static inline int fblocks(int Nf) { return (Nf + FNT - 1) / FNT; }

// ---------------------------------------------------------------- quasi-static kernels
// Vf0 = 2 v[iFlt] + Vpl ; Vf = Vf0 ; d[iFlt] = F = dPre[iFlt] + v[iFlt] dt  (main.jl:231-238)
__global__ void __launch_bounds__(FNT) k_qs_begin(double* __restrict__ d, const double* __restrict__ dPre, const double* __restrict__ v,
                           double* Vf0, double* Vf, int Nf, const Ctrl* C) {
    EQC_GRID_WAIT();
    const double dt = C->dt, Vpl = C->Vpl;
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < Nf; k += blockDim.x * gridDim.x) {
        const double a = 2 * v[k] + Vpl;
        Vf0[k] = a;
        Vf[k] = a;
        d[k] = dPre[k] + v[k] * dt;
    }
}

// Start of a quasi-static step on the bulk rows: dPre = d (main.jl:230) and, when asked and the
// last step was quasi-static, the extrapolated initial guess d += g with
// g = (dt / dt_prev) (d - dPre_old) (g also kept in FP32 for the residual correction).
__global__ void k_qs_begin_bulk(double* __restrict__ d, double* __restrict__ dPre, float* __restrict__ g, int64_t n,
                                int64_t ld, int extrap, const Ctrl* C, int round_g) {
    EQC_GRID_WAIT();
    const bool use = extrap && C->qs_prev && C->dt_prev > 0;
    const double ratio = use ? C->dt / C->dt_prev : 0.0;
    const float ratio_f = (float)ratio;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double dn = d[i], dp = dPre[i];
        dPre[i] = dn;
        if (i >= ld) {
            if (round_g) {
                // mixed precision: the increment added is the FP32 one the solver accounts for (its
                // intermediate reliable updates correct the residual by K of x's change), formed
                // from the FP32-rounded difference (integer conversions: two FP64 operations)
                const float gf = use ? __fmul_rn(ratio_f, f64_to_f32(dn - dp)) : 0.f;
                if (use) d[i] = dn + f32_to_f64(gf);
                g[i] = gf;
            } else {
                const double gi = use ? ratio * (dn - dp) : 0.0;
                d[i] = dn + gi;
                g[i] = (float)gi;
            }
        } else {
            g[i] = 0.f;
        }
    }
}

// After a pass's solve (main.jl:265-279): tau1 = -(K d)[iFlt]/FltB with a[FltIglobBC] = 0,
// slrFunc!, Vf1[iFBC] = Vpl, Vf = (Vf0+Vf1)/2, v[iFlt] = (Vf - Vpl)/2.  If next_F, also
// writes the next pass's F into d[iFlt].
struct FaultArgs {
    const double *fo, *Vo, *xLf, *cca, *ccb, *Seff, *tauo, *XiLf, *FltB, *FltZ, *Mf;
    double *psi, *psi1, *psi2, *tau, *tau1, *tau2, *Vf, *Vf0, *Vf1, *Vf2, *FltVfree, *vPre;
    const int* creep;     // iFBC membership
    const int* bcflag;   // FltIglobBC membership
    int Nf, NFBC0;
};

__global__ void __launch_bounds__(FNT) k_qs_fault(const double* __restrict__ Kd0, double* __restrict__ v, double* __restrict__ d,
                           const double* __restrict__ dPre, FaultArgs f, const Ctrl* C, int next_F) {
    EQC_GRID_WAIT();
    const double dt = C->dt, Vpl = C->Vpl;
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < f.Nf; k += blockDim.x * gridDim.x) {
        const double ak = f.bcflag[k] ? 0. : Kd0[k];
        const double t1 = -ak / f.FltB[k];
        f.tau1[k] = t1;
        if (k >= f.NFBC0) {
            const double p1 = dev_IDS(f.xLf[k], f.Vo[k], f.psi[k], dt, f.Vf[k], 1e-6);
            f.psi1[k] = p1;
            f.Vf1[k] = dev_slr_V(f.fo[k], f.Vo[k], f.cca[k], f.ccb[k], f.Seff[k], f.tauo[k], t1, p1);
        }
        if (f.creep[k]) f.Vf1[k] = Vpl;
        const double vf = (f.Vf0[k] + f.Vf1[k]) / 2;
        f.Vf[k] = vf;
        const double vk = 0.5 * (vf - Vpl);
        v[k] = vk;
        if (next_F) d[k] = dPre[k] + vk * dt;
    }
}

// End of the quasi-static step on the fault (main.jl:283-288).
__global__ void __launch_bounds__(FNT) k_qs_end_fault(double* __restrict__ v, FaultArgs f, const Ctrl* C) {
    EQC_GRID_WAIT();
    const double Vpl = C->Vpl;
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < f.Nf; k += blockDim.x * gridDim.x) {
        f.psi[k] = f.psi1[k];
        double t = f.tau1[k];
        if (f.creep[k]) {
            t = 0.;
            f.Vf1[k] = Vpl;
        }
        f.tau[k] = t;
        v[k] = 0.5 * (f.Vf1[k] - Vpl);
    }
}

// v[FltNI] = (d - dPre)/dt ; a = 0  (main.jl:289-292), rows >= 1; recip (mixed precision): times
// 1/dt (an FP64 division is many FP64 operations, of which GB300 issues few)
__global__ void k_qs_end_bulk(const double* __restrict__ d, const double* __restrict__ dPre, double* __restrict__ v,
                              double* __restrict__ a, int64_t ld, int64_t n, Ctrl* C, int recip) {
    EQC_GRID_WAIT();
    const double dt = C->dt, inv = 1.0 / dt;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        C->kd_valid = 0;   // d changed: no incremental K d
        C->v_half = 0;     // v and a as the reference keeps them
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (i >= ld) v[i] = recip ? (d[i] - dPre[i]) * inv : (d[i] - dPre[i]) / dt;
        a[i] = 0.;
    }
}

// x[list] = 0 for up to three arrays
__global__ void k_zero_list(const int64_t* __restrict__ idx, int n, double* x, double* y, double* z) {
    EQC_GRID_WAIT();
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < n; k += blockDim.x * gridDim.x) {
        const int64_t g = idx[k];
        if (x) x[g] = 0.;
        if (y) y[g] = 0.;
        if (z) z[g] = 0.;
    }
}

// ---------------------------------------------------------------- dynamic kernels
// vPre on the fault; d += dt v + dt^2/2 a ; v += dt/2 a   (main.jl:299-306)
__global__ void k_dyn_predict(double* __restrict__ d, double* __restrict__ v, const double* __restrict__ a,
                              double* __restrict__ vPre_f, int Nf, int64_t n, Ctrl* C) {
    EQC_GRID_WAIT();
    const double dt = C->dt, hdt = C->half_dt, hdt2 = C->half_dt_sq;
    if (blockIdx.x == 0 && threadIdx.x == 0) {   // d changes: no carried residual, no QS history
        C->r_valid = 0;
        C->qs_prev = 0;
    }
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double vi = v[i], ai = a[i];
        if (i < Nf) vPre_f[i] = vi;
        d[i] = d[i] + dt * vi + (hdt2)*ai;
        v[i] = vi + hdt * ai;
    }
}

// Mixed-precision predictor: the increment dd = dt v + dt^2/2 a in FP64, d += dd, dd32 = (float) dd.
// The mixed method's Newmark vector kernels are bound by GB300's FP64 issue rate, not by HBM:
// 4-wide accesses and fused multiply-adds (this method does not reproduce the reference's
// operation order; the plain method's kernels do).
// Its first thread also chooses how the step gets K d: a full FP64 apply (start of a dynamic phase,
// every KD_REFRESH steps) or the FP32 apply of the increment (the two conditional bodies after it).
__global__ void __launch_bounds__(256) k_dyn_predict_inc(double* __restrict__ d, double* __restrict__ v,
                                                         const double* __restrict__ a, double* __restrict__ vPre_f,
                                                         float* __restrict__ dd32, int Nf, int64_t n, Ctrl* C,
                                                         cudaGraphConditionalHandle hf, cudaGraphConditionalHandle hi,
                                                         int use_cond) {
    EQC_GRID_WAIT();
    const double dt = C->dt, hdt = C->half_dt, hdt2 = C->half_dt_sq;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        C->r_valid = 0;
        C->qs_prev = 0;
        const int full = (!C->kd_valid || C->kd_age >= KD_REFRESH) ? 1 : 0;
        C->kd_full = full;
        if (use_cond) {
            cudaGraphSetConditional(hf, full ? 1u : 0u);
            cudaGraphSetConditional(hi, full ? 0u : 1u);
        }
    }
    for (int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n; i += 4 * (int64_t)gridDim.x * blockDim.x) {
        double dd4[4], vv[4], aa[4];
        float f[4];
        ld4(d + i, dd4);
        ld4(v + i, vv);
        ld4(a + i, aa);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (i + k < Nf) vPre_f[i + k] = vv[k];
            const double inc = __fma_rn(dt, vv[k], __dmul_rn(hdt2, aa[k]));
            dd4[k] = __dadd_rn(dd4[k], inc);
            f[k] = (float)inc;
            vv[k] = __fma_rn(hdt, aa[k], vv[k]);
        }
        st4(d + i, dd4);
        st4(v + i, vv);
        st4(dd32 + i, f);
    }
}


// The mixed method's predictor with the step counter of main.jl:221-222 (it += 1, t += dt)
// folded in: vPre on the fault, v += dt/2 a, then d += dt v with that v (dt v + dt^2/2 a as one
// product), and the FP32 increment dd32 = dt v for the FP32 apply.  Two FP64 operations per
// node (GB300's FP64 rate bounds these vector kernels); the conversion to FP32 uses integer
// operations.  Off the fault row in a dynamic phase (C->v_half) v already holds the half-step
// velocity that the previous step's end stored: one FP64 operation, no read of a, no write of v.  The step runs as two launches over [i0, n): the node rows of the first element
// row (lead = 1: the step's bookkeeping -- it, t, the choice how the step gets K d -- after which
// the fault row's work can start), then the rest (lead = 0: the step's dt is read from dt_step,
// since the control at the end of the fault row's work may already have replaced dt with the
// next step's).
__global__ void __launch_bounds__(256) k_dyn_predict_nm(double* __restrict__ d, double* __restrict__ v,
                                                        const double* __restrict__ a, double* __restrict__ vPre_f,
                                                        float* __restrict__ dd32, int Nf, int64_t i0, int64_t n,
                                                        int64_t n0_row, Ctrl* C, int lead) {
    EQC_GRID_WAIT();
    const double dt = lead ? C->dt : C->dt_step, hdt = C->half_dt;
    const float dt_hi = __double2float_rn(dt), dt_lo = __double2float_rn(dt - (double)dt_hi);
    const int vm = C->v_half;
    const int64_t ld = n0_row;
    if (lead && blockIdx.x == 0 && threadIdx.x == 0) {
        C->dt_step = dt;
        C->it += 1;
        C->t = C->t + dt;
        C->r_valid = 0;
        C->qs_prev = 0;
        const int full = (!C->kd_valid || C->kd_age >= KD_REFRESH) ? 1 : 0;
        C->kd_full = full;
        C->kd_valid = 1;
        C->kd_age = full ? 0 : C->kd_age + 1;
    }
    for (int64_t i = i0 + 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n;
         i += 4 * (int64_t)gridDim.x * blockDim.x) {
        double dd4[4], vv[4], aa[4];
        float f[4];
        const bool full = !vm || i < ld;   // 4-entry groups never straddle rows (ld % 8 == 0)
        ld4(d + i, dd4);
        ld4(v + i, vv);
        if (full) ld4(a + i, aa);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (i + k < Nf) vPre_f[i + k] = vv[k];
            const double vh = full ? __fma_rn(hdt, aa[k], vv[k]) : vv[k];
            dd4[k] = __fma_rn(dt, vh, dd4[k]);
            f[k] = nm_incr32(vh, dt_hi, dt_lo);
            vv[k] = vh;
        }
        st4(d + i, dd4);
        if (full) st4(v + i, vv);
        st4(dd32 + i, f);
    }
}

// The end of the mixed Newmark step (NmEpi) on every real node off the fault row: K d += K dd
// (t32, the FP32 apply of the step's increment, unless K d was just recomputed in FP64),
// a = -K d with the absorbing terms, a *= 1/M, then the next step's half-step velocity
// v + dt/2 a + dt/2 a into v (v_half: a is not stored; nm_state_at gives v and a on request).
__global__ void __launch_bounds__(256) k_dyn_finish(NmEpi N, const float* __restrict__ t32) {
    EQC_GRID_WAIT();
    const double hdt = *N.hdt;
    if (*N.kd_full) t32 = nullptr;
    if (blockIdx.x == 0 && threadIdx.x == 0) *N.v_half = 1;   // read by the next step's predictors
    const int gx = N.ld / 4;
    const int64_t ng = (int64_t)gx * N.ny;   // groups of 4 nodes; row 0 is the fault kernel's
    for (int64_t g = gx + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += (int64_t)gridDim.x * blockDim.x) {
        const int iy = (int)(g / gx), ix0 = 4 * (int)(g - (int64_t)iy * gx);
        if (ix0 >= N.nx) continue;
        const int64_t off = (int64_t)iy * N.ld + ix0;
        float t[4] = {0.f, 0.f, 0.f, 0.f};
        if (t32) ld4(t32 + off, t);
        newmark4(N, off, ix0, iy, t, t32 != nullptr, hdt);
    }
}

// a = -K d with K d either refreshed (Kd written by the FP64 apply) or Kd += K dd (t32, FP32).
__global__ void __launch_bounds__(256) k_dyn_force(double* __restrict__ Kd, const float* __restrict__ t32,
                                                   double* __restrict__ a, int64_t n, Ctrl* C) {
    EQC_GRID_WAIT();
    const int full = C->kd_full;
    for (int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n; i += 4 * (int64_t)gridDim.x * blockDim.x) {
        double k[4];
        ld4(Kd + i, k);
        if (!full) {
            float t[4];
            ld4(t32 + i, t);
#pragma unroll
            for (int q = 0; q < 4; ++q) k[q] = __dadd_rn(k[q], (double)t[q]);
            st4(Kd + i, k);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) k[q] = -k[q];
        st4(a + i, k);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        C->kd_valid = 1;
        C->kd_age = full ? 0 : C->kd_age + 1;
    }
}

// a[FltIglobBC] = 0 ; absorbing boundaries (main.jl:314-318), one CTA, L then T.
__global__ void k_dyn_bc(double* __restrict__ a, const double* __restrict__ v, const int64_t* iBC, int nBC,
                         const int64_t* iL, const double* CL, int nL, const int64_t* iT, const double* CT, int nT) {
    EQC_GRID_WAIT();
    for (int k = threadIdx.x; k < nBC; k += blockDim.x) a[iBC[k]] = 0.;
    __syncthreads();
    for (int k = threadIdx.x; k < nL; k += blockDim.x) a[iL[k]] = a[iL[k]] - CL[k] * v[iL[k]];
    __syncthreads();
    for (int k = threadIdx.x; k < nT; k += blockDim.x) a[iT[k]] = a[iT[k]] - CT[k] * v[iT[k]];
}

// The same boundary operations over the union of the three lists, one thread per node, each
// node's operations in k_dyn_bc's order (zero, left term, top term): many CTAs instead of one.
__global__ void k_dyn_bc_nodes(double* __restrict__ a, const double* __restrict__ v, const int64_t* __restrict__ node,
                               const int* __restrict__ ops, const double* __restrict__ cl, const double* __restrict__ ct,
                               int n) {
    EQC_GRID_WAIT();
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += blockDim.x * gridDim.x) {
        const int64_t i = node[k];
        const int op = ops[k];
        double ai = a[i];
        if (op & 1) ai = 0.;
        if (op & 2) ai = ai - cl[k] * v[i];
        if (op & 4) ai = ai - ct[k] * v[i];
        a[i] = ai;
    }
}

// Fault boundary condition (main.jl:321-331): FltVfree, Vf, FBC! (two NR solves per node),
// tau = tau2 - tauo, psi = psi2, a[iFlt] -= FltB tau.
__global__ void __launch_bounds__(FNT) k_dyn_fault(double* __restrict__ a, const double* __restrict__ v, FaultArgs f, Ctrl* C) {
    EQC_GRID_WAIT();
    const double dt = C->dt, hdt = C->half_dt, Vpl = C->Vpl;
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < f.Nf; k += blockDim.x * gridDim.x) {
        const double vfree = 2 * v[k] + 2 * hdt * a[k] / f.Mf[k];
        f.FltVfree[k] = vfree;
        const double vf = 2 * f.vPre[k] + Vpl;
        f.Vf[k] = vf;
        if (k >= f.NFBC0) {
            const double p1 = dev_IDS(f.xLf[k], f.Vo[k], f.psi[k], dt, vf, 1e-5);
            f.psi1[k] = p1;
            double V1, T1;
            dev_NR(f.fo[k], f.Vo[k], f.cca[k], f.ccb[k], f.Seff[k], 0.0, f.tauo[k], p1, f.FltZ[k], vfree, &V1, &T1);
            f.Vf1[k] = V1;
            f.tau1[k] = T1;
            if (vf > 1e10 || isnan(vf) || isnan(T1)) atomicMin(&C->fail, k + 1);
            const double p2 = dev_IDS2(f.xLf[k], f.Vo[k], f.psi[k], p1, dt, vf, V1);
            f.psi2[k] = p2;
            double V2, T2;
            dev_NR(f.fo[k], f.Vo[k], f.cca[k], f.ccb[k], f.Seff[k], T1, f.tauo[k], p2, f.FltZ[k], vfree, &V2, &T2);
            f.Vf2[k] = V2;
            f.tau2[k] = T2;
        }
        double t = f.tau2[k] - f.tauo[k];
        if (f.creep[k]) t = 0.;
        f.tau[k] = t;
        f.psi[k] = f.psi2[k];
        a[k] = a[k] - f.FltB[k] * t;
    }
}

// a = a / M ; v += dt/2 a   (main.jl:336-339).  inv: M holds 1/M (mixed method: a multiply
// instead of GB300's slow FP64 division; the plain method divides as the reference does).
__global__ void k_dyn_correct(double* __restrict__ a, double* __restrict__ v, const double* __restrict__ M, int64_t n,
                              const Ctrl* C, int inv) {
    EQC_GRID_WAIT();
    const double hdt = C->half_dt;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double ai = inv ? a[i] * M[i] : a[i] / M[i];
        a[i] = ai;
        v[i] = v[i] + hdt * ai;
    }
}
// The mixed method's correction: a *= 1/M ; v += dt/2 a (4-wide, one multiply and one FMA); the
// first nzero nodes (the creeping fault nodes, a prefix of the fault row) end with a = v = 0.
__global__ void __launch_bounds__(256) k_dyn_correct_inv(double* __restrict__ a, double* __restrict__ v,
                                                         const double* __restrict__ invM, int64_t n, const Ctrl* C,
                                                         int64_t nzero) {
    EQC_GRID_WAIT();
    const double hdt = C->half_dt;
    for (int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n; i += 4 * (int64_t)gridDim.x * blockDim.x) {
        double aa[4], vv[4], mm[4];
        ld4(a + i, aa);
        ld4(v + i, vv);
        ld4(invM + i, mm);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            aa[k] = __dmul_rn(aa[k], mm[k]);
            vv[k] = __fma_rn(hdt, aa[k], vv[k]);
            if (i + k < nzero) aa[k] = vv[k] = 0.0;
        }
        st4(a + i, aa);
        st4(v + i, vv);
    }
}

// ---------------------------------------------------------------- control
// Vfmax (main.jl:348), hypocentre argmax (main.jl:367), regime switch (main.jl:439-443),
// next dt (dtevol!, src/dtevol.jl:5-44).  The reductions are a maximum with its first index
// and a minimum, so their value does not depend on how the nodes are grouped: one CTA of any
// size (k_control), or per-CTA partials combined by the last CTA of the dynamic fault kernel.
struct CtlAcc {
    double vmax;   // largest v over the fault (NaN flagged apart: Julia's maximum propagates it)
    int imax;      // its first index
    int nan;
    double dmin;   // dtevol!: min over the friction nodes of XiLf / |V| where |V| dtmax > XiLf
};
static_assert(sizeof(CtlAcc) == 3 * sizeof(double), "the fault kernel's partials take three doubles each");
static_assert(FNT == 32, "the dynamic fault kernel reduces with one warp per CTA");
constexpr double DTMAX = 50.0 * 24 * 60 * 60;   // src/dtevol.jl:7
__device__ __forceinline__ CtlAcc ctl_init() { return CtlAcc{-INFINITY, 0x7fffffff, 0, DTMAX}; }
__device__ __forceinline__ void ctl_add(CtlAcc& c, int k, double vk, double xilf, int nfbc0, double Vpl) {
    if (vk > c.vmax) { c.vmax = vk; c.imax = k; }
    if (vk != vk) c.nan = 1;
    if (k >= nfbc0) {
        const double sr = fabs(2 * vk + Vpl);
        if (sr * DTMAX > xilf) c.dmin = fmin(c.dmin, xilf / sr);
    }
}
__device__ __forceinline__ void ctl_merge(CtlAcc& c, const CtlAcc& o) {
    if (o.vmax > c.vmax || (o.vmax == c.vmax && o.imax < c.imax)) { c.vmax = o.vmax; c.imax = o.imax; }
    c.nan |= o.nan;
    c.dmin = fmin(c.dmin, o.dmin);
}
__device__ __forceinline__ CtlAcc ctl_warp(CtlAcc c) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        CtlAcc x;
        x.vmax = __shfl_down_sync(0xffffffffu, c.vmax, o);
        x.imax = __shfl_down_sync(0xffffffffu, c.imax, o);
        x.nan = __shfl_down_sync(0xffffffffu, c.nan, o);
        x.dmin = __shfl_down_sync(0xffffffffu, c.dmin, o);
        ctl_merge(c, x);
    }
    return c;
}
// The decision of the step (one thread): Vfmax, hypocentre, next regime, next dt.
__device__ __forceinline__ void ctl_finish(const CtlAcc& c, Ctrl* C) {
    const double bv = c.nan ? __longlong_as_double(0x7ff8000000000000LL) : c.vmax;
    const double Vfmax = 2 * bv + C->Vpl;
    C->Vfmax = Vfmax;
    C->vhypo = Vfmax;
    C->ihypo = c.nan ? 0 : c.imax;
    const int iso = C->isolver;
    const int next = ((iso == 1 && Vfmax < 5e-3) || (iso == 2 && Vfmax < 2e-3)) ? 1 : 2;
    C->isolver = next;
    C->dt_prev = C->dt;
    if (iso == 1) C->qs_prev = 1;
    if (next == 2) {
        C->dt = C->dtmin;   // dtevol!: the dynamic step takes dtmin
    } else {                // a quasi-static next step: min over XiLf / |V|, capped at 1.2 dt
        double dtnx = c.dmin;
        if (C->dtmin > dtnx) dtnx = C->dtmin;
        if (dtnx > 1.2 * C->dt_prev) dtnx = 1.2 * C->dt_prev;
        C->dt = dtnx;
    }
}

// One CTA (up to 1024 threads) over the fault row.
__global__ void __launch_bounds__(FT) k_control(const double* __restrict__ v, FaultArgs f, Ctrl* C) {
    EQC_GRID_WAIT();
    __shared__ CtlAcc sh[32];
    const double Vpl = C->Vpl;
    CtlAcc c = ctl_init();
    for (int k = threadIdx.x; k < f.Nf; k += blockDim.x) ctl_add(c, k, v[k], f.XiLf[k], f.NFBC0, Vpl);
    c = ctl_warp(c);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        CtlAcc t = sh[0];
        for (int q = 1; q < (int)(blockDim.x >> 5); ++q) ctl_merge(t, sh[q]);
        ctl_finish(t, C);
    }
}

// The fault row of the mixed method's dynamic step, from a = -(K d)[iFlt] (t0, the FP64 strip
// apply of the predicted displacement, on the steps that refresh K d; else K d += q0) to the end
// of the step, then the control of k_control: the creeping nodes' a = 0 and the absorbing term
// of the fault's bottom node (main.jl:314-318), the friction Newton solves (dev_NR_warm:
// warm-started) and a[iFlt] -= FltB tau (main.jl:321-331), a *= 1/M, v += dt/2 a,
// creeping nodes a = v = 0 (main.jl:336-344); the last CTA to finish (counted in *count, which
// it clears again) combines the per-CTA partials in part[], reduces Vfmax, switches the regime and
// takes the next dt.  It runs beside the end of the step on the other rows, which it shares no
// node with.  One warp (FNT threads) per CTA.
__global__ void __launch_bounds__(FNT) k_dyn_fault_nm(double* __restrict__ a, double* __restrict__ v,
                                                      const double* __restrict__ t0, const float* __restrict__ q0,
                                                      double* __restrict__ Kd, FaultArgs f, Ctrl* C,
                                                      const double* __restrict__ invM, int hasL0, double cL0,
                                                      CtlAcc* part, unsigned* count) {
    EQC_GRID_WAIT();
    __shared__ bool last;
    const double dt = C->dt_step, hdt = C->half_dt, Vpl = C->Vpl;
    const int full = C->kd_full;
    CtlAcc acc = ctl_init();
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < f.Nf; k += blockDim.x * gridDim.x) {
        // every input is loaded before the first store: through FaultArgs' pointers (which may
        // alias for all the compiler knows) a load after a store waits for it, and the node's
        // work is one thread's latency chain
        const double vk0 = v[k], vpre = f.vPre[k], Mf = __ldg(f.Mf + k), psi = f.psi[k], tau_c = f.tau[k];
        const double tauo = __ldg(f.tauo + k), FltB = __ldg(f.FltB + k), iM = __ldg(invM + k);
        const double xilf = __ldg(f.XiLf + k), tau2_old = f.tau2[k], psi2_old = f.psi2[k];
        const int bc = __ldg(f.bcflag + k), cr = __ldg(f.creep + k);
        const bool fr = k >= f.NFBC0;
        double xLf = 0, Vo = 0, fo = 0, cca = 0, ccb = 0, Seff = 0, FltZ = 0;
        if (fr) {
            xLf = __ldg(f.xLf + k);
            Vo = __ldg(f.Vo + k);
            fo = __ldg(f.fo + k);
            cca = __ldg(f.cca + k);
            ccb = __ldg(f.ccb + k);
            Seff = __ldg(f.Seff + k);
            FltZ = __ldg(f.FltZ + k);
        }
        // K d on the fault row as on the other rows: recomputed in FP64 (t0) on the steps that
        // refresh it (the full FP64 apply beside this kernel stores it), else K d += K dd (q0, the
        // FP32 apply of the increment on the fault's element row, whose row 0 has the bits of the
        // full FP32 apply's: every row's K d then carries the same FP32 rounding.  A strip kernel
        // with another summation order let the fault row's K d drift from its neighbours', a net
        // force that made the displacement error ten times larger after 300 steps.)
        const double kd = full ? t0[k] : __dadd_rn(Kd[k], f32_to_f64(q0[k]));
        double a0 = -kd;
        if (bc) a0 = 0.0;
        if (k == 0 && hasL0) a0 = a0 - cL0 * vk0;
        const double vfree = 2 * vk0 + 2 * hdt * a0 / Mf;
        const double vf = 2 * vpre + Vpl;
        double p1 = 0, V1 = 0, T1 = 0, p2 = psi2_old, V2 = 0, T2 = tau2_old;
        if (fr) {
            p1 = dev_IDS(xLf, Vo, psi, dt, vf, 1e-5);
            // the first search starts from the node's current shear stress (tau + tauo)
            dev_NR_warm(fo, Vo, cca, ccb, Seff, tau_c + tauo, tauo, p1, FltZ, vfree, &V1, &T1);
            if (vf > 1e10 || isnan(vf) || isnan(T1)) atomicMin(&C->fail, k + 1);
            p2 = dev_IDS2(xLf, Vo, psi, p1, dt, vf, V1);
            dev_NR_warm(fo, Vo, cca, ccb, Seff, T1, tauo, p2, FltZ, vfree, &V2, &T2);
        }
        double t = T2 - tauo;
        if (cr) t = 0.;
        double am = __dmul_rn(a0 - FltB * t, iM), vk = __fma_rn(hdt, am, vk0);
        if (cr) am = vk = 0.0;
        if (!full) Kd[k] = kd;
        f.FltVfree[k] = vfree;
        f.Vf[k] = vf;
        if (fr) {
            f.psi1[k] = p1;
            f.Vf1[k] = V1;
            f.tau1[k] = T1;
            f.psi2[k] = p2;
            f.Vf2[k] = V2;
            f.tau2[k] = T2;
        }
        f.tau[k] = t;
        f.psi[k] = p2;
        a[k] = am;
        v[k] = vk;
        ctl_add(acc, k, vk, xilf, f.NFBC0, Vpl);
    }
    acc = ctl_warp(acc);
    if (threadIdx.x == 0) {
        part[blockIdx.x] = acc;
        __threadfence();
        last = atomicAdd(count, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    CtlAcc c = ctl_init();
    for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) {
        CtlAcc o;
        o.vmax = __ldcg(&part[q].vmax);
        o.imax = __ldcg(&part[q].imax);
        o.nan = __ldcg(&part[q].nan);
        o.dmin = __ldcg(&part[q].dmin);
        ctl_merge(c, o);
    }
    c = ctl_warp(c);
    if (threadIdx.x == 0) {
        ctl_finish(c, C);
        *count = 0u;
    }
}

// Gather d, v, a at receivers (main.jl:433-435) into out[3*ns] (v and a of the step's end where
// v holds the next half-step velocity).
__global__ void k_gather_seis(const int64_t* idx, int ns, const double* d, const double* v, const double* a,
                              double* out, const Ctrl* C, NmEpi N) {
    EQC_GRID_WAIT();
    const int k = threadIdx.x;
    if (k < ns) {
        const int64_t g = idx[k];
        double vg = v[g], ag = a[g];
        if (C->v_half && g >= N.ld) nm_state_at(N, g, C->half_dt, &vg, &ag);
        out[k] = d[g];
        out[ns + k] = vg;
        out[2 * ns + k] = ag;
    }
}

// v and a of the step's end off the fault row, in place, where v holds the next half-step
// velocity (before a caller reads or sets them); the host then clears v_half, after the launch,
// so that every CTA reads the same flag.
__global__ void k_nm_materialize(Ctrl* C, NmEpi N) {
    EQC_GRID_WAIT();
    if (!C->v_half) return;
    const double hdt = C->half_dt;
    const int64_t n = (int64_t)N.ld * N.ny;
    for (int64_t i = N.ld + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (i % N.ld >= N.nx) continue;
        double ve, ae;
        nm_state_at(N, i, hdt, &ve, &ae);
        N.v[i] = ve;
        N.a[i] = ae;
    }
}

// ---------------------------------------------------------------- host side
static FaultArgs fargs(Handle& h, const int* bcflag) {
    FaultDev& F = h.F;
    FaultArgs f;
    f.fo = F.fo.p; f.Vo = F.Vo.p; f.xLf = F.xLf.p; f.cca = F.cca.p; f.ccb = F.ccb.p; f.Seff = F.Seff.p;
    f.tauo = F.tauo.p; f.XiLf = F.XiLf.p; f.FltB = F.FltB.p; f.FltZ = F.FltZ.p; f.Mf = F.Mf.p;
    f.psi = F.psi.p; f.psi1 = F.psi1.p; f.psi2 = F.psi2.p; f.tau = F.tau.p; f.tau1 = F.tau1.p; f.tau2 = F.tau2.p;
    f.Vf = F.Vf.p; f.Vf0 = F.Vf0.p; f.Vf1 = F.Vf1.p; f.Vf2 = F.Vf2.p; f.FltVfree = F.FltVfree.p; f.vPre = F.vPre.p;
    f.creep = F.creep.p;
    f.bcflag = bcflag;
    f.Nf = F.Nf;
    f.NFBC0 = F.NFBC0;
    return f;
}

static inline int vblocks(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 4 * 152); }
// 4 entries per thread: every SM's threads resident at once (8 CTAs of 256)
static inline int vblocks4(int64_t n) { return (int)std::min<int64_t>((n / 4 + 255) / 256, 8 * 152); }

static void launch_check() { EQC_CHECK_LAUNCH(); }

// --- fault-only API helpers (eqc_slrFunc / eqc_FBC / eqc_dtevol) ---------------------------
__global__ void __launch_bounds__(FNT) k_api_slr(FaultArgs f, double dt) {
    EQC_GRID_WAIT();
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < f.Nf; k += blockDim.x * gridDim.x) {
        if (k < f.NFBC0) continue;
        const double p1 = dev_IDS(f.xLf[k], f.Vo[k], f.psi[k], dt, f.Vf[k], 1e-6);
        f.psi1[k] = p1;
        f.Vf1[k] = dev_slr_V(f.fo[k], f.Vo[k], f.cca[k], f.ccb[k], f.Seff[k], f.tauo[k], f.tau1[k], p1);
    }
}
__global__ void __launch_bounds__(FNT) k_api_fbc(FaultArgs f, double dt, int* fail) {
    EQC_GRID_WAIT();
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < f.Nf; k += blockDim.x * gridDim.x) {
        if (k < f.NFBC0) continue;
        const double vf = f.Vf[k], vfree = f.FltVfree[k];
        const double p1 = dev_IDS(f.xLf[k], f.Vo[k], f.psi[k], dt, vf, 1e-5);
        f.psi1[k] = p1;
        double V1, T1;
        dev_NR(f.fo[k], f.Vo[k], f.cca[k], f.ccb[k], f.Seff[k], 0.0, f.tauo[k], p1, f.FltZ[k], vfree, &V1, &T1);
        f.Vf1[k] = V1;
        f.tau1[k] = T1;
        if (vf > 1e10 || isnan(vf) || isnan(T1)) atomicMin(fail, k + 1);
        const double p2 = dev_IDS2(f.xLf[k], f.Vo[k], f.psi[k], p1, dt, vf, V1);
        f.psi2[k] = p2;
        double V2, T2;
        dev_NR(f.fo[k], f.Vo[k], f.cca[k], f.ccb[k], f.Seff[k], T1, f.tauo[k], p2, f.FltZ[k], vfree, &V2, &T2);
        f.Vf2[k] = V2;
        f.tau2[k] = T2;
    }
}

void fault_slrFunc(Handle& h, const double* psi, double* psi1, const double* Vf, double* Vf1, const double* tau1,
                   double dt) {
    FaultDev& F = h.F;
    const int Nf = F.Nf;
    cudaStream_t s = h.stream;
    F.psi.upload(psi, Nf, s);
    F.Vf.upload(Vf, Nf, s);
    F.tau1.upload(tau1, Nf, s);
    F.psi1.upload(psi1, Nf, s);
    F.Vf1.upload(Vf1, Nf, s);
    k_api_slr<<<fblocks(h.F.Nf), FNT, 0, s>>>(fargs(h, h.bcflag.p), dt);
    launch_check();
    count_launch();
    F.psi1.download(psi1, Nf, s);
    F.Vf1.download(Vf1, Nf, s);
    EQC_CUDA(cudaStreamSynchronize(s));
}

int fault_FBC(Handle& h, double* psi1, double* Vf1, double* tau1, double* psi2, double* Vf2, double* tau2,
              const double* psi, const double* Vf, const double* FltVfree, double dt) {
    FaultDev& F = h.F;
    const int Nf = F.Nf;
    cudaStream_t s = h.stream;
    F.psi.upload(psi, Nf, s);
    F.Vf.upload(Vf, Nf, s);
    F.FltVfree.upload(FltVfree, Nf, s);
    F.psi1.upload(psi1, Nf, s);
    F.Vf1.upload(Vf1, Nf, s);
    F.tau1.upload(tau1, Nf, s);
    F.psi2.upload(psi2, Nf, s);
    F.Vf2.upload(Vf2, Nf, s);
    F.tau2.upload(tau2, Nf, s);
    int big = 0x7fffffff;
    EQC_CUDA(cudaMemcpyAsync(&h.ctrl.p->fail, &big, sizeof(int), cudaMemcpyHostToDevice, s));
    k_api_fbc<<<fblocks(h.F.Nf), FNT, 0, s>>>(fargs(h, h.bcflag.p), dt, &h.ctrl.p->fail);
    launch_check();
    count_launch();
    F.psi1.download(psi1, Nf, s);
    F.Vf1.download(Vf1, Nf, s);
    F.tau1.download(tau1, Nf, s);
    F.psi2.download(psi2, Nf, s);
    F.Vf2.download(Vf2, Nf, s);
    F.tau2.download(tau2, Nf, s);
    int fail = 0;
    EQC_CUDA(cudaMemcpyAsync(&fail, &h.ctrl.p->fail, sizeof(int), cudaMemcpyDeviceToHost, s));
    EQC_CUDA(cudaStreamSynchronize(s));
    return fail == 0x7fffffff ? 0 : fail;
}

__global__ void k_api_dtevol(const double* Vf, FaultArgs f, double dt, double dtmin, int isolver, double* out) {
    EQC_GRID_WAIT();
    __shared__ double smin[FT / 32];
    const double dtmax = 50.0 * 24 * 60 * 60;
    double dmin = dtmax;
    for (int k = threadIdx.x; k < f.Nf; k += blockDim.x) {
        if (k < f.NFBC0) continue;
        const double sr = fabs(Vf[k]);
        if (sr * dtmax > f.XiLf[k]) dmin = fmin(dmin, f.XiLf[k] / sr);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dmin = fmin(dmin, __shfl_down_sync(0xffffffffu, dmin, o));
    if ((threadIdx.x & 31) == 0) smin[threadIdx.x >> 5] = dmin;
    __syncthreads();
    if (threadIdx.x == 0) {
        double bm = dtmax;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) bm = fmin(bm, smin[q]);
        double r;
        if (isolver == 1) {
            double dtnx = bm;
            if (dtmin > dtnx) dtnx = dtmin;
            if (dtnx > 1.2 * dt) dtnx = 1.2 * dt;
            r = dtnx;
        } else {
            r = dtmin;
        }
        *out = r;
    }
}

double fault_dtevol(Handle& h, double dt, double dtmin, const double* Vf, int isolver) {
    FaultDev& F = h.F;
    cudaStream_t s = h.stream;
    F.Vf2.upload(Vf, F.Nf, s);
    k_api_dtevol<<<1, FT, 0, s>>>(F.Vf2.p, fargs(h, h.bcflag.p), dt, dtmin, isolver, h.scal.p + 15);
    launch_check();
    count_launch();
    double r = 0;
    EQC_CUDA(cudaMemcpyAsync(&r, h.scal.p + 15, sizeof(double), cudaMemcpyDeviceToHost, s));
    EQC_CUDA(cudaStreamSynchronize(s));
    return r;
}

// --- state initialisation (main.jl:89-190) -----------------------------------------------
__global__ void __launch_bounds__(FNT) k_init_psi(const double* v, FaultArgs f) {
    EQC_GRID_WAIT();
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < f.Nf; k += blockDim.x * gridDim.x)
        f.psi[k] = f.tauo[k] / (f.Seff[k] * f.ccb[k]) - f.fo[k] / f.ccb[k] -
                   (f.cca[k] / f.ccb[k]) * log(2 * v[k] / f.Vo[k]);
}
// Fill value only on real nodes (row padding stays zero).
__global__ void k_fill_nodes(double* x, double val, Layout L) {
    EQC_GRID_WAIT();
    const int64_t n = L.size();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = ((i % L.ld) < L.nx) ? val : 0.0;
}
__global__ void __launch_bounds__(FNT) k_init_Vf(const double* v, FaultArgs f) {
    EQC_GRID_WAIT();
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < f.Nf; k += blockDim.x * gridDim.x)
        f.Vf[k] = f.creep[k] ? 0. : 2 * v[k];
}

void init_state(Handle& h, double V_init) {
    cudaStream_t s = h.stream;
    const Layout& L = h.L;
    const int64_t n = L.size();
        FaultArgs f = fargs(h, h.bcflag.p);
    h.d.zero(s);
    h.a.zero(s);
    h.dPre.zero(s);
    k_fill_nodes<<<vblocks(n), 256, 0, s>>>(h.v.p, 0.5 * V_init, L);
    k_init_psi<<<fblocks(h.F.Nf), FNT, 0, s>>>(h.v.p, f);
    // v = v - Vpl/2 (main.jl:183)
    k_fill_nodes<<<vblocks(n), 256, 0, s>>>(h.v.p, 0.5 * V_init - 0.5 * h.Vpl, L);
    k_init_Vf<<<fblocks(h.F.Nf), FNT, 0, s>>>(h.v.p, f);
    if (h.nCreep) k_zero_list<<<1, 256, 0, s>>>(h.iCreep.p, h.nCreep, h.v.p, nullptr, nullptr);
    launch_check();
    count_launch(h.nCreep ? 5 : 4);
    for (DBuf<double>* b : {&h.F.psi1, &h.F.psi2, &h.F.tau, &h.F.tau1, &h.F.tau2, &h.F.Vf0, &h.F.Vf1, &h.F.Vf2,
                            &h.F.FltVfree, &h.F.vPre})
        b->zero(s);
    Ctrl c{};
    c.dt = h.dt0;
    c.dtmin = h.dt0;
    c.half_dt = 0.5 * h.dt0;
    c.half_dt_sq = 0.5 * (h.dt0 * h.dt0);
    c.Vpl = h.Vpl;
    c.t = 0.;
    c.isolver = 1;
    c.fail = 0x7fffffff;
    c.it = 0;
    *h.h_ctrl = c;
    EQC_CUDA(cudaMemcpyAsync(h.ctrl.p, h.h_ctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, s));
    EQC_CUDA(cudaStreamSynchronize(s));
    // output bookkeeping (main.jl:166-181)
    h.res = Handle::Results();
    h.tvsx = 5 * h.yr2sec;
    h.tvsxinc = h.tvsx;
    h.tevneinc = 0.5;
    h.tevneb = h.tevne = 0;
    h.idelevne = h.ntvsx = h.nevne = h.slipstart = h.idd = h.it_s = h.it_e = h.rit = 0;
    h.delfref.assign(h.F.Nf, 0.0);
    h.initialized = true;
}

// capacities of the reference's preallocated outputs (main.jl:154-163)
constexpr int64_t CAP_SEISMIC = 30000, CAP_IS = 4000, CAP_SEIS = 190000, CAP_EV = 400;
constexpr int STEP_BATCH = 512;   // default steps per batched launch (the size of the device logs)

static void fault_columns(Handle& h, std::vector<double>& dF, std::vector<double>& vF, std::vector<double>& tauF) {
    const int Nf = h.F.Nf;
    dF.resize(Nf);
    vF.resize(Nf);
    tauF.resize(Nf);
    EQC_CUDA(cudaMemcpyAsync(dF.data(), h.d.p, sizeof(double) * Nf, cudaMemcpyDeviceToHost, h.stream));
    EQC_CUDA(cudaMemcpyAsync(vF.data(), h.v.p, sizeof(double) * Nf, cudaMemcpyDeviceToHost, h.stream));
    EQC_CUDA(cudaMemcpyAsync(tauF.data(), h.F.tau.p, sizeof(double) * Nf, cudaMemcpyDeviceToHost, h.stream));
    EQC_CUDA(cudaStreamSynchronize(h.stream));
}

// it = it + 1 ; t = t + dt  (main.jl:221-222), dt of this step = C->dt
__global__ void k_step_begin(Ctrl* C) {
    EQC_GRID_WAIT();
    C->it += 1;
    C->t = C->t + C->dt;
}

// Quasi-static step (main.jl:226-295): two predictor-corrector passes.
static void enqueue_qs(Handle& h, bool graph) {
    cudaStream_t s = h.stream;
    const Layout& L = h.L;
    const int64_t n = L.size();
    FaultArgs f = fargs(h, h.bcflag.p);
    const bool extrap = h.opt.guess == EQC_GUESS_EXTRAPOLATE;
    if (extrap) {
        k_qs_begin_bulk<<<vblocks(n), 256, 0, s>>>(h.d.p, h.dPre.p, h.g32.p, n, L.ld, 1, h.ctrl.p,
                                                   h.opt.precision == EQC_MIXED ? 1 : 0);
        count_launch();
    } else {
        EQC_CUDA(cudaMemcpyAsync(h.dPre.p, h.d.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    }
    k_qs_begin<<<fblocks(h.F.Nf), FNT, 0, s>>>(h.d.p, h.dPre.p, h.v.p, h.F.Vf0.p, h.F.Vf.p, h.F.Nf, h.ctrl.p);
    launch_check();
    count_launch();
    // learned guess for the first solve (a trained network), and/or logging of training pairs
    const bool learned = !extrap && h.opt.guess == EQC_GUESS_LEARNED && h.net && h.net->trained;
    const bool logging = h.net && h.net->log_cap > 0;
    if (learned || logging) gn_enqueue_features(h);
    if (learned) gn_enqueue_guess(h);
    for (int p1 = 0; p1 < 2; ++p1) {
        enqueue_solve(h, h.opt.cg_tol, h.opt.cg_maxit, graph, true,
                      (p1 == 0 && (extrap || learned)) ? h.g32.p : nullptr);
        if (p1 == 0 && logging) gn_enqueue_log(h);
        apply_K<double>(h.d.p, h.tmp64b.p, args64(h), 1.0, 3, s);  // (K d)[iFlt]
        k_qs_fault<<<fblocks(h.F.Nf), FNT, 0, s>>>(h.tmp64b.p, h.v.p, h.d.p, h.dPre.p, f, h.ctrl.p, p1 == 0);
        launch_check();
        count_launch();
    }
    k_qs_end_fault<<<fblocks(h.F.Nf), FNT, 0, s>>>(h.v.p, f, h.ctrl.p);
    k_qs_end_bulk<<<vblocks(n), 256, 0, s>>>(h.d.p, h.dPre.p, h.v.p, h.a.p, L.ld, n, h.ctrl.p,
                                             h.opt.precision == EQC_MIXED ? 1 : 0);
    count_launch(2);
    if (h.nCreep) {
        k_zero_list<<<1, 256, 0, s>>>(h.iCreep.p, h.nCreep, h.d.p, h.v.p, nullptr);
        count_launch();
    }
    launch_check();
}

// Dynamic step (main.jl:297-345): Newmark predictor, K d, boundaries, fault, corrector.
static NmEpi nm_args(Handle& h) {
    NmEpi N;
    N.Kd = h.Kd.p;
    N.v = h.v.p;
    N.a = h.a.p;
    N.invM = h.invM.p;
    N.cL = h.edgeL.p;
    N.cT = h.edgeT.p;
    N.hasL = h.edgeLhas.p;
    N.hasT = h.edgeThas.p;
    N.hdt = &h.ctrl.p->half_dt;
    N.kd_full = &h.ctrl.p->kd_full;
    N.v_half = &h.ctrl.p->v_half;
    N.ld = h.L.ld;
    N.nx = h.L.nx;
    N.ny = h.L.ny;
    return N;
}

// The mixed method's dynamic step, on three streams:
//   main:  predictor of the first element row's node rows (the step's bookkeeping) -> predictor
//          of the other rows -> FP32 apply of the increment -> end of the step off the fault row
//          (k_dyn_finish: K d += K dd, boundary terms, a /= M, v += dt/2 a);
//   side:  the apply of the fault's element row (FP32 of the increment, or FP64 of d on the
//          steps that refresh K d) -> the fault kernel, which ends the step on the fault row and
//          runs the control;
//   side2: on the steps that refresh K d, the FP64 apply of d (forked after the predictor).
// At the start of a dynamic phase and every KD_REFRESH steps K d is recomputed in FP64.  The
// lead predictor's choice reaches the applies through gates (ApplyArgs::gate) rather than
// conditional graph nodes, so the step is the same straight sequence of launches eagerly and in
// a graph.  The step graphs keep ordinary edges here (no programmatic launches): a dependent
// launched early parks its CTAs on the SMs while it waits, and those slots are what the other
// streams' kernels need (measured on dz480: 70 us per step without, 87 us with).
static void enqueue_dyn_mixed_fused(Handle& h) {
    cudaStream_t s = h.stream;
    if (h.capturing) h.pdl_off = true;
    const int64_t n = h.L.size();
    const int* full = &h.ctrl.p->kd_full;
    auto gated = [&](auto A, int val) {
        A.gate = full;
        A.gate_val = val;
        return A;
    };
    const int64_t n0 = std::min<int64_t>(5 * (int64_t)h.L.ld, n);
    k_dyn_predict_nm<<<vblocks4(n0), 256, 0, s>>>(h.d.p, h.v.p, h.a.p, h.F.vPre.p, h.g32.p, h.F.Nf, 0, n0, h.L.ld,
                                                  h.ctrl.p, 1);
    EQC_CHECK_LAUNCH();
    EQC_CUDA(cudaEventRecord(h.ev_fork, s));
    // fault row
    EQC_CUDA(cudaStreamWaitEvent(h.side_stream, h.ev_fork, 0));
    const ApplyArgs<float> a32f = gated(args32(h), 0);
    if (!apply_K_fault32(h.g32.p, h.z32.p, a32f, h.side_stream))
        apply_K<float>(h.g32.p, h.z32.p, a32f, 1.0f, 3, h.side_stream);
    apply_K<double>(h.d.p, h.tmp64c.p, gated(args64(h), 1), 1.0, 3, h.side_stream);
    k_dyn_fault_nm<<<fblocks(h.F.Nf), FNT, 0, h.side_stream>>>(h.a.p, h.v.p, h.tmp64c.p, h.z32.p, h.Kd.p,
                                                               fargs(h, h.bcflag.p), h.ctrl.p,
                                                               h.invM.p, h.edgeL0has, h.edgeL0,
                                                               reinterpret_cast<CtlAcc*>(h.fault_part.p),
                                                               h.fault_count.p);
    EQC_CHECK_LAUNCH();
    EQC_CUDA(cudaEventRecord(h.ev_join, h.side_stream));
    // K d off the fault row
    k_dyn_predict_nm<<<vblocks4(n - n0), 256, 0, s>>>(h.d.p, h.v.p, h.a.p, h.F.vPre.p, h.g32.p, h.F.Nf, n0, n,
                                                      h.L.ld, h.ctrl.p, 0);
    EQC_CHECK_LAUNCH();
    EQC_CUDA(cudaEventRecord(h.ev_fork2, s));
    EQC_CUDA(cudaStreamWaitEvent(h.side_stream2, h.ev_fork2, 0));
    apply_K<double>(h.d.p, h.Kd.p, gated(args64(h), 1), 1.0, 0, h.side_stream2);
    EQC_CUDA(cudaEventRecord(h.ev_join2, h.side_stream2));
    apply_K<float>(h.g32.p, h.q32.p, gated(args32(h), 0), 1.0f, 0, s);
    EQC_CUDA(cudaStreamWaitEvent(s, h.ev_join2, 0));
    k_dyn_finish<<<vblocks(n / 4), 256, 0, s>>>(nm_args(h), h.q32.p);
    EQC_CHECK_LAUNCH();
    count_launch(4);
    EQC_CUDA(cudaStreamWaitEvent(s, h.ev_join, 0));
    launch_check();
}

static void enqueue_dyn(Handle& h, bool graph) {
    cudaStream_t s = h.stream;
    const int64_t n = h.L.size();
    FaultArgs f = fargs(h, h.bcflag.p);
    if (h.opt.precision == EQC_MIXED && h.nm_fused) {
        enqueue_dyn_mixed_fused(h);
        return;
    }
    if (h.opt.precision == EQC_MIXED) {
        // FP64 accumulation of d and of K d, FP32 apply of the step's increment
        if (graph) {
            const cudaGraphConditionalHandle hf = cond_handle(h), hi = cond_handle(h);
            k_dyn_predict_inc<<<vblocks4(n), 256, 0, s>>>(h.d.p, h.v.p, h.a.p, h.F.vPre.p, h.g32.p, h.F.Nf, n,
                                                          h.ctrl.p, hf, hi, 1);
            count_launch();
            const int64_t t0 = capture_tally();
            cond_begin(h, cudaGraphCondTypeIf, hf);
            apply_K<double>(h.d.p, h.Kd.p, args64(h), 1.0, 0, h.stream);
            cond_end(h);
            const int64_t t1 = capture_tally();
            cond_begin(h, cudaGraphCondTypeIf, hi);
            apply_K<float>(h.g32.p, h.q32.p, args32(h), 1.0f, 0, h.stream);
            cond_end(h);
            if (h.capturing) {
                h.capturing->k_bodies += capture_tally() - t0;
                h.capturing->k_fixed_extra += std::max(t1 - t0, capture_tally() - t1);   // one of the two runs
            }
        } else {
            k_dyn_predict_inc<<<vblocks4(n), 256, 0, s>>>(h.d.p, h.v.p, h.a.p, h.F.vPre.p, h.g32.p, h.F.Nf, n,
                                                          h.ctrl.p, 0, 0, 0);
            count_launch();
            int full = 0;
            EQC_CUDA(cudaMemcpyAsync(&full, &h.ctrl.p->kd_full, sizeof(int), cudaMemcpyDeviceToHost, s));
            EQC_CUDA(cudaStreamSynchronize(s));
            if (full) apply_K<double>(h.d.p, h.Kd.p, args64(h), 1.0, 0, s);
            else apply_K<float>(h.g32.p, h.q32.p, args32(h), 1.0f, 0, s);
        }
        k_dyn_force<<<vblocks4(n), 256, 0, s>>>(h.Kd.p, h.q32.p, h.a.p, n, h.ctrl.p);
        count_launch();
    } else {
        k_dyn_predict<<<vblocks(n), 256, 0, s>>>(h.d.p, h.v.p, h.a.p, h.F.vPre.p, h.F.Nf, n, h.ctrl.p);
        count_launch();
        apply_K<double>(h.d.p, h.a.p, args64(h), -1.0, 0, s);
    }
    if (h.nBcNodes > 0)
        k_dyn_bc_nodes<<<(h.nBcNodes + 127) / 128, 128, 0, s>>>(h.a.p, h.v.p, h.bcNode.p, h.bcOps.p, h.bcL.p, h.bcT.p,
                                                               h.nBcNodes);
    else
        k_dyn_bc<<<1, 1024, 0, s>>>(h.a.p, h.v.p, h.iCreep.p, h.nCreep, h.iBcL.p, h.BcLC.p, h.nBcL, h.iBcT.p, h.BcTC.p,
                                    h.nBcT);
    k_dyn_fault<<<fblocks(h.F.Nf), FNT, 0, s>>>(h.a.p, h.v.p, f, h.ctrl.p);
    const bool mixed = h.opt.precision == EQC_MIXED;
    const bool zero_fused = mixed && h.creep_prefix;
    if (mixed) k_dyn_correct_inv<<<vblocks4(n), 256, 0, s>>>(h.a.p, h.v.p, h.invM.p, n, h.ctrl.p,
                                                            zero_fused ? (int64_t)h.F.NFBC0 : 0);
    else k_dyn_correct<<<vblocks(n), 256, 0, s>>>(h.a.p, h.v.p, h.M.p, n, h.ctrl.p, 0);
    count_launch(3);
    if (h.nCreep && !zero_fused) {
        k_zero_list<<<1, 256, 0, s>>>(h.iCreep.p, h.nCreep, h.v.p, h.a.p, nullptr);
        count_launch();
    }
    launch_check();
}

// One whole time step, ending with the control kernel (Vfmax, regime, next dt).
void materialize_dyn_state(Handle& h) {
    if (!h.nm_fused || h.opt.precision != EQC_MIXED) return;
    k_nm_materialize<<<vblocks(h.L.size()), 256, 0, h.stream>>>(h.ctrl.p, nm_args(h));
    EQC_CHECK_LAUNCH();
    count_launch();
    EQC_CUDA(cudaMemsetAsync(&h.ctrl.p->v_half, 0, sizeof(int), h.stream));   // after every CTA read it
    if (h.h_ctrl) h.h_ctrl->v_half = 0;
}

void enqueue_step(Handle& h, int iso, bool graph) {
    // the mixed method's dynamic step advances it and t in its predictor and runs the control in
    // its fault kernel
    const bool fused = iso == 2 && h.opt.precision == EQC_MIXED && h.nm_fused;
    if (!fused) {
        k_step_begin<<<1, 1, 0, h.stream>>>(h.ctrl.p);
        count_launch();
    }
    if (iso == 1) enqueue_qs(h, graph);
    else enqueue_dyn(h, graph);
    if (!fused) {
        k_control<<<1, FT, 0, h.stream>>>(h.v.p, fargs(h, h.bcflag.p), h.ctrl.p);
        launch_check();
        count_launch();
    }
}

void destroy_graphs(Handle& h) {
    for (StepGraph* arr : {h.graphs, h.batched})
        for (int k = 0; k < 2; ++k) {
            StepGraph& g = arr[k];
            if (g.exec) cudaGraphExecDestroy(g.exec);
            if (g.graph) cudaGraphDestroy(g.graph);
            g = StepGraph();
        }
}

// End of a step inside a batched launch: log time_ and Vfmax (and, every 10th step, the receivers,
// main.jl:433-435), then decide on the device whether the loop of steps goes on.  It stops on any
// step whose outputs need the host (main.jl:361-436: event start or end, a 5-year snapshot, a
// seismic snapshot or its end), on a regime switch, a failure flag, t_end, a full log, or verbose
// progress printing; the host then treats that last step exactly like a single step.
__global__ void k_step_end(Ctrl* C, double* __restrict__ log_t, double* __restrict__ log_vf,
                           double* __restrict__ log_seis, const int64_t* __restrict__ iSeis, int ns,
                           const double* __restrict__ d, const double* __restrict__ v, const double* __restrict__ a,
                           NmEpi N, int regime, cudaGraphConditionalHandle hw) {
    EQC_GRID_WAIT();
    __shared__ int rec;
    const long long it = C->it;
    const int k = C->nlog;
    if (threadIdx.x == 0) {
        log_t[k] = C->t;
        log_vf[k] = C->Vfmax;
        rec = (ns > 0 && it % 10 == 0) ? C->nrec : -1;
    }
    __syncthreads();
    if (rec >= 0 && (int)threadIdx.x < ns) {
        const int64_t g = iSeis[threadIdx.x];
        double* o = log_seis + (int64_t)rec * 3 * ns;
        double vg = v[g], ag = a[g];
        if (C->v_half && g >= N.ld) nm_state_at(N, g, C->half_dt, &vg, &ag);
        o[threadIdx.x] = d[g];
        o[ns + threadIdx.x] = vg;
        o[2 * ns + threadIdx.x] = ag;
    }
    if (threadIdx.x == 0) {
        C->nlog = k + 1;
        if (rec >= 0) C->nrec = rec + 1;
        const double t = C->t, Vf = C->Vfmax;
        int stop = 0;
        if (C->isolver != regime) stop = 1;
        if (C->fail != 0x7fffffff || C->apply_err || C->cg_fail || !isfinite(Vf)) stop = 1;
        if (Vf > 1.01 * C->Vthres && C->slipstart == 0) stop = 1;
        if (Vf < 0.99 * C->Vthres && C->slipstart == 1) stop = 1;
        if (t > C->tvsx) stop = 1;
        if (Vf > C->Vevne) {
            if (C->idelevne == 0 || (t - C->tevneb) > C->tevne) stop = 1;
        } else if (C->idelevne == 1) {
            stop = 1;
        }
        if (C->verbose && it % 500 == 0) stop = 1;
        if (k + 1 >= C->max_batch || t >= C->t_end) stop = 1;
        if (rec >= 0 && rec + 1 >= C->rec_cap) stop = 1;
        cudaGraphSetConditional(hw, stop ? 0u : 1u);
    }
}

// Captures the batched steps of regime iso: a device-driven WHILE loop over whole steps.
static StepGraph& batched_graph(Handle& h, int iso) {
    StepGraph& G = h.batched[iso == 1 ? 0 : 1];
    if (G.exec) return G;
    G = StepGraph();
    h.capturing = &G;
    capture_counting(true);
    try {
        h.pdl_off = false;
        EQC_CUDA(cudaStreamBeginCapture(h.stream, cudaStreamCaptureModeThreadLocal));
        const cudaGraphConditionalHandle hw = cond_handle(h, 1);   // the first step always runs
        cond_begin(h, cudaGraphCondTypeWhile, hw);
        enqueue_step(h, iso, true);
        k_step_end<<<1, 32, 0, h.stream>>>(h.ctrl.p, h.log_t.p, h.log_vf.p, h.log_seis.p, h.iSeis.p, h.nSeis, h.d.p,
                                            h.v.p, h.a.p, nm_args(h), iso, hw);
        EQC_CHECK_LAUNCH();
        count_launch();
        cond_end(h);
        EQC_CUDA(cudaStreamEndCapture(h.stream, &G.graph));
        if (!h.pdl_off) h.pdl_edges += make_programmatic(G.graph);
        h.pdl_off = false;
    } catch (...) {
        abort_capture(h);
        h.capturing = nullptr;
        throw;
    }
    G.k_fixed = capture_tally() - G.k_bodies + G.k_fixed_extra;   // kernels of one step (the loop body)
    capture_counting(false);
    h.capturing = nullptr;
    EQC_CUDA(cudaGraphInstantiate(&G.exec, G.graph, 0));
    return G;
}

// Captures the step of regime iso (1 quasi-static, 2 dynamic) into a graph, once.
static StepGraph& step_graph(Handle& h, int iso) {
    StepGraph& G = h.graphs[iso == 1 ? 0 : 1];
    if (G.exec) return G;
    G = StepGraph();
    h.capturing = &G;
    capture_counting(true);
    try {
        h.pdl_off = false;
        EQC_CUDA(cudaStreamBeginCapture(h.stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(h, iso, true);
        EQC_CUDA(cudaStreamEndCapture(h.stream, &G.graph));
        if (!h.pdl_off) h.pdl_edges += make_programmatic(G.graph);
        h.pdl_off = false;
    } catch (...) {
        abort_capture(h);
        h.capturing = nullptr;
        throw;
    }
    G.k_fixed = capture_tally() - G.k_bodies + G.k_fixed_extra;
    capture_counting(false);
    h.capturing = nullptr;
    EQC_CUDA(cudaGraphInstantiate(&G.exec, G.graph, 0));
    return G;
}

// Host side of one finished step (the control block is in h.h_ctrl): failure checks and the
// output triggers of main.jl:361-436.
void post_step(Handle& h, int iso, eqc_run_stats& stats, PostBufs& pb, bool logged) {
    cudaStream_t s = h.stream;
    const int Nf = h.F.Nf;
    const double Vpl = h.Vpl;
    const std::vector<double>& tauo = h.h_tauo;
    const std::vector<double>& FltX = h.h_FltX;
    Ctrl& C = *h.h_ctrl;
    std::vector<double>& dF = pb.dF;
    std::vector<double>& vF = pb.vF;
    std::vector<double>& tauF = pb.tauF;
    std::vector<double>& seis = pb.seis;
    if (seis.size() < (size_t)(3 * std::max(h.nSeis, 1))) seis.resize(3 * std::max(h.nSeis, 1));
    if (!logged) {
        if (iso == 1) stats.qs_steps++;
        else stats.dyn_steps++;
    }
    const double tnow = C.t;
    if (!logged && (int64_t)h.res.time_.size() >= h.cap_time)
        throw Error(EQC_E_CAPACITY, "time_ capacity (" + std::to_string(h.cap_time) + ") exceeded");
    if (!logged) h.res.time_.push_back(tnow);
    if (C.fail != 0x7fffffff)
        throw Error(EQC_E_NR, "NR SEARCH FAILED at fault node " + std::to_string(C.fail));
    if (C.apply_err) check_apply_err(h);
    if (C.cg_fail & 2) throw Error(EQC_E_NAN, "non-finite residual in CG");
    if (C.cg_fail & 1)
        throw Error(EQC_E_CG, "CG did not converge within maxit (relres " + std::to_string(C.cg_last_relres) + ")");
    const double Vfmax = C.Vfmax;
    if (!std::isfinite(Vfmax)) throw Error(EQC_E_NAN, "non-finite slip rate");
    // ---- outputs (main.jl:361-436) ----
    bool need_cols = (Vfmax > 1.01 * h.Vthres && h.slipstart == 0) ||
                     (Vfmax < 0.99 * h.Vthres && h.slipstart == 1) || (tnow > h.tvsx) || (Vfmax > h.Vevne);
    if (need_cols) fault_columns(h, dF, vF, tauF);
    auto push_col = [&](std::vector<double>& dst, int which) {
        for (int k = 0; k < Nf; ++k) {
            double val;
            if (which == 0) val = 2 * dF[k] + Vpl * tnow;
            else if (which == 1) val = 2 * vF[k] + Vpl;
            else val = (tauF[k] + tauo[k]) / 1e6;
            dst.push_back(val);
        }
    };
    if (Vfmax > 1.01 * h.Vthres && h.slipstart == 0) {
        if (h.it_s >= CAP_EV) throw Error(EQC_E_CAPACITY, "event capacity (400) exceeded");
        h.it_s += 1;
        for (int k = 0; k < Nf; ++k) h.delfref[k] = 2 * dF[k] + Vpl * tnow;
        h.slipstart = 1;
        h.res.tStart.push_back(tnow);
        push_col(h.res.taubefore, 2);
        h.res.hypo.push_back(FltX[C.ihypo]);
    }
    if (Vfmax < 0.99 * h.Vthres && h.slipstart == 1) {
        h.it_e += 1;
        for (int k = 0; k < Nf; ++k) h.res.delfafter.push_back(2 * dF[k] + Vpl * tnow - h.delfref[k]);
        push_col(h.res.tauafter, 2);
        h.res.tEnd.push_back(tnow);
        h.slipstart = 0;
        // damage grows at the end of each earthquake (main.jl:377-378, damageEvol.jl:5-7)
        if (!h.damage_el.empty() && h.damage_factor != 1.0) damage_evolve(h);
    }
    if (tnow > h.tvsx) {
        if (h.ntvsx >= CAP_IS) throw Error(EQC_E_CAPACITY, "interseismic snapshot capacity (4000) exceeded");
        h.ntvsx += 1;
        h.idd += 1;
        push_col(h.res.is_slip, 0);
        push_col(h.res.is_slipvel, 1);
        push_col(h.res.is_stress, 2);
        h.tvsx = h.tvsx + h.tvsxinc;
    }
    if (Vfmax > h.Vevne) {
        if (h.idelevne == 0) {
            if (h.nevne >= CAP_SEISMIC) throw Error(EQC_E_CAPACITY, "seismic snapshot capacity exceeded");
            h.nevne += 1;
            h.idd += 1;
            h.idelevne = 1;
            h.tevneb = tnow;
            h.tevne = h.tevneinc;
            push_col(h.res.seismic_slip, 0);
            push_col(h.res.seismic_slipvel, 1);
            push_col(h.res.seismic_stress, 2);
        }
        if (h.idelevne == 1 && (tnow - h.tevneb) > h.tevne) {
            if (h.nevne >= CAP_SEISMIC) throw Error(EQC_E_CAPACITY, "seismic snapshot capacity exceeded");
            h.nevne += 1;
            h.idd += 1;
            push_col(h.res.seismic_slip, 0);
            push_col(h.res.seismic_slipvel, 1);
            push_col(h.res.seismic_stress, 2);
            h.tevne = h.tevne + h.tevneinc;
        }
    } else {
        h.idelevne = 0;
    }
    if (h.opt.verbose && C.it % 500 == 0) printf("Time (yr) = %1.5g\n", tnow / h.yr2sec);
    if (!logged && C.it % 10 == 0 && h.nSeis > 0) {
        if (h.rit >= CAP_SEIS) throw Error(EQC_E_CAPACITY, "receiver capacity (190000) exceeded");
        h.rit += 1;
        k_gather_seis<<<1, 32, 0, s>>>(h.iSeis.p, h.nSeis, h.d.p, h.v.p, h.a.p, h.seis.p, h.ctrl.p, nm_args(h));
        count_launch();
        EQC_CUDA(cudaMemcpyAsync(seis.data(), h.seis.p, sizeof(double) * 3 * h.nSeis, cudaMemcpyDeviceToHost, s));
        EQC_CUDA(cudaStreamSynchronize(s));
        for (int k = 0; k < h.nSeis; ++k) {
            h.res.dSeis.push_back(seis[k]);
            h.res.vSeis.push_back(seis[h.nSeis + k]);
            h.res.aSeis.push_back(seis[2 * h.nSeis + k]);
        }
    }
    if (!logged) {
        h.res.Vfmax.push_back(Vfmax);
        stats.steps++;
    }
}

void run_steps(Handle& h, int64_t max_steps, double t_end, eqc_run_stats* st) {
    if (!h.initialized) throw Error(EQC_E_STATE, "eqc_run before eqc_init");
    cudaStream_t s = h.stream;
    const int Nf = h.F.Nf;
    const double Vpl = h.Vpl;
    const std::vector<double>& tauo = h.h_tauo;
    const std::vector<double>& FltX = h.h_FltX;
    auto t0 = std::chrono::steady_clock::now();
    eqc_run_stats stats{};
    PostBufs pb;
    Ctrl& C = *h.h_ctrl;
    EQC_CUDA(cudaMemcpyAsync(h.h_ctrl, h.ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
    EQC_CUDA(cudaStreamSynchronize(s));
    const long long cg0 = C.cg_iters, qs0 = C.cg_solves;
    cudaEvent_t ev0, ev1;
    EQC_CUDA(cudaEventCreate(&ev0));
    EQC_CUDA(cudaEventCreate(&ev1));
    EQC_CUDA(cudaEventRecord(ev0, s));
    const int batch = h.opt.step_batch == 0 ? STEP_BATCH : h.opt.step_batch;
    while (C.t < t_end && stats.steps < max_steps) {
        if ((int64_t)h.res.time_.size() >= h.cap_time)
            throw Error(EQC_E_CAPACITY, "time_ capacity (" + std::to_string(h.cap_time) + ") exceeded");
        const int iso = C.isolver;
        if (h.opt.use_graphs && batch > 1) {   // several steps per launch, outputs logged on the device
            const long long it_before = C.cg_iters, up_before = C.cg_updates, ca_before = C.cg_carried,
                            so_before = C.cg_solves;
            C.tvsx = h.tvsx;
            C.tevneb = h.tevneb;
            C.tevne = h.tevne;
            C.t_end = t_end;
            C.Vthres = h.Vthres;
            C.Vevne = h.Vevne;
            C.slipstart = (int)h.slipstart;
            C.idelevne = (int)h.idelevne;
            C.verbose = h.opt.verbose;
            C.max_batch = (int)std::min<int64_t>({(int64_t)batch, max_steps - stats.steps,
                                                  h.cap_time - (int64_t)h.res.time_.size()});
            C.rec_cap = (int)std::min<int64_t>(STEP_BATCH / 10 + 2, CAP_SEIS - h.rit);
            if (h.nSeis > 0 && C.rec_cap < 1) throw Error(EQC_E_CAPACITY, "receiver capacity (190000) exceeded");
            C.nlog = 0;
            C.nrec = 0;
            StepGraph& G = batched_graph(h, iso);
            EQC_CUDA(cudaMemcpyAsync(h.ctrl.p, h.h_ctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, s));
            EQC_CUDA(cudaGraphLaunch(G.exec, s));
            EQC_CUDA(cudaMemcpyAsync(h.h_ctrl, h.ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
            EQC_CUDA(cudaStreamSynchronize(s));
            const int nl = C.nlog, nr = C.nrec;
            std::vector<double> lt(nl), lv(nl), ls((size_t)nr * 3 * std::max(h.nSeis, 1));
            h.log_t.download(lt.data(), nl, s);
            h.log_vf.download(lv.data(), nl, s);
            if (nr) h.log_seis.download(ls.data(), (size_t)nr * 3 * h.nSeis, s);
            EQC_CUDA(cudaStreamSynchronize(s));
            h.res.time_.insert(h.res.time_.end(), lt.begin(), lt.end());
            h.res.Vfmax.insert(h.res.Vfmax.end(), lv.begin(), lv.end());
            for (int r = 0; r < nr; ++r)
                for (int k = 0; k < h.nSeis; ++k) {
                    h.res.dSeis.push_back(ls[(size_t)r * 3 * h.nSeis + k]);
                    h.res.vSeis.push_back(ls[(size_t)r * 3 * h.nSeis + h.nSeis + k]);
                    h.res.aSeis.push_back(ls[(size_t)r * 3 * h.nSeis + 2 * h.nSeis + k]);
                }
            h.rit += nr;
            stats.steps += nl;
            if (iso == 1) stats.qs_steps += nl;
            else stats.dyn_steps += nl;
            const long long carried = C.cg_carried - ca_before;
            g_launches += (int64_t)nl * G.k_fixed + G.k_iter * (C.cg_iters - it_before) +
                          G.k_update * (C.cg_updates - up_before) + G.k_carry * carried +
                          G.k_full * (C.cg_solves - so_before - carried);
            post_step(h, iso, stats, pb, true);   // the outputs of the last step (the one that stopped)
            continue;
        }
        const long long it_before = C.cg_iters, up_before = C.cg_updates, ca_before = C.cg_carried,
                        so_before = C.cg_solves;
        if (h.opt.use_graphs) {
            StepGraph& G = step_graph(h, iso);
            EQC_CUDA(cudaGraphLaunch(G.exec, s));
            // kernels the replay executes: fixed part plus the conditional bodies that ran
            EQC_CUDA(cudaMemcpyAsync(h.h_ctrl, h.ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
            EQC_CUDA(cudaStreamSynchronize(s));
            const long long carried = C.cg_carried - ca_before;
            g_launches += G.k_fixed + G.k_iter * (C.cg_iters - it_before) + G.k_update * (C.cg_updates - up_before) +
                          G.k_carry * carried + G.k_full * (C.cg_solves - so_before - carried);
        } else {
            enqueue_step(h, iso, false);
            EQC_CUDA(cudaMemcpyAsync(h.h_ctrl, h.ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost, s));
            EQC_CUDA(cudaStreamSynchronize(s));
        }
        post_step(h, iso, stats, pb);
    }
    EQC_CUDA(cudaEventRecord(ev1, s));
    EQC_CUDA(cudaEventSynchronize(ev1));
    float gms = 0.f;
    EQC_CUDA(cudaEventElapsedTime(&gms, ev0, ev1));
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    stats.gpu_ms = gms;
    stats.cg_iters = C.cg_iters - cg0;
    stats.qs_solves = C.cg_solves - qs0;
    stats.t = C.t;
    stats.dt = C.dt;
    stats.isolver = C.isolver;
    stats.events = (int32_t)h.it_s;
    stats.wall_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st) *st = stats;
}

}  // namespace eqc
