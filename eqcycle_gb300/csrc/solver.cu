// Quasi-static displacement solve (K3 + preconditioner), src/main.jl:236-262.
//
// The reference solves  -K_II d_I = (K F)_I  with cg!(dnew, kni, rhs, Pl = AMG, tol)
// (IterativeSolvers.jl 0.8: x0 = previous displacement, rho0 = 1, u0 = 0, stop when
// ||r_k||_2 <= tol * ||rhs||_2).  Here the equivalent SPD system K_II d_I = -(K F)_I is
// solved on the layout's rows 1.. (the fault is row 0 and holds F), so every vector is
// a contiguous slice [ld, ld*ny) of a full node array.
//
// Plain FP64 path: FP64 apply, FP64 preconditioner, FP64 vectors.
// Mixed path: CG with reliable updates (van der Vorst & Ye residual replacement): the
// Krylov recurrences run on FP32 vectors with an FP32 apply and FP32 preconditioner
// (dot products accumulated in FP64); the iterate is accumulated in FP64 and, whenever
// the recurrence residual has dropped by a factor `delta` since the last update, the
// true residual b - K_II x is recomputed with the FP64 apply and replaces the FP32 one.
// Convergence is always certified on an FP64 true residual.
#include "model.h"
#include "reduce.cuh"
#include "vec.cuh"
#include "epi.cuh"
#include <cmath>
#include <cstddef>

namespace eqc {

// Slots of the scalar block the vector kernels address (the leading doubles of CGState).
enum { S_RHO = 0, S_RHOP = 1, S_PQ = 2, S_RR = 3, S_BB = 4 };
static_assert(offsetof(CGState, rho_prev) == 8 * S_RHOP && offsetof(CGState, pq) == 8 * S_PQ &&
                  offsetof(CGState, rr) == 8 * S_RR && offsetof(CGState, bb) == 8 * S_BB,
              "CGState must start with rho, rho_prev, pq, rr, bb");

// The vector kernels run on a fixed grid of VEC_BLOCKS x VEC_THREADS threads over 4-wide
// chunks (n is a multiple of 4: every vector is a whole number of 8-entry-aligned rows);
// reductions are deterministic (fixed slices, partials summed in CTA order).

// dot into S_RHO, shifting the previous value into S_RHOP
template <class T>
__global__ void __launch_bounds__(VEC_THREADS) k_dot_rho(const T* __restrict__ x, const T* __restrict__ y, int64_t n,
                                                         double* part, unsigned* count, double* S) {
    EQC_GRID_WAIT();
    __shared__ double sh[32];
    DotAcc<T> acc;
    for (int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n; i += 4 * (int64_t)gridDim.x * blockDim.x) {
        T a[4], b[4];
        ld4(x + i, a);
        ld4(y + i, b);
#pragma unroll
        for (int k = 0; k < 4; ++k) acc.add(a[k], b[k]);
    }
    const double s = block_sum(acc.value(), sh);
    finish_reduction(s, part, count, sh, [&](double t) {
        S[S_RHOP] = S[S_RHO];
        S[S_RHO] = t;
    });
}

// u = z + (rho / rho_prev) u   (u = z after a restart)
template <class T>
__global__ void __launch_bounds__(VEC_THREADS) k_pupdate(const T* __restrict__ z, T* __restrict__ u, int64_t n,
                                                         const double* S, const int* restart) {
    EQC_GRID_WAIT();
    const T b = *restart ? T(0) : (T)(S[S_RHO] / S[S_RHOP]);
    for (int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n; i += 4 * (int64_t)gridDim.x * blockDim.x) {
        T zz[4], uu[4];
        ld4(z + i, zz);
        ld4(u + i, uu);
#pragma unroll
        for (int k = 0; k < 4; ++k) uu[k] = zz[k] + b * uu[k];
        st4(u + i, uu);
    }
}

// The update decision (cg_check_a) run by the last CTA of k_xr_update (on = 0: not run), and the
// loop's condition for an iteration without an update (with one, k_cg_check_b in the update's
// body sets it again): without an update the loop goes on unless the residual is not finite.
struct CheckA {
    int on = 0, use_cond = 0;   // on: 1 the mixed iteration's decision, 2 the FP64 iteration's check
    double delta = 0.0;
    cudaGraphConditionalHandle hi = 0, hw = 0;
};
__device__ __forceinline__ int cg_check_a(CGState* S, double delta);
__device__ __forceinline__ int cg_check64(CGState* S);

// x += alpha u ; r -= alpha q ; S_RR = r.r   (alpha = rho / (u.q)); then the update decision
// (ck.on: S is the CGState)
template <class TX, class T>
__global__ void __launch_bounds__(VEC_THREADS) k_xr_update(TX* __restrict__ x, T* __restrict__ r, const T* __restrict__ u,
                                                           const T* __restrict__ q, int64_t n, double* part,
                                                           unsigned* count, double* S, CheckA ck) {
    EQC_GRID_WAIT();
    __shared__ double sh[32];
    const double alpha = S[S_RHO] / S[S_PQ];
    const T a = (T)alpha;
    const TX ax = (TX)alpha;
    DotAcc<T> acc;
    for (int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n; i += 4 * (int64_t)gridDim.x * blockDim.x) {
        TX xx[4];
        T rr[4], uu[4], qq[4];
        ld4(x + i, xx);
        ld4(r + i, rr);
        ld4(u + i, uu);
        ld4(q + i, qq);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            xx[k] = xx[k] + ax * (TX)uu[k];
            rr[k] = rr[k] - a * qq[k];
            acc.add(rr[k], rr[k]);
        }
        st4(x + i, xx);
        st4(r + i, rr);
    }
    const double s = block_sum(acc.value(), sh);
    finish_reduction(s, part, count, sh, [&](double t) {
        S[S_RR] = t;
        CGState* cs = reinterpret_cast<CGState*>(S);
        if (ck.on == 1) {
            const int need = cg_check_a(cs, ck.delta);
            if (ck.use_cond) {
                cudaGraphSetConditional(ck.hi, need ? 1u : 0u);
                cudaGraphSetConditional(ck.hw, cs->done == 0 ? 1u : 0u);
            }
        } else if (ck.on == 2) {
            const int st = cg_check64(cs);
            if (ck.use_cond) cudaGraphSetConditional(ck.hw, st == 0 ? 1u : 0u);
        }
    });
}

template <class T>
__global__ void k_jacobi(const T* __restrict__ r, const T* __restrict__ dg, T* __restrict__ z, int64_t n) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        z[i] = r[i] / dg[i];
}

// x64 += (double) y32 / sigma ; y32 = 0   (sigma a power of two: the division is exact); for an
// intermediate reliable update (S->upd_incr) also dx64 += y32: dx64 is sigma times x's change since
// r64 was last exact, whose K dx updates the residual (in the recurrence's scaled units, so that
// the steady-sliding start's 1e-25 m increments stay inside double-float's range).
// The widening and the scaling use integer operations (f32_to_f64, pow2_scale): one FP64 add per
// vector and node, the same bits as (double) y / sigma.
__global__ void __launch_bounds__(VEC_THREADS) k_fold(double* __restrict__ x, float* __restrict__ y,
                                                      double* __restrict__ dx, int64_t n, const CGState* S) {
    EQC_GRID_WAIT();
    const double inv = 1.0 / S->sigma;
    const int es = -ilogb(S->sigma);
    const bool incr = dx && S->upd_incr;
    for (int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n; i += 4 * (int64_t)gridDim.x * blockDim.x) {
        double xx[4], dd[4];
        float yy[4];
        ld4(x + i, xx);
        ld4(y + i, yy);
        if (incr) ld4(dx + i, dd);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const double yw = f32_to_f64(yy[k]);
            xx[k] += pow2_scale(yw, es, inv);
            if (incr) dd[k] += yw;
        }
        st4(x + i, xx);
        if (incr) st4(dx + i, dd);
        const float zero[4] = {0.f, 0.f, 0.f, 0.f};
        st4(y + i, zero);
    }
}

// dx64 = sigma times the kept initial-guess increment (r64 is the residual without it), else 0.
// (widening and the power-of-two scaling by integer operations: the bits of (double) g * sigma)
__global__ void k_dx_init(double* __restrict__ dx, const float* __restrict__ g, const CGState* S, int64_t n) {
    EQC_GRID_WAIT();
    const bool keep = g && S->guess_keep;
    const double sg = S->sigma;
    const int es = ilogb(sg);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        dx[i] = keep ? pow2_scale(f32_to_f64(g[i]), es, sg) : 0.0;
}
// [intermediate reliable update (kdx given and S->upd_incr): r64 += kdx / sigma, kdx the
// double-float -K dx of the scaled change] ; r32 = (float) (sigma r64) ; S->rr = r32.r32 (the
// scaled norm, of the FP32 residual: within 1e-7 of sigma^2 r64.r64)
// (kdx given: a reliable update's end; r64 is then exact for x, so dx64 = 0.)  The scaling and
// the rounding to FP32 use integer operations (pow2_scale, f64_to_f32) and the norm the FP32
// compensated sum: GB300's FP64 rate is a small fraction of its FP32 and integer rates.
__global__ void __launch_bounds__(VEC_THREADS) k_demote_norm(double* __restrict__ r64, float* __restrict__ r32,
                                                             int64_t n, double* part, unsigned* count, CGState* S,
                                                             const double* __restrict__ kdx, double* __restrict__ dx) {
    EQC_GRID_WAIT();
    __shared__ double sh[32];
    const double sg = S->sigma;
    const int es = ilogb(sg);
    const bool incr = kdx && S->upd_incr;
    DotAcc<float> acc;
    for (int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n; i += 4 * (int64_t)gridDim.x * blockDim.x) {
        double v[4];
        float f[4];
        ld4(r64 + i, v);
        if (incr) {
            const double inv = 1.0 / sg;   // a power of two: exact
            double t[4];
            ld4(kdx + i, t);
#pragma unroll
            for (int k = 0; k < 4; ++k) v[k] = __fma_rn(t[k], inv, v[k]);
            st4(r64 + i, v);
        }
        if (dx) {
            const double zero[4] = {0.0, 0.0, 0.0, 0.0};
            st4(dx + i, zero);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            f[k] = f64_to_f32(pow2_scale(v[k], es, sg));
            acc.add(f[k], f[k]);
        }
        st4(r32 + i, f);
    }
    const double s = block_sum(acc.value(), sh);
    finish_reduction(s, part, count, sh, [&](double t) { S->rr = t; });
}

// Scale of the FP32 recurrence for this solve: sigma = 2^-e with 2^e <= ||b|| < 2^(e+1)
// (1 in FP64, or when b = 0).
__global__ void k_set_sigma(CGState* S, int mixed) {
    EQC_GRID_WAIT();
    const double nb = sqrt(S->bb);
    S->sigma = (mixed && nb > 0 && isfinite(nb)) ? ldexp(1.0, -ilogb(nb)) : 1.0;
}

static inline dim3 vgrid() { return dim3(vec_blocks()); }

// ---- device-side control of the CG loop -----------------------------------------------
// Every control kernel is a single thread: it owns the CGState and is the only caller of
// cudaGraphSetConditional for its node (concurrent calls on one handle are undefined).

// Start of a solve: S->bb, S->rr hold ||b||^2 and ||r0||^2.
__global__ void k_cg_init(CGState* S, double tol, int maxit, int rule, int incr_ok, cudaGraphConditionalHandle hw,
                          int use_cond) {
    EQC_GRID_WAIT();
    S->incr_ok = incr_ok;
    S->upd_incr = 0;
    const double nb = sqrt(S->bb), r = sqrt(S->rr) / S->sigma;
    const double reltol = (rule == EQC_TOL_R0 ? r : nb) * tol;
    S->nb = nb;
    S->reltol = reltol;
    S->res = r;
    S->rmax = r;
    S->it = 0;
    S->maxit = maxit;
    S->rho = 1.0;
    S->rho_prev = 1.0;
    S->need_update = 0;
    S->restart = 0;
    const int st = !isfinite(r) ? 3 : (r <= reltol ? 1 : (maxit <= 0 ? 2 : 0));
    S->done = st;
    if (use_cond) cudaGraphSetConditional(hw, st == 0 ? 1u : 0u);
}

// End of an FP64 iteration: the loop goes on until ||r|| <= reltol or maxit.
__device__ __forceinline__ int cg_check64(CGState* S) {
    S->it += 1;
    const double r = sqrt(S->rr) / S->sigma;
    S->res = r;
    const int st = !isfinite(r) ? 3 : (r <= S->reltol ? 1 : (S->it >= S->maxit ? 2 : 0));
    S->done = st;
    return st;
}

// Mixed precision, after the FP32 recurrences: decide whether a reliable update is due
// (the recurrence residual fell by `delta` since the last one, or the loop would stop).
__device__ __forceinline__ int cg_check_a(CGState* S, double delta) {
    S->it += 1;
    S->restart = 0;   // consumed by this iteration's direction update
    const double rs = sqrt(S->rr) / S->sigma;
    int need = 0;
    if (!isfinite(rs)) {
        S->done = 3;
    } else {
        S->rmax = fmax(S->rmax, rs);
        need = (rs < delta * S->rmax || rs <= S->reltol || S->it >= S->maxit) ? 1 : 0;
    }
    S->res = rs;
    S->need_update = need;
    // a certifying update (the loop would stop) recomputes b - K x in FP64
    S->upd_incr = (need && rs > S->reltol && S->it < S->maxit && S->incr_ok) ? 1 : 0;
    return need;
}

// Mixed precision, end of the iteration: take the FP64 residual of a reliable update and
// decide whether the loop goes on.
__global__ void k_cg_check_b(CGState* S, Ctrl* C, cudaGraphConditionalHandle hw, int use_cond) {
    EQC_GRID_WAIT();
    if (S->done != 3) {
        if (S->need_update) {
            const double rs = sqrt(S->rr) / S->sigma;
            // the true residual left the recurrence's (the FP32 recurrences drifted, e.g. from a
            // guess far from the solution): continue from the true residual with a fresh direction
            if (rs > 2.0 * S->res) {
                S->restart = 1;
                C->cg_restarts += 1;
            }
            S->res = rs;
            S->rmax = rs;
            S->need_update = 0;
            C->cg_updates += 1;
        }
        const double r = S->res;
        S->done = !isfinite(r) ? 3 : (r <= S->reltol ? 1 : (S->it >= S->maxit ? 2 : 0));
    }
    if (use_cond) cudaGraphSetConditional(hw, S->done == 0 ? 1u : 0u);
}

// After the loop: solve counters and failure flags in the control block.  mark_valid: the
// loop ended on an FP64 true residual (mixed precision), which the next solve may carry.
__global__ void k_cg_finish(const CGState* S, Ctrl* C, int mark_valid) {
    EQC_GRID_WAIT();
    C->r_valid = (mark_valid && S->done == 1) ? 1 : 0;
    C->cg_iters += S->it;
    C->cg_solves += 1;
    C->cg_last_it = S->it;
    C->cg_last_relres = S->nb > 0 ? S->res / S->nb : S->res;
    if (S->done == 2) C->cg_fail |= 1;
    if (S->done == 3) C->cg_fail |= 2;
}

// Fault row: dF = d[k] - Flast[k] into row 0 of a work vector, Flast = d[k].
__global__ void k_fault_delta(const double* __restrict__ d, double* __restrict__ Flast, double* __restrict__ dF,
                              int Nf) {
    EQC_GRID_WAIT();
    for (int k = threadIdx.x + blockIdx.x * blockDim.x; k < Nf; k += blockDim.x * gridDim.x) {
        const double f = d[k];
        dF[k] = f - Flast[k];
        Flast[k] = f;
    }
}

// Carried residual, rows 1..4 (the only rows K_IF reaches): r64 += t.
__global__ void k_carry_rows(double* __restrict__ r64, const double* __restrict__ t, int64_t n) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r64[i] += t[i];
}

// Carried residual after the guess increment g: r32 -= sigma K_II g (t = K_II g in FP32),
// S->rr_guess = ||r32||^2 (S->rr keeps the residual without the increment).
__global__ void __launch_bounds__(VEC_THREADS) k_guess_residual(float* __restrict__ r32, const float* __restrict__ t,
                                                                int64_t n, double* part, unsigned* count, CGState* S) {
    EQC_GRID_WAIT();
    __shared__ double sh[32];
    const float sg = (float)S->sigma;
    DotAcc<float> acc;
    for (int64_t i = 4 * ((int64_t)blockIdx.x * blockDim.x + threadIdx.x); i < n; i += 4 * (int64_t)gridDim.x * blockDim.x) {
        float rr[4], tt[4];
        ld4(r32 + i, rr);
        ld4(t + i, tt);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            rr[k] -= sg * tt[k];
            acc.add(rr[k], rr[k]);
        }
        st4(r32 + i, rr);
    }
    const double s = block_sum(acc.value(), sh);
    finish_reduction(s, part, count, sh, [&](double tt2) { S->rr_guess = tt2; });
}

// The previous-step guess judges the increment: keep it only if it lowered ||r||.
__global__ void k_guess_decide(CGState* S, Ctrl* C) {
    EQC_GRID_WAIT();
    const int keep = S->rr_guess < S->rr ? 1 : 0;
    S->guess_keep = keep;
    if (keep) S->rr = S->rr_guess;
    C->guess_tried += 1;
    C->guess_kept += keep;
}
// Rejected increment: d -= g, r32 = (float) (sigma r64) (the residual without it).
__global__ void __launch_bounds__(VEC_THREADS) k_guess_revert(const CGState* S, double* __restrict__ d,
                                                              const float* __restrict__ g, float* __restrict__ r32,
                                                              const double* __restrict__ r64, int64_t n) {
    EQC_GRID_WAIT();
    if (S->guess_keep) return;
    const double sg = S->sigma;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        d[i] -= (double)g[i];
        r32[i] = (float)(r64[i] * sg);
    }
}

// Chooses the residual set-up of a solve: carry (r_valid) or a full FP64 apply.
__global__ void k_setup_select(Ctrl* C, cudaGraphConditionalHandle hc, cudaGraphConditionalHandle hf, int use_cond) {
    EQC_GRID_WAIT();
    const unsigned v = C->r_valid ? 1u : 0u;
    C->cg_carried += v;
    if (use_cond) {
        cudaGraphSetConditional(hc, v);
        cudaGraphSetConditional(hf, 1u - v);
    }
}

static const CGState& read_cg(Handle& h) {
    EQC_CUDA(cudaMemcpyAsync(h.h_cg, h.cg.p, sizeof(CGState), cudaMemcpyDeviceToHost, h.stream));
    EQC_CUDA(cudaStreamSynchronize(h.stream));
    return *h.h_cg;
}

template <class T>
static void precond(Handle& h, const T* r, T* z, int64_t n);

template <>
void precond<double>(Handle& h, const double* r, double* z, int64_t n) {
    if (h.opt.precond == EQC_PC_AMG) {
        mg_apply64(h, r, z);
    } else {
        k_jacobi<double><<<vgrid(), VEC_THREADS, 0, h.stream>>>(r, h.diag64.p + h.L.ld, z, n);
        EQC_CHECK_LAUNCH();
        count_launch();
    }
}
template <>
void precond<float>(Handle& h, const float* r, float* z, int64_t n) {
    if (h.opt.precond == EQC_PC_AMG) {
        mg_apply32(h, r, z);
    } else {
        k_jacobi<float><<<vgrid(), VEC_THREADS, 0, h.stream>>>(r, h.diag32.p + h.L.ld, z, n);
        EQC_CHECK_LAUNCH();
        count_launch();
    }
}

// Right-hand side: S->bb = ||b||^2 with b = -K_IF F on rows 1..4 (d holds F on row 0).
static void setup_rhs(Handle& h, bool mixed) {
    const int64_t ld = h.L.ld;
    apply_K<double>(h.d.p, h.tmp64a.p, args64(h), -1.0, 2, h.stream);
    dot64(h, h.tmp64a.p + ld, h.tmp64a.p + ld, 4 * ld, &h.cg.p->bb);
    k_set_sigma<<<1, 1, 0, h.stream>>>(h.cg.p, mixed ? 1 : 0);
    EQC_CHECK_LAUNCH();
    count_launch();
}

// Full initial residual: r64 = b - K_II d_I (rows >= 1, row 0 zero), S->rr = ||r||^2, and in
// mixed precision r32 = (float) r64.
static void setup_residual_full(Handle& h, bool mixed) {
    const Layout& L = h.L;
    const int64_t ld = L.ld, n = L.size() - ld;
    CGState* S = h.cg.p;
    apply_K<double>(h.d.p, h.r64.p, args64(h), -1.0, 1, h.stream);     // r = -(K d)_I
    if (mixed) {
        k_demote_norm<<<vgrid(), VEC_THREADS, 0, h.stream>>>(h.r64.p + ld, h.r32.p + ld, n, h.red_part.p,
                                                             h.red_count.p, S, nullptr, h.dx64.p ? h.dx64.p + ld : nullptr);
        EQC_CHECK_LAUNCH();
        count_launch();
    } else {
        dot64(h, h.r64.p + ld, h.r64.p + ld, n, &S->rr);
    }
}

// Carried residual: r64 -= K_IF (F - Flast) on rows 1..4 (tmp64b row 0 holds F - Flast), then
// r32 = sigma r64 for this solve's sigma; with a guess increment g in d: r32 -= sigma K_II g
// (the first reliable update recomputes r64).
static void setup_residual_carry(Handle& h, const float* guess) {
    const int64_t ld = h.L.ld, n = h.L.size() - ld;
    apply_K<double>(h.tmp64b.p, h.tmp64c.p, args64(h), -1.0, 2, h.stream);
    k_carry_rows<<<vgrid(), VEC_THREADS, 0, h.stream>>>(h.r64.p + ld, h.tmp64c.p + ld, 4 * ld);
    k_demote_norm<<<vgrid(), VEC_THREADS, 0, h.stream>>>(h.r64.p + ld, h.r32.p + ld, n, h.red_part.p,
                                                         h.red_count.p, h.cg.p, nullptr, h.dx64.p ? h.dx64.p + ld : nullptr);
    EQC_CHECK_LAUNCH();
    count_launch(2);
    if (guess) {
        apply_K<float>(guess, h.q32.p, args32(h), 1.0f, 1, h.stream);
        k_guess_residual<<<vgrid(), VEC_THREADS, 0, h.stream>>>(h.r32.p + ld, h.q32.p + ld, n, h.red_part.p,
                                                                h.red_count.p, h.cg.p);
        k_guess_decide<<<1, 1, 0, h.stream>>>(h.cg.p, h.ctrl.p);
        k_guess_revert<<<vgrid(), VEC_THREADS, 0, h.stream>>>(h.cg.p, h.d.p + ld, guess + ld, h.r32.p + ld,
                                                              h.r64.p + ld, n);
        EQC_CHECK_LAUNCH();
        count_launch(3);
        if (h.dx64.p) {   // r64 is the residual without the kept increment
            k_dx_init<<<vgrid(), VEC_THREADS, 0, h.stream>>>(h.dx64.p + ld, guess + ld, h.cg.p, n);
            EQC_CHECK_LAUNCH();
            count_launch();
        }
    }
}

// One FP64 iteration, ending with the loop decision.
static void iter_fp64(Handle& h, cudaGraphConditionalHandle hw, int use_cond) {
    const Layout& L = h.L;
    const int64_t ld = L.ld, n = L.size() - ld;
    CGState* S = h.cg.p;
    double* x = h.d.p + ld;
    double* r = h.r64.p + ld;
    double* z = h.z64.p + ld;
    double* u = h.p64.p + ld;
    double* q = h.q64.p + ld;
    precond<double>(h, r, z, n);
    k_dot_rho<double><<<vgrid(), VEC_THREADS, 0, h.stream>>>(z, r, n, h.red_part.p, h.red_count.p, &S->rho);
    k_pupdate<double><<<vgrid(), VEC_THREADS, 0, h.stream>>>(z, u, n, &S->rho, &S->restart);
    apply_K<double>(h.p64.p, h.q64.p, args64(h), 1.0, 1, h.stream);
    dot64(h, u, q, n, &S->pq);
    CheckA ck;
    ck.on = 2;
    ck.use_cond = use_cond;
    ck.hw = hw;
    k_xr_update<double, double><<<vgrid(), VEC_THREADS, 0, h.stream>>>(x, r, u, q, n, h.red_part.p, h.red_count.p,
                                                                       &S->rho, ck);
    EQC_CHECK_LAUNCH();
    count_launch(3);
}

// Mixed precision: FP32 recurrences of one iteration, ending with the update decision (hi) and,
// for an iteration without an update, the loop's condition (hw).
static void iter_mixed_a(Handle& h, double delta, cudaGraphConditionalHandle hi, cudaGraphConditionalHandle hw,
                         int use_cond) {
    const Layout& L = h.L;
    const int64_t ld = L.ld, n = L.size() - ld;
    CGState* S = h.cg.p;
    float* r = h.r32.p + ld;
    float* z = h.z32.p + ld;
    float* u = h.p32.p + ld;
    float* q = h.q32.p + ld;
    float* y = h.x32.p + ld;   // correction accumulated since the last reliable update
    precond<float>(h, r, z, n);
    k_dot_rho<float><<<vgrid(), VEC_THREADS, 0, h.stream>>>(z, r, n, h.red_part.p, h.red_count.p, &S->rho);
    k_pupdate<float><<<vgrid(), VEC_THREADS, 0, h.stream>>>(z, u, n, &S->rho, &S->restart);
    apply_K<float>(h.p32.p, h.q32.p, args32(h), 1.0f, 1, h.stream);
    dot32(h, u, q, n, &S->pq);
    CheckA ck;
    ck.on = 1;
    ck.use_cond = use_cond;
    ck.delta = delta;
    ck.hi = hi;
    ck.hw = hw;
    k_xr_update<float, float><<<vgrid(), VEC_THREADS, 0, h.stream>>>(y, r, u, q, n, h.red_part.p, h.red_count.p,
                                                                     &S->rho, ck);
    EQC_CHECK_LAUNCH();
    count_launch(3);
}

// Reliable update: x += y ; r = b - K_II x in FP64 ; r32 = r ; S->rr = ||r||^2.
// An intermediate update (the recurrence residual fell by the update factor and the loop goes on)
// instead computes r -= K_II dx with the double-float apply of the correction dx folded since the
// previous update (69 against 139 us on dz480): K dx has the size of the residual it corrects, so
// the double-float error stays far below the residual left.  The update that certifies
// convergence recomputes b - K_II x with the FP64 apply: the full K x's double-float error would
// floor the residual near 1e-5 of |b| late in a cycle (|K||x| / |b| large; measured).  Both
// forms run as gated launches (ApplyArgs::gate on S->upd_incr).
static int incr_updates(const Handle& h, bool mixed) {
    return (mixed && h.df_ok && h.dx64.p && h.kdx64.p) ? 1 : 0;
}
static void update_mixed(Handle& h) {
    const Layout& L = h.L;
    const int64_t ld = L.ld, n = L.size() - ld;
    CGState* S = h.cg.p;
    const bool incr = incr_updates(h, true) != 0;
    k_fold<<<vgrid(), VEC_THREADS, 0, h.stream>>>(h.d.p + ld, h.x32.p + ld, incr ? h.dx64.p + ld : nullptr, n, S);
    ApplyArgs<double> a64 = args64(h);
    if (incr) {
        a64.gate = &S->upd_incr;
        a64.gate_val = 0;
        apply_K_df(h, h.dx64.p, h.kdx64.p, -1.0, 1, h.stream, &S->upd_incr, 1);   // -K_II dx
    }
    apply_K<double>(h.d.p, h.r64.p, a64, -1.0, 1, h.stream);                    // r = -(K d)_I
    k_demote_norm<<<vgrid(), VEC_THREADS, 0, h.stream>>>(h.r64.p + ld, h.r32.p + ld, n, h.red_part.p, h.red_count.p,
                                                         S, incr ? h.kdx64.p + ld : nullptr, incr ? h.dx64.p + ld : nullptr);
    EQC_CHECK_LAUNCH();
    count_launch(2);
}

constexpr double RELIABLE_DELTA = 1e-3;   // default residual-replacement factor

void enqueue_solve(Handle& h, double tol, int maxit, bool graph, bool carry, const float* guess) {
    if (maxit <= 0) maxit = (int)std::min<int64_t>(h.L.size() - h.L.ld, 1 << 30);
    const Layout& L = h.L;
    // the 4-wide vector kernels need whole 8-entry rows (the layout's row pitch)
    if (L.ld % 8) throw Error(EQC_E_STATE, "row pitch must be a multiple of 8");
    CGState* S = h.cg.p;
    const bool mixed = h.opt.precision == EQC_MIXED;
    carry = carry && mixed;
    const double delta = h.opt.reliable_delta > 0 ? h.opt.reliable_delta : RELIABLE_DELTA;
    setup_rhs(h, mixed);
    if (carry) {
        k_fault_delta<<<(h.F.Nf + 255) / 256, 256, 0, h.stream>>>(h.d.p, h.F.Flast.p, h.tmp64b.p, h.F.Nf);
        EQC_CHECK_LAUNCH();
        count_launch();
        if (graph) {
            const cudaGraphConditionalHandle hc = cond_handle(h), hf = cond_handle(h);
            k_setup_select<<<1, 1, 0, h.stream>>>(h.ctrl.p, hc, hf, 1);
            count_launch();
            const int64_t t0 = capture_tally();
            cond_begin(h, cudaGraphCondTypeIf, hc);
            setup_residual_carry(h, guess);
            cond_end(h);
            const int64_t t1 = capture_tally();
            cond_begin(h, cudaGraphCondTypeIf, hf);
            setup_residual_full(h, mixed);
            cond_end(h);
            if (h.capturing) {
                h.capturing->k_carry = t1 - t0;
                h.capturing->k_full = capture_tally() - t1;
                h.capturing->k_bodies += capture_tally() - t0;
            }
        } else {
            k_setup_select<<<1, 1, 0, h.stream>>>(h.ctrl.p, 0, 0, 0);
            count_launch();
            int valid = 0;
            EQC_CUDA(cudaMemcpyAsync(&valid, &h.ctrl.p->r_valid, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
            EQC_CUDA(cudaStreamSynchronize(h.stream));
            if (valid) setup_residual_carry(h, guess);
            else setup_residual_full(h, mixed);
        }
    } else {
        setup_residual_full(h, mixed);
    }
    if (mixed) {
        EQC_CUDA(cudaMemsetAsync(h.p32.p, 0, sizeof(float) * L.size(), h.stream));
        EQC_CUDA(cudaMemsetAsync(h.x32.p, 0, sizeof(float) * L.size(), h.stream));
    } else {
        EQC_CUDA(cudaMemsetAsync(h.p64.p, 0, sizeof(double) * L.size(), h.stream));
    }
    if (graph) {
        // k_cg_init (upstream of the while node) sets the node's first value
        const cudaGraphConditionalHandle hw = cond_handle(h);
        k_cg_init<<<1, 1, 0, h.stream>>>(S, tol, maxit, h.opt.tol_rule, incr_updates(h, mixed), hw, 1);
        count_launch();
        const int64_t t0 = capture_tally();
        cond_begin(h, cudaGraphCondTypeWhile, hw);
        if (mixed) {
            const cudaGraphConditionalHandle hi = cond_handle(h);
            iter_mixed_a(h, delta, hi, hw, 1);
            const int64_t t1 = capture_tally();
            cond_begin(h, cudaGraphCondTypeIf, hi);
            update_mixed(h);
            k_cg_check_b<<<1, 1, 0, h.stream>>>(S, h.ctrl.p, hw, 1);
            count_launch();
            cond_end(h);
            if (h.capturing) {
                h.capturing->k_update = capture_tally() - t1;
                h.capturing->k_iter = t1 - t0;
                h.capturing->k_bodies += capture_tally() - t0;
            }
        } else {
            iter_fp64(h, hw, 1);
            if (h.capturing) {
                h.capturing->k_iter = capture_tally() - t0;
                h.capturing->k_bodies += capture_tally() - t0;
            }
        }
        cond_end(h);
    } else {
        k_cg_init<<<1, 1, 0, h.stream>>>(S, tol, maxit, h.opt.tol_rule, incr_updates(h, mixed), 0, 0);
        count_launch();
        const CGState* hs = &read_cg(h);
        while (hs->done == 0) {
            if (mixed) {
                iter_mixed_a(h, delta, 0, 0, 0);
                hs = &read_cg(h);
                if (hs->need_update) {
                    update_mixed(h);
                    k_cg_check_b<<<1, 1, 0, h.stream>>>(S, h.ctrl.p, 0, 0);
                    count_launch();
                }
            } else {
                iter_fp64(h, 0, 0);
            }
            hs = &read_cg(h);
        }
    }
    k_cg_finish<<<1, 1, 0, h.stream>>>(S, h.ctrl.p, carry ? 1 : 0);
    EQC_CHECK_LAUNCH();
    count_launch();
}

void invalidate_residual(Handle& h) {
    EQC_CUDA(cudaMemsetAsync(&h.ctrl.p->r_valid, 0, sizeof(int), h.stream));
    EQC_CUDA(cudaMemsetAsync(&h.ctrl.p->qs_prev, 0, sizeof(int), h.stream));
    EQC_CUDA(cudaMemsetAsync(&h.ctrl.p->kd_valid, 0, sizeof(int), h.stream));
    if (h.h_ctrl) h.h_ctrl->r_valid = h.h_ctrl->qs_prev = h.h_ctrl->kd_valid = 0;
}

// Solves for d_I given d row 0 = F (eager); returns iterations (negative: maxit reached).
int qs_solve_device(Handle& h, double tol, int maxit, double* relres) {
    enqueue_solve(h, tol, maxit, false);
    const CGState& S = read_cg(h);
    check_apply_err(h);
    if (S.done == 3) throw Error(EQC_E_NAN, "non-finite residual in CG");
    if (relres) *relres = S.nb > 0 ? S.res / S.nb : S.res;
    return S.done == 1 ? S.it : -S.it;
}

// Reports (EQC_E_TIMEOUT) and clears the flag a TMA-fed apply sets when a bounded wait gave up,
// so that the handle stays usable after the error.
void check_apply_err(Handle& h) {
    int err = 0;
    EQC_CUDA(cudaMemcpyAsync(&err, &h.ctrl.p->apply_err, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    EQC_CUDA(cudaStreamSynchronize(h.stream));
    if (!err) return;
    EQC_CUDA(cudaMemsetAsync(&h.ctrl.p->apply_err, 0, sizeof(int), h.stream));
    EQC_CUDA(cudaStreamSynchronize(h.stream));
    h.h_ctrl->apply_err = 0;
    throw Error(EQC_E_TIMEOUT, "stiffness apply: bounded wait for a TMA tile gave up");
}

}  // namespace eqc
