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
#include <cmath>

namespace eqc {

enum { S_RHO = 0, S_RHOP = 1, S_PQ = 2, S_RR = 3, S_BB = 4, S_R0 = 5, S_NSLOT = 16 };

// dot into S_RHO, shifting the previous value into S_RHOP
template <class T>
__global__ void __launch_bounds__(RED_THREADS) k_dot_rho(const T* __restrict__ x, const T* __restrict__ y, int64_t n,
                                                         double* part, unsigned* count, double* S) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        s += (double)x[i] * (double)y[i];
    s = block_sum(s, sh);
    finish_reduction(s, part, count, sh, [&](double t) {
        S[S_RHOP] = S[S_RHO];
        S[S_RHO] = t;
    });
}

// u = z + (rho / rho_prev) u
template <class T>
__global__ void k_pupdate(const T* __restrict__ z, T* __restrict__ u, int64_t n, const double* S) {
    const double beta = S[S_RHO] / S[S_RHOP];
    const T b = (T)beta;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        u[i] = z[i] + b * u[i];
}

// x += alpha u ; r -= alpha q ; S_RR = r.r   (alpha = rho / (u.q))
template <class TX, class T>
__global__ void __launch_bounds__(RED_THREADS) k_xr_update(TX* __restrict__ x, T* __restrict__ r, const T* __restrict__ u,
                                                           const T* __restrict__ q, int64_t n, double* part,
                                                           unsigned* count, double* S) {
    __shared__ double sh[32];
    const double alpha = S[S_RHO] / S[S_PQ];
    const T a = (T)alpha;
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] = x[i] + (TX)alpha * (TX)u[i];
        const T ri = r[i] - a * q[i];
        r[i] = ri;
        s += (double)ri * (double)ri;
    }
    s = block_sum(s, sh);
    finish_reduction(s, part, count, sh, [&](double t) { S[S_RR] = t; });
}

template <class T>
__global__ void k_jacobi(const T* __restrict__ r, const T* __restrict__ dg, T* __restrict__ z, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        z[i] = r[i] / dg[i];
}

__global__ void k_set_scalar(double* S, int slot, double v) { S[slot] = v; }

// x64 += (double) y32 ; y32 = 0
__global__ void k_fold(double* __restrict__ x, float* __restrict__ y, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        x[i] += (double)y[i];
        y[i] = 0.f;
    }
}
// r32 = (float) r64 ; S_RR = r64.r64
__global__ void __launch_bounds__(RED_THREADS) k_demote_norm(const double* __restrict__ r64, float* __restrict__ r32,
                                                             int64_t n, double* part, unsigned* count, double* S) {
    __shared__ double sh[32];
    double s = 0.0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double v = r64[i];
        r32[i] = (float)v;
        s += v * v;
    }
    s = block_sum(s, sh);
    finish_reduction(s, part, count, sh, [&](double t) { S[S_RR] = t; });
}

static inline dim3 vgrid() { return dim3(RED_BLOCKS); }

static void read_scalars(Handle& h) {
    EQC_CUDA(cudaMemcpyAsync(h.h_scal, h.scal.p, sizeof(double) * S_NSLOT, cudaMemcpyDeviceToHost, h.stream));
    EQC_CUDA(cudaStreamSynchronize(h.stream));
}

template <class T>
static void precond(Handle& h, const T* r, T* z, int64_t n);

template <>
void precond<double>(Handle& h, const double* r, double* z, int64_t n) {
    if (h.opt.precond == EQC_PC_AMG) {
        mg_apply64(h, r, z);
    } else {
        k_jacobi<double><<<vgrid(), RED_THREADS, 0, h.stream>>>(r, h.diag64.p + h.L.ld, z, n);
        EQC_CHECK_LAUNCH();
        count_launch();
    }
}
template <>
void precond<float>(Handle& h, const float* r, float* z, int64_t n) {
    if (h.opt.precond == EQC_PC_AMG) {
        mg_apply32(h, r, z);
    } else {
        k_jacobi<float><<<vgrid(), RED_THREADS, 0, h.stream>>>(r, h.diag32.p + h.L.ld, z, n);
        EQC_CHECK_LAUNCH();
        count_launch();
    }
}

// Right-hand-side norm and initial residual; d holds F on row 0 and the guess elsewhere.
// Returns ||b|| (host) and leaves r64 = b - K_II d_I (rows >= 1, row 0 zero).
static double setup_residual(Handle& h) {
    const Layout& L = h.L;
    const int64_t ld = L.ld;
    apply_K<double>(h.d.p, h.r64.p, args64(h), -1.0, 1, h.stream);     // r = -(K d)_I
    apply_K<double>(h.d.p, h.tmp64a.p, args64(h), -1.0, 2, h.stream);  // b on rows 1..4
    dot64(h, h.tmp64a.p + ld, h.tmp64a.p + ld, 4 * ld, h.scal.p + S_BB);
    dot64(h, h.r64.p + ld, h.r64.p + ld, L.size() - ld, h.scal.p + S_RR);
    read_scalars(h);
    return std::sqrt(h.h_scal[S_BB]);
}

static int pcg_fp64(Handle& h, double tol, int maxit, double* relres) {
    const Layout& L = h.L;
    const int64_t ld = L.ld, n = L.size() - ld;
    const double nb = setup_residual(h);
    const double reltol = (h.opt.tol_rule == EQC_TOL_R0 ? std::sqrt(h.h_scal[S_RR]) : nb) * tol;
    double res = std::sqrt(h.h_scal[S_RR]);
    double* x = h.d.p + ld;
    double* r = h.r64.p + ld;
    double* z = h.z64.p + ld;
    double* u = h.p64.p + ld;
    double* q = h.q64.p + ld;
    EQC_CUDA(cudaMemsetAsync(h.p64.p, 0, sizeof(double) * L.size(), h.stream));
    k_set_scalar<<<1, 1, 0, h.stream>>>(h.scal.p, S_RHO, 1.0);
    count_launch();
    int it = 0;
    while (!(it >= maxit || res <= reltol)) {
        precond<double>(h, r, z, n);
        k_dot_rho<double><<<vgrid(), RED_THREADS, 0, h.stream>>>(z, r, n, h.red_part.p, h.red_count.p, h.scal.p);
        k_pupdate<double><<<vgrid(), RED_THREADS, 0, h.stream>>>(z, u, n, h.scal.p);
        apply_K<double>(h.p64.p, h.q64.p, args64(h), 1.0, 1, h.stream);
        dot64(h, u, q, n, h.scal.p + S_PQ);
        k_xr_update<double, double><<<vgrid(), RED_THREADS, 0, h.stream>>>(x, r, u, q, n, h.red_part.p,
                                                                           h.red_count.p, h.scal.p);
        EQC_CHECK_LAUNCH();
        count_launch(3);
        read_scalars(h);
        res = std::sqrt(h.h_scal[S_RR]);
        ++it;
        if (!std::isfinite(res)) throw Error(EQC_E_NAN, "non-finite residual in CG");
    }
    if (relres) *relres = nb > 0 ? res / nb : res;
    return res <= reltol ? it : -it;
}

// CG with reliable updates: FP32 recurrences, FP64 iterate and true residual.
static int pcg_mixed(Handle& h, double tol, int maxit, double* relres) {
    const Layout& L = h.L;
    const int64_t ld = L.ld, n = L.size() - ld;
    const double delta = 0.1;
    const double nb = setup_residual(h);
    const double reltol = (h.opt.tol_rule == EQC_TOL_R0 ? std::sqrt(h.h_scal[S_RR]) : nb) * tol;
    double res = std::sqrt(h.h_scal[S_RR]);
    double* x = h.d.p + ld;
    float* r = h.r32.p + ld;
    float* z = h.z32.p + ld;
    float* u = h.p32.p + ld;
    float* q = h.q32.p + ld;
    float* y = h.x32.p + ld;   // correction accumulated since the last reliable update
    EQC_CUDA(cudaMemsetAsync(h.p32.p, 0, sizeof(float) * L.size(), h.stream));
    EQC_CUDA(cudaMemsetAsync(h.x32.p, 0, sizeof(float) * L.size(), h.stream));
    k_demote_norm<<<vgrid(), RED_THREADS, 0, h.stream>>>(h.r64.p + ld, r, n, h.red_part.p, h.red_count.p, h.scal.p);
    k_set_scalar<<<1, 1, 0, h.stream>>>(h.scal.p, S_RHO, 1.0);
    count_launch(2);
    double rmax = res;  // largest recurrence residual since the last update
    int it = 0;
    while (!(it >= maxit || res <= reltol)) {
        precond<float>(h, r, z, n);
        k_dot_rho<float><<<vgrid(), RED_THREADS, 0, h.stream>>>(z, r, n, h.red_part.p, h.red_count.p, h.scal.p);
        k_pupdate<float><<<vgrid(), RED_THREADS, 0, h.stream>>>(z, u, n, h.scal.p);
        apply_K<float>(h.p32.p, h.q32.p, args32(h), 1.0f, 1, h.stream);
        dot32(h, u, q, n, h.scal.p + S_PQ);
        k_xr_update<float, float><<<vgrid(), RED_THREADS, 0, h.stream>>>(y, r, u, q, n, h.red_part.p,
                                                                         h.red_count.p, h.scal.p);
        EQC_CHECK_LAUNCH();
        count_launch(3);
        read_scalars(h);
        double rs = std::sqrt(h.h_scal[S_RR]);
        ++it;
        if (!std::isfinite(rs)) throw Error(EQC_E_NAN, "non-finite residual in CG");
        rmax = std::max(rmax, rs);
        if (rs < delta * rmax || rs <= reltol || it >= maxit) {
            // reliable update: x += y ; r = b - K_II x in FP64
            k_fold<<<vgrid(), RED_THREADS, 0, h.stream>>>(x, y, n);
            apply_K<double>(h.d.p, h.r64.p, args64(h), -1.0, 1, h.stream);
            k_demote_norm<<<vgrid(), RED_THREADS, 0, h.stream>>>(h.r64.p + ld, r, n, h.red_part.p, h.red_count.p,
                                                                 h.scal.p);
            count_launch(2);
            read_scalars(h);
            rs = std::sqrt(h.h_scal[S_RR]);
            rmax = rs;
        }
        res = rs;
    }
    if (relres) *relres = nb > 0 ? res / nb : res;
    return res <= reltol ? it : -it;
}

// Solves for d_I given d row 0 = F; returns iterations (negative: maxit reached).
int qs_solve_device(Handle& h, double tol, int maxit, double* relres) {
    if (maxit <= 0) maxit = (int)std::min<int64_t>(h.L.size() - h.L.ld, 1 << 30);
    int it = (h.opt.precision == EQC_MIXED) ? pcg_mixed(h, tol, maxit, relres) : pcg_fp64(h, tol, maxit, relres);
    int err = 0;
    EQC_CUDA(cudaMemcpyAsync(&err, &h.ctrl.p->apply_err, sizeof(int), cudaMemcpyDeviceToHost, h.stream));
    EQC_CUDA(cudaStreamSynchronize(h.stream));
    if (err) throw Error(EQC_E_TIMEOUT, "stiffness apply: bounded wait for a TMA tile gave up");
    h.cg_iters_total += it < 0 ? -it : it;
    h.qs_solves_total += 1;
    return it;
}

}  // namespace eqc
