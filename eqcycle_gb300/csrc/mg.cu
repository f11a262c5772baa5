// Multigrid V-cycle on the device (see mg.h for the hierarchy).
#include "mg.h"
#include "reduce.cuh"
#include "epi.cuh"
#include "mg_pt.cuh"
#include <cmath>
#include <random>
#include <utility>

namespace eqc {

// ------------------------------------------------------------------ device kernels
template <class T>
__global__ void k_stencil(const T* __restrict__ A, const T* __restrict__ x, T* __restrict__ y, int cx, int cy,
                          OpEpi<T> E) {
    EQC_GRID_WAIT();
    const int64_t N = (int64_t)cx * cy;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x)
        epi_store1(E, y, i, stencil_pt<T>(A, x, cx, cy, N, i, LdPlain()));
}

// xf[fine] += sum_{a,b} wx_a wy_b xc[coarse]   (fine rows >= 1); xc + pend where the coarse
// level's post-smoothing left its first step's direction pending (pend non-null)
template <class T>
__global__ void k_prolong_add(const T* __restrict__ xc, T* __restrict__ xf, int nfx, int nfy, int ldf, int ldc,
                              const int* __restrict__ px, const int* __restrict__ py, const T* __restrict__ wx,
                              const T* __restrict__ wy, const T* __restrict__ pend) {
    EQC_GRID_WAIT();
    const int64_t N = (int64_t)nfx * nfy;
    LdPend ld;
    ld.base = xc;
    ld.pend = pend;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const int ix = (int)(i % nfx), iy = (int)(i / nfx);
        if (iy == 0) continue;
        T* o = xf + (int64_t)iy * ldf + ix;
        *o = add_rn<T>(*o, prolong_pt<T>(xc, ldc, px, py, wx, wy, ix, iy, ld));
    }
}

// bc[coarse] = sum over restriction lists of rf[fine]  (coarse rows >= 1; row 0 = 0)
template <class T>
__global__ void k_restrict(const T* __restrict__ rf, T* __restrict__ bc, int ncx, int ncy, int ldf, int ldc,
                           const int* __restrict__ rpx, const int* __restrict__ rix, const T* __restrict__ rwx,
                           const int* __restrict__ rpy, const int* __restrict__ riy, const T* __restrict__ rwy,
                           ChebFirst<T> F) {
    EQC_GRID_WAIT();
    const int64_t N = (int64_t)ncx * ncy;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (int64_t)gridDim.x * blockDim.x) {
        const int cxi = (int)(i % ncx), cyi = (int)(i / ncx);
        const T s = restrict_pt<T>(rf, ldf, rpx, rix, rwx, rpy, riy, rwy, cxi, cyi, LdPlain());
        bc[(int64_t)cyi * ldc + cxi] = s;
        cheb_first_pt(F, (int64_t)cyi * ldc + cxi, s);
    }
}

// ---- transfers between the spectral-element grid and the element-vertex grid ----------
// The GLL node at local index k of an element interpolates the element's two vertices with
// weights lo[k] (lower vertex) and hi[k] (upper vertex), k = 0..3; the last node of the
// lattice is the last vertex.  Structured: no index tables, no integer division.
template <class T>
struct GllW {
    T lo[4], hi[4];
};

// xf[iy, 4ex + k] += P0 xc  for node rows iy >= 1; one thread per (element column, node row),
// the thread of the last element column also takes the lattice's last node.
template <class T>
__global__ void k_prolong_sem(const T* __restrict__ xc, T* __restrict__ xf, Layout L, int ldc, GllW<T> w,
                              const T* __restrict__ pend) {
    EQC_GRID_WAIT();
    const int ex = blockIdx.x * blockDim.x + threadIdx.x;
    const int iy = blockIdx.y + 1;
    if (ex >= L.NelX || iy >= L.ny) return;
    LdPend ld;
    ld.base = xc;
    ld.pend = pend;
    const int ey = min(iy >> 2, L.NelY - 1), ky = iy - 4 * ey;
    const T wyl = ky == 4 ? T(0) : w.lo[ky], wyh = ky == 4 ? T(1) : w.hi[ky];
    const T* c0 = xc + (int64_t)ey * ldc + ex;
    const T* c1 = c0 + ldc;
    const T a0 = wyl * ld(c0) + wyh * ld(c1);           // vertex column ex
    const T a1 = wyl * ld(c0 + 1) + wyh * ld(c1 + 1);   // vertex column ex + 1
    T* row = xf + (int64_t)iy * L.ld + 4 * ex;
#pragma unroll
    for (int k = 0; k < 4; ++k) row[k] += w.lo[k] * a0 + w.hi[k] * a1;
    if (ex == L.NelX - 1) row[4] += a1;
}

// bc[vy, vx] = (P0^T rf)[vy, vx] over fine rows iy >= 1; coarse row 0 = 0.  One thread per vertex.
template <class T>
__global__ void k_restrict_sem(const T* __restrict__ rf, T* __restrict__ bc, Layout L, int ldc, GllW<T> w,
                               ChebFirst<T> F) {
    EQC_GRID_WAIT();
    const int vx = blockIdx.x * blockDim.x + threadIdx.x;
    const int vy = blockIdx.y;
    const int ncx = L.NelX + 1;
    if (vx >= ncx) return;
    T acc = T(0);
    if (vy >= 1) {
        for (int dy = -3; dy <= 3; ++dy) {
            const int iy = 4 * vy + dy;
            if (iy < 1 || iy >= L.ny) continue;
            const T wy = dy == 0 ? T(1) : (dy > 0 ? (vy < L.NelY ? w.lo[dy] : T(0)) : w.hi[4 + dy]);
            const T* row = rf + (int64_t)iy * L.ld;
            T sx = T(0);
#pragma unroll
            for (int dx = -3; dx <= 3; ++dx) {
                const int ix = 4 * vx + dx;
                if (ix < 0 || ix >= L.nx) continue;
                const T wx = dx == 0 ? T(1) : (dx > 0 ? (vx < L.NelX ? w.lo[dx] : T(0)) : w.hi[4 + dx]);
                sx += wx * row[ix];
            }
            acc += wy * sx;
        }
    }
    bc[(int64_t)vy * ldc + vx] = acc;
    cheb_first_pt(F, (int64_t)vy * ldc + vx, acc);
}

// Chebyshev, first step.  with_x: r = Dinv (b - t) with t = A x ; else r = Dinv b, x = 0.
// d = r/theta ; x += d
template <class T>
__global__ void k_cheb_first(T* __restrict__ x, T* __restrict__ r, T* __restrict__ d, const T* __restrict__ b,
                             const T* __restrict__ t, const T* __restrict__ Dinv, int64_t n, T inv_theta, int with_x) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        cheb_first_step_pt<T>(x, r, d, b, t, Dinv, i, inv_theta, with_x != 0, LdPlain());
}
// Chebyshev, later step: r -= Dinv t (t = A d) ; d = c1 d + c2 r ; x += d
template <class T>
__global__ void k_cheb_step(T* __restrict__ x, T* __restrict__ r, T* __restrict__ d, const T* __restrict__ t,
                            const T* __restrict__ Dinv, int64_t n, T c1, T c2) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        T ri = r[i], di = d[i], xi = x[i];
        cheb_step_pt<T>(ri, di, xi, t[i], Dinv[i], c1, c2);
        r[i] = ri;
        d[i] = di;
        x[i] = xi;
    }
}
// x += d: a post-smoothing's pending first-step direction (OpEpi mode 3) with no later reader
// to add it
template <class T>
__global__ void k_add_pend(T* __restrict__ x, const T* __restrict__ d, int64_t n) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = add_rn<T>(x[i], d[i]);
}
// r = b - t
template <class T>
__global__ void k_sub(const T* __restrict__ b, const T* __restrict__ t, T* __restrict__ r, int64_t n) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        r[i] = b[i] - t[i];
}
// x[cx + k] = sum_j Cinv[k][j] b[cx + j]  (one warp per row).  Accumulates in T: FP32 for the
// FP32 cycle (a preconditioner; GB300's FP64 rate would make this the slowest kernel of it).
template <class T>
__global__ void k_dense_mv(const T* __restrict__ Cinv, const T* __restrict__ b, T* __restrict__ x, int n, int off) {
    EQC_GRID_WAIT();
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (warp >= n) return;
    const T s = dense_row<T>(Cinv, b, n, off, warp, lane, LdPlain());
    if (lane == 0) x[off + warp] = s;
}
template <class T>
__global__ void k_scale(T* x, int64_t n, double s) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = (T)((double)x[i] * s);
}
template <class T>
__global__ void k_mul(const T* a, T* x, int64_t n) {
    EQC_GRID_WAIT();
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] = a[i] * x[i];
}

static inline int vb(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 8 * 152); }

// ------------------------------------------------------------------ typed access
template <class T> struct Sel;
template <> struct Sel<double> {
    static double* x(MGWork& w) { return w.x64.p; }
    static double* b(MGWork& w) { return w.b64.p; }
    static double* r(MGWork& w) { return w.r64.p; }
    static double* d(MGWork& w) { return w.d64.p; }
    static double* t(MGWork& w) { return w.t64.p; }
    static const double* A(StencilLevel& l) { return l.A64.p; }
    static const double* Di(StencilLevel& l) { return l.Dinv64.p; }
    static const double* Di0(MGHier& m) { return m.Dinv0_64.p; }
    static const double* C(MGHier& m) { return m.Cinv64.p; }
    static const double* wx(DevTransfer& t) { return t.wx64.p; }
    static const double* wy(DevTransfer& t) { return t.wy64.p; }
    static const double* rwx(DevTransfer& t) { return t.rwx64.p; }
    static const double* rwy(DevTransfer& t) { return t.rwy64.p; }
    static ApplyArgs<double> args(Handle& h) { return args64(h); }
};
template <> struct Sel<float> {
    static float* x(MGWork& w) { return w.x32.p; }
    static float* b(MGWork& w) { return w.b32.p; }
    static float* r(MGWork& w) { return w.r32.p; }
    static float* d(MGWork& w) { return w.d32.p; }
    static float* t(MGWork& w) { return w.t32.p; }
    static const float* A(StencilLevel& l) { return l.A32.p; }
    static const float* Di(StencilLevel& l) { return l.Dinv32.p; }
    static const float* Di0(MGHier& m) { return m.Dinv0_32.p; }
    static const float* C(MGHier& m) { return m.Cinv32.p; }
    static const float* wx(DevTransfer& t) { return t.wx32.p; }
    static const float* wy(DevTransfer& t) { return t.wy32.p; }
    static const float* rwx(DevTransfer& t) { return t.rwx32.p; }
    static const float* rwy(DevTransfer& t) { return t.rwy32.p; }
    static ApplyArgs<float> args(Handle& h) { return args32(h); }
};

template <class T>
static GllW<T> gll_weights(const MGHier& m) {
    GllW<T> g;
    for (int k = 0; k < 4; ++k) {
        g.lo[k] = (T)m.gll_lo[k];
        g.hi[k] = (T)m.gll_hi[k];
    }
    return g;
}

// y = A_l x on level l (0 = spectral-element grid)
template <class T>
static void level_apply(Handle& h, int l, const T* x, T* y) {
    MGHier& m = *h.mg;
    if (l == 0) {
        apply_K<T>(x, y, Sel<T>::args(h), T(1), 1, h.stream);
    } else {
        StencilLevel& L = m.lev[l - 1];
        k_stencil<T><<<vb((int64_t)L.cx * L.cy), 256, 0, h.stream>>>(Sel<T>::A(L), x, y, L.cx, L.cy, OpEpi<T>());
        EQC_CHECK_LAUNCH();
        count_launch();
    }
}

// The operator of level l applied to x with the epilogue E (the level's residual or Chebyshev
// step) in the same launch; false when level 0's selected apply kernel has no epilogue.
static bool epi_apply(Handle& h, int l, const float* x, const OpEpi<float>& E) {
    if (!h.fuse) return false;
    if (l == 0) return apply_K_epi(x, args32(h), 1, E, h.stream);
    StencilLevel& L = h.mg->lev[l - 1];
    k_stencil<float><<<vb((int64_t)L.cx * L.cy), 256, 0, h.stream>>>(L.A32.p, x, nullptr, L.cx, L.cy, E);
    EQC_CHECK_LAUNCH();
    count_launch();
    return true;
}
static bool epi_apply(Handle& h, int l, const double* x, const OpEpi<double>& E) {
    if (l == 0 || !h.fuse) return false;   // the FP64 spectral-element apply has no epilogue
    StencilLevel& L = h.mg->lev[l - 1];
    k_stencil<double><<<vb((int64_t)L.cx * L.cy), 256, 0, h.stream>>>(L.A64.p, x, nullptr, L.cx, L.cy, E);
    EQC_CHECK_LAUNCH();
    count_launch();
    return true;
}

static int64_t level_size(Handle& h, int l) {
    return l == 0 ? h.L.size() : (int64_t)h.mg->lev[l - 1].cx * h.mg->lev[l - 1].cy;
}

// The Chebyshev smoother's coefficients on level l (0: the spectral-element level): 1/theta of
// the first step and (c1[k], c2[k]) of steps k = 1..deg-1.
static void cheb_coeffs(const MGHier& m, int l, int deg, double* inv_theta, double* c1, double* c2) {
    const double lmax = (l == 0) ? m.lmax0 : m.lev[l - 1].lmax;
    const double lmin = lmax / m.lo_ratio;
    const double theta = 0.5 * (lmax + lmin), delta = 0.5 * (lmax - lmin);
    const double sigma = theta / delta;
    double rho = 1.0 / sigma;
    *inv_theta = 1.0 / theta;
    for (int k = 1; k < deg; ++k) {
        const double rho_new = 1.0 / (2.0 * sigma - rho);
        c1[k] = rho_new * rho;
        c2[k] = 2.0 * rho_new / delta;
        rho = rho_new;
    }
}

// Chebyshev smoothing of A_l x = b (deg steps), x = 0 initially when !with_x.  first_done: the
// first step (from x = 0) already ran inside the restriction that produced b.  Steps run fused
// into the operator (r, x updated in place, the direction alternating between the d and t work
// vectors) when the level's operator kernel has the epilogue; the first step from x then leaves
// x += d pending (OpEpi mode 3) for the second step, or, with one step, returns d for the
// caller's next reader of x to add (null: x is complete).
template <class T>
static const T* chebyshev(Handle& h, int l, T* x, const T* b, bool with_x, bool first_done = false) {
    MGHier& m = *h.mg;
    MGWork& w = m.work[l];
    const int64_t n = level_size(h, l);
    const T* Dinv = (l == 0) ? Sel<T>::Di0(m) : Sel<T>::Di(m.lev[l - 1]);
    const int deg = (l == 0) ? m.deg : m.deg_coarse;
    std::vector<double> cc1(std::max(deg, 1)), cc2(std::max(deg, 1));
    double inv_theta = 0.0;
    cheb_coeffs(m, l, deg, &inv_theta, cc1.data(), cc2.data());
    T* r = Sel<T>::r(w);
    T* d = Sel<T>::d(w);
    T* t = Sel<T>::t(w);
    bool pend = false;
    if (!first_done) {
        OpEpi<T> E;
        E.mode = 3;
        E.b = b;
        E.r = r;
        E.dinv = Dinv;
        E.dnew = d;
        E.inv_theta = (T)inv_theta;
        if (with_x && epi_apply(h, l, x, E)) {
            pend = true;
        } else {
            if (with_x) level_apply<T>(h, l, x, t);
            k_cheb_first<T><<<vb(n), 256, 0, h.stream>>>(x, r, d, b, t, Dinv, n, (T)inv_theta, with_x ? 1 : 0);
            count_launch();
        }
    }
    T* dcur = d;
    T* dnext = t;
    for (int k = 1; k < deg; ++k) {
        const T c1 = (T)cc1[k], c2 = (T)cc2[k];
        OpEpi<T> E;
        E.mode = 2;
        E.r = r;
        E.dinv = Dinv;
        E.dold = dcur;
        E.dnew = dnext;
        E.x = x;
        E.c1 = c1;
        E.c2 = c2;
        E.x_pend = pend;
        if (epi_apply(h, l, dcur, E)) {
            std::swap(dcur, dnext);
        } else {
            if (pend) {
                k_add_pend<T><<<vb(n), 256, 0, h.stream>>>(x, dcur, n);
                count_launch();
            }
            level_apply<T>(h, l, dcur, t);
            k_cheb_step<T><<<vb(n), 256, 0, h.stream>>>(x, r, dcur, t, Dinv, n, c1, c2);
            count_launch();
        }
        pend = false;
    }
    EQC_CHECK_LAUNCH();
    return pend ? dcur : nullptr;
}

// 1 / theta of level l's Chebyshev interval (as chebyshev() computes it)
static double cheb_inv_theta(const MGHier& m, int l) {
    double it = 0.0;
    cheb_coeffs(m, l, 1, &it, nullptr, nullptr);
    return it;
}

// first_done: the restriction that produced b already took level l's first smoothing step.
// Returns the post-smoothing's pending direction (chebyshev), null when x is complete.
template <class T>
static const T* vcycle(Handle& h, int l, T* x, const T* b, bool first_done = false) {
    MGHier& m = *h.mg;
    const int L = (int)m.lev.size();
    if (l == L) {  // coarsest: dense solve on rows >= 1
        StencilLevel& c = m.lev[L - 1];
        const int64_t n = (int64_t)c.cx * c.cy;
        EQC_CUDA(cudaMemsetAsync(x, 0, sizeof(T) * c.cx, h.stream));
        k_dense_mv<T><<<(m.nc * 32 + 255) / 256, 256, 0, h.stream>>>(Sel<T>::C(m), b, x, m.nc, c.cx);
        EQC_CHECK_LAUNCH();
        count_launch();
        (void)n;
        return nullptr;
    }
    MGWork& w = m.work[l];
    const int64_t n = level_size(h, l);
    chebyshev<T>(h, l, x, b, false, first_done);   // from x = 0: nothing pending
    // residual r = b - A x, fused into the operator where it has the epilogue
    T* t = Sel<T>::t(w);
    T* r = Sel<T>::r(w);
    OpEpi<T> E;
    E.mode = 1;
    E.b = b;
    E.r = r;
    if (!epi_apply(h, l, x, E)) {
        level_apply<T>(h, l, x, t);
        k_sub<T><<<vb(n), 256, 0, h.stream>>>(b, t, r, n);
        count_launch();
    }
    DevTransfer& tr = m.T[l];
    MGWork& wc = m.work[l + 1];
    T* bc = Sel<T>::b(wc);
    T* xc = Sel<T>::x(wc);
    const GllW<T> gw = gll_weights<T>(m);
    // the coarse level's first smoothing step rides on the restriction (not into the dense level)
    ChebFirst<T> F;
    const bool fuse = h.fuse && l + 1 < L;
    if (fuse) {
        F.dinv = Sel<T>::Di(m.lev[l]);
        F.x = xc;
        F.r = Sel<T>::r(wc);
        F.d = Sel<T>::d(wc);
        F.inv_theta = (T)cheb_inv_theta(m, l + 1);
    }
    if (l == 0) {
        k_restrict_sem<T><<<dim3((tr.ncx + 127) / 128, tr.ncy), 128, 0, h.stream>>>(r, bc, h.L, tr.ldc, gw, F);
    } else {
        k_restrict<T><<<vb((int64_t)tr.ncx * tr.ncy), 256, 0, h.stream>>>(r, bc, tr.ncx, tr.ncy, tr.ldf, tr.ldc,
                                                                           tr.rpx.p, tr.rix.p, Sel<T>::rwx(tr), tr.rpy.p,
                                                                           tr.riy.p, Sel<T>::rwy(tr), F);
    }
    count_launch();
    const T* pc = vcycle<T>(h, l + 1, xc, bc, fuse);
    if (l == 0) {
        k_prolong_sem<T><<<dim3((h.L.NelX + 127) / 128, h.L.ny - 1), 128, 0, h.stream>>>(xc, x, h.L, tr.ldc, gw, pc);
    } else {
        k_prolong_add<T><<<vb((int64_t)tr.nfx * tr.nfy), 256, 0, h.stream>>>(xc, x, tr.nfx, tr.nfy, tr.ldf, tr.ldc,
                                                                             tr.px.p, tr.py.p, Sel<T>::wx(tr),
                                                                             Sel<T>::wy(tr), pc);
    }
    count_launch();
    EQC_CHECK_LAUNCH();
    return chebyshev<T>(h, l, x, b, true);
}

// The whole V-cycle on level 0 with any pending direction added to x.
template <class T>
static void vcycle0(Handle& h, T* x, const T* b) {
    const T* p = vcycle<T>(h, 0, x, b);
    if (p) {
        const int64_t n = level_size(h, 0);
        k_add_pend<T><<<vb(n), 256, 0, h.stream>>>(x, p, n);
        EQC_CHECK_LAUNCH();
        count_launch();
    }
}

// z = M^{-1} r for the CG: r, z are the interior slices (rows >= 1) of level-0 vectors.
void mg_apply64(Handle& h, const double* r, double* z) {
    if (!h.mg) throw Error(EQC_E_STATE, "multigrid not built");
    const int64_t ld = h.L.ld;
    vcycle0<double>(h, z - ld, r - ld);
}
void mg_apply32(Handle& h, const float* r, float* z) {
    if (!h.mg) throw Error(EQC_E_STATE, "multigrid not built");
    const int64_t ld = h.L.ld;
    vcycle0<float>(h, z - ld, r - ld);
}

// ------------------------------------------------------------------ setup
static void upload_transfer(Handle& h, DevTransfer& d, const Transfer1D& tx, const Transfer1D& ty, int ldf, int ldc) {
    cudaStream_t s = h.stream;
    d.nfx = tx.nf;
    d.nfy = ty.nf;
    d.ncx = tx.nc;
    d.ncy = ty.nc;
    d.ldf = ldf;
    d.ldc = ldc;
    auto up_i = [&](DBuf<int>& b, const std::vector<int>& v) { b.alloc(v.size()); b.upload(v.data(), v.size(), s); };
    auto up_w = [&](DBuf<double>& b64, DBuf<float>& b32, const std::vector<double>& v) {
        b64.alloc(v.size());
        b64.upload(v.data(), v.size(), s);
        std::vector<float> f(v.begin(), v.end());
        b32.alloc(f.size());
        b32.upload(f.data(), f.size(), s);
    };
    up_i(d.px, tx.p_idx);
    up_i(d.py, ty.p_idx);
    up_w(d.wx64, d.wx32, tx.p_w);
    up_w(d.wy64, d.wy32, ty.p_w);
    up_i(d.rpx, tx.r_ptr);
    up_i(d.rix, tx.r_idx);
    up_w(d.rwx64, d.rwx32, tx.r_w);
    up_i(d.rpy, ty.r_ptr);
    up_i(d.riy, ty.r_idx);
    up_w(d.rwy64, d.rwy32, ty.r_w);
    EQC_CUDA(cudaStreamSynchronize(s));
}

static void alloc_work(MGWork& w, int64_t n) {
    for (DBuf<double>* b : {&w.x64, &w.b64, &w.r64, &w.d64, &w.t64}) b->alloc(n);
    for (DBuf<float>* b : {&w.x32, &w.b32, &w.r32, &w.d32, &w.t32}) b->alloc(n);
}

// Largest eigenvalue of D^-1 A_l by power iteration (FP64, 30 steps), times 1.1.
static double estimate_lmax(Handle& h, int l) {
    MGHier& m = *h.mg;
    MGWork& w = m.work[l];
    const int64_t n = level_size(h, l);
    const double* Dinv = (l == 0) ? m.Dinv0_64.p : m.lev[l - 1].Dinv64.p;
    std::vector<double> x0(n);
    std::mt19937_64 rng(1234 + l);
    std::uniform_real_distribution<double> U(0.5, 1.5);
    const int nx = (l == 0) ? h.L.ld : m.lev[l - 1].cx;
    const int nreal = (l == 0) ? h.L.nx : nx;
    for (int64_t i = 0; i < n; ++i) x0[i] = (i < nx || (i % nx) >= nreal) ? 0.0 : U(rng);
    w.x64.upload(x0.data(), n, h.stream);
    double lam = 0.0;
    for (int it = 0; it < 30; ++it) {
        level_apply<double>(h, l, w.x64.p, w.t64.p);
        k_mul<double><<<vb(n), 256, 0, h.stream>>>(Dinv, w.t64.p, n);
        dot64(h, w.t64.p, w.t64.p, n, h.scal.p + 14);
        dot64(h, w.x64.p, w.t64.p, n, h.scal.p + 13);
        dot64(h, w.x64.p, w.x64.p, n, h.scal.p + 12);
        double sc[3];
        EQC_CUDA(cudaMemcpyAsync(sc, h.scal.p + 12, sizeof(double) * 3, cudaMemcpyDeviceToHost, h.stream));
        EQC_CUDA(cudaStreamSynchronize(h.stream));
        lam = std::sqrt(sc[2] / sc[0]);
        EQC_CUDA(cudaMemcpyAsync(w.x64.p, w.t64.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, h.stream));
        k_scale<double><<<vb(n), 256, 0, h.stream>>>(w.x64.p, n, 1.0 / std::sqrt(sc[2]));
        count_launch(2);
    }
    EQC_CHECK_LAUNCH();
    return 1.1 * lam;
}

void mg_build(Handle& h) {
    mg_destroy(h);
    h.mg = new MGHier();
    MGHier& m = *h.mg;
    const Layout& L = h.L;
    cudaStream_t s = h.stream;
    static const double xg[5] = {-1.0, -0.65465367070797714, 0.0, 0.65465367070797714, 1.0};
    // level 0 Jacobi scaling
    {
        std::vector<double> dg(L.size());
        h.diag64.download(dg.data(), dg.size(), s);
        EQC_CUDA(cudaStreamSynchronize(s));
        std::vector<double> di(L.size(), 0.0);
        for (int64_t i = L.ld; i < L.size(); ++i) di[i] = ((i % L.ld) < L.nx) ? 1.0 / dg[i] : 0.0;
        std::vector<float> df(di.begin(), di.end());
        m.Dinv0_64.alloc(L.size());
        m.Dinv0_64.upload(di.data(), di.size(), s);
        m.Dinv0_32.alloc(L.size());
        m.Dinv0_32.upload(df.data(), df.size(), s);
    }
    // level 1: vertex grid
    std::vector<double> Wh((size_t)25 * h.Nel);
    h.W64.download(Wh.data(), Wh.size(), s);
    EQC_CUDA(cudaStreamSynchronize(s));
    std::vector<Transfer1D> tx, ty;
    tx.push_back(make_gll_transfer(L.NelX, xg));
    ty.push_back(make_gll_transfer(L.NelY, xg));
    for (int k = 0; k < 4; ++k) {   // weights of local node k (identical in every element)
        m.gll_lo[k] = tx[0].p_w[2 * k];
        m.gll_hi[k] = tx[0].p_w[2 * k + 1];
    }
    StencilLevel l1;
    l1.cx = L.NelX + 1;
    l1.cy = L.NelY + 1;
    l1.A = vertex_operator(h, Wh.data());
    m.lev.push_back(std::move(l1));
    // coarser vertex grids
    const int64_t coarse_max = h.opt.mg_coarse_max > 0 ? h.opt.mg_coarse_max : 2048;
    if (h.opt.mg_degree > 0) m.deg = h.opt.mg_degree;
    m.deg_coarse = h.opt.mg_degree_coarse > 0 ? h.opt.mg_degree_coarse : 3;
    while ((int64_t)m.lev.back().cx * (m.lev.back().cy - 1) > coarse_max && m.lev.back().cx >= 5 &&
           m.lev.back().cy >= 5) {
        StencilLevel& f = m.lev.back();
        Transfer1D ax = make_coarsen_transfer(f.cx), ay = make_coarsen_transfer(f.cy);
        StencilLevel c;
        c.cx = ax.nc;
        c.cy = ay.nc;
        c.A = galerkin_stencil(f.A, f.cx, f.cy, ax, ay, c.cx, c.cy);
        tx.push_back(std::move(ax));
        ty.push_back(std::move(ay));
        m.lev.push_back(std::move(c));
    }
    // upload stencils and diagonal scalings
    for (StencilLevel& lv : m.lev) {
        const size_t N = (size_t)lv.cx * lv.cy;
        std::vector<float> a32(lv.A.begin(), lv.A.end());
        lv.A64.alloc(9 * N);
        lv.A64.upload(lv.A.data(), 9 * N, s);
        lv.A32.alloc(9 * N);
        lv.A32.upload(a32.data(), 9 * N, s);
        std::vector<double> di(N, 0.0);
        for (size_t i = lv.cx; i < N; ++i) di[i] = 1.0 / lv.A[4 * N + i];
        std::vector<float> df(di.begin(), di.end());
        lv.Dinv64.alloc(N);
        lv.Dinv64.upload(di.data(), N, s);
        lv.Dinv32.alloc(N);
        lv.Dinv32.upload(df.data(), N, s);
        EQC_CUDA(cudaStreamSynchronize(s));
    }
    // transfers: T[0] SEM -> vertex grid, T[k] lev[k-1] -> lev[k]
    m.T.resize(m.lev.size());
    upload_transfer(h, m.T[0], tx[0], ty[0], L.ld, m.lev[0].cx);
    for (size_t k = 1; k < m.lev.size(); ++k)
        upload_transfer(h, m.T[k], tx[k], ty[k], m.lev[k - 1].cx, m.lev[k].cx);
    // coarsest dense inverse
    {
        StencilLevel& c = m.lev.back();
        std::vector<double> inv = dense_inverse_spd(c.A, c.cx, c.cy, m.nc);
        std::vector<float> f(inv.begin(), inv.end());
        m.Cinv64.alloc(inv.size());
        m.Cinv64.upload(inv.data(), inv.size(), s);
        m.Cinv32.alloc(f.size());
        m.Cinv32.upload(f.data(), f.size(), s);
    }
    // work vectors
    m.work.resize(m.lev.size() + 1);
    alloc_work(m.work[0], L.size());
    for (size_t k = 0; k < m.lev.size(); ++k) alloc_work(m.work[k + 1], (int64_t)m.lev[k].cx * m.lev[k].cy);
    EQC_CUDA(cudaStreamSynchronize(s));
    // spectral bounds for Chebyshev (all levels but the coarsest, which is solved directly)
    m.lmax0 = estimate_lmax(h, 0);
    for (size_t k = 0; k + 1 < m.lev.size(); ++k) m.lev[k].lmax = estimate_lmax(h, (int)k + 1);
    EQC_CUDA(cudaStreamSynchronize(s));
    // the V-cycle recursion below the coarsest smoothed level uses lev[L-1] as the dense level
}

void mg_destroy(Handle& h) {
    delete h.mg;
    h.mg = nullptr;
}

}  // namespace eqc
