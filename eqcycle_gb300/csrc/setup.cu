// Model setup on the device for structured box meshes (par.jl:99-152 with MeshBox.jl,
// Assemble.jl and Kassemble.jl's diagonal): the element weights W, the lumped mass M with the
// absorbing-boundary terms, 1/M and the diagonal of K, computed straight into the node layout
// instead of on the host.  The arithmetic is the host setup's operation by operation (this file
// is compiled without FMA contraction), and every node sums its <= 4 element contributions in
// element order, as the host's element-by-element accumulation does, so both give the same bits.
#include "model.h"

namespace eqc {

struct SetupArgs {
    Layout L;
    eqc_material mat;
    double dxe, dye, jac, c1, c2, half_dt;
    double xg[5], wg[5], H[25];
};

// Material (rho, mu) at local node (i, j) of element (ex, ey): Assemble.jl:34-35's rectangle
// rule per element, or the trapezoid per GLL node from the node's coordinates (MeshBox: the
// last element that writes a node defines its coordinate).
__device__ __forceinline__ void material(const SetupArgs& a, int ex, int ey, int i, int j, double& rho, double& mu) {
    const eqc_material& m = a.mat;
    bool dmg = false;
    if (m.rule == 1) {
        dmg = ((double)(ex + 1) * a.dxe >= m.ThickX) && (a.dye <= (double)(ey + 1) * a.dye) &&
              ((double)(ey + 1) * a.dye <= m.ThickY);
    } else if (m.rule == 2) {
        const int ix = 4 * ex + i, iy = 4 * ey + j;
        const int exw = min(ix / 4, a.L.NelX - 1), eyw = min(iy / 4, a.L.NelY - 1);
        const int iw = ix - 4 * exw, jw = iy - 4 * eyw;
        const double xcol = a.dxe * (double)exw + a.dxe * (0.5 * (1.0 + a.xg[iw]));
        const double y = a.dye * (double)eyw + a.dye * (0.5 * (1.0 + a.xg[jw]));
        const double x = xcol - m.LX;
        const double z = -x;
        const double wdt = m.trap_w0 + (m.trap_w1 - m.trap_w0) * (z / m.trap_z1);
        dmg = (z <= m.trap_z1) && (y <= wdt);
    }
    const double r = dmg ? m.rho2 : m.rho1, vs = dmg ? m.vs2 : m.vs1;
    rho = r;
    mu = r * (vs * vs);
}

// One thread per element: W (FP64, FP32 and the copies padded for TMA element tiles).
__global__ void k_setup_W(SetupArgs a, double* __restrict__ W64, float* __restrict__ W32, double* __restrict__ W64p,
                          float* __restrict__ W32p, float* __restrict__ W32lo) {
    EQC_GRID_WAIT();
    const int64_t Nel = (int64_t)a.L.NelX * a.L.NelY;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < Nel; e += (int64_t)gridDim.x * blockDim.x) {
        const int ex = (int)(e % a.L.NelX), ey = (int)(e / a.L.NelX);
        for (int j = 0; j < 5; ++j)
            for (int i = 0; i < 5; ++i) {
                double rho, mu;
                material(a, ex, ey, i, j, rho, mu);
                const double w = (a.wg[i] * a.wg[j]) * mu;
                W64[25 * e + i + 5 * j] = w;
                W32[25 * e + i + 5 * j] = (float)w;
                W64p[(int64_t)WPad<double>::v * e + i + 5 * j] = w;
                W32p[(int64_t)WPad<float>::v * e + i + 5 * j] = (float)w;
                W32lo[(int64_t)WPad<float>::v * e + i + 5 * j] = (float)(w - (double)(float)w);
            }
        for (int q = 25; q < WPad<double>::v; ++q) W64p[(int64_t)WPad<double>::v * e + q] = 0.0;
        for (int q = 25; q < WPad<float>::v; ++q) {
            W32p[(int64_t)WPad<float>::v * e + q] = 0.f;
            W32lo[(int64_t)WPad<float>::v * e + q] = 0.f;
        }
    }
}

// One thread per layout node: lumped mass (Assemble.jl:165, element order), 1/M and the
// diagonal of K (Kassemble.jl:50-58 with i = k, j = l).  Row padding: M = 1, diag = 1; the fault
// row's diagonal is 1 (not part of the quasi-static system).
__global__ void k_setup_nodes(SetupArgs a, double* __restrict__ M, double* __restrict__ dg64, float* __restrict__ dg32) {
    EQC_GRID_WAIT();
    const Layout L = a.L;
    const int64_t N = L.size();
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x) {
        const int iy = (int)(n / L.ld), ix = (int)(n % L.ld);
        if (ix >= L.nx) {
            M[n] = 1.0;
            dg64[n] = 1.0;
            dg32[n] = 1.f;
            continue;
        }
        // elements holding the node, in element order: (x left/right) x (y below/above)
        const int exs[2] = {(ix % 4 == 0 && ix > 0) ? ix / 4 - 1 : -1, ix / 4 < L.NelX ? ix / 4 : -1};
        const int eys[2] = {(iy % 4 == 0 && iy > 0) ? iy / 4 - 1 : -1, iy / 4 < L.NelY ? iy / 4 : -1};
        double m = 0.0, d = 0.0;
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 2; ++c) {
                const int ex = exs[c], ey = eys[b];
                if (ex < 0 || ey < 0) continue;
                const int i = ix - 4 * ex, j = iy - 4 * ey;
                double rho, mu;
                material(a, ex, ey, i, j, rho, mu);
                m += ((a.wg[i] * a.wg[j]) * rho) * a.jac;
                double t1 = 0.0, t2 = 0.0;
                for (int p = 0; p < 5; ++p) {
                    double rp, mp, rq, mq;
                    material(a, ex, ey, i, p, rp, mp);   // W(i, p)
                    material(a, ex, ey, p, j, rq, mq);   // W(p, j)
                    const double wip = (a.wg[i] * a.wg[p]) * mp, wpj = (a.wg[p] * a.wg[j]) * mq;
                    t1 += wip * a.c2 * a.H[j + 5 * p] * a.H[j + 5 * p];
                    t2 += wpj * a.c1 * a.H[i + 5 * p] * a.H[i + 5 * p];
                }
                d += t1 + t2;
            }
        M[n] = m;
        if (iy == 0) d = 1.0;
        dg64[n] = d;
        dg32[n] = (float)d;
    }
}

// M[iB] += half_dt * Bc (par.jl:173-174), the left boundary first, then the top one.
__global__ void k_setup_boundary(double* __restrict__ M, const int64_t* __restrict__ iB, const double* __restrict__ Bc,
                                 int n, double half_dt) {
    EQC_GRID_WAIT();
    for (int k = threadIdx.x; k < n; k += blockDim.x) M[iB[k]] = M[iB[k]] + half_dt * Bc[k];
}

__global__ void k_setup_inv(const double* __restrict__ M, double* __restrict__ invM, int64_t N) {
    EQC_GRID_WAIT();
    for (int64_t n = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; n < N; n += (int64_t)gridDim.x * blockDim.x)
        invM[n] = 1.0 / M[n];
}

static SetupArgs setup_args(const Handle& h, const eqc_material& mat, const double* xg, const double* wg) {
    SetupArgs a;
    a.L = h.L;
    a.mat = mat;
    a.dxe = h.dxe;
    a.dye = h.dye;
    const double dx_dxi = 0.5 * h.dxe, dy_deta = 0.5 * h.dye;
    a.jac = dx_dxi * dy_deta;
    a.c1 = h.c1;
    a.c2 = h.c2;
    a.half_dt = 0.5 * h.dt0;
    for (int k = 0; k < 5; ++k) {
        a.xg[k] = xg[k];
        a.wg[k] = wg[k];
    }
    for (int k = 0; k < 25; ++k) a.H[k] = h.H[k];
    return a;
}

void setup_element_data_device(Handle& h, const eqc_material& mat) {
    const SetupArgs a = setup_args(h, mat, mat.xgll, mat.wgll);
    const int64_t Nel = (int64_t)h.L.NelX * h.L.NelY;
    h.W64.alloc((size_t)25 * Nel);
    h.W32.alloc((size_t)25 * Nel);
    h.W64p.alloc((size_t)WPad<double>::v * Nel);
    h.W32p.alloc((size_t)WPad<float>::v * Nel);
    h.W32lo.alloc((size_t)WPad<float>::v * Nel);
    h.diag64.alloc(h.L.size());
    h.diag32.alloc(h.L.size());
    const int blocks = (int)std::min<int64_t>((Nel + 255) / 256, 4096);
    k_setup_W<<<blocks, 256, 0, h.stream>>>(a, h.W64.p, h.W32.p, h.W64p.p, h.W32p.p, h.W32lo.p);
    EQC_CHECK_LAUNCH();
    count_launch();
}

void setup_node_data_device(Handle& h, const eqc_material& mat, const std::vector<int64_t>& lBcL, const double* BcLC,
                            const std::vector<int64_t>& lBcT, const double* BcTC) {
    const SetupArgs a = setup_args(h, mat, mat.xgll, mat.wgll);
    const int64_t N = h.L.size();
    cudaStream_t s = h.stream;
    const int blocks = (int)std::min<int64_t>((N + 255) / 256, 8192);
    k_setup_nodes<<<blocks, 256, 0, s>>>(a, h.M.p, h.diag64.p, h.diag32.p);
    EQC_CHECK_LAUNCH();
    count_launch();
    DBuf<int64_t> ib;
    DBuf<double> bc;
    for (int side = 0; side < 2; ++side) {
        const std::vector<int64_t>& idx = side == 0 ? lBcL : lBcT;
        const double* B = side == 0 ? BcLC : BcTC;
        if (idx.empty()) continue;
        ib.alloc(idx.size());
        bc.alloc(idx.size());
        ib.upload(idx.data(), idx.size(), s);
        bc.upload(B, idx.size(), s);
        k_setup_boundary<<<1, 256, 0, s>>>(h.M.p, ib.p, bc.p, (int)idx.size(), a.half_dt);
        EQC_CHECK_LAUNCH();
        count_launch();
        EQC_CUDA(cudaStreamSynchronize(s));
    }
    h.invM.alloc(N);
    k_setup_inv<<<blocks, 256, 0, s>>>(h.M.p, h.invM.p, N);
    EQC_CHECK_LAUNCH();
    count_launch();
    EQC_CUDA(cudaStreamSynchronize(s));
}

}  // namespace eqc
