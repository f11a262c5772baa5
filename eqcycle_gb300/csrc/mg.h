// Multigrid preconditioner for the quasi-static solve (replaces the AMG V-cycle of
// src/main.jl:200-201, aspreconditioner(ruge_stuben(kni))).
//
// Hierarchy, built once on the host because K is constant (src/main.jl:193-211):
//   level 0   the spectral-element grid (matrix-free K_II, kapply.cu)
//   level 1   the element-vertex grid: P_0 interpolates vertex values bilinearly to the
//             25 GLL nodes of every element (p-coarsening 4 -> 1), A_1 = P_0^T K_II P_0
//             assembled element by element
//   level k+1 the vertex grid coarsened by two in each direction, bilinear P_k,
//             A_{k+1} = P_k^T A_k P_k (Galerkin products; every A_k is a 9-point stencil)
//   coarsest  dense inverse (Cholesky on the host) applied as a matrix-vector product
// Smoothing: Chebyshev polynomial in D^-1 A (degree `deg`) on every level, symmetric pre and
// post, so the V-cycle is a symmetric preconditioner for CG.
#pragma once
#include "model.h"

namespace eqc {

// 1-D transfer between a fine index range [0, nf) and a coarse one [0, nc):
// prolongation rows (<= 2 coarse neighbours per fine index) and restriction rows
// (the transpose, as a CSR list per coarse index).
struct Transfer1D {
    int nf = 0, nc = 0;
    std::vector<int> p_idx;      // [2*nf]
    std::vector<double> p_w;     // [2*nf]
    std::vector<int> r_ptr;      // [nc+1]
    std::vector<int> r_idx;      // fine indices
    std::vector<double> r_w;
};

struct DevTransfer {
    int nfx, nfy, ncx, ncy;      // grid sizes (with the fault row)
    int ldf, ldc;                // row pitches
    int rmaxx, rmaxy;            // max restriction row lengths
    DBuf<int> px, py, rpx, rpy, rix, riy;
    DBuf<double> wx64, wy64, rwx64, rwy64;
    DBuf<float> wx32, wy32, rwx32, rwy32;
};

struct StencilLevel {
    int cx = 0, cy = 0;          // vertex grid size including the fault row (row 0 unused)
    std::vector<double> A;       // host [9][cx*cy], offsets (dx,dy) in {-1,0,1}^2, k = (dy+1)*3+(dx+1)
    DBuf<double> A64, Dinv64;
    DBuf<float> A32, Dinv32;
    double lmax = 0;
};

struct MGWork {                  // per-level vectors, full layout of the level
    DBuf<double> x64, b64, r64, d64, t64;
    DBuf<float> x32, b32, r32, d32, t32;
};


struct MGHier {
    int deg = 4;          // Chebyshev steps on the spectral-element level
    int deg_coarse = 3;   // ... on the vertex levels
    double lo_ratio = 30.0;
    double lmax0 = 0;
    double gll_lo[4] = {0, 0, 0, 0}, gll_hi[4] = {0, 0, 0, 0};   // SEM <-> vertex weights
    DBuf<double> Dinv0_64;
    DBuf<float> Dinv0_32;
    std::vector<StencilLevel> lev;    // levels 1..L
    std::vector<DevTransfer> T;       // T[0]: SEM -> lev[0]; T[k]: lev[k-1] -> lev[k]
    std::vector<MGWork> work;         // work[0]: SEM level; work[k]: lev[k-1]
    int nc = 0;                       // coarsest dense size
    DBuf<double> Cinv64;
    DBuf<float> Cinv32;
    int64_t launches_per_vcycle = 0;
};

// host setup helpers (mg_setup.cpp)
Transfer1D make_gll_transfer(int nel, const double* xgll);          // GLL lattice -> vertices
Transfer1D make_coarsen_transfer(int nf);                          // factor-2 coarsening
std::vector<double> vertex_operator(const Handle& h, const double* W);  // A_1 stencil
std::vector<double> galerkin_stencil(const std::vector<double>& A, int cx, int cy, const Transfer1D& tx,
                                     const Transfer1D& ty, int ncx, int ncy);
std::vector<double> dense_inverse_spd(const std::vector<double>& A9, int cx, int cy, int& n);

}  // namespace eqc
