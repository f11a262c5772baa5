// Host construction of the multigrid hierarchy (see mg.h): transfer tables, the vertex
// operator A_1 = P_0^T K_II P_0 (element by element), Galerkin stencils of the coarser
// vertex grids and the dense inverse of the coarsest operator.
#include "mg.h"
#include <cmath>
#include <algorithm>
#include "host_par.h"

namespace eqc {

static void finish_restriction(Transfer1D& t) {
    t.r_ptr.assign(t.nc + 1, 0);
    for (int i = 0; i < t.nf; ++i)
        for (int a = 0; a < 2; ++a)
            if (t.p_w[2 * i + a] != 0.0) t.r_ptr[t.p_idx[2 * i + a] + 1]++;
    for (int c = 0; c < t.nc; ++c) t.r_ptr[c + 1] += t.r_ptr[c];
    t.r_idx.assign(t.r_ptr[t.nc], 0);
    t.r_w.assign(t.r_ptr[t.nc], 0.0);
    std::vector<int> pos(t.r_ptr.begin(), t.r_ptr.end() - 1);
    for (int i = 0; i < t.nf; ++i)
        for (int a = 0; a < 2; ++a)
            if (t.p_w[2 * i + a] != 0.0) {
                const int c = t.p_idx[2 * i + a];
                t.r_idx[pos[c]] = i;
                t.r_w[pos[c]] = t.p_w[2 * i + a];
                pos[c]++;
            }
}

// GLL lattice of nel elements (4*nel+1 points) -> the nel+1 element vertices:
// linear interpolation in the element's reference coordinate t = (1+xi)/2.
Transfer1D make_gll_transfer(int nel, const double* xgll) {
    Transfer1D t;
    t.nf = 4 * nel + 1;
    t.nc = nel + 1;
    t.p_idx.assign(2 * t.nf, 0);
    t.p_w.assign(2 * t.nf, 0.0);
    for (int i = 0; i < t.nf; ++i) {
        const int e = std::min(i / 4, nel - 1);
        const int k = i - 4 * e;
        const double s = 0.5 * (1.0 + xgll[k]);
        t.p_idx[2 * i] = e;
        t.p_idx[2 * i + 1] = e + 1;
        t.p_w[2 * i] = (k == 0) ? 1.0 : (k == 4 ? 0.0 : 1.0 - s);
        t.p_w[2 * i + 1] = (k == 0) ? 0.0 : (k == 4 ? 1.0 : s);
    }
    finish_restriction(t);
    return t;
}

// Factor-2 coarsening of nf points: coarse points at fine indices 0, 2, 4, ... and the last
// fine index; fine points between two coarse points interpolate linearly by index.
Transfer1D make_coarsen_transfer(int nf) {
    std::vector<int> cpos;
    for (int i = 0; i < nf; i += 2) cpos.push_back(i);
    if (cpos.back() != nf - 1) cpos.push_back(nf - 1);
    Transfer1D t;
    t.nf = nf;
    t.nc = (int)cpos.size();
    t.p_idx.assign(2 * nf, 0);
    t.p_w.assign(2 * nf, 0.0);
    int c = 0;
    for (int i = 0; i < nf; ++i) {
        while (c + 1 < t.nc && cpos[c + 1] <= i) ++c;
        if (cpos[c] == i) {
            t.p_idx[2 * i] = c;
            t.p_w[2 * i] = 1.0;
            t.p_idx[2 * i + 1] = c;
            t.p_w[2 * i + 1] = 0.0;
        } else {
            const double s = double(i - cpos[c]) / double(cpos[c + 1] - cpos[c]);
            t.p_idx[2 * i] = c;
            t.p_w[2 * i] = 1.0 - s;
            t.p_idx[2 * i + 1] = c + 1;
            t.p_w[2 * i + 1] = s;
        }
    }
    finish_restriction(t);
    return t;
}

// A_1 = P_0^T K_II P_0 on the (NelX+1) x (NelY+1) vertex grid, element by element: the
// element operator (src/PCG.jl:82 form) applied to the four bilinear vertex functions.
std::vector<double> vertex_operator(const Handle& h, const double* W) {
    const Layout& L = h.L;
    const int cx = L.NelX + 1, cy = L.NelY + 1;
    std::vector<double> A((size_t)9 * cx * cy, 0.0);
    const double* H = h.H;  // H[i + 5j] = h'_i(x_j)
    double xg[5];
    {   // GLL nodes are the zeros of the derivative matrix's row structure; recover them
        // from H: x_j for a 5-point rule is -1, -sqrt(3/7), 0, sqrt(3/7), 1.
        xg[0] = -1.0; xg[1] = -std::sqrt(3.0 / 7.0); xg[2] = 0.0; xg[3] = std::sqrt(3.0 / 7.0); xg[4] = 1.0;
    }
    double Lb[2][5];
    for (int i = 0; i < 5; ++i) {
        const double s = 0.5 * (1.0 + xg[i]);
        Lb[0][i] = (i == 0) ? 1.0 : (i == 4 ? 0.0 : 1.0 - s);
        Lb[1][i] = (i == 0) ? 0.0 : (i == 4 ? 1.0 : s);
    }
    // the 16 vertex-pair entries of every element (in parallel), then their sum in element order
    const int64_t Nel = (int64_t)L.NelX * L.NelY;
    std::vector<double> E((size_t)16 * Nel);
    parallel_for(Nel, [&](int64_t e) {
            const double* w = W + e * 25;
            double y[4][25];
            for (int v = 0; v < 4; ++v) {
                const int av = v & 1, bv = v >> 1;
                double u[5][5], t1[5][5], t2[5][5];
                for (int j = 0; j < 5; ++j)
                    for (int i = 0; i < 5; ++i) u[i][j] = Lb[av][i] * Lb[bv][j];
                for (int j = 0; j < 5; ++j)
                    for (int p = 0; p < 5; ++p) {
                        double s1 = 0, s2 = 0;
                        for (int k = 0; k < 5; ++k) {
                            s1 += H[k + 5 * p] * u[k][j];
                            s2 += u[p][k] * H[k + 5 * j];
                        }
                        t1[p][j] = w[p + 5 * j] * s1;
                        t2[p][j] = w[p + 5 * j] * s2;
                    }
                for (int j = 0; j < 5; ++j)
                    for (int i = 0; i < 5; ++i) {
                        double s1 = 0, s2 = 0;
                        for (int p = 0; p < 5; ++p) {
                            s1 += H[i + 5 * p] * t1[p][j];
                            s2 += t2[i][p] * H[j + 5 * p];
                        }
                        y[v][i + 5 * j] = h.c1 * s1 + h.c2 * s2;
                    }
            }
            for (int u = 0; u < 4; ++u) {
                const int au = u & 1, bu = u >> 1;
                for (int v = 0; v < 4; ++v) {
                    double s = 0;
                    for (int j = 0; j < 5; ++j)
                        for (int i = 0; i < 5; ++i) s += Lb[au][i] * Lb[bu][j] * y[v][i + 5 * j];
                    E[(size_t)16 * e + 4 * u + v] = s;
                }
            }
        });
    for (int ey = 0; ey < L.NelY; ++ey)
        for (int ex = 0; ex < L.NelX; ++ex) {
            const int64_t e = (int64_t)ey * L.NelX + ex;
            for (int u = 0; u < 4; ++u) {
                const int au = u & 1, bu = u >> 1;
                const int vx = ex + au, vy = ey + bu;
                for (int v = 0; v < 4; ++v) {
                    const int av = v & 1, bv = v >> 1;
                    const int k = (bv - bu + 1) * 3 + (av - au + 1);
                    A[(size_t)k * cx * cy + (size_t)vy * cx + vx] += E[(size_t)16 * e + 4 * u + v];
                }
            }
        }
    // fault row is Dirichlet: no equations on row 0, no couplings into row 0
    for (int k = 0; k < 9; ++k)
        for (int vx = 0; vx < cx; ++vx) A[(size_t)k * cx * cy + vx] = 0.0;
    for (int vx = 0; vx < cx; ++vx)
        for (int dx = -1; dx <= 1; ++dx) A[(size_t)((0) * 3 + (dx + 1)) * cx * cy + (size_t)1 * cx + vx] = 0.0;
    return A;
}

// Galerkin product P^T A P for a 9-point stencil A on (cx, cy) and P = Py (x) Px.  Coarse rows
// are independent (in parallel); each sums its contributions in fine-point order.
std::vector<double> galerkin_stencil(const std::vector<double>& A, int cx, int cy, const Transfer1D& tx,
                                     const Transfer1D& ty, int ncx, int ncy) {
    std::vector<double> Ac((size_t)9 * ncx * ncy, 0.0);
    const size_t N = (size_t)cx * cy, Nc = (size_t)ncx * ncy;
    // fine rows whose interpolation reaches coarse row Jy, ascending
    std::vector<std::vector<int>> rows(ncy);
    for (int fy = 1; fy < cy; ++fy)
        for (int q = 0; q < 2; ++q) {
            const int Jy = ty.p_idx[2 * fy + q];
            if (ty.p_w[2 * fy + q] != 0.0 && Jy > 0 && (rows[Jy].empty() || rows[Jy].back() != fy))
                rows[Jy].push_back(fy);
        }
    std::vector<char> bad(ncy, 0);
    parallel_for(ncy, [&](int64_t jy) {
        const int Jrow = (int)jy;
        for (int fy : rows[Jrow])
            for (int fx = 0; fx < cx; ++fx) {
                const size_t f = (size_t)fy * cx + fx;
                for (int k = 0; k < 9; ++k) {
                    const double a = A[k * N + f];
                    if (a == 0.0) continue;
                    const int gx = fx + (k % 3) - 1, gy = fy + (k / 3) - 1;
                    if (gx < 0 || gx >= cx || gy < 1 || gy >= cy) continue;
                    for (int p = 0; p < 2; ++p)
                        for (int q = 0; q < 2; ++q) {
                            const double wJ = tx.p_w[2 * fx + p] * ty.p_w[2 * fy + q];
                            if (wJ == 0.0) continue;
                            const int Jx = tx.p_idx[2 * fx + p], Jy = ty.p_idx[2 * fy + q];
                            if (Jy != Jrow) continue;
                            for (int r = 0; r < 2; ++r)
                                for (int s = 0; s < 2; ++s) {
                                    const double wK = tx.p_w[2 * gx + r] * ty.p_w[2 * gy + s];
                                    if (wK == 0.0) continue;
                                    const int Kx = tx.p_idx[2 * gx + r], Ky = ty.p_idx[2 * gy + s];
                                    if (Ky == 0) continue;
                                    const int dx = Kx - Jx, dy = Ky - Jy;
                                    if (dx < -1 || dx > 1 || dy < -1 || dy > 1) {
                                        bad[Jrow] = 1;
                                        continue;
                                    }
                                    Ac[(size_t)((dy + 1) * 3 + dx + 1) * Nc + (size_t)Jy * ncx + Jx] += wJ * a * wK;
                                }
                        }
                }
            }
    });
    for (char b : bad)
        if (b) throw Error(EQC_E_ARG, "Galerkin operator left the 9-point stencil");
    return Ac;
}

// Dense inverse of the SPD operator on rows >= 1 of a small grid (Cholesky).  With rows
// numbered lexicographically the 9-point stencil couples rows at most bw = cx + 1 apart and the
// Cholesky factor L keeps that bandwidth, so M and L are held as bands (row i, columns
// i - bw .. i + bw of M and i - bw .. i of L); only the inverse is dense.
std::vector<double> dense_inverse_spd(const std::vector<double>& A9, int cx, int cy, int& n) {
    n = cx * (cy - 1);
    const size_t N = (size_t)cx * cy;
    const int bw = std::min(n - 1, cx + 1);
    const int mw = 2 * bw + 1, lw = bw + 1;
    std::vector<double> Mb((size_t)n * mw, 0.0);   // M(r, c) at Mb[r * mw + c - r + bw]
    for (int iy = 1; iy < cy; ++iy)
        for (int ix = 0; ix < cx; ++ix) {
            const int r = (iy - 1) * cx + ix;
            for (int k = 0; k < 9; ++k) {
                const int gx = ix + (k % 3) - 1, gy = iy + (k / 3) - 1;
                if (gx < 0 || gx >= cx || gy < 1 || gy >= cy) continue;
                const int c = (gy - 1) * cx + gx;
                Mb[(size_t)r * mw + c - r + bw] += A9[k * N + (size_t)iy * cx + ix];
            }
        }
    auto Mat = [&](int r, int c) -> double& { return Mb[(size_t)r * mw + c - r + bw]; };
    // symmetrise round-off (entries outside the band are zero on both sides)
    for (int i = 0; i < n; ++i)
        for (int j = std::max(0, i - bw); j < i; ++j) {
            const double s = 0.5 * (Mat(i, j) + Mat(j, i));
            Mat(i, j) = Mat(j, i) = s;
        }
    // banded Cholesky M = L L^T
    std::vector<double> Lb((size_t)n * lw, 0.0);    // L(i, k) at Lb[i * lw + k - i + bw]
    auto Lf = [&](int i, int k) -> double& { return Lb[(size_t)i * lw + k - i + bw]; };
    for (int j = 0; j < n; ++j) {
        double d = Mat(j, j);
        for (int k = std::max(0, j - bw); k < j; ++k) d -= Lf(j, k) * Lf(j, k);
        if (!(d > 0)) throw Error(EQC_E_ARG, "coarsest multigrid operator is not positive definite");
        d = std::sqrt(d);
        Lf(j, j) = d;
        for (int i = j + 1; i <= std::min(n - 1, j + bw); ++i) {
            double s = Mat(i, j);
            for (int k = std::max(0, i - bw); k < j; ++k) s -= Lf(i, k) * Lf(j, k);
            Lf(i, j) = s / d;
        }
    }
    // L^T by rows (row i holds L(k, i) for k = i .. i + bw), for the back substitution
    std::vector<double> LTb((size_t)n * lw, 0.0);
    for (int i = 0; i < n; ++i)
        for (int k = i; k <= std::min(n - 1, i + bw); ++k) LTb[(size_t)i * lw + k - i] = Lf(k, i);
    // column c of the inverse (into row c of T; columns are independent, in parallel), then
    // T transposed into the row-major inverse
    std::vector<double> T((size_t)n * n, 0.0);
    parallel_for(n, [&](int64_t c64) {
        const int c = (int)c64;
        double* col = T.data() + (size_t)c * n;
        col[c] = 1.0;
        for (int i = c; i < n; ++i) {  // L y = e_c (y = 0 above row c)
            const double* Li = Lb.data() + (size_t)i * lw - i + bw;
            double s = col[i];
            for (int k = std::max(c, i - bw); k < i; ++k) s -= Li[k] * col[k];
            col[i] = s / Li[i];
        }
        for (int i = n - 1; i >= 0; --i) {  // L^T x = y
            const double* Ui = LTb.data() + (size_t)i * lw - i;
            double s = col[i];
            for (int k = i + 1; k <= std::min(n - 1, i + bw); ++k) s -= Ui[k] * col[k];
            col[i] = s / Ui[i];
        }
    });
    std::vector<double> Inv((size_t)n * n);
    constexpr int TB = 64;
    parallel_for((n + TB - 1) / TB, [&](int64_t bi) {
        const int i0 = (int)bi * TB, i1 = std::min(n, i0 + TB);
        for (int c0 = 0; c0 < n; c0 += TB)
            for (int i = i0; i < i1; ++i)
                for (int c = c0; c < std::min(n, c0 + TB); ++c) Inv[(size_t)i * n + c] = T[(size_t)c * n + i];
    }, 1);
    return Inv;
}

}  // namespace eqc
