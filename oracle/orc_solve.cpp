// CPU oracle -- linear algebra restatement (test infrastructure; see orc_api.h).
//
//   y = K x, assembled            SparseArrays SpMV used at src/main.jl:246,267,311
//   y = K x, element form         src/PCG.jl:71-86 (element_computation!), src/dump.jl:54-64
//   AMG hierarchy                 src/main.jl:195-201: ruge_stuben(kni), aspreconditioner(ml)
//                                 (AlgebraicMultigrid.jl, unpinned version: Classical(0.25)
//                                 strength, RS C/F splitting, direct interpolation, symmetric
//                                 Gauss-Seidel pre/post smoothing, max_levels 10,
//                                 max_coarse 10, dense pseudo-inverse coarse solve)
//   CG                            src/main.jl:256 cg!(dnew, kni, rhs, Pl=p, tol=...)
//                                 (IterativeSolvers.jl 0.8, unpinned: stop when
//                                 ||r_k||_2 <= tol * ||b||_2, r_k the unpreconditioned residual)
#include "orc_internal.h"
#include <cmath>
#include <algorithm>
#include <cstring>
#include <omp.h>

namespace orc {

void CSR::spmv(const double* x, double* y) const {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int64_t k = ptr[i]; k < ptr[i + 1]; ++k) s += val[k] * x[col[k]];
        y[i] = s;
    }
}

CSR transpose(const CSR& A) {
    CSR T;
    T.n = A.m;
    T.m = A.n;
    T.ptr.assign(T.n + 1, 0);
    for (int64_t k = 0; k < A.nnz(); ++k) T.ptr[A.col[k] + 1]++;
    for (int64_t i = 0; i < T.n; ++i) T.ptr[i + 1] += T.ptr[i];
    T.col.resize(A.nnz());
    T.val.resize(A.nnz());
    std::vector<int64_t> pos(T.ptr.begin(), T.ptr.end() - 1);
    for (int64_t i = 0; i < A.n; ++i)
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            int64_t p = pos[A.col[k]]++;
            T.col[p] = i;
            T.val[p] = A.val[k];
        }
    return T;
}

// Gustavson row-by-row product, columns sorted within each row.
CSR matmul(const CSR& A, const CSR& B) {
    CSR C;
    C.n = A.n;
    C.m = B.m;
    C.ptr.assign(C.n + 1, 0);
    const int nt = omp_get_max_threads();
    std::vector<std::vector<int64_t>> rcol(C.n);
    std::vector<vec> rval(C.n);
#pragma omp parallel num_threads(nt)
    {
        std::vector<int64_t> mark(B.m, -1);
        vec acc(B.m, 0.0);
        std::vector<int64_t> cols;
#pragma omp for schedule(dynamic, 256)
        for (int64_t i = 0; i < A.n; ++i) {
            cols.clear();
            for (int64_t ka = A.ptr[i]; ka < A.ptr[i + 1]; ++ka) {
                const int64_t j = A.col[ka];
                const double av = A.val[ka];
                for (int64_t kb = B.ptr[j]; kb < B.ptr[j + 1]; ++kb) {
                    const int64_t c = B.col[kb];
                    if (mark[c] != i) {
                        mark[c] = i;
                        acc[c] = 0.0;
                        cols.push_back(c);
                    }
                    acc[c] += av * B.val[kb];
                }
            }
            std::sort(cols.begin(), cols.end());
            rcol[i] = cols;
            rval[i].resize(cols.size());
            for (size_t q = 0; q < cols.size(); ++q) rval[i][q] = acc[cols[q]];
        }
    }
    for (int64_t i = 0; i < C.n; ++i) C.ptr[i + 1] = C.ptr[i] + (int64_t)rcol[i].size();
    C.col.resize(C.ptr[C.n]);
    C.val.resize(C.ptr[C.n]);
    for (int64_t i = 0; i < C.n; ++i) {
        std::copy(rcol[i].begin(), rcol[i].end(), C.col.begin() + C.ptr[i]);
        std::copy(rval[i].begin(), rval[i].end(), C.val.begin() + C.ptr[i]);
    }
    return C;
}

// ---------------------------------------------------------------------------------------
// Ruge-Stueben pieces.
// Strength (Classical, theta): off-diagonal a_ij of row i is strong when
// |a_ij| >= theta * max_{k != i} |a_ik|.  The returned S keeps A's values on the strong
// pattern (what direct interpolation consumes) and has no diagonal.
static CSR strength_classical(const CSR& A, double theta) {
    CSR S;
    S.n = A.n;
    S.m = A.m;
    S.ptr.assign(S.n + 1, 0);
    std::vector<std::vector<int64_t>> rc(A.n);
    std::vector<vec> rv(A.n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < A.n; ++i) {
        double mx = 0.0;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k)
            if (A.col[k] != i) mx = std::max(mx, std::fabs(A.val[k]));
        const double thr = theta * mx;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            if (A.col[k] == i) continue;
            if (std::fabs(A.val[k]) >= thr && A.val[k] != 0.0) {
                rc[i].push_back(A.col[k]);
                rv[i].push_back(A.val[k]);
            }
        }
    }
    for (int64_t i = 0; i < S.n; ++i) S.ptr[i + 1] = S.ptr[i] + (int64_t)rc[i].size();
    S.col.resize(S.ptr[S.n]);
    S.val.resize(S.ptr[S.n]);
    for (int64_t i = 0; i < S.n; ++i) {
        std::copy(rc[i].begin(), rc[i].end(), S.col.begin() + S.ptr[i]);
        std::copy(rv[i].begin(), rv[i].end(), S.val.begin() + S.ptr[i]);
    }
    return S;
}

enum { F_NODE = 0, C_NODE = 1, U_NODE = 2 };

// First-pass Ruge-Stueben C/F splitting with the bucketed lambda measure: repeatedly take
// the undecided node with the largest lambda (number of undecided/F nodes that depend on
// it), make it C, make its dependants F, and update lambdas.  S[i] lists the nodes i
// depends on strongly; T = S^T lists the nodes that depend on i.
static std::vector<int> rs_cf_splitting(const CSR& S) {
    const int64_t n = S.n;
    CSR T = transpose(S);
    std::vector<int64_t> lambda(n), iptr(n + 1, 0), icount(n + 1, 0), i2n(n), n2i(n);
    for (int64_t i = 0; i < n; ++i) {
        lambda[i] = T.ptr[i + 1] - T.ptr[i];
        icount[lambda[i]]++;
    }
    for (int64_t k = 0; k < n; ++k) iptr[k + 1] = iptr[k] + icount[k];
    std::fill(icount.begin(), icount.end(), 0);
    for (int64_t i = 0; i < n; ++i) {
        const int64_t li = lambda[i];
        const int64_t idx = iptr[li] + icount[li];
        icount[li]++;
        i2n[idx] = i;
        n2i[i] = idx;
    }
    std::vector<int> split(n, U_NODE);
    for (int64_t i = 0; i < n; ++i)
        if (lambda[i] == 0) split[i] = F_NODE;
    for (int64_t top = n - 1; top >= 0; --top) {
        const int64_t i = i2n[top];
        const int64_t li = lambda[i];
        icount[li]--;
        if (split[i] == F_NODE) continue;
        split[i] = C_NODE;
        // nodes that depend on i become F
        for (int64_t k = T.ptr[i]; k < T.ptr[i + 1]; ++k) {
            const int64_t j = T.col[k];
            if (split[j] != U_NODE) continue;
            split[j] = F_NODE;
            // every undecided node that j depends on gains one in lambda
            for (int64_t q = S.ptr[j]; q < S.ptr[j + 1]; ++q) {
                const int64_t r = S.col[q];
                if (split[r] != U_NODE) continue;
                const int64_t lr = lambda[r];
                const int64_t old_pos = n2i[r];
                const int64_t new_pos = iptr[lr] + icount[lr] - 1;
                const int64_t sw = i2n[new_pos];
                i2n[old_pos] = sw;
                i2n[new_pos] = r;
                n2i[r] = new_pos;
                n2i[sw] = old_pos;
                icount[lr]--;
                icount[lr + 1]++;
                iptr[lr + 1] = new_pos;
                lambda[r]++;
            }
        }
        // every undecided node that i depends on loses one in lambda
        for (int64_t q = S.ptr[i]; q < S.ptr[i + 1]; ++q) {
            const int64_t r = S.col[q];
            if (split[r] != U_NODE) continue;
            const int64_t lr = lambda[r];
            const int64_t old_pos = n2i[r];
            const int64_t new_pos = iptr[lr];
            const int64_t sw = i2n[new_pos];
            i2n[old_pos] = sw;
            i2n[new_pos] = r;
            n2i[r] = new_pos;
            n2i[sw] = old_pos;
            icount[lr]--;
            icount[lr - 1]++;
            iptr[lr]++;
            lambda[r]--;
        }
    }
    return split;
}

// Direct interpolation: F row i interpolates from its strong C neighbours, negative and
// positive couplings scaled separately so that row sums are preserved.
static CSR direct_interpolation(const CSR& A, const CSR& S, const std::vector<int>& split) {
    const int64_t n = A.n;
    std::vector<int64_t> cmap(n, -1);
    int64_t nc = 0;
    for (int64_t i = 0; i < n; ++i)
        if (split[i] == C_NODE) cmap[i] = nc++;
    CSR P;
    P.n = n;
    P.m = nc;
    P.ptr.assign(n + 1, 0);
    for (int64_t i = 0; i < n; ++i) {
        if (split[i] == C_NODE) {
            P.ptr[i + 1] = 1;
        } else {
            int64_t c = 0;
            for (int64_t k = S.ptr[i]; k < S.ptr[i + 1]; ++k)
                if (split[S.col[k]] == C_NODE) ++c;
            P.ptr[i + 1] = c;
        }
    }
    for (int64_t i = 0; i < n; ++i) P.ptr[i + 1] += P.ptr[i];
    P.col.resize(P.ptr[n]);
    P.val.resize(P.ptr[n]);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t q = P.ptr[i];
        if (split[i] == C_NODE) {
            P.col[q] = cmap[i];
            P.val[q] = 1.0;
            continue;
        }
        double ssp = 0.0, ssn = 0.0, sap = 0.0, san = 0.0, diag = 0.0;
        for (int64_t k = S.ptr[i]; k < S.ptr[i + 1]; ++k)
            if (split[S.col[k]] == C_NODE) {
                if (S.val[k] < 0) ssn += S.val[k];
                else ssp += S.val[k];
            }
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            if (A.col[k] == i) diag += A.val[k];
            else if (A.val[k] < 0) san += A.val[k];
            else sap += A.val[k];
        }
        double alpha = san / ssn, beta = sap / ssp;
        if (ssp == 0.0) {
            diag += sap;
            beta = 0.0;
        }
        const double nc_ = -alpha / diag, pc = -beta / diag;
        for (int64_t k = S.ptr[i]; k < S.ptr[i + 1]; ++k)
            if (split[S.col[k]] == C_NODE) {
                P.col[q] = cmap[S.col[k]];
                P.val[q] = (S.val[k] < 0 ? nc_ : pc) * S.val[k];
                ++q;
            }
    }
    return P;
}

// Dense symmetric pseudo-inverse through Jacobi eigen-decomposition (tiny coarse grid).
static void pinv_dense(int64_t n, const vec& A, vec& X) {
    vec a(A), V(n * n, 0.0);
    for (int64_t i = 0; i < n; ++i) V[i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0;
        for (int64_t p = 0; p < n; ++p)
            for (int64_t q = p + 1; q < n; ++q) off += a[p * n + q] * a[p * n + q];
        if (off < 1e-30) break;
        for (int64_t p = 0; p < n; ++p)
            for (int64_t q = p + 1; q < n; ++q) {
                double apq = a[p * n + q];
                if (std::fabs(apq) < 1e-300) continue;
                double th = (a[q * n + q] - a[p * n + p]) / (2 * apq);
                double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
                double cs = 1 / std::sqrt(t * t + 1), sn = t * cs;
                for (int64_t k = 0; k < n; ++k) {
                    double akp = a[k * n + p], akq = a[k * n + q];
                    a[k * n + p] = cs * akp - sn * akq;
                    a[k * n + q] = sn * akp + cs * akq;
                }
                for (int64_t k = 0; k < n; ++k) {
                    double apk = a[p * n + k], aqk = a[q * n + k];
                    a[p * n + k] = cs * apk - sn * aqk;
                    a[q * n + k] = sn * apk + cs * aqk;
                }
                for (int64_t k = 0; k < n; ++k) {
                    double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = cs * vkp - sn * vkq;
                    V[k * n + q] = sn * vkp + cs * vkq;
                }
            }
    }
    double emax = 0.0;
    for (int64_t i = 0; i < n; ++i) emax = std::max(emax, std::fabs(a[i * n + i]));
    X.assign(n * n, 0.0);
    for (int64_t k = 0; k < n; ++k) {
        double ev = a[k * n + k];
        if (std::fabs(ev) <= 1e-14 * emax) continue;
        for (int64_t i = 0; i < n; ++i)
            for (int64_t j = 0; j < n; ++j) X[i * n + j] += V[i * n + k] * V[j * n + k] / ev;
    }
}

void AMG::build(const CSR& A0, double theta, int max_levels, int max_coarse) {
    levels.clear();
    CSR A = A0;
    while ((int)levels.size() + 1 < max_levels && A.n > max_coarse) {
        CSR S = strength_classical(A, theta);
        std::vector<int> split = rs_cf_splitting(S);
        CSR P = direct_interpolation(A, S, split);
        CSR R = transpose(P);
        CSR Ac = matmul(R, matmul(A, P));
        levels.push_back({std::move(A), std::move(P), std::move(R)});
        A = std::move(Ac);
    }
    Acoarse = std::move(A);
    nc = Acoarse.n;
    vec dense(nc * nc, 0.0);
    for (int64_t i = 0; i < nc; ++i)
        for (int64_t k = Acoarse.ptr[i]; k < Acoarse.ptr[i + 1]; ++k) dense[i * nc + Acoarse.col[k]] = Acoarse.val[k];
    pinv_dense(nc, dense, coarse_pinv);
    res.resize(levels.size());
    cb.resize(levels.size());
    cx.resize(levels.size());
    for (size_t l = 0; l < levels.size(); ++l) {
        res[l].assign(levels[l].A.n, 0.0);
        cb[l].assign(levels[l].P.m, 0.0);
        cx[l].assign(levels[l].P.m, 0.0);
    }
}

double AMG::operator_complexity() const {
    double s = 0, f = levels.empty() ? 1 : (double)levels[0].A.nnz();
    for (auto& L : levels) s += (double)L.A.nnz();
    s += (double)Acoarse.nnz();
    return s / f;
}

// Gauss-Seidel sweep over rows start..stop (inclusive) with step +-1.
static void gs_sweep(const CSR& A, const double* b, double* x, int64_t start, int64_t step, int64_t stop) {
    for (int64_t i = start;; i += step) {
        double rsum = 0.0, d = 0.0;
        for (int64_t k = A.ptr[i]; k < A.ptr[i + 1]; ++k) {
            if (A.col[k] == i) d = A.val[k];
            else rsum += A.val[k] * x[A.col[k]];
        }
        if (d != 0.0) x[i] = (b[i] - rsum) / d;
        if (i == stop) break;
    }
}
static void gs_symmetric(const CSR& A, const double* b, double* x) {
    gs_sweep(A, b, x, 0, 1, A.n - 1);
    gs_sweep(A, b, x, A.n - 1, -1, 0);
}

void AMG::vcycle(int lvl, double* x, const double* b) {
    const AMGLevel& L = levels[lvl];
    const int64_t n = L.A.n;
    gs_symmetric(L.A, b, x);
    L.A.spmv(x, res[lvl].data());
    for (int64_t i = 0; i < n; ++i) res[lvl][i] = b[i] - res[lvl][i];
    L.R.spmv(res[lvl].data(), cb[lvl].data());
    std::fill(cx[lvl].begin(), cx[lvl].end(), 0.0);
    if (lvl + 1 == (int)levels.size()) {
        for (int64_t i = 0; i < nc; ++i) {
            double s = 0.0;
            for (int64_t j = 0; j < nc; ++j) s += coarse_pinv[i * nc + j] * cb[lvl][j];
            cx[lvl][i] = s;
        }
    } else {
        vcycle(lvl + 1, cx[lvl].data(), cb[lvl].data());
    }
    L.P.spmv(cx[lvl].data(), res[lvl].data());
    for (int64_t i = 0; i < n; ++i) x[i] += res[lvl][i];
    gs_symmetric(L.A, b, x);
}

void AMG::precond(double* x, const double* b) {
    if (levels.empty()) {
        for (int64_t i = 0; i < nc; ++i) {
            double s = 0.0;
            for (int64_t j = 0; j < nc; ++j) s += coarse_pinv[i * nc + j] * b[j];
            x[i] = s;
        }
        return;
    }
    std::fill(x, x + levels[0].A.n, 0.0);
    vcycle(0, x, b);
}

// Partial sums over fixed blocks of 4096 entries, added in block order: the same bits for any
// thread count and any run (an OpenMP reduction combines the threads' sums in arrival order).
static double dot(int64_t n, const double* a, const double* b) {
    constexpr int64_t BS = 4096;
    const int64_t nb = (n + BS - 1) / BS;
    vec part(nb, 0.0);
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < nb; ++q) {
        double s = 0.0;
        const int64_t e = std::min(n, (q + 1) * BS);
        for (int64_t i = q * BS; i < e; ++i) s += a[i] * b[i];
        part[q] = s;
    }
    double s = 0.0;
    for (int64_t q = 0; q < nb; ++q) s += part[q];
    return s;
}

void qs_prepare(orc_model* m) {
    if (m->qs_ready) return;
    const int64_t nglob = m->nglob, nI = (int64_t)m->FltNI.size(), Nf = m->FltNglob;
    std::vector<int64_t> mapI(nglob, -1), mapF(nglob, -1);
    for (int64_t k = 0; k < nI; ++k) mapI[m->FltNI[k]] = k;
    for (int64_t k = 0; k < Nf; ++k) mapF[m->iFlt[k]] = k;
    CSR& A = m->Kni;
    CSR& B = m->Knf;
    A.n = A.m = nI;
    B.n = nI;
    B.m = Nf;
    A.ptr.assign(nI + 1, 0);
    B.ptr.assign(nI + 1, 0);
    for (int64_t r = 0; r < nI; ++r) {
        const int64_t g = m->FltNI[r];
        for (int64_t k = m->K.ptr[g]; k < m->K.ptr[g + 1]; ++k) {
            const int64_t c = m->K.col[k];
            if (mapI[c] >= 0) {
                A.col.push_back(mapI[c]);
                A.val.push_back(-m->K.val[k]);
            } else {
                B.col.push_back(mapF[c]);
                B.val.push_back(m->K.val[k]);
            }
        }
        A.ptr[r + 1] = (int64_t)A.col.size();
        B.ptr[r + 1] = (int64_t)B.col.size();
    }
    m->diagKni.assign(nI, 0.0);
    for (int64_t r = 0; r < nI; ++r)
        for (int64_t k = A.ptr[r]; k < A.ptr[r + 1]; ++k)
            if (A.col[k] == r) m->diagKni[r] = A.val[k];
    m->amg.build(A);
    m->qs_ready = true;
}

// PCG restating IterativeSolvers.jl 0.8 cg! (x0 = guess, rho0 = 1, u0 = 0).
static int pcg(orc_model* m, int mode, const vec& b, vec& x, double tol, int maxit, double* relres) {
    const CSR& A = m->Kni;
    const int64_t n = A.n;
    vec r(n), c(n), u(n, 0.0);
    A.spmv(x.data(), c.data());
    for (int64_t i = 0; i < n; ++i) r[i] = b[i] - c[i];
    const double nb = std::sqrt(dot(n, b.data(), b.data()));
    const double reltol = nb * tol;
    double res = std::sqrt(dot(n, r.data(), r.data()));
    double rho = 1.0;
    int it = 0;
    while (!(it >= maxit || res <= reltol)) {
        if (mode == 0) m->amg.precond(c.data(), r.data());
        else
            for (int64_t i = 0; i < n; ++i) c[i] = r[i] / m->diagKni[i];
        const double rho_prev = rho;
        rho = dot(n, c.data(), r.data());
        const double beta = rho / rho_prev;
        for (int64_t i = 0; i < n; ++i) u[i] = c[i] + beta * u[i];
        A.spmv(u.data(), c.data());
        const double alpha = rho / dot(n, u.data(), c.data());
        for (int64_t i = 0; i < n; ++i) {
            x[i] += alpha * u[i];
            r[i] -= alpha * c[i];
        }
        res = std::sqrt(dot(n, r.data(), r.data()));
        ++it;
    }
    if (relres) *relres = nb > 0 ? res / nb : res;
    return res <= reltol ? it : -it;
}

}  // namespace orc

using namespace orc;

extern "C" void orc_apply_K_csr(const orc_model* m, const double* x, double* y) { m->K.spmv(x, y); }

extern "C" void orc_apply_K_elem(const orc_model* m, const double* x, double* y) {
    const int N = (int)m->NGLL;
    const double* H = m->H.data();
    const double c1 = m->coefint1, c2 = m->coefint2;
    std::fill(y, y + m->nglob, 0.0);
    // Element results first, then a serial scatter (Conn * a_elem, PCG.jl:266).
    std::vector<double> ae((size_t)N * N * m->Nel);
#pragma omp parallel for schedule(static)
    for (int64_t e = 0; e < m->Nel; ++e) {
        const int64_t* ig = &m->iglob[(size_t)N * N * e];
        const double* Wl = &m->W[(size_t)N * N * e];
        double u[5][5], t1[5][5], t2[5][5];
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) u[i][j] = x[ig[i + N * j]];
        // t1 = W .* (H' u), t2 = W .* (u H)
        for (int j = 0; j < N; ++j)
            for (int p = 0; p < N; ++p) {
                double s1 = 0.0, s2 = 0.0;
                for (int k = 0; k < N; ++k) {
                    s1 += H[k + N * p] * u[k][j];
                    s2 += u[p][k] * H[k + N * j];
                }
                t1[p][j] = Wl[p + N * j] * s1;
                t2[p][j] = Wl[p + N * j] * s2;
            }
        // c1 * H t1 + c2 * t2 H'
        for (int j = 0; j < N; ++j)
            for (int i = 0; i < N; ++i) {
                double s1 = 0.0, s2 = 0.0;
                for (int p = 0; p < N; ++p) {
                    s1 += H[i + N * p] * t1[p][j];
                    s2 += t2[i][p] * H[j + N * p];
                }
                ae[i + N * j + (size_t)N * N * e] = c1 * s1 + c2 * s2;
            }
    }
    for (int64_t e = 0; e < m->Nel; ++e)
        for (int q = 0; q < N * N; ++q) y[m->iglob[q + (size_t)N * N * e]] += ae[q + (size_t)N * N * e];
}

extern "C" int orc_qs_solve(orc_model* m, const double* F_fault, double* d_full, double tol, int mode,
                            int maxit, double* relres) {
    qs_prepare(m);
    const int64_t nI = (int64_t)m->FltNI.size();
    vec b(nI), x(nI);
    m->Knf.spmv(F_fault, b.data());  // rhs = (K F)[FltNI]
    for (int64_t k = 0; k < nI; ++k) x[k] = d_full[m->FltNI[k]];
    int it = pcg(m, mode, b, x, tol, maxit <= 0 ? (int)nI : maxit, relres);
    for (int64_t k = 0; k < nI; ++k) d_full[m->FltNI[k]] = x[k];
    for (int64_t k = 0; k < m->FltNglob; ++k) d_full[m->iFlt[k]] = F_fault[k];
    return it;
}

namespace orc {
int qs_solve_internal(orc_model* m, const vec& Ffault, vec& d, double tol, int mode, int maxit) {
    return orc_qs_solve(m, Ffault.data(), d.data(), tol, mode, maxit, nullptr);
}
}  // namespace orc
