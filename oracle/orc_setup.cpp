// CPU oracle -- setup restatement (test infrastructure; see orc_api.h).
//
// Follows, in order, par.jl:15-231 (setParameters) and the files it includes:
//   GLL tables           src/GetGLL.jl:17-28 (values recomputed from Legendre polynomials)
//   mesh numbering       src/MeshBox.jl:27-88
//   mass / dt / muMax    src/Assemble.jl:7-71
//   W                    src/MaterialProperties.jl:3-21 (rectangle), :77-101 (per-node)
//   stiffness            src/Kassemble.jl:3-63
//   boundary matrices    src/BoundaryMatrix.jl:7-61
//   receivers            src/FindNearestNode.jl:3-19
//   depth profiles       src/initialConditions/defaultInitialConditions.jl:9-84
//   XiLf                 par.jl:304-339
#include "orc_internal.h"
#include <cmath>
#include <algorithm>
#include <stdexcept>
#include <numeric>

namespace orc {

// --- GLL nodes/weights/derivatives from Legendre polynomials -------------------------
// Newton iteration x <- x - (x P_N - P_{N-1}) / ((N+1) P_N) from Chebyshev-Lobatto
// starting points converges to the zeros of (1-x^2) P_N'(x) (the GLL nodes).
static void legendre(int N, double x, double* P) {  // P[0..N]
    P[0] = 1.0;
    if (N >= 1) P[1] = x;
    for (int k = 2; k <= N; ++k) P[k] = ((2.0 * k - 1.0) * x * P[k - 1] - (k - 1.0) * P[k - 2]) / k;
}

void gll(int ngll, double* xo, double* wo, double* Ho) {
    const int N = ngll - 1;
    std::vector<double> x(ngll), P(ngll + 1);
    for (int i = 0; i < ngll; ++i) x[i] = -std::cos(M_PI * i / N);
    for (int i = 0; i < ngll; ++i) {
        if (i == 0 || i == N) continue;
        for (int itn = 0; itn < 100; ++itn) {
            legendre(N, x[i], P.data());
            double dx = (x[i] * P[N] - P[N - 1]) / ((N + 1) * P[N]);
            x[i] -= dx;
            if (std::fabs(dx) < 1e-17) break;
        }
    }
    // Symmetrise: x[N-i] = -x[i] computed from the lower half.
    for (int i = 0; i < ngll / 2; ++i) x[N - i] = -x[i];
    if (N % 2 == 0) x[N / 2] = 0.0;
    std::vector<double> PN(ngll);
    for (int i = 0; i < ngll; ++i) {
        legendre(N, x[i], P.data());
        PN[i] = P[N];
        xo[i] = x[i];
        wo[i] = 2.0 / (N * (N + 1.0) * P[N] * P[N]);
    }
    // H[i,j] = h'_i(x_j) (GetGLL.jl:14) ; column-major H[i + ngll*j].
    for (int j = 0; j < ngll; ++j)
        for (int i = 0; i < ngll; ++i) {
            double v;
            if (i != j) v = PN[j] / (PN[i] * (x[j] - x[i]));
            else if (i == 0) v = -N * (N + 1.0) / 4.0;
            else if (i == N) v = N * (N + 1.0) / 4.0;
            else v = 0.0;
            Ho[i + ngll * j] = v;
        }
}

// --- seeded uniform(-1,1) stream (splitmix64) ----------------------------------------
struct SplitMix {
    uint64_t s;
    uint64_t next() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    double uniform_pm1() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0; }
};

static double Int1D(double p1v, double p1z, double p2v, double p2z, double val) {
    // Int1D, defaultInitialConditions.jl:2-5
    return p1v + ((p2v - p1v) / (p2z - p1z)) * (val - p1z);
}

// Material at a GLL node for the per-node (trapezoid) model.
static void trap_props(const orc_config& c, double xn, double yn, double& rho, double& vs) {
    double z = -xn;  // depth
    rho = c.rho1;
    vs = c.vs1;
    if (z <= c.trap_z1) {
        double w = c.trap_w0 + (c.trap_w1 - c.trap_w0) * (z / c.trap_z1);
        if (yn <= w) {
            rho = c.rho2;
            vs = c.vs2;
        }
    }
}

static void csr_from_coo(int64_t n, std::vector<int64_t>& I, std::vector<int64_t>& J, vec& V, CSR& A) {
    // sum duplicates, drop exact zeros (Kassemble.jl:204 dropzeros!)
    const int64_t nz = (int64_t)I.size();
    std::vector<int64_t> cnt(n + 1, 0);
    for (int64_t k = 0; k < nz; ++k) cnt[I[k] + 1]++;
    for (int64_t i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
    std::vector<int64_t> pos(cnt.begin(), cnt.end() - 1);
    std::vector<int64_t> cj(nz);
    vec cv(nz);
    for (int64_t k = 0; k < nz; ++k) {
        int64_t p = pos[I[k]]++;
        cj[p] = J[k];
        cv[p] = V[k];
    }
    A.n = A.m = n;
    A.ptr.assign(n + 1, 0);
    A.col.clear();
    A.val.clear();
    A.col.reserve(nz / 4);
    A.val.reserve(nz / 4);
    std::vector<int64_t> perm;
    for (int64_t i = 0; i < n; ++i) {
        int64_t b = cnt[i], e = cnt[i + 1];
        perm.resize(e - b);
        std::iota(perm.begin(), perm.end(), b);
        std::stable_sort(perm.begin(), perm.end(), [&](int64_t a, int64_t c) { return cj[a] < cj[c]; });
        int64_t k = 0;
        while (k < (int64_t)perm.size()) {
            int64_t c = cj[perm[k]];
            double s = 0.0;
            while (k < (int64_t)perm.size() && cj[perm[k]] == c) s += cv[perm[k++]];
            if (s != 0.0) {
                A.col.push_back(c);
                A.val.push_back(s);
            }
        }
        A.ptr[i + 1] = (int64_t)A.col.size();
    }
}

// Stiffness assembly from the element weights W (Kassemble.jl:3-63): the element matrix of
// every element, summed into CSR through the connectivity (FEMSparse's COO sum).
void assemble_K(orc_model* m) {
    const int NGLL = 5;
    const int64_t nglob = (int64_t)m->x.size();
    auto IG = [&](int i, int j, int64_t e) { return m->iglob[i + NGLL * j + (int64_t)NGLL * NGLL * e]; };
    const double* H = m->H.data();
    auto Hm = [&](int i, int j) { return H[i + NGLL * j]; };
    const double cy = m->jac / (m->dy_deta * m->dy_deta);  // multiplies the eta terms
    const double cx = m->jac / (m->dx_dxi * m->dx_dxi);
    std::vector<int64_t> I, J;
    vec V;
    const size_t per = (size_t)NGLL * NGLL * (2 * NGLL - 1);
    I.reserve(per * m->Nel);
    J.reserve(per * m->Nel);
    V.reserve(per * m->Nel);
    for (int64_t eo = 0; eo < m->Nel; ++eo) {
        const double* ww = &m->W[(int64_t)NGLL * NGLL * eo];
        auto w = [&](int i, int j) { return ww[i + NGLL * j]; };
        for (int l = 0; l < NGLL; ++l)
            for (int k = 0; k < NGLL; ++k)
                for (int j = 0; j < NGLL; ++j)
                    for (int i = 0; i < NGLL; ++i) {
                        if (i != k && j != l) continue;
                        double term1 = 0.0, term2 = 0.0;
                        for (int p = 0; p < NGLL; ++p) {
                            term1 += (i == k ? 1.0 : 0.0) * w(k, p) * cy * Hm(j, p) * Hm(l, p);
                            term2 += (j == l ? 1.0 : 0.0) * w(p, j) * cx * Hm(i, p) * Hm(k, p);
                        }
                        I.push_back(IG(i, j, eo));
                        J.push_back(IG(k, l, eo));
                        V.push_back(term1 + term2);
                    }
    }
    csr_from_coo(nglob, I, J, V, m->K);
}

// damageEvol.jl:5-7: W[:, :, damage_idx] .*= factor, then K is assembled again (the quasi-
// static solver pieces are rebuilt on next use).
void damage_evolve(orc_model* m) {
    for (int64_t e : m->damage_el)
        for (int q = 0; q < 25; ++q) m->W[(size_t)25 * e + q] *= m->damage_factor;
    assemble_K(m);
    m->qs_ready = false;
    m->damage_count += 1;
}

void setup_model(orc_model* m) {
    const orc_config& c = m->cfg;
    const int NGLL = 5;
    m->NGLL = NGLL;
    m->NelX = c.NelX;
    m->NelY = c.NelY;
    const int64_t NelX = c.NelX, NelY = c.NelY;
    m->dxe = c.LX / NelX;
    m->dye = c.LY / NelY;
    m->Nel = NelX * NelY;
    m->FltNglob = NelX * (NGLL - 1) + 1;
    m->dx_dxi = 0.5 * m->dxe;
    m->dy_deta = 0.5 * m->dye;
    m->jac = m->dx_dxi * m->dy_deta;
    m->coefint1 = m->jac / (m->dx_dxi * m->dx_dxi);
    m->coefint2 = m->jac / (m->dy_deta * m->dy_deta);
    m->yr2sec = 365.0 * 24 * 60 * 60;
    m->Total_time = c.total_years * m->yr2sec;
    m->IDstate = 2;
    m->ETA = 0.0;
    m->Vpl = c.Vpl;
    m->Vthres = c.Vthres;
    m->Vevne = c.Vthres;

    m->xgll.resize(NGLL);
    m->wgll.resize(NGLL);
    m->H.resize(NGLL * NGLL);
    gll(NGLL, m->xgll.data(), m->wgll.data(), m->H.data());
    const double* XG = m->xgll.data();
    const double* wg = m->wgll.data();

    // ---- MeshBox (src/MeshBox.jl:27-88) ----
    const int64_t nglob = m->FltNglob * (NelY * (NGLL - 1) + 1);
    m->nglob = nglob;
    m->iglob.assign((size_t)NGLL * NGLL * m->Nel, 0);
    m->x.assign(nglob, 0.0);
    m->y.assign(nglob, 0.0);
    auto IG = [&](int i, int j, int64_t e) -> int64_t& { return m->iglob[i + NGLL * j + (int64_t)NGLL * NGLL * e]; };
    double xg[NGLL][NGLL], yg[NGLL][NGLL];
    for (int i = 0; i < NGLL; ++i)
        for (int j = 0; j < NGLL; ++j) {
            xg[i][j] = m->dxe * (0.5 * (1.0 + XG[i]));
            yg[i][j] = m->dye * (0.5 * (1.0 + XG[j]));
        }
    int64_t ig[NGLL][NGLL];
    int64_t last = 0;
    int64_t et = -1;
    for (int64_t ey = 0; ey < NelY; ++ey)
        for (int64_t ex = 0; ex < NelX; ++ex) {
            ++et;
            if (et == 0) {
                for (int j = 0; j < NGLL; ++j)
                    for (int i = 0; i < NGLL; ++i) ig[i][j] = i + NGLL * j;
            } else if (ey == 0) {  // bottom row: left edge shared
                for (int j = 0; j < NGLL; ++j) ig[0][j] = IG(NGLL - 1, j, et - 1);
                for (int j = 0; j < NGLL; ++j)
                    for (int i = 1; i < NGLL; ++i) ig[i][j] = last + (i - 1) + (NGLL - 1) * j + 1;
            } else if (ex == 0) {  // left column: bottom edge shared
                for (int i = 0; i < NGLL; ++i) ig[i][0] = IG(i, NGLL - 1, et - NelX);
                for (int j = 1; j < NGLL; ++j)
                    for (int i = 0; i < NGLL; ++i) ig[i][j] = last + i + NGLL * (j - 1) + 1;
            } else {
                for (int j = 0; j < NGLL; ++j) ig[0][j] = IG(NGLL - 1, j, et - 1);
                for (int i = 0; i < NGLL; ++i) ig[i][0] = IG(i, NGLL - 1, et - NelX);
                for (int j = 1; j < NGLL; ++j)
                    for (int i = 1; i < NGLL; ++i) ig[i][j] = last + (i - 1) + (NGLL - 1) * (j - 1) + 1;
            }
            for (int j = 0; j < NGLL; ++j)
                for (int i = 0; i < NGLL; ++i) IG(i, j, et) = ig[i][j];
            last = ig[NGLL - 1][NGLL - 1];
            for (int j = 0; j < NGLL; ++j)
                for (int i = 0; i < NGLL; ++i) {
                    m->x[ig[i][j]] = m->dxe * (double)ex + xg[i][j];
                    m->y[ig[i][j]] = m->dye * (double)ey + yg[i][j];
                }
        }
    for (auto& xv : m->x) xv = xv - c.LX;  // par.jl:101

    // ---- Mass matrix, dt, muMax (Assemble.jl:7-71) and W (MaterialProperties.jl) ----
    m->M.assign(nglob, 0.0);
    m->W.assign((size_t)NGLL * NGLL * m->Nel, 0.0);
    if (c.damage == 2) {
        m->rho_node.assign(nglob, 0.0);
        m->mu_node.assign(nglob, 0.0);
        for (int64_t g = 0; g < nglob; ++g) {
            double r, vs;
            trap_props(c, m->x[g], m->y[g], r, vs);
            m->rho_node[g] = r;
            m->mu_node[g] = r * (vs * vs);
        }
    }
    double dt = INFINITY, muMax = 0.0;
    double dxg[NGLL - 1];
    for (int i = 0; i < NGLL - 1; ++i) dxg[i] = XG[i + 1] - XG[i];
    for (int64_t ey = 0; ey < NelY; ++ey)
        for (int64_t ex = 0; ex < NelX; ++ex) {
            const int64_t eo = ey * NelX + ex;
            double rho[NGLL][NGLL], mu[NGLL][NGLL];
            if (c.damage == 2) {
                for (int j = 0; j < NGLL; ++j)
                    for (int i = 0; i < NGLL; ++i) {
                        int64_t g = IG(i, j, eo);
                        rho[i][j] = m->rho_node[g];
                        mu[i][j] = m->mu_node[g];
                    }
            } else {
                bool dmg = (c.damage == 1) && ((double)(ex + 1) * m->dxe >= c.ThickX) &&
                           (m->dye <= (double)(ey + 1) * m->dye && (double)(ey + 1) * m->dye <= c.ThickY);
                double r = dmg ? c.rho2 : c.rho1;
                double mv = dmg ? c.rho2 * (c.vs2 * c.vs2) : c.rho1 * (c.vs1 * c.vs1);
                for (int j = 0; j < NGLL; ++j)
                    for (int i = 0; i < NGLL; ++i) {
                        rho[i][j] = r;
                        mu[i][j] = mv;
                    }
            }
            {   // element of the damage zone: the rectangle rule (Assemble.jl:34-35), or, for the
                // per-node trapezoid, any node with the damaged material
                bool in = false;
                for (int j = 0; j < NGLL; ++j)
                    for (int i = 0; i < NGLL; ++i) in = in || mu[i][j] != c.rho1 * (c.vs1 * c.vs1);
                if (in && c.damage != 0) m->damage_idx.push_back(eo);
            }
            for (int j = 0; j < NGLL; ++j)
                for (int i = 0; i < NGLL; ++i) muMax = std::max(muMax, mu[i][j]);
            for (int j = 0; j < NGLL; ++j)
                for (int i = 0; i < NGLL; ++i) {
                    m->M[IG(i, j, eo)] += ((wg[i] * wg[j]) * rho[i][j]) * m->jac;
                    m->W[i + NGLL * j + (int64_t)NGLL * NGLL * eo] = (wg[i] * wg[j]) * mu[i][j];
                }
            double vso[NGLL][NGLL];
            for (int j = 0; j < NGLL; ++j)
                for (int i = 0; i < NGLL; ++i) vso[i][j] = std::sqrt(mu[i][j] / rho[i][j]);
            for (int a = 0; a < NGLL - 1; ++a)
                for (int b = 0; b < NGLL; ++b) {
                    double vs, dx;
                    if (m->dxe < m->dye) {
                        vs = std::max(vso[a][b], vso[a + 1][b]);
                        dx = dxg[a] * 0.5 * m->dxe;
                    } else {
                        vs = std::max(vso[b][a], vso[b][a + 1]);
                        dx = dxg[a] * 0.5 * m->dye;
                    }
                    dt = std::min(dt, dx / vs);
                }
        }
    m->muMax = muMax;

    // ---- stiffness assembly (Kassemble.jl:3-63) ----
    assemble_K(m);

    // ---- time-step (par.jl:155-158) ----
    dt = c.CFL * dt;
    m->dt0 = dt;
    const double half_dt = 0.5 * dt;

    // ---- boundary matrices (BoundaryMatrix.jl:7-61) ----
    auto boundary = [&](char side, vec& B, ivec& iB) {
        std::vector<int64_t> eB;
        int igll = -1, jgll = -1;
        double jac1D, imp;
        if (side == 'L') {
            for (int64_t k = 0; k < NelY; ++k) eB.push_back(k * NelX);
            igll = 0;
            jac1D = m->dy_deta;
            imp = c.rho1 * c.vs1;
        } else if (side == 'R') {
            for (int64_t k = 0; k < NelY; ++k) eB.push_back(k * NelX + NelX - 1);
            igll = NGLL - 1;
            jac1D = m->dy_deta;
            imp = c.rho1 * c.vs1;
        } else if (side == 'T') {
            for (int64_t k = 0; k < NelX; ++k) eB.push_back((NelY - 1) * NelX + k);
            jgll = NGLL - 1;
            jac1D = m->dx_dxi;
            imp = c.rho1 * c.vs1;
        } else {
            for (int64_t k = 0; k < NelX; ++k) eB.push_back(k);
            jgll = 0;
            jac1D = m->dx_dxi;
            imp = 1.0;
        }
        const int64_t NelB = (int64_t)eB.size();
        const int64_t ng = NelB * (NGLL - 1) + 1;
        iB.assign(ng, 0);
        B.assign(ng, 0.0);
        for (int64_t e = 0; e < NelB; ++e)
            for (int k = 0; k < NGLL; ++k) {
                int64_t ip = (NGLL - 1) * e + k;
                iB[ip] = (igll >= 0) ? IG(igll, k, eB[e]) : IG(k, jgll, eB[e]);
                B[ip] += (jac1D * wg[k]) * imp;
            }
    };
    boundary('L', m->BcLC, m->iBcL);
    boundary('T', m->BcTC, m->iBcT);
    for (size_t k = 0; k < m->iBcL.size(); ++k) m->M[m->iBcL[k]] = m->M[m->iBcL[k]] + half_dt * m->BcLC[k];
    for (size_t k = 0; k < m->iBcT.size(); ++k) m->M[m->iBcT[k]] = m->M[m->iBcT[k]] + half_dt * m->BcTC[k];
    boundary('B', m->FltB, m->iFlt);
    const int64_t Nf = m->FltNglob;
    m->FltZ.resize(Nf);
    m->FltX.resize(Nf);
    for (int64_t k = 0; k < Nf; ++k) {
        m->FltZ[k] = ((m->M[m->iFlt[k]] / m->FltB[k]) / half_dt) * 0.5;
        m->FltX[k] = m->x[m->iFlt[k]];
    }

    // ---- friction parameters and fault profiles ----
    m->fo.assign(Nf, c.fo);
    m->Vo.assign(Nf, c.Vo);
    m->xLf.assign(Nf, c.Dc);
    m->cca.resize(Nf);
    m->ccb.resize(Nf);
    m->Seff.resize(Nf);
    m->tauo.resize(Nf);
    if (c.profile == 0) {
        for (int64_t k = 0; k < Nf; ++k) {
            const double X = m->FltX[k], z = std::fabs(X);
            double ab = 0.015 - 0.019;
            if (z <= 2e3) ab = Int1D(0.012, 0e3, -0.0041, -2e3, X);
            else if (z <= 12e3) ab = Int1D(-0.0041, -2e3, -0.0041, -12e3, X);
            else if (z <= 17e3) ab = Int1D(-0.0041, -12e3, 0.015, -17e3, X);
            else if (z <= 24e3) ab = Int1D(0.015, -17e3, 0.024, -24e3, X);
            else ab = 0.0047;
            m->ccb[k] = 0.019;
            m->cca[k] = 0.019 + ab;
            m->Seff[k] = (z <= 2e3) ? Int1D(10e6, 0, 50e6, -2e3, X) : 50e6;
            double t0 = 22.5e6;
            if (z <= 2e3) t0 = Int1D(0.01e6, 0, 30e6, -2e3, X);
            else if (z <= 12e3) t0 = Int1D(30e6, -2e3, 30e6, -12e3, X);
            else if (z <= 17e3) t0 = Int1D(30e6, -12e3, 22.5e6, -17e3, X);
            else if (z <= 24e3) t0 = Int1D(22.5e6, -17e3, 22.5e6, -24e3, X);
            m->tauo[k] = t0;
        }
    } else {
        SplitMix rng{c.seed};
        for (int64_t k = 0; k < Nf; ++k) {
            const double z = std::fabs(m->FltX[k]);
            double b;
            if (z <= c.zb0) b = c.b0;
            else if (z >= c.zb1) b = c.b1;
            else b = c.b0 + (c.b1 - c.b0) * ((z - c.zb0) / (c.zb1 - c.zb0));
            m->cca[k] = c.a0;
            m->ccb[k] = b;
            m->Seff[k] = c.sigma;
            const double theta = (c.Dc / c.Vpl) * (1.0 + c.noise_amp * rng.uniform_pm1());
            const double psi0 = std::log(c.Vo * theta / c.Dc);
            m->tauo[k] = m->Seff[k] * (c.fo + m->ccb[k] * psi0 + m->cca[k] * std::log(c.V_init / c.Vo));
        }
    }

    // ---- XiLf (par.jl:304-339) ----
    {
        const double hcell = c.LX / (double)(Nf - 1);
        const double gamma_ = M_PI / 4.0, Ximax = 0.5, Xithf = 1.0;
        m->XiLf.resize(Nf);
        for (int64_t j = 0; j < Nf; ++j) {
            double expr1 = -(m->cca[j] - m->ccb[j]) / m->cca[j];
            double expr2 = gamma_ * muMax / hcell * m->xLf[j] / (m->cca[j] * m->Seff[j]);
            double ro = expr2 - expr1;
            double Xith = (0.25 * ro * ro - expr2 >= 0) ? 1.0 / ro : 1.0 - expr1 / expr2;
            m->XiLf[j] = (Xithf * Xith > Ximax) ? Ximax * m->xLf[j] : Xithf * Xith * m->xLf[j];
        }
    }

    // ---- FltNI (par.jl:209) ----
    {
        std::vector<char> onf(nglob, 0);
        for (auto g : m->iFlt) onf[g] = 1;
        m->FltNI.clear();
        m->FltNI.reserve(nglob - Nf);
        for (int64_t g = 0; g < nglob; ++g)
            if (!onf[g]) m->FltNI.push_back(g);
    }

    // ---- creeping fault nodes: FltIglobBC (par.jl:214-217) / iFBC (main.jl:185) ----
    auto creeps = [&](double X) {
        return c.creep_inclusive ? (std::fabs(X) >= c.creep_depth) : (std::fabs(X) > c.creep_depth);
    };
    m->FltIglobBC.clear();
    {
        // fbc = iglob[:,1,:][:]: bottom-line nodes of every element, element by element.
        std::vector<int64_t> fbc;
        for (int64_t e = 0; e < m->Nel; ++e)
            for (int i = 0; i < NGLL; ++i) fbc.push_back(IG(i, 0, e));
        int64_t last_creep = -1;
        for (int64_t k = 0; k < Nf; ++k)
            if (creeps(m->FltX[k])) last_creep = m->iFlt[k];
        if (last_creep >= 0) {
            size_t idx = 0;
            while (fbc[idx] != last_creep) ++idx;
            m->FltIglobBC.assign(fbc.begin(), fbc.begin() + idx + 1);
        }
    }
    m->iFBC.clear();
    for (int64_t k = 0; k < Nf; ++k)
        if (creeps(m->FltX[k])) m->iFBC.push_back(k);
    m->NFBC = (int64_t)m->iFBC.size();  // 0-based first friction node

    // ---- receivers (par.jl:118-122, FindNearestNode.jl) ----
    m->out_seis.clear();
    m->xout.clear();
    m->yout.clear();
    for (int r = 0; r < c.nrec; ++r) {
        int64_t best = 0;
        double bd = INFINITY;
        for (int64_t g = 0; g < nglob; ++g) {
            double dd = (m->x[g] - c.rec_x[r]) * (m->x[g] - c.rec_x[r]) + (m->y[g] - c.rec_y[r]) * (m->y[g] - c.rec_y[r]);
            if (dd < bd) {
                bd = dd;
                best = g;
            }
        }
        m->out_seis.push_back(best);
        m->xout.push_back(m->x[best]);
        m->yout.push_back(m->y[best]);
    }
}

}  // namespace orc
