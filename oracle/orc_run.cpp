// CPU oracle -- time loop restatement of src/main.jl:67-477 (test infrastructure).
#include "orc_internal.h"
#include <cmath>
#include <algorithm>
#include <cstdio>

namespace orc {
int qs_solve_internal(orc_model* m, const vec& Ffault, vec& d, double tol, int mode, int maxit);

void init_state(orc_model* m) {
    const int64_t n = m->nglob, Nf = m->FltNglob;
    // main.jl:89-97 (ETA == 0)
    m->dt = m->dt0;
    m->dtmin = m->dt;
    m->half_dt = 0.5 * m->dtmin;
    m->half_dt_sq = 0.5 * (m->dtmin * m->dtmin);
    // main.jl:100-103: v = V_init / 2 everywhere
    m->d.assign(n, 0.0);
    m->v.assign(n, 0.5 * m->cfg.V_init);
    m->a.assign(n, 0.0);
    m->tau.assign(Nf, 0.0);
    m->Vf.assign(Nf, 0.0);
    m->Vf0.assign(Nf, 0.0);
    m->Vf1.assign(Nf, 0.0);
    m->Vf2.assign(Nf, 0.0);
    m->psi1.assign(Nf, 0.0);
    m->psi2.assign(Nf, 0.0);
    m->tau1.assign(Nf, 0.0);
    m->tau2.assign(Nf, 0.0);
    m->FltVfree.assign(Nf, 0.0);
    m->psi.assign(Nf, 0.0);
    // main.jl:125
    for (int64_t k = 0; k < Nf; ++k)
        m->psi[k] = m->tauo[k] / (m->Seff[k] * m->ccb[k]) - m->fo[k] / m->ccb[k] -
                    (m->cca[k] / m->ccb[k]) * std::log(2 * m->v[m->iFlt[k]] / m->Vo[k]);
    m->isolver = 1;
    m->F.assign(n, 0.0);
    m->dPre.assign(n, 0.0);
    m->vPre.assign(n, 0.0);
    // main.jl:166-181
    m->tvsx = 5 * m->yr2sec;
    m->tvsxinc = m->tvsx;
    m->tevneinc = 0.5;
    m->delfref.assign(Nf, 0.0);
    m->idelevne = 0;
    m->tevneb = 0;
    m->tevne = 0;
    m->ntvsx = m->nevne = m->slipstart = m->idd = m->it_s = m->it_e = m->rit = 0;
    // main.jl:183-190
    for (auto& vv : m->v) vv = vv - 0.5 * m->Vpl;
    for (int64_t k = 0; k < Nf; ++k) m->Vf[k] = 2 * m->v[m->iFlt[k]];
    for (auto k : m->iFBC) m->Vf[k] = 0.;
    for (auto g : m->FltIglobBC) m->v[g] = 0.;
    m->it = 0;
    m->t = 0.;
    m->out = Results();
}

static void record_fault(const orc_model* m, std::vector<vec>& dst, int which) {
    const int64_t Nf = m->FltNglob;
    vec col(Nf);
    for (int64_t k = 0; k < Nf; ++k) {
        const int64_t g = m->iFlt[k];
        if (which == 0) col[k] = 2 * m->d[g] + m->Vpl * m->t;
        else if (which == 1) col[k] = 2 * m->v[g] + m->Vpl;
        else col[k] = (m->tau[k] + m->tauo[k]) / 1e6;
    }
    dst.push_back(std::move(col));
}

}  // namespace orc

using namespace orc;

extern "C" int64_t orc_run(orc_model* m, int64_t nsteps, double t_end_s, int qs_mode, double qs_tol, int qs_maxit) {
    const int64_t Nf = m->FltNglob, n = m->nglob;
    const double Vpl = m->Vpl;
    vec Ffault(Nf), a_tmp(n);
    int64_t steps = 0;
    while (m->t < t_end_s && steps < nsteps) {
        m->it = m->it + 1;
        m->t = m->t + m->dt;
        const double dt = m->dt;
        m->out.time_.push_back(m->t);
        m->out.regime.push_back(m->isolver);
        int cgsum = 0;
        if (m->isolver == 1) {
            // ---------------- quasi-static (main.jl:226-295) ----------------
            m->vPre = m->v;
            m->dPre = m->d;
            for (int64_t k = 0; k < Nf; ++k) {
                m->Vf0[k] = 2 * m->v[m->iFlt[k]] + Vpl;
                m->Vf[k] = m->Vf0[k];
            }
            for (int p1 = 0; p1 < 2; ++p1) {
                for (int64_t k = 0; k < Nf; ++k) Ffault[k] = m->dPre[m->iFlt[k]] + m->v[m->iFlt[k]] * dt;
                int its = qs_solve_internal(m, Ffault, m->d, qs_tol, qs_mode, qs_maxit);
                cgsum += its < 0 ? -its : its;
                // a = K d ; a[FltIglobBC] = 0 ; tau1 = -a[iFlt] / FltB
                m->K.spmv(m->d.data(), m->a.data());
                for (auto g : m->FltIglobBC) m->a[g] = 0.;
                for (int64_t k = 0; k < Nf; ++k) m->tau1[k] = -m->a[m->iFlt[k]] / m->FltB[k];
                orc_slrFunc(m, m->psi.data(), m->psi1.data(), m->Vf.data(), m->Vf1.data(), m->tau1.data(), dt);
                for (auto k : m->iFBC) m->Vf1[k] = Vpl;
                for (int64_t k = 0; k < Nf; ++k) {
                    m->Vf[k] = (m->Vf0[k] + m->Vf1[k]) / 2;
                    m->v[m->iFlt[k]] = 0.5 * (m->Vf[k] - Vpl);
                }
            }
            m->psi = m->psi1;
            m->tau = m->tau1;
            for (auto k : m->iFBC) {
                m->tau[k] = 0.;
                m->Vf1[k] = Vpl;
            }
            for (int64_t k = 0; k < Nf; ++k) m->v[m->iFlt[k]] = 0.5 * (m->Vf1[k] - Vpl);
            for (auto g : m->FltNI) m->v[g] = (m->d[g] - m->dPre[g]) / dt;
            std::fill(m->a.begin(), m->a.end(), 0.);
            for (auto g : m->FltIglobBC) {
                m->d[g] = 0.;
                m->v[g] = 0.;
            }
        } else {
            // ---------------- dynamic (main.jl:297-345) ----------------
            m->dPre = m->d;
            m->vPre = m->v;
            for (int64_t g = 0; g < n; ++g) {
                m->d[g] = m->d[g] + dt * m->v[g] + (m->half_dt_sq) * m->a[g];
                m->v[g] = m->v[g] + m->half_dt * m->a[g];
            }
            m->K.spmv(m->d.data(), a_tmp.data());
            for (int64_t g = 0; g < n; ++g) m->a[g] = -a_tmp[g];
            for (auto g : m->FltIglobBC) m->a[g] = 0.;
            for (size_t k = 0; k < m->iBcL.size(); ++k) m->a[m->iBcL[k]] = m->a[m->iBcL[k]] - m->BcLC[k] * m->v[m->iBcL[k]];
            for (size_t k = 0; k < m->iBcT.size(); ++k) m->a[m->iBcT[k]] = m->a[m->iBcT[k]] - m->BcTC[k] * m->v[m->iBcT[k]];
            for (int64_t k = 0; k < Nf; ++k) {
                const int64_t g = m->iFlt[k];
                m->FltVfree[k] = 2 * m->v[g] + 2 * m->half_dt * m->a[g] / m->M[g];
                m->Vf[k] = 2 * m->vPre[g] + Vpl;
            }
            int fail = orc_FBC(m, m->psi1.data(), m->Vf1.data(), m->tau1.data(), m->psi2.data(), m->Vf2.data(),
                               m->tau2.data(), m->psi.data(), m->Vf.data(), m->FltVfree.data(), dt);
            if (fail) return -(int64_t)fail;
            for (int64_t k = 0; k < Nf; ++k) m->tau[k] = m->tau2[k] - m->tauo[k];
            for (auto k : m->iFBC) m->tau[k] = 0.;
            m->psi = m->psi2;
            for (int64_t k = 0; k < Nf; ++k) m->a[m->iFlt[k]] = m->a[m->iFlt[k]] - m->FltB[k] * m->tau[k];
            for (int64_t g = 0; g < n; ++g) {
                m->a[g] = m->a[g] / m->M[g];
                m->v[g] = m->v[g] + m->half_dt * m->a[g];
            }
            for (auto g : m->FltIglobBC) {
                m->v[g] = 0.;
                m->a[g] = 0.;
            }
        }
        m->out.cg_iters.push_back(cgsum);
        // main.jl:348
        double vmax = -INFINITY;
        for (int64_t k = 0; k < Nf; ++k) vmax = std::max(vmax, m->v[m->iFlt[k]]);
        const double Vfmax = 2 * vmax + Vpl;
        const double tnow = m->t;
        // event start / end (main.jl:361-380)
        if (Vfmax > 1.01 * m->Vthres && m->slipstart == 0) {
            m->it_s = m->it_s + 1;
            for (int64_t k = 0; k < Nf; ++k) m->delfref[k] = 2 * m->d[m->iFlt[k]] + Vpl * tnow;
            m->slipstart = 1;
            m->out.tStart.push_back(tnow);
            record_fault(m, m->out.taubefore, 2);
            int64_t indx = 0;
            double vh = -INFINITY;
            for (int64_t k = 0; k < Nf; ++k) {
                const double s = 2 * m->v[m->iFlt[k]] + Vpl;
                if (s > vh) {
                    vh = s;
                    indx = k;
                }
            }
            m->out.hypo.push_back(m->FltX[indx]);
        }
        if (Vfmax < 0.99 * m->Vthres && m->slipstart == 1) {
            m->it_e = m->it_e + 1;
            vec col(Nf);
            for (int64_t k = 0; k < Nf; ++k) col[k] = 2 * m->d[m->iFlt[k]] + Vpl * tnow - m->delfref[k];
            m->out.delfafter.push_back(col);
            record_fault(m, m->out.tauafter, 2);
            m->out.tEnd.push_back(tnow);
            m->slipstart = 0;
            // damage grows at the end of each earthquake (main.jl:377-378)
            if (!m->damage_el.empty() && m->damage_factor != 1.0) orc::damage_evolve(m);
        }
        // interseismic snapshots (main.jl:384-393)
        if (tnow > m->tvsx) {
            m->ntvsx = m->ntvsx + 1;
            m->idd += 1;
            record_fault(m, m->out.is_slip, 0);
            record_fault(m, m->out.is_slipvel, 1);
            record_fault(m, m->out.is_stress, 2);
            m->tvsx = m->tvsx + m->tvsxinc;
        }
        // coseismic snapshots (main.jl:395-422)
        if (Vfmax > m->Vevne) {
            if (m->idelevne == 0) {
                m->nevne = m->nevne + 1;
                m->idd += 1;
                m->idelevne = 1;
                m->tevneb = tnow;
                m->tevne = m->tevneinc;
                record_fault(m, m->out.seismic_slip, 0);
                record_fault(m, m->out.seismic_slipvel, 1);
                record_fault(m, m->out.seismic_stress, 2);
            }
            if (m->idelevne == 1 && (tnow - m->tevneb) > m->tevne) {
                m->nevne = m->nevne + 1;
                m->idd += 1;
                record_fault(m, m->out.seismic_slip, 0);
                record_fault(m, m->out.seismic_slipvel, 1);
                record_fault(m, m->out.seismic_stress, 2);
                m->tevne = m->tevne + m->tevneinc;
            }
        } else {
            m->idelevne = 0;
        }
        // receivers every 10 steps (main.jl:431-436)
        if (m->it % 10 == 0) {
            m->rit += 1;
            vec dd, vv, aa;
            for (auto g : m->out_seis) {
                dd.push_back(m->d[g]);
                vv.push_back(m->v[g]);
                aa.push_back(m->a[g]);
            }
            m->out.dSeis.push_back(dd);
            m->out.vSeis.push_back(vv);
            m->out.aSeis.push_back(aa);
        }
        // regime switch (main.jl:439-443)
        if ((m->isolver == 1 && Vfmax < 5e-3) || (m->isolver == 2 && Vfmax < 2e-3)) m->isolver = 1;
        else m->isolver = 2;
        m->out.Vfmax.push_back(Vfmax);
        // next dt (main.jl:447-450)
        vec sr(Nf);
        for (int64_t k = 0; k < Nf; ++k) sr[k] = 2 * m->v[m->iFlt[k]] + Vpl;
        m->dt = orc_dtevol(m, m->dt, m->dtmin, sr.data(), m->isolver);
        ++steps;
    }
    return steps;
}
