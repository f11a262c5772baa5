// CPU oracle -- C API (test infrastructure; see orc_api.h).
#include "orc_internal.h"
#include <cstring>
#include <cmath>
#include <string>
#include <omp.h>

using namespace orc;

extern "C" orc_model* orc_create(const orc_config* cfg) {
    orc_model* m = new orc_model();
    m->cfg = *cfg;
    setup_model(m);
    init_state(m);
    return m;
}

extern "C" void orc_destroy(orc_model* m) { delete m; }

extern "C" int orc_gll(int ngll, double* x, double* w, double* H) {
    if (ngll < 2 || ngll > 32) return -1;
    gll(ngll, x, w, H);
    return 0;
}

extern "C" void orc_reset(orc_model* m) { init_state(m); }

extern "C" void orc_set_threads(int n) { omp_set_num_threads(n); }
extern "C" int orc_get_threads(void) { return omp_get_max_threads(); }

namespace {
struct ArrRef {
    const void* p;
    int64_t n;
    int kind;  // 0 double, 1 int64 (converted to 1-based), 2 int64 raw
};

ArrRef lookup(const orc_model* m, const std::string& s) {
    auto D = [](const vec& v) { return ArrRef{v.data(), (int64_t)v.size(), 0}; };
    auto I = [](const ivec& v) { return ArrRef{v.data(), (int64_t)v.size(), 1}; };
    if (s == "x") return D(m->x);
    if (s == "y") return D(m->y);
    if (s == "xgll") return D(m->xgll);
    if (s == "wgll") return D(m->wgll);
    if (s == "H") return D(m->H);
    if (s == "W") return D(m->W);
    if (s == "iglob") return I(m->iglob);
    if (s == "damage_idx") return I(m->damage_idx);
    if (s == "M") return D(m->M);
    if (s == "BcLC") return D(m->BcLC);
    if (s == "BcTC") return D(m->BcTC);
    if (s == "FltB") return D(m->FltB);
    if (s == "FltZ") return D(m->FltZ);
    if (s == "FltX") return D(m->FltX);
    if (s == "fo") return D(m->fo);
    if (s == "Vo") return D(m->Vo);
    if (s == "xLf") return D(m->xLf);
    if (s == "cca") return D(m->cca);
    if (s == "ccb") return D(m->ccb);
    if (s == "Seff") return D(m->Seff);
    if (s == "tauo") return D(m->tauo);
    if (s == "XiLf") return D(m->XiLf);
    if (s == "xout") return D(m->xout);
    if (s == "yout") return D(m->yout);
    if (s == "iFlt") return I(m->iFlt);
    if (s == "iBcL") return I(m->iBcL);
    if (s == "iBcT") return I(m->iBcT);
    if (s == "FltIglobBC") return I(m->FltIglobBC);
    if (s == "FltNI") return I(m->FltNI);
    if (s == "out_seis") return I(m->out_seis);
    if (s == "K_ptr") return ArrRef{m->K.ptr.data(), (int64_t)m->K.ptr.size(), 2};
    if (s == "K_col") return ArrRef{m->K.col.data(), (int64_t)m->K.col.size(), 2};
    if (s == "K_val") return D(m->K.val);
    // state
    if (s == "d") return D(m->d);
    if (s == "v") return D(m->v);
    if (s == "a") return D(m->a);
    if (s == "psi") return D(m->psi);
    if (s == "tau") return D(m->tau);
    if (s == "Vf") return D(m->Vf);
    // results
    if (s == "time_") return D(m->out.time_);
    if (s == "Vfmax") return D(m->out.Vfmax);
    if (s == "tStart") return D(m->out.tStart);
    if (s == "tEnd") return D(m->out.tEnd);
    if (s == "hypo") return D(m->out.hypo);
    return ArrRef{nullptr, -1, 0};
}

const std::vector<vec>* lookup_cols(const orc_model* m, const std::string& s) {
    const Results& r = m->out;
    if (s == "seismic_stress") return &r.seismic_stress;
    if (s == "seismic_slipvel") return &r.seismic_slipvel;
    if (s == "seismic_slip") return &r.seismic_slip;
    if (s == "is_stress") return &r.is_stress;
    if (s == "is_slipvel") return &r.is_slipvel;
    if (s == "is_slip") return &r.is_slip;
    if (s == "dSeis") return &r.dSeis;
    if (s == "vSeis") return &r.vSeis;
    if (s == "aSeis") return &r.aSeis;
    if (s == "taubefore") return &r.taubefore;
    if (s == "tauafter") return &r.tauafter;
    if (s == "delfafter") return &r.delfafter;
    return nullptr;
}
}  // namespace

extern "C" int64_t orc_size(const orc_model* m, const char* name) {
    std::string s(name);
    if (s == "regime") return (int64_t)m->out.regime.size();
    if (s == "cg_iters") return (int64_t)m->out.cg_iters.size();
    ArrRef r = lookup(m, s);
    if (r.n >= 0) return r.n;
    auto c = lookup_cols(m, s);
    if (c) {
        int64_t tot = 0;
        for (auto& v : *c) tot += (int64_t)v.size();
        return tot;
    }
    return -1;
}

extern "C" int orc_get(const orc_model* m, const char* name, void* out) {
    std::string s(name);
    if (s == "regime" || s == "cg_iters") {
        const auto& v = (s == "regime") ? m->out.regime : m->out.cg_iters;
        int64_t* o = (int64_t*)out;
        for (size_t k = 0; k < v.size(); ++k) o[k] = v[k];
        return 0;
    }
    ArrRef r = lookup(m, s);
    if (r.n >= 0) {
        if (r.kind == 0) std::memcpy(out, r.p, sizeof(double) * r.n);
        else {
            const int64_t* src = (const int64_t*)r.p;
            int64_t* o = (int64_t*)out;
            for (int64_t k = 0; k < r.n; ++k) o[k] = src[k] + (r.kind == 1 ? 1 : 0);
        }
        return 0;
    }
    auto c = lookup_cols(m, s);
    if (c) {
        double* o = (double*)out;
        for (auto& v : *c) {
            std::memcpy(o, v.data(), sizeof(double) * v.size());
            o += v.size();
        }
        return 0;
    }
    return -1;
}

extern "C" double orc_scalar(const orc_model* m, const char* name) {
    std::string s(name);
    if (s == "dt0") return m->dt0;
    if (s == "dt") return m->dt;
    if (s == "t") return m->t;
    if (s == "it") return (double)m->it;
    if (s == "isolver") return m->isolver;
    if (s == "muMax") return m->muMax;
    if (s == "nglob") return (double)m->nglob;
    if (s == "FltNglob") return (double)m->FltNglob;
    if (s == "Nel") return (double)m->Nel;
    if (s == "NFBC") return (double)(m->NFBC + 1);
    if (s == "dxe") return m->dxe;
    if (s == "dye") return m->dye;
    if (s == "coefint1") return m->coefint1;
    if (s == "coefint2") return m->coefint2;
    if (s == "Total_time") return m->Total_time;
    if (s == "yr2sec") return m->yr2sec;
    if (s == "Vpl") return m->Vpl;
    if (s == "amg_levels") {
        return (double)m->amg.levels.size() + (m->qs_ready ? 1 : 0);
    }
    if (s == "damage_count") return (double)m->damage_count;
    if (s == "amg_complexity") return m->qs_ready ? m->amg.operator_complexity() : -1.0;
    if (s == "amg_coarse") return (double)m->amg.nc;
    if (s == "n_events") return (double)m->out.tStart.size();
    return NAN;
}

extern "C" int orc_state(const orc_model* m, const char* name, void* out) { return orc_get(m, name, out); }

extern "C" int orc_set_state(orc_model* m, const char* name, const void* in) {
    std::string s(name);
    vec* dst = nullptr;
    if (s == "d") dst = &m->d;
    else if (s == "v") dst = &m->v;
    else if (s == "a") dst = &m->a;
    else if (s == "psi") dst = &m->psi;
    else if (s == "tau") dst = &m->tau;
    if (dst) {
        std::memcpy(dst->data(), in, sizeof(double) * dst->size());
        return 0;
    }
    const double v = *(const double*)in;
    if (s == "t") m->t = v;
    else if (s == "dt") m->dt = v;
    else if (s == "isolver") m->isolver = (int)v;
    else return -1;
    return 0;
}

extern "C" int orc_set_damage(orc_model* m, const int64_t* idx, int64_t n, double factor) {
    m->damage_el.clear();
    for (int64_t k = 0; k < n; ++k) {
        if (idx[k] < 1 || idx[k] > m->Nel) return -1;
        m->damage_el.push_back(idx[k] - 1);
    }
    m->damage_factor = factor;
    return 0;
}

extern "C" void orc_damage_evolve(orc_model* m) { orc::damage_evolve(m); }
