// C ABI of libeqc (include/eqc.h): model upload, reference-numbering <-> layout
// permutation, host-array entry points.
#include "model.h"
#include "learn.h"
#include "host_par.h"
#include <cmath>
#include <cstring>
#include <cstdlib>
#include <algorithm>
#include <unordered_map>
#include <chrono>

namespace eqc {

Handle::~Handle() {
    destroy_graphs(*this);
    mg_destroy(*this);
    delete net;
    if (h_ctrl) cudaFreeHost(h_ctrl);
    if (h_scal) cudaFreeHost(h_scal);
    if (h_cg) cudaFreeHost(h_cg);
    for (cudaStream_t c : cap_streams)
        if (c) cudaStreamDestroy(c);
    for (cudaStream_t c : {side_stream, side_stream2})
        if (c) cudaStreamDestroy(c);
    for (cudaEvent_t e : {ev_fork, ev_join, ev_fork2, ev_join2})
        if (e) cudaEventDestroy(e);
    if (own_stream) cudaStreamDestroy(own_stream);
}

static void fail_if(bool cond, const std::string& msg) {
    if (cond) throw Error(EQC_E_ARG, msg);
}

// Diagonal of K in the layout (Kassemble.jl:50-58 with i=k, j=l).
static std::vector<double> diag_K(const Handle& h, const double* W) {
    const Layout& L = h.L;
    std::vector<double> dg(L.size(), 0.0);
    const double* H = h.H;
    for (int ey = 0; ey < L.NelY; ++ey)
        for (int ex = 0; ex < L.NelX; ++ex) {
            const double* w = W + ((int64_t)ey * L.NelX + ex) * 25;
            for (int j = 0; j < 5; ++j)
                for (int i = 0; i < 5; ++i) {
                    double t1 = 0, t2 = 0;
                    for (int p = 0; p < 5; ++p) {
                        t1 += w[i + 5 * p] * h.c2 * H[j + 5 * p] * H[j + 5 * p];
                        t2 += w[p + 5 * j] * h.c1 * H[i + 5 * p] * H[i + 5 * p];
                    }
                    dg[(int64_t)(4 * ey + j) * L.ld + 4 * ex + i] += t1 + t2;
                }
        }
    return dg;
}

// W (FP64, FP32, and both copies padded per element for TMA element tiles) and the diagonal
// of K on the device.  Buffers are allocated once; a later call (damage evolution) rewrites
// them in place, so the tensor maps of the element data stay valid.
static void load_element_data(Handle& h, const double* W) {
    const Layout& L = h.L;
    cudaStream_t s = h.stream;
    const int64_t Nel = (int64_t)L.NelX * L.NelY;
    const size_t nW = (size_t)25 * Nel;
    const bool first = h.W64.p == nullptr;
    if (first) {
        h.W64.alloc(nW);
        h.W32.alloc(nW);
        h.W32p.alloc((size_t)WPad<float>::v * Nel);
        h.W64p.alloc((size_t)WPad<double>::v * Nel);
        h.diag64.alloc(L.size());
        h.diag32.alloc(L.size());
    }
    if (!h.W32lo.p) h.W32lo.alloc((size_t)WPad<float>::v * Nel);
    std::vector<float> w32(nW);
    for (size_t k = 0; k < nW; ++k) w32[k] = (float)W[k];
    const int p32 = WPad<float>::v, p64 = WPad<double>::v;
    std::vector<float> a((size_t)p32 * Nel, 0.f), alo((size_t)p32 * Nel, 0.f);
    std::vector<double> b((size_t)p64 * Nel, 0.0);
    for (int64_t e = 0; e < Nel; ++e)
        for (int q = 0; q < 25; ++q) {
            a[(size_t)p32 * e + q] = w32[(size_t)25 * e + q];
            alo[(size_t)p32 * e + q] = (float)(W[(size_t)25 * e + q] - (double)w32[(size_t)25 * e + q]);
            b[(size_t)p64 * e + q] = W[(size_t)25 * e + q];
        }
    std::vector<double> dg = diag_K(h, W);
    for (int64_t i = 0; i < L.size(); ++i)   // fault row and row padding are not part of the system
        if (i < L.ld || (i % L.ld) >= L.nx) dg[i] = 1.0;
    std::vector<float> dg32(dg.begin(), dg.end());
    h.W64.upload(W, nW, s);
    h.W32.upload(w32.data(), nW, s);
    h.W32p.upload(a.data(), a.size(), s);
    h.W32lo.upload(alo.data(), alo.size(), s);
    h.W64p.upload(b.data(), b.size(), s);
    h.diag64.upload(dg.data(), dg.size(), s);
    h.diag32.upload(dg32.data(), dg32.size(), s);
    EQC_CUDA(cudaStreamSynchronize(s));
}

void damage_evolve(Handle& h) {
    if (h.damage_el.empty()) return;
    const int64_t Nel = (int64_t)h.L.NelX * h.L.NelY;
    std::vector<double> W((size_t)25 * Nel);
    h.W64.download(W.data(), W.size(), h.stream);
    EQC_CUDA(cudaStreamSynchronize(h.stream));
    for (int64_t e : h.damage_el)   // damageEvol!: W[:, :, damage_idx] .*= factor
        for (int q = 0; q < 25; ++q) W[(size_t)25 * e + q] *= h.damage_factor;
    load_element_data(h, W.data());
    if (h.opt.precond == EQC_PC_AMG) mg_build(h);   // K changed: new Galerkin hierarchy and bounds
    invalidate_residual(h);   // carried residual, extrapolation history and K d refer to the old K
    destroy_graphs(h);        // the step graphs hold the old hierarchy's buffers
    h.damage_count += 1;
    h.gen += 1;
}

// Reference node id (0-based) of lexicographic node (ix, iy) by MeshBox.jl:27-88's numbering:
// a node gets its id from the first element (in element order) that contains it, in the order
// that element creates its new nodes.
static int64_t meshbox_id(int64_t ix, int64_t iy, int64_t nx) {
    const int64_t exc = ix == 0 ? 0 : (ix - 1) / 4, i = ix - 4 * exc;
    const int64_t eyc = iy == 0 ? 0 : (iy - 1) / 4, j = iy - 4 * eyc;
    const int64_t rowstart = eyc == 0 ? 0 : 5 * nx + (eyc - 1) * 4 * nx;
    if (eyc == 0 && exc == 0) return i + 5 * j;
    if (eyc == 0) return 25 + 20 * (exc - 1) + (i - 1) + 4 * j;
    if (exc == 0) return rowstart + i + 5 * (j - 1);
    return rowstart + 20 + 16 * (exc - 1) + (i - 1) + 4 * (j - 1);
}

// mat == nullptr: the element data come from the caller (iglob, W, M of setParameters);
// otherwise the mesh numbering is MeshBox's and W, M, 1/M and diag(K) are built on the device.
static void create(Handle& h, const eqc_model& m, const eqc_material* mat) {
    fail_if(m.NGLL != 5, "NGLL must be 5");
    fail_if(m.NelX < 1 || m.NelY < 1 || m.Nel != m.NelX * m.NelY, "Nel != NelX*NelY");
    fail_if(m.FltNglob != 4 * m.NelX + 1, "FltNglob != 4*NelX+1");
    fail_if(m.nglob != (4 * m.NelX + 1) * (4 * m.NelY + 1), "nglob != (4NelX+1)(4NelY+1)");
    fail_if(!m.H || !m.iFlt, "null model array");
    if (mat) {
        fail_if(!mat->xgll || !mat->wgll, "eqc_material needs the GLL nodes and weights");
        fail_if(mat->rule < 0 || mat->rule > 2, "eqc_material.rule must be 0, 1 or 2");
        fail_if(mat->rule == 2 && !(mat->trap_z1 > 0), "eqc_material.trap_z1 must be positive");
    } else {
        fail_if(!m.iglob || !m.W || !m.M, "null model array");
    }
    fail_if(m.IDstate != 2, "only IDstate = 2 (aging law, log form) is on the hot path");
    fail_if(m.ETA != 0.0, "Kelvin-Voigt damping (ETA != 0) is not on the hot path");
    EQC_CUDA(cudaSetDevice(h.opt.device));
    h.fuse = std::getenv("EQC_NO_FUSE") == nullptr;
    EQC_CUDA(cudaStreamCreateWithFlags(&h.own_stream, cudaStreamNonBlocking));
    for (cudaStream_t* c : {&h.side_stream, &h.side_stream2})
        EQC_CUDA(cudaStreamCreateWithFlags(c, cudaStreamNonBlocking));
    for (cudaEvent_t* e : {&h.ev_fork, &h.ev_join, &h.ev_fork2, &h.ev_join2})
        EQC_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
    h.stream = h.own_stream;
    cudaStream_t s = h.stream;
    Layout& L = h.L;
    L.NelX = (int)m.NelX;
    L.NelY = (int)m.NelY;
    L.nx = 4 * L.NelX + 1;
    L.ny = 4 * L.NelY + 1;
    L.ld = (L.nx + 7) / 8 * 8;   // rows start on 32-byte (FP32) / 64-byte (FP64) boundaries
    h.nglob = m.nglob;
    h.Nel = m.Nel;
    h.dxe = m.dxe;
    h.dye = m.dye;
    const double dx_dxi = 0.5 * m.dxe, dy_deta = 0.5 * m.dye, jac = dx_dxi * dy_deta;
    h.c1 = jac / (dx_dxi * dx_dxi);
    h.c2 = jac / (dy_deta * dy_deta);
    h.Vpl = m.Vpl;
    h.Vthres = m.Vthres;
    h.Vevne = m.Vevne;
    h.dt0 = m.dt0;
    h.Total_time = m.Total_time;
    h.yr2sec = (double)m.yr2sec;
    std::memcpy(h.H, m.H, sizeof(h.H));
    set_H(h.H, s);
    set_H_df(h.H, s);
    {   // the double-float apply uses the even-odd form: H must be centro-antisymmetric
        double hmax = 0.0, asym = 0.0;
        for (int k = 0; k < 25; ++k) hmax = std::max(hmax, std::fabs(h.H[k]));
        for (int i = 0; i < 5; ++i)
            for (int j = 0; j < 5; ++j) asym = std::max(asym, std::fabs(h.H[i + 5 * j] + h.H[(4 - i) + 5 * (4 - j)]));
        h.df_ok = asym <= 1e-12 * hmax && std::getenv("EQC_NO_DF") == nullptr;
    }
    using clk = std::chrono::steady_clock;
    auto ms_since = [](clk::time_point t) { return std::chrono::duration<double, std::milli>(clk::now() - t).count(); };
    auto t0 = clk::now();

    // reference node -> layout index, from the connectivity (or MeshBox's numbering rule)
    h.ref2lay.resize(m.nglob);
    constexpr int64_t CH = 1 << 14;   // nodes per work item of the host loops
    parallel_for((m.nglob + CH - 1) / CH, [&](int64_t c) {
        std::fill(h.ref2lay.begin() + c * CH, h.ref2lay.begin() + std::min(m.nglob, (c + 1) * CH), (int64_t)-1);
    }, 1);
    if (mat) {   // MeshBox's numbering is a bijection of the nx x ny nodes: rows write disjoint entries
        parallel_for(L.ny, [&](int64_t iy) {
            for (int64_t ix = 0; ix < L.nx; ++ix) h.ref2lay[meshbox_id(ix, iy, L.nx)] = iy * L.ld + ix;
        });
    }
    for (int64_t e = 0; e < (mat ? 0 : m.Nel); ++e) {
        const int ex = (int)(e % m.NelX), ey = (int)(e / m.NelX);
        for (int j = 0; j < 5; ++j)
            for (int i = 0; i < 5; ++i) {
                const int64_t ref = m.iglob[i + 5 * j + 25 * e] - 1;
                fail_if(ref < 0 || ref >= m.nglob, "iglob entry out of range");
                const int64_t lay = (int64_t)(4 * ey + j) * L.ld + 4 * ex + i;
                fail_if(h.ref2lay[ref] >= 0 && h.ref2lay[ref] != lay, "iglob is not a structured box mesh");
                h.ref2lay[ref] = lay;
            }
    }
    {
        const int64_t nc = (m.nglob + CH - 1) / CH;
        std::vector<char> hole(nc, 0);
        parallel_for(nc, [&](int64_t c) {
            for (int64_t g = c * CH; g < std::min(m.nglob, (c + 1) * CH); ++g) hole[c] |= h.ref2lay[g] < 0;
        }, 1);
        for (char x : hole) fail_if(x != 0, "iglob does not cover every node");
    }
    const int Nf = (int)m.FltNglob;
    for (int k = 0; k < Nf; ++k)
        fail_if(h.ref2lay[m.iFlt[k] - 1] != k, "iFlt must run along the y = 0 edge from x = -LX (BoundaryMatrix 'B')");

    h.setup_ms[0] = ms_since(t0);   // node numbering
    t0 = clk::now();
    // element data
    if (mat) setup_element_data_device(h, *mat);
    else load_element_data(h, m.W);
    EQC_CUDA(cudaStreamSynchronize(s));
    h.setup_ms[1] = ms_since(t0);   // W and its copies (and diag K on the host path)
    t0 = clk::now();

    // node arrays
    const int64_t N = L.size();
    for (DBuf<double>* b : {&h.M, &h.d, &h.v, &h.a, &h.dPre, &h.tmp64a, &h.tmp64b, &h.tmp64c, &h.r64, &h.z64, &h.p64,
                             &h.q64, &h.Kd})
        b->alloc(N);
    for (DBuf<float>* b : {&h.r32, &h.z32, &h.p32, &h.q32, &h.x32, &h.g32}) b->alloc(N);
    if (h.opt.precision == EQC_MIXED && std::getenv("EQC_NO_DF_UPDATE") == nullptr) {
        h.dx64.alloc(N);    // the intermediate reliable updates' correction and its K dx
        h.kdx64.alloc(N);
    }
    if (!mat) {
        std::vector<double> Mlay(N, 1.0);
        for (int64_t g = 0; g < m.nglob; ++g) Mlay[h.ref2lay[g]] = m.M[g];
        h.M.upload(Mlay.data(), N, s);
        std::vector<double> inv(N);
        for (int64_t i = 0; i < N; ++i) inv[i] = 1.0 / Mlay[i];
        h.invM.alloc(N);
        h.invM.upload(inv.data(), N, s);
        EQC_CUDA(cudaStreamSynchronize(s));
    }

    // boundary lists
    auto to_lay = [&](const int64_t* idx, int64_t n) {
        std::vector<int64_t> o(n);
        for (int64_t k = 0; k < n; ++k) {
            fail_if(idx[k] < 1 || idx[k] > m.nglob, "node index out of range");
            o[k] = h.ref2lay[idx[k] - 1];
        }
        return o;
    };
    auto up_i = [&](DBuf<int64_t>& b, const std::vector<int64_t>& v) {
        b.alloc(std::max<size_t>(v.size(), 1));
        b.upload(v.data(), v.size(), s);
    };
    auto up_d = [&](DBuf<double>& b, const double* v, int64_t n) {
        b.alloc(std::max<int64_t>(n, 1));
        b.upload(v, n, s);
    };
    std::vector<int64_t> lBcL = to_lay(m.iBcL, m.n_iBcL), lBcT = to_lay(m.iBcT, m.n_iBcT);
    std::vector<int64_t> lCreep = to_lay(m.FltIglobBC, m.n_FltIglobBC), lSeis = to_lay(m.out_seis, m.n_out_seis);
    {   // per-node boundary operations (k_dyn_bc_nodes), nodes in first-appearance order
        std::vector<int64_t> node;
        std::vector<int> ops;
        std::vector<double> cl, ct;
        std::unordered_map<int64_t, size_t> at;
        auto slot = [&](int64_t g) {
            auto it = at.find(g);
            if (it != at.end()) return it->second;
            at[g] = node.size();
            node.push_back(g);
            ops.push_back(0);
            cl.push_back(0.0);
            ct.push_back(0.0);
            return node.size() - 1;
        };
        for (int64_t g : lCreep) ops[slot(g)] |= 1;
        bool dup = false;   // a node twice in the left or the top list: keep the list kernel
        for (size_t k = 0; k < lBcL.size(); ++k) {
            const size_t q = slot(lBcL[k]);
            dup = dup || (ops[q] & 2);
            ops[q] |= 2;
            cl[q] = m.BcLC[k];
        }
        for (size_t k = 0; k < lBcT.size(); ++k) {
            const size_t q = slot(lBcT[k]);
            dup = dup || (ops[q] & 4);
            ops[q] |= 4;
            ct[q] = m.BcTC[k];
        }
        if (!dup && !node.empty()) {
            h.bcNode.alloc(node.size());
            h.bcNode.upload(node.data(), node.size(), s);
            h.bcOps.alloc(ops.size());
            h.bcOps.upload(ops.data(), ops.size(), s);
            h.bcL.alloc(cl.size());
            h.bcL.upload(cl.data(), cl.size(), s);
            h.bcT.alloc(ct.size());
            h.bcT.upload(ct.data(), ct.size(), s);
            h.nBcNodes = (int)node.size();
            EQC_CUDA(cudaStreamSynchronize(s));
        }
    }
    up_i(h.iBcL, lBcL);
    up_i(h.iBcT, lBcT);
    up_i(h.iCreep, lCreep);
    up_i(h.iSeis, lSeis);
    up_d(h.BcLC, m.BcLC, m.n_iBcL);
    up_d(h.BcTC, m.BcTC, m.n_iBcT);
    h.nBcL = (int)m.n_iBcL;
    h.nBcT = (int)m.n_iBcT;
    h.nCreep = (int)m.n_FltIglobBC;
    h.nSeis = (int)m.n_out_seis;
    fail_if(h.nSeis > 32, "at most 32 receivers");
    h.seis.alloc(3 * std::max(h.nSeis, 1));
    if (mat) setup_node_data_device(h, *mat, lBcL, m.BcLC, lBcT, m.BcTC);   // M (+ boundary terms), 1/M, diag K

    // fault arrays (fault order == layout row 0)
    FaultDev& F = h.F;
    F.Nf = Nf;
    std::vector<int> creep(Nf, 0), bcflag(Nf, 0);
    for (auto g : lCreep)
        if (g < Nf) bcflag[g] = 1;
    // iFBC (main.jl:185) is the creeping set; it must be a prefix of the fault order.
    for (int k = 0; k < Nf; ++k) creep[k] = bcflag[k];
    int nfbc = 0;
    while (nfbc < Nf && creep[nfbc]) ++nfbc;
    for (int k = nfbc; k < Nf; ++k) fail_if(creep[k], "creeping fault nodes must be the deepest ones");
    F.NFBC0 = nfbc;
    h.creep_prefix = true;
    for (auto g : lCreep) h.creep_prefix = h.creep_prefix && g < nfbc;
    {   // the mixed method's four-kernel dynamic step needs iBcL on column ix = 0 and iBcT on row
        // iy = ny - 1, each node listed once (the reference's BoundaryMatrix edges x = -LX, y = LY)
        std::vector<double> cL(L.ny, 0.0), cT(L.nx, 0.0);
        std::vector<int> hL(L.ny, 0), hT(L.nx, 0);
        bool ok = h.creep_prefix;
        for (size_t k = 0; k < lBcL.size() && ok; ++k) {
            const int64_t g = lBcL[k], iy = g / L.ld, ix = g % L.ld;
            ok = ix == 0 && iy < L.ny && !hL[iy];
            if (ok) { hL[iy] = 1; cL[iy] = m.BcLC[k]; }
        }
        for (size_t k = 0; k < lBcT.size() && ok; ++k) {
            const int64_t g = lBcT[k], iy = g / L.ld, ix = g % L.ld;
            ok = iy == L.ny - 1 && ix < L.nx && !hT[ix];
            if (ok) { hT[ix] = 1; cT[ix] = m.BcTC[k]; }
        }
        h.nm_fused = ok && std::getenv("EQC_NO_NM_FUSE") == nullptr;
        if (h.nm_fused) {
            h.edgeL0has = hL[0];
            h.edgeL0 = cL[0];
            h.fault_count.alloc(1);
            h.fault_part.alloc(3 * (size_t)((Nf + 31) / 32));
            up_d(h.edgeL, cL.data(), L.ny);
            up_d(h.edgeT, cT.data(), L.nx);
            h.edgeLhas.alloc(L.ny);
            h.edgeLhas.upload(hL.data(), L.ny, s);
            h.edgeThas.alloc(L.nx);
            h.edgeThas.upload(hT.data(), L.nx, s);
            EQC_CUDA(cudaStreamSynchronize(s));
        }
    }
    for (DBuf<double>* b : {&F.fo, &F.Vo, &F.xLf, &F.cca, &F.ccb, &F.Seff, &F.tauo, &F.XiLf, &F.FltB, &F.FltZ, &F.FltX,
                            &F.Mf, &F.psi, &F.psi1, &F.psi2, &F.tau, &F.tau1, &F.tau2, &F.Vf, &F.Vf0, &F.Vf1, &F.Vf2,
                            &F.FltVfree, &F.vPre, &F.Flast})
        b->alloc(Nf);
    F.fo.upload(m.fo, Nf, s);
    F.Vo.upload(m.Vo, Nf, s);
    F.xLf.upload(m.xLf, Nf, s);
    F.cca.upload(m.cca, Nf, s);
    F.ccb.upload(m.ccb, Nf, s);
    F.Seff.upload(m.Seff, Nf, s);
    F.tauo.upload(m.tauo, Nf, s);
    F.XiLf.upload(m.XiLf, Nf, s);
    F.FltB.upload(m.FltB, Nf, s);
    F.FltZ.upload(m.FltZ, Nf, s);
    F.FltX.upload(m.FltX, Nf, s);
    std::vector<double> Mf(Nf);
    if (mat) {   // fault order == layout row 0
        h.M.download(Mf.data(), Nf, s);
        EQC_CUDA(cudaStreamSynchronize(s));
    } else {
        for (int k = 0; k < Nf; ++k) Mf[k] = m.M[m.iFlt[k] - 1];
    }
    F.Mf.upload(Mf.data(), Nf, s);
    F.creep.alloc(Nf);
    F.creep.upload(creep.data(), Nf, s);
    h.bcflag.alloc(Nf);
    h.bcflag.upload(bcflag.data(), Nf, s);
    h.h_tauo.assign(m.tauo, m.tauo + Nf);
    h.h_FltX.assign(m.FltX, m.FltX + Nf);

    EQC_CUDA(cudaStreamSynchronize(s));
    h.setup_ms[2] = ms_since(t0);   // node and fault arrays (M, 1/M; diag K on the device path)
    t0 = clk::now();
    // control, reductions
    h.ctrl.alloc(1);
    EQC_CUDA(cudaStreamSynchronize(s));
    tma_init(h);
    EQC_CUDA(cudaMallocHost(&h.h_ctrl, sizeof(Ctrl)));
    std::memset(h.h_ctrl, 0, sizeof(Ctrl));
    h.red_part.alloc(4096);
    h.red_count.alloc(64);
    h.scal.alloc(16);
    EQC_CUDA(cudaMallocHost(&h.h_scal, sizeof(double) * 16));
    h.cg.alloc(1);
    EQC_CUDA(cudaMallocHost(&h.h_cg, sizeof(CGState)));
    {   // device logs of batched steps (512 steps, a receiver record every 10th)
        const int nb = std::max(h.opt.step_batch, 512);
        h.log_t.alloc(nb);
        h.log_vf.alloc(nb);
        h.log_seis.alloc((size_t)(nb / 10 + 2) * 3 * std::max(h.nSeis, 1));
    }
    std::memset(h.h_cg, 0, sizeof(CGState));
    EQC_CUDA(cudaStreamSynchronize(s));
    h.setup_ms[3] = ms_since(t0);
    t0 = clk::now();
    if (h.opt.precond == EQC_PC_AMG) mg_build(h);
    EQC_CUDA(cudaStreamSynchronize(s));
    h.setup_ms[4] = ms_since(t0);   // multigrid hierarchy (host Galerkin products, device bounds)
}

// Reference numbering <-> node layout on the host's cores: ref2lay is one-to-one, so the
// chunks write disjoint entries (the layout's row padding stays zero).
static void to_layout(const Handle& h, const double* ref, std::vector<double>& lay) {
    constexpr int64_t CH = 1 << 14;   // nodes per work item
    const int64_t N = h.L.size();
    lay.resize(N);
    parallel_for((N + CH - 1) / CH, [&](int64_t c) {
        std::fill(lay.begin() + c * CH, lay.begin() + std::min(N, (c + 1) * CH), 0.0);
    }, 1);
    parallel_for((h.nglob + CH - 1) / CH, [&](int64_t c) {
        for (int64_t g = c * CH; g < std::min(h.nglob, (c + 1) * CH); ++g) lay[h.ref2lay[g]] = ref[g];
    }, 1);
}
static void from_layout(const Handle& h, const std::vector<double>& lay, double* ref) {
    constexpr int64_t CH = 1 << 14;
    parallel_for((h.nglob + CH - 1) / CH, [&](int64_t c) {
        for (int64_t g = c * CH; g < std::min(h.nglob, (c + 1) * CH); ++g) ref[g] = lay[h.ref2lay[g]];
    }, 1);
}

// The same maps on the device, for the state transfers of eqc_get_state / eqc_set_state: the
// field crosses PCIe / C2C in the reference numbering and is permuted by a kernel (the padding
// entries of the layout are zero).
__global__ void k_ref_to_layout(const double* __restrict__ ref, const int* __restrict__ map, int64_t n,
                                double* __restrict__ lay) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
        lay[map[g]] = ref[g];
}
__global__ void k_layout_to_ref(const double* __restrict__ lay, const int* __restrict__ map, int64_t n,
                                double* __restrict__ ref) {
    for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += (int64_t)gridDim.x * blockDim.x)
        ref[g] = lay[map[g]];
}
static void ensure_ref_maps(Handle& h) {
    if (h.d_ref2lay.p) return;
    fail_if(h.L.size() > INT32_MAX, "node layout too large for 32-bit indices");
    std::vector<int> m32(h.nglob);
    for (int64_t g = 0; g < h.nglob; ++g) m32[g] = (int)h.ref2lay[g];
    h.d_ref2lay.alloc(h.nglob);
    h.d_ref2lay.upload(m32.data(), m32.size(), h.stream);
    h.ref_stage.alloc(h.nglob);
    EQC_CUDA(cudaStreamSynchronize(h.stream));
}
static int ref_blocks(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 8 * 152); }

static thread_local std::string g_create_err;
void set_thread_error(const std::string& msg) { g_create_err = msg; }

}  // namespace eqc

using namespace eqc;


template <class F>
static eqc_status guarded(eqc_handle* H, F&& f) {
    try {
        f();
        return EQC_OK;
    } catch (const Error& e) {
        if (H) H->h.err = e.what();
        return e.code;
    } catch (const std::exception& e) {
        if (H) H->h.err = e.what();
        return EQC_E_ARG;
    }
}

extern "C" {

void eqc_default_options(eqc_options* o) {
    std::memset(o, 0, sizeof(*o));
    o->precision = EQC_FP64;
    o->precond = EQC_PC_AMG;
    o->guess = EQC_GUESS_PREVIOUS;
    o->tol_rule = EQC_TOL_RHS;
    o->cg_tol = 1e-8;
    o->cg_maxit = 0;
    o->device = 0;
    o->use_graphs = 1;
    o->verbose = 0;
}


eqc_status eqc_create(const eqc_model* model, const eqc_options* opt, eqc_handle** out) {
    if (!model || !out) return EQC_E_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        g_create_err = "no CUDA device";
        return EQC_E_NOGPU;
    }
    eqc_handle* H = new eqc_handle();
    if (opt) H->h.opt = *opt;
    else eqc_default_options(&H->h.opt);
    eqc_status st = guarded(H, [&] { create(H->h, *model, nullptr); });
    if (st != EQC_OK) {
        g_create_err = H->h.err;
        delete H;
        return st;
    }
    *out = H;
    return EQC_OK;
}

eqc_status eqc_create_structured(const eqc_model* model, const eqc_material* mat, const eqc_options* opt,
                                 eqc_handle** out) {
    if (!model || !mat || !out) return EQC_E_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        g_create_err = "no CUDA device";
        return EQC_E_NOGPU;
    }
    eqc_handle* H = new eqc_handle();
    if (opt) H->h.opt = *opt;
    else eqc_default_options(&H->h.opt);
    eqc_status st = guarded(H, [&] { create(H->h, *model, mat); });
    if (st != EQC_OK) {
        g_create_err = H->h.err;
        delete H;
        return st;
    }
    *out = H;
    return EQC_OK;
}

eqc_status eqc_destroy(eqc_handle* H) {
    if (!H) return EQC_E_ARG;
    delete H;
    return EQC_OK;
}

const char* eqc_last_error(const eqc_handle* H) { return H ? H->h.err.c_str() : g_create_err.c_str(); }

eqc_status eqc_apply_K(eqc_handle* H, const double* x, double* y) {
    if (!H || !x || !y) return EQC_E_ARG;
    return guarded(H, [&] {
        Handle& h = H->h;
        std::vector<double> xl, yl(h.L.size());
        to_layout(h, x, xl);
        h.tmp64a.upload(xl.data(), xl.size(), h.stream);
        apply_K<double>(h.tmp64a.p, h.tmp64b.p, args64(h), 1.0, 0, h.stream);
        h.tmp64b.download(yl.data(), yl.size(), h.stream);
        EQC_CUDA(cudaStreamSynchronize(h.stream));
        check_apply_err(h);
        from_layout(h, yl, y);
    });
}

eqc_status eqc_qs_solve(eqc_handle* H, const double* F_fault, double* d_inout, double tol, int32_t maxit,
                        int32_t* iters, double* relres) {
    if (!H || !F_fault || !d_inout) return EQC_E_ARG;
    return guarded(H, [&] {
        Handle& h = H->h;
        const int64_t N = h.L.size();
        // keep the time-loop displacement intact
        EQC_CUDA(cudaMemcpyAsync(h.dPre.p, h.d.p, sizeof(double) * N, cudaMemcpyDeviceToDevice, h.stream));
        std::vector<double> dl;
        to_layout(h, d_inout, dl);
        for (int k = 0; k < h.F.Nf; ++k) dl[k] = F_fault[k];
        h.d.upload(dl.data(), N, h.stream);
        double rr = 0;
        int it = qs_solve_device(h, tol, maxit, &rr);
        h.d.download(dl.data(), N, h.stream);
        EQC_CUDA(cudaMemcpyAsync(h.d.p, h.dPre.p, sizeof(double) * N, cudaMemcpyDeviceToDevice, h.stream));
        EQC_CUDA(cudaStreamSynchronize(h.stream));
        from_layout(h, dl, d_inout);
        if (iters) *iters = it;
        if (relres) *relres = rr;
        if (it < 0) throw Error(EQC_E_CG, "CG reached maxit");
    });
}

eqc_status eqc_slrFunc(eqc_handle* H, const double* psi, double* psi1, const double* Vf, double* Vf1,
                       const double* tau1, double dt) {
    if (!H || !psi || !psi1 || !Vf || !Vf1 || !tau1) return EQC_E_ARG;
    return guarded(H, [&] { fault_slrFunc(H->h, psi, psi1, Vf, Vf1, tau1, dt); });
}

eqc_status eqc_FBC(eqc_handle* H, double* psi1, double* Vf1, double* tau1, double* psi2, double* Vf2, double* tau2,
                   const double* psi, const double* Vf, const double* FltVfree, double dt, int64_t* fail_node) {
    if (!H || !psi1 || !Vf1 || !tau1 || !psi2 || !Vf2 || !tau2 || !psi || !Vf || !FltVfree) return EQC_E_ARG;
    return guarded(H, [&] {
        int f = fault_FBC(H->h, psi1, Vf1, tau1, psi2, Vf2, tau2, psi, Vf, FltVfree, dt);
        if (fail_node) *fail_node = f;
        if (f) throw Error(EQC_E_NR, "NR SEARCH FAILED at fault node " + std::to_string(f));
    });
}

eqc_status eqc_dtevol(eqc_handle* H, double dt, double dtmin, const double* Vf, int32_t isolver, double* dt_out) {
    if (!H || !Vf || !dt_out) return EQC_E_ARG;
    return guarded(H, [&] { *dt_out = fault_dtevol(H->h, dt, dtmin, Vf, isolver); });
}

eqc_status eqc_init(eqc_handle* H, double V_init) {
    if (!H || !(V_init > 0)) return EQC_E_ARG;
    return guarded(H, [&] { init_state(H->h, V_init); });
}

eqc_status eqc_run(eqc_handle* H, int64_t max_steps, double t_end, eqc_run_stats* stats) {
    if (!H) return EQC_E_ARG;
    return guarded(H, [&] { run_steps(H->h, max_steps, t_end, stats); });
}

static DBuf<double>* state_buf(Handle& h, const std::string& s, bool& fault) {
    fault = false;
    if (s == "d") return &h.d;
    if (s == "v") return &h.v;
    if (s == "a") return &h.a;
    fault = true;
    if (s == "psi") return &h.F.psi;
    if (s == "tau") return &h.F.tau;
    return nullptr;
}

eqc_status eqc_get_state(eqc_handle* H, const char* name, double* out) {
    if (!H || !name || !out) return EQC_E_ARG;
    return guarded(H, [&] {
        Handle& h = H->h;
        bool fault;
        DBuf<double>* b = state_buf(h, name, fault);
        if (!b) throw Error(EQC_E_ARG, std::string("unknown state ") + name);
        if (b == &h.v || b == &h.a) materialize_dyn_state(h);
        if (fault) {
            b->download(out, h.F.Nf, h.stream);
        } else {
            ensure_ref_maps(h);
            k_layout_to_ref<<<ref_blocks(h.nglob), 256, 0, h.stream>>>(b->p, h.d_ref2lay.p, h.nglob, h.ref_stage.p);
            EQC_CHECK_LAUNCH();
            count_launch();
            h.ref_stage.download(out, h.nglob, h.stream);
        }
        EQC_CUDA(cudaStreamSynchronize(h.stream));
    });
}

eqc_status eqc_set_state(eqc_handle* H, const char* name, const double* in) {
    if (!H || !name || !in) return EQC_E_ARG;
    return guarded(H, [&] {
        Handle& h = H->h;
        bool fault;
        DBuf<double>* b = state_buf(h, name, fault);
        if (!b) throw Error(EQC_E_ARG, std::string("unknown state ") + name);
        if (b == &h.v || b == &h.a) materialize_dyn_state(h);   // the other one stays valid
        if (fault) {
            b->upload(in, h.F.Nf, h.stream);
        } else {
            ensure_ref_maps(h);
            h.ref_stage.upload(in, h.nglob, h.stream);
            b->zero(h.stream);
            k_ref_to_layout<<<ref_blocks(h.nglob), 256, 0, h.stream>>>(h.ref_stage.p, h.d_ref2lay.p, h.nglob, b->p);
            EQC_CHECK_LAUNCH();
            count_launch();
        }
        invalidate_residual(h);
        EQC_CUDA(cudaStreamSynchronize(h.stream));
    });
}

eqc_status eqc_get_scalar(eqc_handle* H, const char* name, double* out) {
    if (!H || !name || !out) return EQC_E_ARG;
    return guarded(H, [&] {
        Handle& h = H->h;
        const std::string s(name);
        const Ctrl& C = *h.h_ctrl;
        if (s == "t") *out = C.t;
        else if (s == "apply_variant") *out = h.opt.apply_variant;
        else if (s == "damage_events") *out = (double)h.damage_count;
        else if (s == "setup_ms_numbering") *out = h.setup_ms[0];
        else if (s == "setup_ms_elements") *out = h.setup_ms[1];
        else if (s == "setup_ms_nodes") *out = h.setup_ms[2];
        else if (s == "setup_ms_other") *out = h.setup_ms[3];
        else if (s == "setup_ms_hierarchy") *out = h.setup_ms[4];
        else if (s == "pdl_edges") *out = (double)h.pdl_edges;
        else if (s == "tma_wait_polls") *out = h.tma_wait_polls;
        else if (s == "time_capacity") *out = (double)h.cap_time;
        else if (s == "reliable_delta") *out = h.opt.reliable_delta > 0 ? h.opt.reliable_delta : 1e-3;
        else if (s == "dt") *out = C.dt;
        else if (s == "isolver") *out = C.isolver;
        else if (s == "it") *out = (double)C.it;
        else if (s == "cg_iters" || s == "qs_solves" || s == "cg_updates" || s == "cg_carried" ||
                 s == "guess_tried" || s == "guess_kept" || s == "cg_restarts") {
            Ctrl c;
            EQC_CUDA(cudaMemcpyAsync(&c, h.ctrl.p, sizeof(Ctrl), cudaMemcpyDeviceToHost, h.stream));
            EQC_CUDA(cudaStreamSynchronize(h.stream));
            *out = (double)(s == "cg_iters" ? c.cg_iters : s == "qs_solves" ? c.cg_solves
                            : s == "cg_updates" ? c.cg_updates : s == "cg_carried" ? c.cg_carried
                            : s == "guess_tried" ? c.guess_tried : s == "guess_kept" ? c.guess_kept
                            : c.cg_restarts);
        }
        else throw Error(EQC_E_ARG, "unknown scalar " + s);
    });
}

eqc_status eqc_set_scalar(eqc_handle* H, const char* name, double value) {
    if (!H || !name) return EQC_E_ARG;
    return guarded(H, [&] {
        Handle& h = H->h;
        const std::string s(name);
        if (s == "tma_wait_polls") {   // bound of the TMA applies' first tile wait (failure tests)
            if (!(value >= 0 && value <= MBAR_SPIN_LIMIT) || value != (double)(int)value)
                throw Error(EQC_E_ARG, "tma_wait_polls must be an integer in [0, " + std::to_string(MBAR_SPIN_LIMIT) + "]");
            h.tma_wait_polls = (int)value;
            destroy_graphs(h);   // captured launches hold the old bound
            return;
        }
        if (s == "time_capacity") {    // length of the time_ / Vfmax records (main.jl:154-163)
            if (!(value >= 1 && value <= 1900000) || value != (double)(int64_t)value)
                throw Error(EQC_E_ARG, "time_capacity must be an integer in [1, 1900000]");
            h.cap_time = (int64_t)value;
            return;
        }
        if (!h.initialized) throw Error(EQC_E_STATE, "eqc_set_scalar before eqc_init");
        Ctrl& C = *h.h_ctrl;
        if (s == "t") C.t = value;
        else if (s == "dt") {
            if (!(value > 0)) throw Error(EQC_E_ARG, "dt must be positive");
            C.dt = value;
        } else if (s == "isolver") {
            if (value != 1 && value != 2) throw Error(EQC_E_ARG, "isolver must be 1 or 2");
            C.isolver = (int)value;
        } else throw Error(EQC_E_ARG, "unknown or read-only scalar " + s);
        C.r_valid = 0;
        EQC_CUDA(cudaMemcpyAsync(h.ctrl.p, h.h_ctrl, sizeof(Ctrl), cudaMemcpyHostToDevice, h.stream));
        EQC_CUDA(cudaStreamSynchronize(h.stream));
    });
}

static const std::vector<double>* result_field(Handle& h, const std::string& s) {
    auto& r = h.res;
    if (s == "seismic_stress") return &r.seismic_stress;
    if (s == "seismic_slipvel") return &r.seismic_slipvel;
    if (s == "seismic_slip") return &r.seismic_slip;
    if (s == "is_stress") return &r.is_stress;
    if (s == "is_slipvel") return &r.is_slipvel;
    if (s == "is_slip") return &r.is_slip;
    if (s == "dSeis") return &r.dSeis;
    if (s == "vSeis") return &r.vSeis;
    if (s == "aSeis") return &r.aSeis;
    if (s == "tStart") return &r.tStart;
    if (s == "tEnd") return &r.tEnd;
    if (s == "hypo") return &r.hypo;
    if (s == "taubefore") return &r.taubefore;
    if (s == "tauafter") return &r.tauafter;
    if (s == "delfafter") return &r.delfafter;
    if (s == "time_") return &r.time_;
    if (s == "Vfmax") return &r.Vfmax;
    return nullptr;
}

int64_t eqc_result_size(eqc_handle* H, const char* field) {
    if (!H || !field) return -1;
    if (std::string(field) == "index_eq") return 0;
    const std::vector<double>* f = result_field(H->h, field);
    return f ? (int64_t)f->size() : -1;
}

// Receiver matrices are stored record-major on the host; the reference's dSeis is
// [rit, nseis] column-major, so transpose on the way out.
eqc_status eqc_get_result(eqc_handle* H, const char* field, double* out) {
    if (!H || !field || !out) return EQC_E_ARG;
    return guarded(H, [&] {
        Handle& h = H->h;
        const std::string s(field);
        const std::vector<double>* f = result_field(h, s);
        if (!f) throw Error(EQC_E_ARG, "unknown result field " + s);
        if ((s == "dSeis" || s == "vSeis" || s == "aSeis") && h.nSeis > 0) {
            const int64_t nr = (int64_t)f->size() / h.nSeis;
            for (int64_t r = 0; r < nr; ++r)
                for (int k = 0; k < h.nSeis; ++k) out[r + nr * k] = (*f)[r * h.nSeis + k];
        } else {
            std::copy(f->begin(), f->end(), out);
        }
    });
}

eqc_status eqc_layout(eqc_handle* H, int64_t* nx, int64_t* ny, int64_t* ld) {
    if (!H) return EQC_E_ARG;
    if (nx) *nx = H->h.L.nx;
    if (ny) *ny = H->h.L.ny;
    if (ld) *ld = H->h.L.ld;
    return EQC_OK;
}

eqc_status eqc_set_damage(eqc_handle* H, const int64_t* damage_idx, int64_t n, double factor) {
    if (!H || n < 0 || (n > 0 && !damage_idx) || !(factor > 0.0) || !std::isfinite(factor)) return EQC_E_ARG;
    return guarded(H, [&] {
        Handle& h = H->h;
        const int64_t Nel = (int64_t)h.L.NelX * h.L.NelY;
        std::vector<int64_t> el((size_t)n);
        for (int64_t k = 0; k < n; ++k) {
            fail_if(damage_idx[k] < 1 || damage_idx[k] > Nel, "damage_idx entries must be element numbers 1..Nel");
            el[(size_t)k] = damage_idx[k] - 1;
        }
        std::sort(el.begin(), el.end());
        el.erase(std::unique(el.begin(), el.end()), el.end());
        h.damage_el = std::move(el);
        h.damage_factor = factor;
    });
}

eqc_status eqc_damage_evolve(eqc_handle* H) {
    if (!H) return EQC_E_ARG;
    return guarded(H, [&] { damage_evolve(H->h); });
}

eqc_status eqc_apply_K_device(eqc_handle* H, const void* x, void* y, int32_t dtype) {
    if (!H || !x || !y || dtype < 0 || dtype > 2) return EQC_E_ARG;
    return guarded(H, [&] {
        Handle& h = H->h;
        if (dtype == 0) apply_K<double>((const double*)x, (double*)y, args64(h), 1.0, 0, h.stream);
        else if (dtype == 1) apply_K<float>((const float*)x, (float*)y, args32(h), 1.0f, 0, h.stream);
        else if (!apply_K_df(h, (const double*)x, (double*)y, 1.0, 0, h.stream))
            throw Error(EQC_E_STATE, "double-float apply unavailable (EQC_NO_DF, or H not centro-antisymmetric)");
    });
}

int64_t eqc_launch_count(eqc_handle* H) { return H ? eqc::g_launches : -1; }

eqc_status eqc_sync(eqc_handle* H) {
    if (!H) return EQC_E_ARG;
    return guarded(H, [&] { EQC_CUDA(cudaStreamSynchronize(H->h.stream)); });
}

}  // extern "C"
