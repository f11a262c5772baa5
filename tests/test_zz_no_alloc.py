"""The allocation-free time-step entry point (eqc_dtevol_noalloc) against eqc_dtevol.

Callers that cannot allocate device memory (a host code with a fixed device arena, an
allocator budget that forbids library allocations) use eqc_dtevol_noalloc on their own
device arrays; its reduction scratch is a static device array inside libeqc.  This test
calls it through the C ABI twice in a row and checks each result against the handle-based
eqc_dtevol on the same slip rates.  It lives in its own file so that pytest collects it
last, and it passes alone in a fresh process as well as after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_dtevol_noalloc_matches_dtevol(eqclib):
    torch = pytest.importorskip("torch")
    from eqcycle_gb300 import EQC_PC_JACOBI, Solver, preset, set_parameters
    P = set_parameters(preset("dz40"))
    Nf = P.int_.FltNglob
    dtmin = P.float_.dt0
    creeping = set(P.iarray.FltIglobBC.tolist()) & set(P.iarray.iFlt.tolist())
    NFBC = len(creeping) + 1                       # src/main.jl:186
    rng = np.random.default_rng(11)
    xi_d = torch.tensor(np.ascontiguousarray(P.farray.XiLf), dtype=torch.float64, device="cuda")
    out_d = torch.zeros(1, dtype=torch.float64, device="cuda")
    with Solver(P, precond=EQC_PC_JACOBI) as s:
        for call in range(2):   # two calls in a row share the static scratch
            Vf = 10 ** rng.uniform(-11, -1, Nf)
            vf_d = torch.tensor(Vf, dtype=torch.float64, device="cuda")
            for iso in (1, 2):
                for dt in (1e3, 3e6):
                    ref = s.dtevol(dt, dtmin, Vf, iso)
                    out_d.fill_(-1.0)
                    st = eqclib.eqc_dtevol_noalloc(C.c_void_p(vf_d.data_ptr()), C.c_void_p(xi_d.data_ptr()),
                                                   Nf, NFBC, dt, dtmin, iso, C.c_void_p(out_d.data_ptr()), None)
                    assert st == 0, eqclib.eqc_last_error(None)
                    torch.cuda.synchronize()
                    assert float(out_d.item()) == ref, (call, iso, dt)   # a minimum: exact
    # sizes beyond the stated maximum are rejected before any launch
    st = eqclib.eqc_dtevol_noalloc(C.c_void_p(xi_d.data_ptr()), C.c_void_p(xi_d.data_ptr()), (1 << 22) + 1, 1,
                                   1e3, dtmin, 1, C.c_void_p(out_d.data_ptr()), None)
    assert st == 1
    assert b"EQC_NOALLOC_MAX_NODES" in eqclib.eqc_last_error(None)


def _dtevol_np(Vf, XiLf, NFBC, dt, dtmin, isolver):
    """dtevol! (src/dtevol.jl:5-44) in numpy: the minimum of XiLf/|V| over the friction nodes
    NFBC..n (1-based) where |V| dtmax > XiLf, clamped to [dtmin, 1.2 dt]; dtmin when dynamic."""
    dtmax = 50.0 * 24 * 60 * 60
    if isolver != 1:
        return dtmin
    sr = np.abs(Vf[NFBC - 1:])
    xi = XiLf[NFBC - 1:]
    sel = sr * dtmax > xi
    dtnx = min(dtmax, float(np.min(xi[sel] / sr[sel]))) if np.any(sel) else dtmax
    return min(max(dtnx, dtmin), 1.2 * dt)


@pytest.mark.parametrize("n,NFBC", [(300_000, 1_001), ((1 << 22) - 3, 17), ((1 << 22), (1 << 22) + 1)],
                         ids=["300k", "near-max", "empty-range"])
def test_dtevol_noalloc_many_ctas(eqclib, n, NFBC):
    """Synthetic device arrays large enough that the reduction runs on its full grid of CTAs
    (each striding over many nodes), with the minimum placed far from the first CTA's range:
    the per-CTA minima, the last-CTA election and its read of the other CTAs' minima must give
    dtevol!'s value exactly, on two calls in a row with different data.  With NFBC = n + 1 the
    friction range is empty: dtmax, then the clamps."""
    torch = pytest.importorskip("torch")
    out_d = torch.zeros(1, dtype=torch.float64, device="cuda")
    dtmin = 3e-3
    for call in range(2):
        rng = np.random.default_rng(100 + call)
        Vf = 10 ** rng.uniform(-12, -9, n)
        XiLf = rng.uniform(1e-4, 1e-2, n)
        if NFBC <= n:
            k = NFBC - 1 + int(rng.integers(0, n - NFBC + 1))
            Vf[k] = 1e-6                          # the winning node, somewhere in the range
            Vf[max(0, NFBC - 2)] = 1.0           # a faster node before the range: ignored
        vf_d = torch.tensor(Vf, dtype=torch.float64, device="cuda")
        xi_d = torch.tensor(XiLf, dtype=torch.float64, device="cuda")
        for iso in (1, 2):
            for dt in (1e3, 3e6, 1e9):
                ref = _dtevol_np(Vf, XiLf, NFBC, dt, dtmin, iso)
                out_d.fill_(-1.0)
                st = eqclib.eqc_dtevol_noalloc(C.c_void_p(vf_d.data_ptr()), C.c_void_p(xi_d.data_ptr()), n, NFBC,
                                               dt, dtmin, iso, C.c_void_p(out_d.data_ptr()), None)
                assert st == 0, eqclib.eqc_last_error(None)
                torch.cuda.synchronize()
                assert float(out_d.item()) == ref, (call, iso, dt)

