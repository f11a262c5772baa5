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
                    assert float(out_d.item()) == pytest.approx(ref, rel=1e-15, abs=0.0), (call, iso, dt)
    # sizes beyond the stated maximum are rejected before any launch
    st = eqclib.eqc_dtevol_noalloc(C.c_void_p(xi_d.data_ptr()), C.c_void_p(xi_d.data_ptr()), (1 << 22) + 1, 1,
                                   1e3, dtmin, 1, C.c_void_p(out_d.data_ptr()), None)
    assert st == 1
    assert b"EQC_NOALLOC_MAX_NODES" in eqclib.eqc_last_error(None)
