"""Failure detection through the C ABI: every error status the time loop and the operator entry
points report, each made to happen by its inputs on the host side (nothing here faults, traps or
hangs the GPU).

  EQC_E_NR       the reference's "NR SEARCH FAILED!" exit of FBC! (src/NRsearch_serial.jl:19-31):
                 an input slip rate above 1e10 or NaN, or a NaN traction from NRsearch!, at the
                 first such node in fault order -- the node the oracle's FBC! returns;
  EQC_E_NAN      a non-finite CG residual or slip rate;
  EQC_E_CG       CG at maxit without meeting its tolerance;
  EQC_E_CAPACITY a full time_ record (the reference preallocates 1.9M entries, main.jl:154-163;
                 the capacity is lowered for the test with the scalar "time_capacity");
  EQC_E_TIMEOUT  a TMA-fed stiffness apply whose first tile wait is given no polls at all (scalar
                 "tma_wait_polls" = 0): the kernel flags the give-up, waits with its full bound
                 for the copies it issued, and returns; the handle keeps working afterwards.
"""
import numpy as np
import pytest

from eqcycle_gb300 import (EQC_FP64, EQC_MIXED, EQC_PC_AMG, EQC_PC_JACOBI, Solver, preset, set_parameters)
from eqcycle_gb300._lib import EqcError

pytestmark = pytest.mark.gpu

E_NR, E_CG, E_NAN, E_CAPACITY, E_TIMEOUT = 3, 4, 5, 6, 7
SMALL = preset("homog48").replace(NelX=12, NelY=16, LX=6e3, LY=8e3, creep_depth=6e3)


def _status(excinfo):
    return excinfo.value.status


@pytest.fixture(scope="module")
def small():
    return SMALL, set_parameters(SMALL)


def test_fbc_failure_node_matches_the_oracle(eqclib, oracle_mod, small):
    cfg, P = small
    o = oracle_mod.Oracle(cfg)
    Nf = P.int_.FltNglob
    rng = np.random.default_rng(3)
    psi = np.log(1e-6 * (cfg.Dc / cfg.Vpl) * rng.uniform(0.5, 2, Nf) / cfg.Dc)
    Vf = 10 ** rng.uniform(-9, 0.5, Nf)
    Vfree = Vf * rng.uniform(0.8, 1.2, Nf)
    dt = P.float_.dt0
    import ctypes as C
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))   # noqa: E731
    nfbc = int(o.scalar("NFBC"))          # 1-based first friction node
    cases = []
    a = Vf.copy(); a[nfbc + 20] = 2e10                                   # slip rate above 1e10
    cases.append((psi, a, nfbc + 21))
    a = Vf.copy(); a[nfbc + 30] = np.nan                                  # NaN slip rate
    cases.append((psi, a, nfbc + 31))
    p = psi.copy(); p[nfbc + 5] = np.nan                                  # NaN traction from NRsearch!
    a = Vf.copy(); a[nfbc + 40] = 3e10
    cases.append((p, a, nfbc + 6))                                        # the first in fault order
    with Solver(P, precond=EQC_PC_JACOBI) as s:
        for ps, vf, want in cases:
            refs = [np.zeros(Nf) for _ in range(6)]
            got_ref = oracle_mod.lib().orc_FBC(o.h, *[dp(r) for r in refs], dp(np.ascontiguousarray(ps)),
                                               dp(np.ascontiguousarray(vf)), dp(Vfree), dt)
            assert got_ref == want
            with pytest.raises(EqcError) as ei:
                s.FBC(*[np.zeros(Nf)] * 6, ps, vf, Vfree, dt)
            assert _status(ei) == E_NR
            assert f"fault node {want}" in str(ei.value)
        # a clean call after the failures
        outs = s.FBC(*[np.zeros(Nf)] * 6, psi, Vf, Vfree, dt)
        assert all(np.all(np.isfinite(x)) for x in outs)


def test_time_loop_nr_failure(eqclib, small):
    """A fault slip rate above 1e10 m/s entering a dynamic step stops the loop with EQC_E_NR."""
    cfg, P = small
    with Solver(P, precond=EQC_PC_AMG) as s:
        s.init(cfg.V_init)
        s.run(2)
        v = s.state("v")
        iF = P.iarray.iFlt - 1
        v[iF[40]] = 1e11
        s.set_state("v", v)
        s.set_scalar("isolver", 2)
        with pytest.raises(EqcError) as ei:
            s.run(1)
        assert _status(ei) == E_NR and "fault node 41" in str(ei.value)


@pytest.mark.parametrize("precision", [EQC_FP64, EQC_MIXED], ids=["fp64", "mixed"])
def test_nan_in_displacement_reports_nan(eqclib, small, precision):
    cfg, P = small
    with Solver(P, precision=precision, precond=EQC_PC_AMG) as s:
        s.init(cfg.V_init)
        s.run(2)
        d = s.state("d")
        d[P.iarray.FltNI[len(P.iarray.FltNI) // 2] - 1] = np.nan
        s.set_state("d", d)
        with pytest.raises(EqcError) as ei:
            s.run(1)
        assert _status(ei) == E_NAN


def test_nan_in_state_reports_nan(eqclib, small):
    """A NaN state variable gives a NaN quasi-static slip rate (slrFunc!), so a NaN Vfmax: the
    loop stops (Julia's maximum propagates NaN; the reference would carry on with it)."""
    cfg, P = small
    with Solver(P, precond=EQC_PC_AMG) as s:
        s.init(cfg.V_init)
        s.run(2)
        psi = s.state("psi")
        psi[P.int_.FltNglob - 10] = np.nan
        s.set_state("psi", psi)
        with pytest.raises(EqcError) as ei:
            s.run(1)
        assert _status(ei) == E_NAN


def test_cg_maxit_reports_cg(eqclib, small):
    cfg, P = small
    rng = np.random.default_rng(1)
    F = rng.uniform(0, 1e-2, P.int_.FltNglob)
    d0 = np.zeros(P.int_.nglob)
    with Solver(P, precond=EQC_PC_JACOBI) as s:
        with pytest.raises(EqcError) as ei:
            s.qs_solve(F, d0, tol=1e-14, maxit=1)
        assert _status(ei) == E_CG
        d, it, rr = s.qs_solve(F, d0, tol=1e-10)        # the handle still solves
        assert it > 1 and rr <= 1e-10
    with Solver(P, precond=EQC_PC_AMG, cg_maxit=1, cg_tol=1e-14) as s:
        s.init(2 * cfg.Vpl)      # off the steady start: the first right-hand side is not zero
        with pytest.raises(EqcError) as ei:
            s.run(3)
        assert _status(ei) == E_CG


def test_time_record_capacity(eqclib, small):
    cfg, P = small
    with Solver(P, precond=EQC_PC_AMG) as s:
        s.set_scalar("time_capacity", 30)
        assert s.scalar("time_capacity") == 30
        s.init(cfg.V_init)
        st = s.run(30)
        assert st["steps"] == 30
        with pytest.raises(EqcError) as ei:
            s.run(5)
        assert _status(ei) == E_CAPACITY
        assert len(s.results().time_) == 30


@pytest.mark.parametrize("variant", [0, 1], ids=["pipelined", "one-tile"])
def test_tma_wait_gives_up_and_the_handle_recovers(eqclib, small, variant):
    """FP64 apply kernels fed by TMA (the persistent pipeline and the one-tile kernel): with no
    polls allowed for the first tile wait every CTA gives up, flags it and drains its own copies;
    the call reports EQC_E_TIMEOUT, and with the bound restored the same handle gives the
    same K x as before."""
    cfg, P = small
    x = np.random.default_rng(0).uniform(-1e-3, 1e-3, P.int_.nglob)
    with Solver(P, precond=EQC_PC_JACOBI, apply_variant=variant) as s:
        y0 = s.apply_K(x)
        default = s.scalar("tma_wait_polls")
        assert default == 1 << 22
        s.set_scalar("tma_wait_polls", 0)
        with pytest.raises(EqcError) as ei:
            s.apply_K(x)
        assert _status(ei) == E_TIMEOUT
        s.set_scalar("tma_wait_polls", default)
        assert np.array_equal(s.apply_K(x), y0)


def test_tma_wait_timeout_in_the_time_loop(eqclib, small):
    """The same give-up inside graph-replayed steps (FP64 apply and multigrid): eqc_run reports
    EQC_E_TIMEOUT; afterwards, with the bound restored and the state initialised again, the
    handle runs the steps a fresh handle runs, bit for bit."""
    cfg, P = small
    with Solver(P, precond=EQC_PC_AMG, cg_maxit=40) as s:
        s.init(cfg.V_init)
        s.set_scalar("tma_wait_polls", 0)
        with pytest.raises(EqcError) as ei:
            s.run(2)
        assert _status(ei) == E_TIMEOUT
        s.set_scalar("tma_wait_polls", 1 << 22)
        s.init(cfg.V_init)
        s.run(5)
        got = {k: s.state(k) for k in ("d", "v", "psi")}
    with Solver(P, precond=EQC_PC_AMG, cg_maxit=40) as s:
        s.init(cfg.V_init)
        s.run(5)
        for k, v in got.items():
            assert np.array_equal(s.state(k), v), k


def test_walk_apply_timeout_in_a_mixed_solve(eqclib, small):
    """The FP32 element-per-lane apply fed by TMA (the walk, apply variant 8) inside a
    mixed-precision solve: EQC_E_TIMEOUT, then a normal solve on the same handle."""
    cfg, P = small
    rng = np.random.default_rng(2)
    F = rng.uniform(0, 1e-2, P.int_.FltNglob)
    d0 = np.zeros(P.int_.nglob)
    with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, apply_variant=8, cg_maxit=40) as s:
        s.set_scalar("tma_wait_polls", 0)
        with pytest.raises(EqcError) as ei:
            s.qs_solve(F, d0, tol=1e-8, maxit=40)
        assert _status(ei) == E_TIMEOUT
        s.set_scalar("tma_wait_polls", 1 << 22)
        d, it, rr = s.qs_solve(F, d0, tol=1e-8)
        assert rr <= 1e-8
