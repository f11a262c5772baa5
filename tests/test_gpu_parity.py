"""GPU parity: libeqc (through the C ABI) against the CPU oracle on the same inputs.

Tolerances (FP64 paths):
  * stiffness apply: 1e-12 relative (max-norm), the bound required of K x;
  * quasi-static solve: both sides solved to a 1e-13 relative residual, solutions agree to
    1e-10 relative (forward error is bounded by cond(K_II) x residual);
  * friction kernels: 1e-12 relative (CUDA vs libm exp/log differ by ulps);
  * time loop: state after the same steps agrees to 1e-8 relative (QS) / 1e-6 (dynamic).
"""
import numpy as np
import pytest

from eqcycle_gb300 import (EQC_FP64, EQC_MIXED, EQC_PC_JACOBI, EQC_PC_AMG, Solver, preset, reference_config,
                           set_parameters)

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


SMALL = preset("homog48").replace(NelX=12, NelY=16, LX=6e3, LY=8e3, creep_depth=6e3)
CFGS = {"ref-res1": reference_config(res=1), "homog48": preset("homog48"), "dz40": preset("dz40")}


@pytest.fixture(scope="module")
def models(eqclib, oracle_mod):
    out = {}
    for k, cfg in CFGS.items():
        P = set_parameters(cfg)
        out[k] = (cfg, P, oracle_mod.Oracle(cfg))
    return out


@pytest.mark.parametrize("name", list(CFGS))
def test_apply_K_matches_oracle(models, name):
    cfg, P, o = models[name]
    with Solver(P, precond=EQC_PC_JACOBI) as s:
        x = np.random.default_rng(0).uniform(-1e-3, 1e-3, P.int_.nglob)
        y = s.apply_K(x)
        y_ref = o.apply_K_csr(x)
        assert rel(y, y_ref) <= 1e-12
        assert np.array_equal(s.apply_K(x), y)   # deterministic, bitwise


@pytest.mark.parametrize("name", ["ref-res1", "dz40"])
def test_qs_solve_matches_oracle(models, name):
    cfg, P, o = models[name]
    rng = np.random.default_rng(1)
    F = rng.uniform(0, 1e-2, P.int_.FltNglob)
    d0 = rng.uniform(-1e-3, 1e-3, P.int_.nglob)
    d_ref, it_ref, rr_ref = o.qs_solve(F, d0, tol=1e-13, mode=1)
    with Solver(P, precond=EQC_PC_JACOBI) as s:
        d, it, rr = s.qs_solve(F, d0, tol=1e-13)
    assert it > 0 and rr <= 1e-13
    assert rel(d, d_ref) <= 1e-10
    iFlt = P.iarray.iFlt - 1
    assert np.array_equal(d[iFlt], F)


def test_friction_kernels_match_oracle(models, oracle_mod):
    cfg, P, o = models["homog48"]
    Nf = P.int_.FltNglob
    rng = np.random.default_rng(2)
    fa = P.farray
    psi = np.log(1e-6 * (cfg.Dc / cfg.Vpl) * rng.uniform(0.5, 2, Nf) / cfg.Dc)
    Vf = 10 ** rng.uniform(-11, 0, Nf)
    tau1 = fa.tauo * rng.uniform(-0.05, 0.05, Nf)
    dt = 1e3
    with Solver(P, precond=EQC_PC_JACOBI) as s:
        psi1, Vf1 = s.slrFunc(psi, np.zeros(Nf), Vf, np.zeros(Nf), tau1, dt)
        p1r, V1r = np.zeros(Nf), np.zeros(Nf)
        import ctypes as C
        dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
        oracle_mod.lib().orc_slrFunc(o.h, dp(psi), dp(p1r), dp(Vf), dp(V1r), dp(tau1), dt)
        assert rel(psi1, p1r) <= 1e-12 and rel(Vf1, V1r) <= 1e-12
        # dynamic: FBC! on a coseismic-like state
        Vfd = 10 ** rng.uniform(-9, 0.5, Nf)
        Vfree = Vfd * rng.uniform(0.8, 1.2, Nf)
        dts = P.float_.dt0
        outs = s.FBC(*[np.zeros(Nf)] * 6, psi, Vfd, Vfree, dts)
        refs = [np.zeros(Nf) for _ in range(6)]
        fail = oracle_mod.lib().orc_FBC(o.h, *[dp(a) for a in refs], dp(psi), dp(Vfd), dp(Vfree), dts)
        assert fail == 0
        for a, b in zip(outs, refs):
            assert rel(a, b) <= 1e-11
        # dtevol!
        for iso in (1, 2):
            for dtp in (1e3, 1e7):
                r = s.dtevol(dtp, P.float_.dt0, Vf, iso)
                assert r == oracle_mod.lib().orc_dtevol(o.h, dtp, P.float_.dt0, dp(Vf), iso)


def _run_both(cfg, nsteps, oracle_mod, tol, **kw):
    P = set_parameters(cfg)
    o = oracle_mod.Oracle(cfg)
    o.run(nsteps, qs_mode=1, qs_tol=tol)
    with Solver(P, cg_tol=tol, **kw) as s:
        s.init(cfg.V_init)
        st = s.run(nsteps)
        got = {k: s.state(k) for k in ("d", "v", "psi", "tau")}
        res = s.results()
    ref = {k: o.state(k) for k in ("d", "v", "psi", "tau")}
    return P, o, st, got, ref, res


def test_time_loop_quasi_static_matches_oracle(eqclib, oracle_mod):
    # the reference's own model (par.jl defaults at res = 1): creeping section below 24 km,
    # V = 1 mm/s initially, so the displacement field is far from round-off
    P, o, st, got, ref, res = _run_both(reference_config(res=1), 40, oracle_mod, 1e-14, precond=EQC_PC_JACOBI)
    assert st["steps"] == 40 and st["qs_steps"] >= 10
    assert int(np.sum(o.get("regime") == 1)) == st["qs_steps"]
    for k in ("d", "v", "psi", "tau"):
        assert rel(got[k], ref[k]) <= 1e-8, k
    assert rel(res.time_, o.get("time_")) <= 1e-12
    assert rel(res.Vfmax, o.get("Vfmax")) <= 1e-8


def test_time_loop_dynamic_matches_oracle(eqclib, oracle_mod):
    # a fast initial slip rate drives the solver into the dynamic regime after one step
    cfg = SMALL.replace(V_init=2e-2)
    P, o, st, got, ref, res = _run_both(cfg, 60, oracle_mod, 1e-12, precond=EQC_PC_JACOBI)
    assert st["dyn_steps"] >= 30
    regime = o.get("regime")
    assert int(np.sum(regime == 2)) == st["dyn_steps"]
    for k in ("d", "v", "psi", "tau"):
        assert rel(got[k], ref[k]) <= 1e-6, k
    assert rel(res.Vfmax, o.get("Vfmax")) <= 1e-6
    assert rel(res.dSeis, o.get("dSeis")) <= 1e-6


def test_mixed_precision_qs_solve(models, oracle_mod):
    cfg, P, o = models["dz40"]
    rng = np.random.default_rng(4)
    F = rng.uniform(0, 1e-2, P.int_.FltNglob)
    d0 = np.zeros(P.int_.nglob)
    d_ref, _, _ = o.qs_solve(F, d0, tol=1e-13, mode=1)
    with Solver(P, precision=EQC_MIXED, precond=EQC_PC_JACOBI) as s:
        d, it, rr = s.qs_solve(F, d0, tol=1e-8)
    assert it > 0 and rr <= 1e-8        # certified on the FP64 true residual
    assert rel(d, d_ref) <= 1e-5


@pytest.mark.parametrize("precision", [EQC_FP64, EQC_MIXED], ids=["fp64", "mixed"])
def test_multigrid_qs_solve_matches_oracle(models, oracle_mod, precision):
    """Multigrid-preconditioned CG: converged solution equals the oracle's, in few iterations."""
    cfg, P, o = models["dz40"]
    rng = np.random.default_rng(6)
    F = rng.uniform(0, 1e-2, P.int_.FltNglob)
    d0 = rng.uniform(-1e-3, 1e-3, P.int_.nglob)
    d_ref, _, _ = o.qs_solve(F, d0, tol=1e-13, mode=1)
    tol = 1e-13 if precision == EQC_FP64 else 1e-10
    with Solver(P, precision=precision, precond=EQC_PC_AMG) as s:
        d, it, rr = s.qs_solve(F, d0, tol=tol)
    assert 0 < it <= 40 and rr <= tol
    assert rel(d, d_ref) <= (1e-10 if precision == EQC_FP64 else 1e-7)


def test_multigrid_time_loop_matches_oracle(eqclib, oracle_mod):
    P, o, st, got, ref, res = _run_both(reference_config(res=1), 30, oracle_mod, 1e-14, precond=EQC_PC_AMG)
    assert st["steps"] == 30
    for k in ("d", "v", "psi", "tau"):
        assert rel(got[k], ref[k]) <= 1e-8, k


@pytest.mark.parametrize("precision,guess", [(EQC_FP64, 0), (EQC_MIXED, 0), (EQC_MIXED, 2)],
                         ids=["fp64", "mixed", "mixed-extrapolate"])
def test_graph_step_equals_eager_step(eqclib, precision, guess):
    """A step replayed from its CUDA graph (device-driven CG loop in conditional nodes) runs
    the same kernels in the same order as the host-driven step: bitwise equal state and the
    same iteration counts, through quasi-static and dynamic steps.  The graphs launch
    consecutive kernels as programmatic dependent launches (pdl_edges > 0); the eager steps do
    not, so equality also shows that every kernel waits for its predecessor."""
    cfg = preset("dz40").replace(V_init=2e-2)
    P = set_parameters(cfg)
    out = []
    for graphs in (0, 1):
        with Solver(P, precision=precision, precond=EQC_PC_AMG, use_graphs=graphs, guess=guess) as s:
            s.init(cfg.V_init)
            st = s.run(12)
            out.append((st, {k: s.state(k) for k in ("d", "v", "a", "psi", "tau")}))
            pdl = s.scalar("pdl_edges")
            assert (pdl > 0) if graphs else (pdl == 0)
    (st0, x0), (st1, x1) = out
    assert st0["qs_steps"] >= 1 and st0["dyn_steps"] >= 1, st0
    for k in ("steps", "qs_steps", "dyn_steps", "cg_iters", "qs_solves", "isolver"):
        assert st0[k] == st1[k], k
    for k in x0:
        assert np.array_equal(x0[k], x1[k]), k


@pytest.mark.parametrize("guess", [0, 2], ids=["previous", "extrapolate"])
def test_mixed_time_loop_matches_fp64_oracle(eqclib, oracle_mod, guess):
    """Mixed precision in the time loop (FP32 apply and multigrid inside the FP64
    reliable-update CG, residual carried from one solve to the next): the state after 15
    quasi-static steps agrees with the FP64 oracle solved tightly."""
    cfg = reference_config(res=1)
    P = set_parameters(cfg)
    o = oracle_mod.Oracle(cfg)
    o.run(15, qs_mode=1, qs_tol=1e-13)
    with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, cg_tol=1e-10, guess=guess) as s:
        s.init(cfg.V_init)
        st = s.run(15)
        got = {k: s.state(k) for k in ("d", "v", "psi", "tau")}
        carried = s.scalar("cg_carried")
    assert st["qs_steps"] == 15
    assert carried >= st["qs_solves"] - 2     # every solve but the first carries
    for k in ("d", "v", "psi", "tau"):
        assert rel(got[k], o.state(k)) <= 1e-6, k


def test_autotune_keeps_the_state_and_chooses_a_valid_smoother(eqclib):
    """eqc_autotune leaves the state and the counters untouched; the run after it converges to
    the same state as a run with the default smoother (same CG tolerance)."""
    cfg = preset("dz40")
    P = set_parameters(cfg)
    out = []
    for tune in (False, True):
        with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=2, cg_tol=1e-10) as s:
            s.init(cfg.V_init)
            s.run(3)   # past the trivial first solves of the steady start
            if tune:
                before = {k: s.state(k) for k in ("d", "v", "a", "psi", "tau")}
                scal = {k: s.scalar(k) for k in ("t", "dt", "isolver", "cg_iters", "qs_solves")}
                res = s.autotune(reps=1)
                assert res["mg_degree"] in (3, 4, 5) and res["mg_degree_coarse"] in (1, 3, 4)
                assert res["apply_variant"] in (0, 7, 4, 8) and res["reliable_delta"] in (1e-2, 1e-3, 1e-4)
                assert res["solve_ms"] > 0
                for k, v in before.items():
                    assert np.array_equal(s.state(k), v), k
                for k, v in scal.items():
                    assert s.scalar(k) == v, k
            st = s.run(8)
            assert st["qs_steps"] == 8
            out.append({k: s.state(k) for k in ("d", "v", "psi")})
    for k in out[0]:
        assert rel(out[1][k], out[0][k]) <= 1e-6, k


def test_mixed_precision_from_the_steady_start(eqclib):
    """From V = Vpl the first increments are ~1e-25 m: the FP32 recurrence works on scaled
    vectors (no underflow) and tracks the FP64 method."""
    cfg = preset("dz40")
    P = set_parameters(cfg)
    res = {}
    for prec in (EQC_FP64, EQC_MIXED):
        with Solver(P, precision=prec, precond=EQC_PC_AMG, cg_tol=1e-10) as s:
            s.init(cfg.V_init)
            st = s.run(12)
            assert st["qs_steps"] == 12
            res[prec] = {k: s.state(k) for k in ("d", "v", "psi")}
    for k in res[EQC_FP64]:
        assert rel(res[EQC_MIXED][k], res[EQC_FP64][k]) <= 1e-6, k


def test_ensemble_equals_members_run_alone(eqclib):
    """Uneven models advanced together by one graph launch per step (one of them in the dynamic
    regime) end bitwise where each ends when run alone."""
    from eqcycle_gb300 import Ensemble
    base = preset("homog48")
    cfgs = [base.replace(NelX=8, NelY=12, LX=4e3, LY=6e3, creep_depth=4e3),
            SMALL.replace(V_init=2e-2),
            base.replace(NelX=10, NelY=20, LX=5e3, LY=10e3, creep_depth=5e3, seed=3)]
    Ps = [set_parameters(c) for c in cfgs]
    alone = []
    for c, P in zip(cfgs, Ps):
        with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=2) as s:
            s.init(c.V_init)
            st = s.run(12)
            alone.append((st, {k: s.state(k) for k in ("d", "v", "psi")}, s.results().Vfmax))
    solvers = [Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=2) for P in Ps]
    try:
        for c, s in zip(cfgs, solvers):
            s.init(c.V_init)
        with Ensemble(solvers) as E:
            stats, ms = E.run(12)
        assert ms > 0
        assert any(st["dyn_steps"] > 0 for st in stats) and any(st["qs_steps"] == 12 for st in stats)
        for (st0, x0, vf0), st, s in zip(alone, stats, solvers):
            for k in ("steps", "qs_steps", "dyn_steps", "cg_iters"):
                assert st[k] == st0[k], k
            for k, v in x0.items():
                assert np.array_equal(s.state(k), v), k
            assert np.array_equal(s.results().Vfmax, vf0)
    finally:
        for s in solvers:
            s.close()


def test_mixed_precision_after_a_dynamic_phase(eqclib):
    """The first quasi-static solves after dynamic steps start from a displacement far from the
    quasi-static solution: the mixed solver restarts its direction when the FP64 residual leaves
    the FP32 recurrence's, converges, and tracks the FP64 method."""
    cfg = SMALL.replace(V_init=2e-2)
    P = set_parameters(cfg)
    out = {}
    for prec in (EQC_FP64, EQC_MIXED):
        with Solver(P, precision=prec, precond=EQC_PC_AMG, cg_tol=1e-10) as s:
            s.init(cfg.V_init)
            st = s.run(20)
            assert st["dyn_steps"] >= 15
            s.set_scalar("isolver", 1)
            st = s.run(6)
            assert st["qs_steps"] >= 1
            out[prec] = ({k: s.state(k) for k in ("d", "v", "psi")}, s.scalar("cg_restarts"))
    for k in out[EQC_FP64][0]:
        assert rel(out[EQC_MIXED][0][k], out[EQC_FP64][0][k]) <= 1e-6, k


def test_batched_steps_equal_single_steps(eqclib):
    """Steps looped on the device (outputs logged there, the launch ending at any step whose outputs
    need the host) give the same state and the same results records as one step per launch."""
    cfg = SMALL.replace(V_init=2e-2)   # fast slip: seismic snapshots, receivers, regime switches
    P = set_parameters(cfg)
    out = []
    for batch in (1, 0):
        with Solver(P, precision=EQC_FP64, precond=EQC_PC_AMG, step_batch=batch) as s:
            s.init(cfg.V_init)
            st = s.run(150)
            out.append((st, {k: s.state(k) for k in ("d", "v", "psi")}, s.results()))
    (st1, x1, r1), (st0, x0, r0) = out
    assert st0["dyn_steps"] > 20
    for k in ("steps", "qs_steps", "dyn_steps", "cg_iters"):
        assert st0[k] == st1[k], k
    for k in x1:
        assert np.array_equal(x0[k], x1[k]), k
    for f in ("time_", "Vfmax", "dSeis", "vSeis", "aSeis", "seismic_slip", "seismic_stress", "tStart", "hypo",
              "taubefore", "is_slip"):
        a, b = getattr(r0, f), getattr(r1, f)
        assert a.shape == b.shape and np.array_equal(a, b), f
    assert len(r1.dSeis) > 0 and r1.seismic_slip.shape[1] > 0


def test_mixed_dynamic_steps_match_oracle(eqclib, oracle_mod):
    """The mixed method's Newmark steps (FP64 d and K d, FP32 apply of each step's increment, FP64
    refresh of K d at the start of the phase) against the FP64 oracle."""
    cfg = SMALL.replace(V_init=2e-2)
    P, o, st, got, ref, res = _run_both(cfg, 60, oracle_mod, 1e-12, precision=EQC_MIXED, precond=EQC_PC_AMG)
    assert st["dyn_steps"] >= 30
    for k in ("d", "v", "psi", "tau"):
        assert rel(got[k], ref[k]) <= 1e-6, k
    assert rel(res.Vfmax, o.get("Vfmax")) <= 1e-6


def test_state_transfers_round_trip_through_pinned_buffers(eqclib):
    """eqc_get_state / eqc_set_state permute node fields between the reference numbering and the
    padded device layout on the device: reading into a caller's (pinned) array gives the same
    bits as a fresh one, and writing a field back and reading it again returns it unchanged, on
    a mesh whose rows carry padding."""
    torch = pytest.importorskip("torch")
    P = set_parameters(preset("homog48"))
    with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG) as s:
        nx, ny, ld = s.layout()
        assert ld > nx   # padded rows
        s.init(P.cfg.V_init)
        s.run(3)
        rng = np.random.default_rng(5)
        for name in ("d", "v", "a", "psi", "tau"):
            x = s.state(name)
            buf = torch.empty(x.size, dtype=torch.float64, pin_memory=True).numpy()
            assert np.array_equal(s.state(name, out=buf), x), name
            y = rng.standard_normal(x.size)
            ybuf = torch.empty(x.size, dtype=torch.float64, pin_memory=True).numpy()
            ybuf[:] = y
            s.set_state(name, ybuf)
            assert np.array_equal(s.state(name), y), name
            s.set_state(name, x)
            assert np.array_equal(s.state(name), x), name
        with pytest.raises(ValueError):
            s.state("d", out=np.zeros(3))
