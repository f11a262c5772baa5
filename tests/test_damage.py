"""Damage evolution (damageEvol.jl:5-7, its event-end call site main.jl:377-378) on the GPU
against the oracle: after a damage step the stiffness apply agrees with the oracle's
reassembled K to 1e-12, and quasi-static solves through the rebuilt multigrid hierarchy
converge to the oracle's solution; in a time loop a damage step follows every event end."""
import numpy as np
import pytest

from eqcycle_gb300 import EQC_FP64, EQC_MIXED, EQC_PC_AMG, Solver, preset, reference_config, set_parameters

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("precision", [EQC_FP64, EQC_MIXED])
def test_damage_step_matches_oracle(eqclib, oracle_mod, precision):
    cfg = reference_config(res=1)
    P = set_parameters(cfg)
    o = oracle_mod.Oracle(cfg)
    rng = np.random.default_rng(5)
    x = rng.uniform(-1e-3, 1e-3, P.int_.nglob)
    F = rng.uniform(0, 1e-2, P.int_.FltNglob)
    d0 = rng.uniform(-1e-3, 1e-3, P.int_.nglob)
    with Solver(P, precision=precision, precond=EQC_PC_AMG) as s:
        y_before = s.apply_K(x)
        s.set_damage(factor=0.9)
        o.set_damage(P.extra["damage_idx"], 0.9)
        for k in range(2):
            s.damage_evolve()
            o.damage_evolve()
        assert s.scalar("damage_events") == 2
        y = s.apply_K(x)
        assert rel(y, o.apply_K_csr(x)) <= 1e-12
        assert rel(y, y_before) > 1e-6   # the operator did change
        d_ref, _, _ = o.qs_solve(F, d0, tol=1e-13, mode=1)
        d, it, rr = s.qs_solve(F, d0, tol=1e-11)
        assert it > 0 and rr <= 1e-11
        assert rel(d, d_ref) <= 1e-8


def test_damage_grows_at_every_event_end(eqclib, oracle_mod):
    """homog48 with a rectangular damage zone through its first event (mixed precision): one
    damage step per event end, and the final operator is the oracle's K after as many steps.
    The event detector of main.jl:361-380 (1.01 / 0.99 Vthres) fires many times while Vfmax
    hovers near Vthres at the end of a rupture, and every end is a damage step; with the 5 %
    of damageEvol.jl the zone loses most of its stiffness in one rupture and the friction
    Newton fails, so this test uses 1 %."""
    cfg = preset("homog48").replace(damage=1, ThickX=12e3, ThickY=1.5e3, rho2=2500.0, vs2=0.6 * 3464.0,
                                    total_years=100.0)
    P = set_parameters(cfg)
    assert len(P.extra["damage_idx"]) > 0
    with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=2) as s:
        s.set_damage(factor=0.99)
        s.init(cfg.V_init)
        s.run(2_000_000)
        res = s.results()
        n_end = len(res.tEnd)
        assert n_end >= 1, "no event ended in the window"
        assert s.scalar("damage_events") == n_end
        o = oracle_mod.Oracle(cfg)
        o.set_damage(P.extra["damage_idx"], 0.99)
        for _ in range(n_end):
            o.damage_evolve()
        x = np.random.default_rng(9).uniform(-1, 1, P.int_.nglob)
        assert rel(s.apply_K(x), o.apply_K_csr(x)) <= 1e-12


def test_ensemble_recaptures_after_a_damage_step(eqclib):
    """A member whose K changed between ensemble launches: the ensemble step is captured again
    and the members end bitwise where they end when run alone with the same damage step."""
    from eqcycle_gb300 import Ensemble
    cfgs = [reference_config(res=1),
            preset("homog48").replace(NelX=10, NelY=20, LX=5e3, LY=10e3, creep_depth=5e3, seed=3, damage=1,
                                      ThickX=2e3, ThickY=1e3, rho2=2500.0, vs2=0.6 * 3464.0)]
    Ps = [set_parameters(c) for c in cfgs]
    assert all(len(P.extra["damage_idx"]) > 0 for P in Ps)
    alone = []
    for c, P in zip(cfgs, Ps):
        with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=2) as s:
            s.set_damage(factor=0.9)
            s.init(c.V_init)
            s.run(6)
            s.damage_evolve()
            s.run(6)
            alone.append({k: s.state(k) for k in ("d", "v", "psi")})
    solvers = [Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=2) for P in Ps]
    try:
        for c, s in zip(cfgs, solvers):
            s.set_damage(factor=0.9)
            s.init(c.V_init)
        with Ensemble(solvers) as E:
            E.run(6)
            for s in solvers:
                s.damage_evolve()
            E.run(6)
        for x0, s in zip(alone, solvers):
            assert s.scalar("damage_events") == 1
            for k, v in x0.items():
                assert np.array_equal(s.state(k), v), k
    finally:
        for s in solvers:
            s.close()
