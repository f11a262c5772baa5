"""The CPU oracle against its own frozen answers (tests/golden/oracle_small.npz, made by
tests/golden/make_oracle_golden.py): the stiffness apply, a quasi-static solve, NRsearch! known
answers, and the first steps of a quasi-static and of a dynamic run, all re-run here and
compared; the event catalogue (47 minutes of oracle time) is checked for consistency only."""
import os

import numpy as np
import pytest

from eqcycle_gb300.config import YR2SEC

GOLD = os.path.join(os.path.dirname(__file__), "golden", "oracle_small.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _cfgs():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_oracle_golden",
                                                  os.path.join(os.path.dirname(GOLD), "make_oracle_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_apply_and_qs_solve_reproduce_the_fixture(oracle_mod, gold):
    g = _cfgs()
    o = oracle_mod.Oracle(g.APPLY_CFG)
    assert rel(o.apply_K_csr(gold["apply_x"]), gold["apply_y"]) <= 1e-14
    d, it, rr = o.qs_solve(gold["qs_F"], gold["qs_d0"], tol=1e-13, mode=1)
    assert rr <= 1e-13 and rel(d, gold["qs_d"]) <= 1e-11


def test_nr_known_answers(oracle_mod, gold):
    rows = gold["nr_in"]
    assert rows.shape == (48, 10)
    for r, f64, q in zip(rows, gold["nr_fp64"], gold["nr_quad"]):
        V, T, st = oracle_mod.NR(*r)
        assert st == f64[2] == q[2]
        assert abs(V - f64[0]) <= 1e-14 * abs(f64[0]) and abs(T - f64[1]) <= 1e-14 * abs(f64[1])
        assert abs(f64[1] - q[1]) <= 1e-12 * abs(q[1])       # FP64 against binary128
    Vs = gold["nr_fp64"][:, 0]
    assert Vs.min() < 1e-10 and Vs.max() > 1.0               # the slip-rate range is spanned


@pytest.mark.parametrize("case,steps,tol", [("loopq", 40, 1e-14), ("loopd", 60, 1e-12)])
def test_first_steps_reproduce_the_fixture(oracle_mod, gold, case, steps, tol):
    g = _cfgs()
    o = oracle_mod.Oracle(g.LOOPQ_CFG if case == "loopq" else g.LOOPD_CFG)
    assert o.run(steps, qs_mode=1, qs_tol=tol) == steps
    iF = o.get("iFlt") - 1
    assert rel(o.state("d")[iF], gold[f"{case}_d_fault"]) <= 1e-10
    assert rel(o.state("v")[iF], gold[f"{case}_v_fault"]) <= 1e-10
    assert rel(o.state("psi"), gold[f"{case}_psi"]) <= 1e-10
    assert rel(o.get("time_"), gold[f"{case}_time"]) <= 1e-12
    assert np.array_equal(o.get("regime"), gold[f"{case}_regime"])
    if case == "loopd":
        assert int(np.sum(gold["loopd_regime"] == 2)) >= 30     # the dynamic phase is covered


def test_event_catalogue_fixture_is_consistent(gold):
    years, steps, _ = gold["ev_info"]
    tS, tE = gold["ev_tStart"], gold["ev_tEnd"]
    assert years == 300.0 and steps > 1000
    assert len(tS) >= 2 and len(tE) == len(tS)
    assert np.all(tE > tS) and np.all(np.diff(tS) > 0) and tE[-1] <= years * YR2SEC
    assert np.all(gold["ev_max_slip"] > 0) and np.all(np.isfinite(gold["ev_Mw"]))


NUCL = os.path.join(os.path.dirname(__file__), "golden", "nucleation_homog48.npz")


def test_nucleation_history_fixture(oracle_mod):
    """The oracle's homog48 history through the first nucleation (make_nucleation_golden.py):
    consistent on its own, and its first 10 steps reproduced by running the oracle again (the
    whole history takes the oracle most of an hour)."""
    from eqcycle_gb300.config import preset
    g = dict(np.load(NUCL))
    nsteps, check, tol = int(g["info"][0]), int(g["info"][1]), float(g["info"][2])
    assert len(g["time"]) == len(g["Vfmax"]) == len(g["regime"]) == nsteps
    cfg = preset("homog48")
    assert g["Vfmax"][-1] > 1.01 * cfg.Vthres and np.all(g["Vfmax"][:-1] <= 1.01 * cfg.Vthres)
    assert np.all(g["regime"] == 1)                      # the nucleation is quasi-static throughout
    assert np.all(np.diff(g["time"]) > 0) and g["check_steps"][-1] == nsteps
    assert list(g["check_steps"][:-1]) == list(range(check, nsteps, check))[:len(g["check_steps"]) - 1]
    assert g["d_fault"].shape == g["v_fault"].shape == g["psi"].shape == (len(g["check_steps"]), 193)
    o = oracle_mod.Oracle(cfg)
    assert o.run(10, qs_mode=0, qs_tol=tol) == 10
    assert rel(o.get("time_"), g["time"][:10]) <= 1e-12
    assert rel(o.get("Vfmax"), g["Vfmax"][:10]) <= 1e-10
