"""GPU against the oracle's frozen answers (tests/golden/oracle_small.npz), through the C ABI:
the stiffness apply (1e-12), a quasi-static solve (1e-10), the first 40 quasi-static and 60
dynamic steps (1e-8 / 1e-6, as the live oracle comparisons), and the event catalogue of the
48 x 48 element model over 300 years, plain FP64 and mixed precision each within 2 % of the
oracle's reference-mode catalogue (recurrence interval, coseismic slip, hypocentre depth), and
the fields of that run's results record (main.jl:479-498) against the oracle's
(tests/golden/catalogue_homog48.npz): event times to 1e-3, hypocentres to two node spacings, the
per-event stress and slip profiles, the 5-year snapshots of slip and stress (and of the slip rate
before the first event) and every 5th coseismic slip snapshot of the first event to 2 % of each
field's largest entry, the coseismic snapshot counts to within three."""
import importlib.util
import os

import numpy as np
import pytest

from eqcycle_gb300 import (EQC_FP64, EQC_GUESS_EXTRAPOLATE, EQC_GUESS_PREVIOUS, EQC_MIXED, EQC_PC_JACOBI, Solver,
                           set_parameters)
from eqcycle_gb300.config import YR2SEC
from eqcycle_gb300.events import EventCatalogue, catalogue, compare

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(__file__), "golden")


def _gen():
    spec = importlib.util.spec_from_file_location("make_oracle_golden", os.path.join(HERE, "make_oracle_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(os.path.join(HERE, "oracle_small.npz")))


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def test_apply_and_qs_solve_match_the_fixture(eqclib, gold):
    P = set_parameters(_gen().APPLY_CFG)
    with Solver(P, precond=EQC_PC_JACOBI) as s:
        assert rel(s.apply_K(gold["apply_x"]), gold["apply_y"]) <= 1e-12
        d, it, rr = s.qs_solve(gold["qs_F"], gold["qs_d0"], tol=1e-13)
    assert rr <= 1e-13 and rel(d, gold["qs_d"]) <= 1e-10


@pytest.mark.parametrize("case,steps,tol,bound", [("loopq", 40, 1e-14, 1e-8), ("loopd", 60, 1e-12, 1e-6)])
def test_first_steps_match_the_fixture(eqclib, gold, case, steps, tol, bound):
    g = _gen()
    cfg = g.LOOPQ_CFG if case == "loopq" else g.LOOPD_CFG
    P = set_parameters(cfg)
    with Solver(P, cg_tol=tol, precond=EQC_PC_JACOBI) as s:
        s.init(cfg.V_init)
        st = s.run(steps)
        iF = P.iarray.iFlt - 1
        got = {"d_fault": s.state("d")[iF], "v_fault": s.state("v")[iF], "psi": s.state("psi")}
        res = s.results()
    assert st["steps"] == steps
    assert st["dyn_steps"] == int(np.sum(gold[f"{case}_regime"] == 2))
    for k, v in got.items():
        assert rel(v, gold[f"{case}_{k}"]) <= bound, k
    assert rel(res.time_, gold[f"{case}_time"]) <= (1e-12 if case == "loopq" else bound)
    assert rel(res.Vfmax, gold[f"{case}_Vfmax"]) <= bound


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_event_catalogue_within_two_percent_of_the_oracle(eqclib, gold, precision):
    g = _gen()
    cfg = g.EV_CFG
    P = set_parameters(cfg)
    t_end = float(gold["ev_info"][0]) * YR2SEC
    prec, guess = (EQC_FP64, EQC_GUESS_PREVIOUS) if precision == "fp64" else (EQC_MIXED, EQC_GUESS_EXTRAPOLATE)
    with Solver(P, precision=prec, cg_tol=1e-8, guess=guess) as s:
        s.init(cfg.V_init)
        while s.scalar("t") < t_end:
            st = s.run(5000, t_end)
            assert st["steps"] > 0
        res = s.results()
    cat = catalogue(res, P.farray.FltX, cfg.rho1 * cfg.vs1 ** 2)
    e = np.zeros(0)
    ref = EventCatalogue(tStart=gold["ev_tStart"], tEnd=gold["ev_tEnd"], hypo=gold["ev_hypo"], slip=e,
                         stress_drop=e, Mw=gold["ev_Mw"], mean_slip=e, mean_drop=e, max_slip=gold["ev_max_slip"])
    c = compare(ref, cat)
    assert c["events_a"] == c["events_b"] == c["compared"]
    for k in ("recurrence", "coseismic_slip", "hypocentre_depth"):
        assert c[k] <= 0.02, (k, c)
    assert np.max(np.abs(cat.Mw - ref.Mw)) <= 0.02
    # every field of the results record against the oracle's 300-year run (catalogue_homog48.npz)
    full = dict(np.load(os.path.join(HERE, "catalogue_homog48.npz")))
    assert np.max(np.abs(res.tStart - full["tStart"]) / full["tStart"]) <= 1e-3
    assert np.max(np.abs(res.tEnd - full["tEnd"]) / full["tEnd"]) <= 1e-3
    assert np.max(np.abs(res.hypo - full["hypo"])) <= 250.0           # two GLL node spacings
    errs = {}
    for f in ("taubefore", "tauafter", "delfafter", "is_slip", "is_stress"):
        a, b = getattr(res, f), full[f].astype(np.float64)
        assert a.shape == b.shape, (f, a.shape, b.shape)
        errs[f] = rel(a, b)
    # the 5-year snapshots of the slip rate before the first event (after it, the slip rate of the
    # slowly creeping parts depends on the exact timing of the rupture: only the event statistics
    # are compared there)
    pre = int(full["tStart"][0] // (5 * YR2SEC))
    errs["is_slipvel before the first event"] = rel(res.is_slipvel[:, :pre],
                                                    full["is_slipvel"][:, :pre].astype(np.float64))
    # coseismic snapshots (every 0.5 s while Vfmax > Vevne, main.jl:395-422): the count may differ
    # by one or two where Vfmax re-crosses Vevne at an event's end (observed: 1,147 in the oracle,
    # 1,148-1,149 on the GPU); the first 400 snapshots lie inside the first event's episode (its
    # ~575 snapshots), aligned at its start in both runs, and their slip is compared every 5th.
    # The snapshots of slip rate and stress sample the rupture front, whose arrival at a fault
    # node shifts by a fraction of a snapshot interval between two solvers stopped at 1e-8
    # (observed 0.18-0.22 of the peak slip rate, 0.04 of the stress, in both GPU methods); they
    # are compared to 1e-9 (FP64) on the short run of tests/test_gpu_results.py instead.
    assert abs(res.seismic_slip.shape[1] - int(full["seismic_count"][0])) <= 3
    a, b = res.seismic_slip[:, :400:5], full["seismic_slip_every5"][:, :80].astype(np.float64)
    assert a.shape == b.shape
    errs["seismic_slip"] = rel(a, b)
    print(precision, {k: f"{v:.2e}" for k, v in errs.items()})
    assert all(v <= 0.02 for v in errs.values()), errs
