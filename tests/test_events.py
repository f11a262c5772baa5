"""Host-side result handling: the serialized results record (save / load round trip), the event
catalogue and its comparison on edge cases, and the clock record bench.py reads from nvidia-smi."""
import os
from dataclasses import fields

import numpy as np

from eqcycle_gb300.events import catalogue, compare, load_results, moment_magnitude, save_results
from eqcycle_gb300.solver import Results


def _results(nev=2, Nf=5, seed=0):
    rng = np.random.default_rng(seed)
    e = np.zeros(0)
    return Results(seismic_stress=rng.uniform(size=(Nf, 3)), seismic_slipvel=rng.uniform(size=(Nf, 3)),
                   seismic_slip=rng.uniform(size=(Nf, 3)), index_eq=np.arange(3, dtype=np.float64),
                   is_stress=e, is_slipvel=e, is_slip=e, dSeis=rng.uniform(size=(4, 6)), vSeis=e, aSeis=e,
                   tStart=np.sort(rng.uniform(0, 1e10, nev)), tEnd=np.sort(rng.uniform(0, 1e10, nev)) + 1.0,
                   taubefore=rng.uniform(20, 30, (Nf, nev)), tauafter=rng.uniform(10, 20, (Nf, nev)),
                   delfafter=rng.uniform(0, 3, (Nf, nev)), hypo=-rng.uniform(0, 1e4, nev),
                   time_=np.cumsum(rng.uniform(size=7)), Vfmax=rng.uniform(size=7))


def test_results_round_trip(tmp_path):
    res = _results()
    p = os.path.join(tmp_path, "run.npz")
    save_results(p, res)
    back = load_results(p)
    for f in fields(Results):
        a, b = np.asarray(getattr(res, f.name)), np.asarray(getattr(back, f.name))
        assert a.shape == b.shape and np.array_equal(a, b), f.name


def test_catalogue_without_events_and_with_unequal_counts():
    FltX = np.linspace(-1e4, 0.0, 5)
    empty = catalogue(_results(nev=0), FltX, 3e10)
    assert len(empty.Mw) == 0 and len(empty.recurrence) == 0
    assert np.isnan(empty.summary()["recurrence_yr"])
    two = catalogue(_results(nev=2), FltX, 3e10)
    c = compare(two, empty)
    assert c == {"events_a": 2, "events_b": 0, "compared": 0}
    three = catalogue(_results(nev=3, seed=1), FltX, 3e10)
    c = compare(two, three)
    assert c["compared"] == 2 and set(c) >= {"recurrence", "coseismic_slip", "hypocentre_depth"}


def test_moment_magnitude_of_a_silent_event():
    FltX = np.linspace(-4.0, 0.0, 5)
    Mw, drop, slip = moment_magnitude(3e10, FltX, np.zeros((5, 1)), np.ones((5, 1)))
    # every node is at or above 1 % of a zero maximum: zero moment, so no magnitude
    assert np.isnan(Mw[0]) and slip[0] == 0.0


def test_clock_record_from_nvidia_smi_lines():
    import bench
    lines = ["0, 2070, 2070, 900.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n",
             "0, 1980, 2070, 1400.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active\n",
             "0, 2070, 2070, 950.0, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n",
             "0, [N/A], 2070, 950.0, 0x0, Not Active, Not Active, Not Active, Not Active\n",
             "0, 2070, 20"]
    rec = bench.parse_clock_csv(lines)
    assert rec["sm_mhz"] == 2070.0 and rec["sm_max_mhz"] == 2070.0 and rec["samples"] == 3
    assert rec["reasons"] == ["sw_power_cap"]
    hot = lines[:1] + ["0, 1200, 2070, 700.0, 0x40, Not Active, Active, Not Active, Not Active\n"]
    assert bench.parse_clock_csv(hot)["reasons"] == ["hw_thermal_slowdown"]
    assert bench.parse_clock_csv([]) is None
