"""Every field of the results record (src/main.jl:479-498, trimmed as in main.jl:455-472) against
the oracle's, on a run that fills all of them: the 12 x 16 element model from a fast start
(V = 2 cm/s), 12 simulated years -- an event that starts at the first step (tStart, hypo,
taubefore), 74 s of dynamic rupture with 0.5-second coseismic snapshots (seismic_*), its end
(tEnd, tauafter, delfafter), then quasi-static steps past the 5- and 10-year marks (is_*), the
receivers every 10th step (dSeis, vSeis, aSeis) and time_/Vfmax at every step: 4,676 steps, 190
of them quasi-static.  Both sides solve every quasi-static step tightly (CG to 1e-12).

Bounds (max-norm relative to the largest entry of the field): 1e-9 for the plain FP64 methods
(observed <= 4e-10, Jacobi-PCG and multigrid alike); the mixed-precision method is held to the
per-field bounds of MIXED_BOUNDS (a few times the errors observed on GB300), which is the error it
carries against the FP64 oracle through this rupture.  Event times and hypocentres agree exactly.
"""
import numpy as np
import pytest

from eqcycle_gb300 import EQC_FP64, EQC_MIXED, EQC_PC_AMG, EQC_PC_JACOBI, Solver, preset, set_parameters

pytestmark = pytest.mark.gpu

CFG = preset("homog48").replace(NelX=12, NelY=16, LX=6e3, LY=8e3, creep_depth=6e3, V_init=2e-2,
                                total_years=12.0)
FIELDS = ("time_", "Vfmax", "tStart", "tEnd", "hypo", "taubefore", "tauafter", "delfafter", "is_slip",
          "is_slipvel", "is_stress", "seismic_slip", "seismic_slipvel", "seismic_stress", "dSeis", "vSeis", "aSeis")
# the mixed method against the FP64 oracle (observed on GB300: Vfmax 5.7e-6, seismic_slipvel 4.5e-6,
# vSeis 3.1e-6, aSeis 5.4e-5, seismic_stress 6.0e-7, the rest <= 2.5e-7)
MIXED_BOUNDS = {"aSeis": 3e-4, "Vfmax": 3e-5, "seismic_slipvel": 3e-5, "vSeis": 3e-5, "seismic_stress": 5e-6}


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def oracle_results(oracle_mod):
    o = oracle_mod.Oracle(CFG)
    steps = o.run(10 ** 9, qs_mode=1, qs_tol=1e-12)
    return steps, {f: o.get(f) for f in FIELDS}


@pytest.mark.parametrize("precision,precond", [(EQC_FP64, EQC_PC_JACOBI), (EQC_FP64, EQC_PC_AMG),
                                               (EQC_MIXED, EQC_PC_AMG)], ids=["fp64-jacobi", "fp64-mg", "mixed-mg"])
def test_every_results_field_matches_the_oracle(eqclib, oracle_results, precision, precond):
    steps, ref = oracle_results
    P = set_parameters(CFG)
    with Solver(P, precision=precision, precond=precond, cg_tol=1e-12 if precision == EQC_FP64 else 1e-10) as s:
        s.init(CFG.V_init)
        st = s.run(10 ** 9)
        res = s.results()
    assert st["steps"] == steps
    assert len(ref["tStart"]) == 1 and len(ref["tEnd"]) == 1          # the run covers every field
    assert ref["is_slip"].shape[1] == 2 and ref["seismic_slip"].shape[1] > 100 and len(ref["dSeis"]) > 400
    for f in FIELDS:
        a, b = getattr(res, f), ref[f]
        assert a.shape == b.shape, (f, a.shape, b.shape)
        if f in ("tStart", "tEnd", "hypo"):
            assert np.array_equal(a, b), f
            continue
        bound = 1e-9 if precision == EQC_FP64 else MIXED_BOUNDS.get(f, 1e-6)
        assert rel(a, b) <= bound, (f, rel(a, b))
