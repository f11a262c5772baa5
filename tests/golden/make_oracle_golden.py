"""Generate tests/golden/oracle_small.npz: the CPU oracle's outputs on small seeded cases.

The reference pins nothing on this path but the GLL table (gll_05.json), so these fixtures are
the oracle's own answers, frozen: tests/test_golden.py checks that the oracle still gives them
(a change to the restatement shows up as a fixture mismatch) and tests/test_gpu_golden.py checks
the CUDA path against them on the GPU.  Cases:

  apply_*   K x on the dz16 damage-zone mesh (8 x 16 elements, 2145 nodes), x ~ U(-1e-3, 1e-3)
  qs_*      one quasi-static solve on dz16 (Jacobi-PCG to a 1e-13 relative residual)
  nr_*      NRsearch! known answers, V over [1e-12, 10] m/s, FP64 and binary128
  loopq_*   40 steps of the reference's own model at res = 1 (quasi-static phase)
  loopd_*   60 steps of a 12 x 16 element model driven into the dynamic phase
  ev_*      the event catalogue of the 48 x 48 element homogeneous model (homog48) over 300
            years, the oracle in its reference mode (Ruge-Stueben AMG in CG to 1e-8, FP64
            friction); about 47 minutes on 8 cores

Run from the repository root:  python tests/golden/make_oracle_golden.py
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from eqcycle_gb300.config import preset, reference_config  # noqa: E402
from eqcycle_gb300.events import catalogue  # noqa: E402
from eqcycle_gb300.params import set_parameters  # noqa: E402
from eqcycle_gb300.solver import Results  # noqa: E402
from oracle import pyoracle  # noqa: E402

EV_YEARS = 300.0

APPLY_CFG = preset("dz16")
LOOPQ_CFG = reference_config(res=1)
LOOPD_CFG = preset("homog48").replace(NelX=12, NelY=16, LX=6e3, LY=8e3, creep_depth=6e3, V_init=2e-2)
EV_CFG = preset("homog48")


def nr_cases(n=48, seed=5):
    """Rows (fo, Vo, cca, ccb, Seff, tau, tauo, psi, FltZ, FltVfree), V log-uniform in [1e-12, 10]."""
    rng = np.random.default_rng(seed)
    rows = []
    for k in range(n):
        V = 10 ** (-12 + 13 * (k + rng.uniform()) / n)
        psi = rng.uniform(-2, 10)
        a, b, sig = 0.015, 0.019, 50e6
        tauo = sig * (0.6 + b * psi + a * np.log(V / 1e-6)) * rng.uniform(0.9, 1.1)
        rows.append([0.6, 1e-6, a, b, sig, 0.0, tauo, psi, 1e7 * rng.uniform(0.5, 2), V * rng.uniform(0.5, 2)])
    return np.array(rows)


def loop_record(o, prefix):
    iF = o.get("iFlt") - 1
    d, v = o.state("d"), o.state("v")
    return {f"{prefix}_d_fault": d[iF], f"{prefix}_v_fault": v[iF], f"{prefix}_psi": o.state("psi"),
            f"{prefix}_tau": o.state("tau"), f"{prefix}_d_norm": np.array([np.linalg.norm(d)]),
            f"{prefix}_v_norm": np.array([np.linalg.norm(v)]), f"{prefix}_time": o.get("time_"),
            f"{prefix}_Vfmax": o.get("Vfmax"), f"{prefix}_regime": o.get("regime")}


def main():
    pyoracle.build()
    out = {}
    o = pyoracle.Oracle(APPLY_CFG)
    x = np.random.default_rng(0).uniform(-1e-3, 1e-3, o.nglob)
    out["apply_x"], out["apply_y"] = x, o.apply_K_csr(x)
    rng = np.random.default_rng(1)
    F = rng.uniform(0, 1e-2, o.Nf)
    d0 = rng.uniform(-1e-3, 1e-3, o.nglob)
    d, it, rr = o.qs_solve(F, d0, tol=1e-13, mode=1)
    out.update(qs_F=F, qs_d0=d0, qs_d=d, qs_info=np.array([it, rr]))
    rows = nr_cases()
    out["nr_in"] = rows
    out["nr_fp64"] = np.array([pyoracle.NR(*r) for r in rows])
    out["nr_quad"] = np.array([pyoracle.NR(*r, quad=True) for r in rows])
    o = pyoracle.Oracle(LOOPQ_CFG)
    o.run(40, qs_mode=1, qs_tol=1e-14)
    out.update(loop_record(o, "loopq"))
    o = pyoracle.Oracle(LOOPD_CFG)
    o.run(60, qs_mode=1, qs_tol=1e-12)
    out.update(loop_record(o, "loopd"))
    t0 = time.time()
    pyoracle.set_threads(os.cpu_count() or 1)
    o = pyoracle.Oracle(EV_CFG.replace(total_years=EV_YEARS))
    steps = o.run(10 ** 9, qs_mode=0, qs_tol=1e-8)
    P = set_parameters(EV_CFG)
    e = np.zeros(0)
    res = Results(seismic_stress=e, seismic_slipvel=e, seismic_slip=e, index_eq=e, is_stress=e, is_slipvel=e,
                  is_slip=e, dSeis=e, vSeis=e, aSeis=e, tStart=o.get("tStart"), tEnd=o.get("tEnd"),
                  taubefore=o.get("taubefore"), tauafter=o.get("tauafter"), delfafter=o.get("delfafter"),
                  hypo=o.get("hypo"), time_=e, Vfmax=e)
    cat = catalogue(res, P.farray.FltX, EV_CFG.rho1 * EV_CFG.vs1 ** 2)
    out.update(ev_tStart=cat.tStart, ev_tEnd=cat.tEnd, ev_hypo=cat.hypo, ev_max_slip=cat.max_slip, ev_Mw=cat.Mw,
               ev_info=np.array([EV_YEARS, steps, time.time() - t0]))
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_small.npz")
    np.savez_compressed(dst, **out)
    print(dst, {k: v.shape for k, v in out.items()}, file=sys.stderr)


if __name__ == "__main__":
    main()
