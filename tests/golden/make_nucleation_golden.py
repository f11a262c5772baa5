"""Generate tests/golden/nucleation_homog48.npz: the CPU oracle's history of the homogeneous 48 x 48
element model (homog48) from the seeded start through its first nucleation, i.e. up to the step at
which the maximum slip rate first exceeds the event threshold (1.01 Vthres, main.jl:361-365).

Stored: for every step, the time, the regime and the maximum slip rate; every CHECK-th step and at
the last one, the fault displacement d[iFlt], the fault velocity v[iFlt] and the state psi.  The
oracle runs its reference mode (Ruge-Stueben AMG in CG), one step per call, which is the same
trajectory as one call for all the steps.  Its CG runs to a 1e-12 relative residual: a residual
of 1e-8, the workloads' tolerance, leaves a solver error of ~1e-8
per step that the nucleation amplifies to ~1e-4 in slip rate, so two correct solvers stopped at
1e-8 differ by that much; converged solves leave only rounding.

Run from the repository root:  python tests/golden/make_nucleation_golden.py
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from eqcycle_gb300.config import preset  # noqa: E402
from oracle import pyoracle  # noqa: E402

CFG = preset("homog48")
CHECK = 50
QS_TOL = 1e-12
MAX_STEPS = 200000


def main():
    pyoracle.build()
    pyoracle.set_threads(os.cpu_count() or 1)
    o = pyoracle.Oracle(CFG)
    iF = o.get("iFlt") - 1
    vthres = CFG.Vthres
    t0 = time.time()
    cks, d_f, v_f, psi = [], [], [], []
    k = 0
    while k < MAX_STEPS:
        if o.run(1, qs_mode=0, qs_tol=QS_TOL) != 1:
            raise RuntimeError(f"oracle stopped at step {k + 1}")
        k += 1
        vfmax = o.get("Vfmax")[-1]
        last = vfmax > 1.01 * vthres
        if k % CHECK == 0 or last:
            cks.append(k)
            d_f.append(o.state("d")[iF])
            v_f.append(o.state("v")[iF])
            psi.append(o.state("psi"))
        if last:
            break
        if k % 200 == 0:
            print(f"step {k}: t = {o.scalar('t'):.4g} s, Vfmax = {vfmax:.3e}, {time.time() - t0:.0f} s",
                  file=sys.stderr, flush=True)
    out = {"time": o.get("time_"), "regime": o.get("regime"), "Vfmax": o.get("Vfmax"), "cg_iters": o.get("cg_iters"),
           "check_steps": np.array(cks), "d_fault": np.array(d_f), "v_fault": np.array(v_f),
           "psi": np.array(psi), "info": np.array([k, CHECK, QS_TOL, time.time() - t0])}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "nucleation_homog48.npz")
    np.savez_compressed(dst, **out)
    print(dst, k, "steps", {n: v.shape for n, v in out.items()}, file=sys.stderr)


if __name__ == "__main__":
    main()
