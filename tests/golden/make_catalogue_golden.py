"""Generate tests/golden/catalogue_homog48.npz: every field of the results record
(src/main.jl:479-498, trimmed as in main.jl:455-472) of the CPU oracle's 300-year run of the
homogeneous 48 x 48 element model (homog48), the oracle in its reference mode (Ruge-Stueben AMG
in CG to a 1e-8 relative residual, FP64 friction).

Stored per event (float64): tStart, tEnd, hypo, taubefore, tauafter, delfafter.
Stored per snapshot (float32, enough for the 2 % comparison they serve): the 5-year interseismic
snapshots is_slip, is_slipvel, is_stress, and every 5th of the 0.5-second coseismic snapshots
seismic_slip, seismic_slipvel, seismic_stress (with their total count).  The receiver records (every 10th step) and time_/Vfmax
(every step) are indexed by step number, which differs between two solvers once the step
sizes differ, so they are left to the short runs compared live.

About 50 minutes on 8 cores.  Run from the repository root:
    python tests/golden/make_catalogue_golden.py
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from eqcycle_gb300.config import preset  # noqa: E402
from oracle import pyoracle  # noqa: E402

YEARS = 300.0
CFG = preset("homog48").replace(total_years=YEARS)


def main():
    pyoracle.build()
    pyoracle.set_threads(os.cpu_count() or 1)
    o = pyoracle.Oracle(CFG)
    t0 = time.time()
    steps = o.run(10 ** 9, qs_mode=0, qs_tol=1e-8)
    out = {"info": np.array([YEARS, steps, time.time() - t0])}
    for f in ("tStart", "tEnd", "hypo", "taubefore", "tauafter", "delfafter"):
        out[f] = np.asarray(o.get(f), dtype=np.float64)
    for f in ("is_slip", "is_slipvel", "is_stress"):
        out[f] = np.asarray(o.get(f), dtype=np.float32)
    for f in ("seismic_slip", "seismic_slipvel", "seismic_stress"):   # every 5th snapshot (2.5 s apart)
        m = np.asarray(o.get(f), dtype=np.float32)
        out[f + "_every5"] = np.ascontiguousarray(m[:, ::5])
        out["seismic_count"] = np.array([m.shape[1]])
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "catalogue_homog48.npz")
    np.savez_compressed(dst, **out)
    print(dst, steps, "steps", {k: v.shape for k, v in out.items()}, file=sys.stderr)


if __name__ == "__main__":
    main()
