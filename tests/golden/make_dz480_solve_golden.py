"""Generate tests/golden/dz480_solve.npz: the CPU oracle's quasi-static solve on the benchmark mesh
(dz480: 480 x 240 elements, 1,846,081 nodes), the oracle in its reference mode (Ruge-Stueben AMG
in CG) run to a 1e-12 relative residual.

Inputs are regenerated from their seed by the test (fault displacement F ~ U(0, 1e-2) m from
numpy's default_rng(1), zero initial guess).  The full solution (15 MB) is not stored; what is:
  idx      20,000 node indices (reference numbering, 0-based) drawn by default_rng(2)
  d_idx    the solution at those nodes
  norms    [||d||_2, ||d||_inf, sum(d * w)] with w ~ U(-1, 1) from default_rng(3)
  info     [iterations, relative residual, seconds]

About 10 minutes on 8 cores.  Run from the repository root:
    python tests/golden/make_dz480_solve_golden.py
"""
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from eqcycle_gb300.config import preset  # noqa: E402
from oracle import pyoracle  # noqa: E402

TOL = 1e-12
NSAMPLE = 20000


def inputs(nglob, nf):
    F = np.random.default_rng(1).uniform(0, 1e-2, nf)
    idx = np.sort(np.random.default_rng(2).choice(nglob, NSAMPLE, replace=False))
    w = np.random.default_rng(3).uniform(-1, 1, nglob)
    return F, idx, w


def main():
    pyoracle.build()
    pyoracle.set_threads(os.cpu_count() or 1)
    o = pyoracle.Oracle(preset("dz480"))
    F, idx, w = inputs(o.nglob, o.Nf)
    t0 = time.time()
    d, it, rr = o.qs_solve(F, np.zeros(o.nglob), tol=TOL, mode=0)
    out = {"idx": idx, "d_idx": d[idx],
           "norms": np.array([np.linalg.norm(d), np.max(np.abs(d)), float(np.dot(d, w))]),
           "info": np.array([it, rr, time.time() - t0])}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "dz480_solve.npz")
    np.savez_compressed(dst, **out)
    print(dst, it, rr, file=sys.stderr)


if __name__ == "__main__":
    main()
