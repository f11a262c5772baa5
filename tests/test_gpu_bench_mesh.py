"""Parity on the benchmark meshes: the 480 x 240 element damage-zone model (dz480, 1,846,081
nodes, the benchmark workload) and its refinement dz960 (7,378,561 nodes).

  * K x through the C ABI (FP64, every apply kernel: the persistent TMA pipeline, the one-tile
    TMA kernel, plain tile loads, and the pipeline with TMA switched off) against the oracle's
    assembled CSR matrix (Kassemble.jl:3-63), 1e-12 of max |K x|;
  * one quasi-static solve on dz480 (FP64 multigrid CG to 1e-12): its residual evaluated with the
    oracle's CSR operator, and the solution against the oracle's own tight solve (reference mode,
    RS-AMG CG to 1e-12, frozen as tests/golden/dz480_solve.npz: 20,000 sampled nodes and three
    norms of the whole vector);
  * the benchmarked mixed-precision solve (FP32 apply and multigrid inside the FP64
    reliable-update CG, tolerance 1e-8): residual under the oracle's operator below 1e-8, and
    the solution within 1e-6 of the FP64 one.
"""
import os

import numpy as np
import pytest

from eqcycle_gb300 import EQC_FP64, EQC_MIXED, EQC_PC_AMG, EQC_PC_JACOBI, Solver, preset, set_parameters

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "dz480_solve.npz")


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.fixture(scope="module")
def meshes(eqclib, oracle_mod):
    oracle_mod.set_threads(os.cpu_count() or 1)
    out = {}
    for name in ("dz480", "dz960"):
        cfg = preset(name)
        out[name] = (cfg, set_parameters(cfg), oracle_mod.Oracle(cfg))
    return out


@pytest.mark.parametrize("name", ["dz480", "dz960"])
@pytest.mark.parametrize("variant", [0, 1, 2], ids=["pipelined", "one-tile", "plain-loads"])
def test_fp64_apply_matches_oracle_csr(meshes, name, variant):
    cfg, P, o = meshes[name]
    x = np.random.default_rng(0).uniform(-1e-3, 1e-3, P.int_.nglob)
    y_ref = o.apply_K_csr(x)
    with Solver(P, precond=EQC_PC_JACOBI, apply_variant=variant) as s:
        y = s.apply_K(x)
    assert rel(y, y_ref) <= 1e-12


def test_fp64_apply_without_tma_matches_oracle_csr(meshes, monkeypatch):
    cfg, P, o = meshes["dz480"]
    monkeypatch.setenv("EQC_NO_TMA", "1")        # read when the handle builds its tensor maps
    x = np.random.default_rng(5).uniform(-1e-3, 1e-3, P.int_.nglob)
    with Solver(P, precond=EQC_PC_JACOBI) as s:
        y = s.apply_K(x)
    assert rel(y, o.apply_K_csr(x)) <= 1e-12


def _oracle_relres(o, P, F, d):
    iF = P.iarray.iFlt - 1
    FltNI = P.iarray.FltNI - 1
    dF = np.zeros(P.int_.nglob)
    dF[iF] = F
    b = -o.apply_K_csr(dF)[FltNI]
    r = o.apply_K_csr(d)[FltNI]          # K_II d_I + K_IF F = -(b - K_II d_I)
    return float(np.linalg.norm(r) / np.linalg.norm(b))


@pytest.fixture(scope="module")
def dz480_solves(meshes):
    cfg, P, o = meshes["dz480"]
    F = np.random.default_rng(1).uniform(0, 1e-2, P.int_.FltNglob)
    d0 = np.zeros(P.int_.nglob)
    with Solver(P, precision=EQC_FP64, precond=EQC_PC_AMG) as s:
        d64, it64, rr64 = s.qs_solve(F, d0, tol=1e-12)
    with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG) as s:
        d32, it32, rr32 = s.qs_solve(F, d0, tol=1e-8)
    return F, (d64, it64, rr64), (d32, it32, rr32)


def test_fp64_solve_on_dz480_solves_the_oracle_system(meshes, dz480_solves):
    cfg, P, o = meshes["dz480"]
    F, (d, it, rr), _ = dz480_solves
    assert 0 < it <= 40 and rr <= 1e-12
    assert _oracle_relres(o, P, F, d) <= 2e-12
    assert np.array_equal(d[P.iarray.iFlt - 1], F)


def test_fp64_solve_on_dz480_matches_the_oracle_solution(meshes, dz480_solves):
    g = dict(np.load(GOLD))
    F, (d, it, rr), _ = dz480_solves
    assert g["info"][1] <= 1e-12                         # the oracle's own tight solve
    ref = g["d_idx"]
    scale = g["norms"][1]
    assert np.max(np.abs(d[g["idx"]] - ref)) <= 1e-9 * scale
    w = np.random.default_rng(3).uniform(-1, 1, len(d))
    assert abs(np.linalg.norm(d) - g["norms"][0]) <= 1e-9 * g["norms"][0]
    assert abs(np.max(np.abs(d)) - scale) <= 1e-9 * scale
    assert abs(float(np.dot(d, w)) - g["norms"][2]) <= 1e-9 * np.sum(np.abs(w)) * scale


def test_mixed_solve_on_dz480(meshes, dz480_solves):
    cfg, P, o = meshes["dz480"]
    F, (d64, _, _), (d32, it, rr) = dz480_solves
    assert 0 < it <= 40 and rr <= 1e-8                  # certified on the FP64 true residual
    assert _oracle_relres(o, P, F, d32) <= 1e-8           # ... which the oracle's operator confirms
    assert rel(d32, d64) <= 1e-6
