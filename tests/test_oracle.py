"""The CPU oracle against the reference's own data and against mathematical invariants.

The GLL table is the only reference-shipped data on this path (pinned below); the rest of
the oracle is a restatement checked through properties the reference's formulas imply.
"""
import json
import os

import numpy as np
import pytest

from eqcycle_gb300.config import preset, reference_config

GOLD = os.path.join(os.path.dirname(__file__), "golden", "gll_05.json")


def test_gll_matches_reference_table(oracle_mod):
    g = json.load(open(GOLD))
    x, w, H = oracle_mod.gll(5)
    assert np.max(np.abs(x - np.array(g["x"]))) <= 2.3e-16
    assert np.max(np.abs(w - np.array(g["w"]))) <= 2.3e-16
    # the table prints 16 significant digits
    assert np.max(np.abs(H - np.array(g["H"]))) <= 4e-15


@pytest.mark.parametrize("cfg", [reference_config(res=1), preset("homog48"), preset("dz40")],
                         ids=["reference-res1", "homog48", "dz40"])
def test_stiffness_invariants(oracle_mod, cfg):
    o = oracle_mod.Oracle(cfg)
    K = o.csr()
    if cfg.NelX == 48:
        assert K.nnz == 407809   # 48x48 mesh, NGLL 5
    scale = abs(K).max()
    assert abs(K - K.T).max() <= 1e-14 * scale                        # symmetric
    assert np.abs(K @ np.ones(o.nglob)).max() <= 1e-14 * scale        # constants in the null space
    x = np.random.default_rng(3).uniform(-1, 1, o.nglob)
    y1, y2 = o.apply_K_csr(x), o.apply_K_elem(x)                      # Kassemble.jl vs PCG.jl:82
    assert np.abs(y1 - y2).max() <= 1e-13 * np.abs(y1).max()
    assert float(x @ y1) > 0                                           # positive semi-definite


def test_element_apply_single_element_check(oracle_mod):
    """src/dump.jl:9-66 compares the element form with Ke*u for one element (seeded here)."""
    cfg = reference_config(res=1).replace(NelX=1, NelY=1, LX=1600.0, LY=1500.0, rec_x=[], rec_y=[])
    o = oracle_mod.Oracle(cfg)
    u = np.random.default_rng(7).uniform(size=o.nglob)
    assert np.allclose(o.apply_K_csr(u), o.apply_K_elem(u), rtol=0, atol=1e-12 * np.abs(o.apply_K_csr(u)).max())


def test_qs_solve_modes_agree(oracle_mod):
    o = oracle_mod.Oracle(reference_config(res=1))
    F = np.random.default_rng(1).uniform(0, 1e-3, o.Nf)
    d0 = np.zeros(o.nglob)
    d_amg, it_amg, rr_amg = o.qs_solve(F, d0, tol=1e-12, mode=0)
    d_jac, it_jac, rr_jac = o.qs_solve(F, d0, tol=1e-12, mode=1)
    assert it_amg > 0 and it_jac > 0 and rr_amg <= 1e-12 and rr_jac <= 1e-12
    assert np.abs(d_amg - d_jac).max() <= 1e-9 * np.abs(d_jac).max()
    # the solution satisfies K[FltNI,:] d = 0 with d[iFlt] = F
    K = o.csr()
    NI = o.get("FltNI") - 1
    r = (K @ d_jac)[NI]
    assert np.linalg.norm(r) <= 1e-11 * np.linalg.norm((K[:, o.get("iFlt") - 1] @ F)[NI])


def test_nr_fp64_vs_binary128(oracle_mod):
    """The reference's NRsearch! iterates in BigFloat; FP64 agrees to round-off."""
    rng = np.random.default_rng(5)
    worst = 0.0
    for _ in range(400):
        V = 10 ** rng.uniform(-12, 1)
        psi = rng.uniform(-2, 10)
        a, b, sig = 0.015, 0.019, 50e6
        tauo = sig * (0.6 + b * psi + a * np.log(V / 1e-6)) * rng.uniform(0.9, 1.1)
        FltZ = 1e7 * rng.uniform(0.5, 2)
        Vfree = V * rng.uniform(0.5, 2)
        r64 = oracle_mod.NR(0.6, 1e-6, a, b, sig, 0.0, tauo, psi, FltZ, Vfree)
        r128 = oracle_mod.NR(0.6, 1e-6, a, b, sig, 0.0, tauo, psi, FltZ, Vfree, quad=True)
        assert r64[2] == r128[2]
        worst = max(worst, abs(r64[1] - r128[1]) / abs(r128[1]))
    assert worst <= 1e-12


def test_time_loop_first_steps(oracle_mod):
    cfg = preset("homog48").replace(NelX=12, NelY=12, LX=6e3, LY=6e3, creep_depth=6e3)
    o = oracle_mod.Oracle(cfg)
    n = o.run(20, qs_mode=1, qs_tol=1e-10)
    assert n == 20
    t = o.get("time_")
    assert np.all(np.diff(t) > 0)
    dt = np.diff(np.concatenate([[0.0], t]))
    assert np.all(dt[1:] <= 1.2 * dt[:-1] * (1 + 1e-12))   # dtevol: growth capped at 1.2x
    assert np.all(np.isfinite(o.state("d"))) and np.all(np.isfinite(o.state("psi")))


def test_guessnet_restatement_gradient_by_finite_differences():
    """The CPU restatement of the learned-guess network: its backward pass agrees with central
    differences of its forward pass (FP64 weights, so the check is not hidden by rounding)."""
    from oracle import guessnet as gn
    Nf = 13
    _, _, offs, n = gn.shapes(Nf)
    rng = np.random.default_rng(0)
    p = rng.uniform(-0.3, 0.3, n).astype(np.float64)
    x0 = rng.uniform(-1, 1, (2, 2 * Nf))
    tgt = rng.uniform(-1, 1, (2, gn.GX * gn.GY))
    loss, g, _ = gn.loss_and_grad(p, x0, tgt, round_bf16=False)
    h = 1e-6
    for name, (o, shp) in offs.items():
        for j in rng.choice(int(np.prod(shp)), size=3, replace=False):
            q = p.copy(); q[o + j] += h
            lp = gn.loss_and_grad(q, x0, tgt, round_bf16=False)[0]
            q[o + j] -= 2 * h
            lm = gn.loss_and_grad(q, x0, tgt, round_bf16=False)[0]
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[o + j]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (name, j, fd, g[o + j])


def test_bf16_rounding_restatement():
    """Round-to-nearest-even to BF16 on known values (ties, carries into the exponent)."""
    from oracle import guessnet as gn
    x = np.array([1.0, 1.00390625, 1.005859375, 1.0078125, -2.5, 3.3e-3], dtype=np.float32)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7 -> even (1.0); 1 + 1.5*2^-8 rounds up
    want = np.array([1.0, 1.0, 1.0078125, 1.0078125, -2.5, 0.0032958984375])
    assert np.array_equal(gn.bf16(x), want)


def test_guessnet_rounds_every_weight_block_and_no_bias():
    from oracle import guessnet as gn
    Nf = 13
    _, _, offs, n = gn.shapes(Nf)
    p = np.full(n, 0.05, dtype=np.float32)   # 0.05 is not a BF16 value
    W = gn.unpack(p.astype(np.float64), Nf)
    for k, v in W.items():
        want = gn.bf16(np.float32(0.05)) if (k.startswith("cw") or k in ("f1w", "f2w")) else np.float32(0.05)
        assert np.all(v == np.float64(want)), k


def test_event_statistics_restatement():
    """post/earthquake_cycles.jl (Coslip, moment_magnitude_new) restated on a hand-built run."""
    from eqcycle_gb300.events import catalogue, compare
    from eqcycle_gb300.solver import Results
    Nf = 11
    FltX = np.linspace(-10.0, 0.0, Nf)            # dx = 1
    slip = np.zeros((Nf, 2))
    slip[2:5, 0] = [1.0, 2.0, 1.0]
    slip[5:8, 1] = [0.5, 0.5, 0.001]              # the last node is below 1 % of the maximum
    tb = np.full((Nf, 2), 30.0)
    ta = np.full((Nf, 2), 28.0)
    e = np.zeros(0)
    res = Results(seismic_stress=e, seismic_slipvel=e, seismic_slip=e, index_eq=e, is_stress=e, is_slipvel=e,
                  is_slip=e, dSeis=e, vSeis=e, aSeis=e, tStart=np.array([0.0, 100.0]), tEnd=np.array([5.0, 106.0]),
                  taubefore=tb, tauafter=ta, delfafter=slip, hypo=np.array([-7.0, -4.0]), time_=e, Vfmax=e)
    mu = 3e10
    cat = catalogue(res, FltX, mu)
    assert np.allclose(cat.max_slip, [2.0, 0.5])
    assert np.allclose(cat.mean_slip, [4.0 / 3.0, 1.0 / 2.0])     # area / zdim over the rupture
    assert np.allclose(cat.mean_drop, [2.0, 2.0])
    want_mw0 = (2.0 / 3.0) * np.log10(mu * 4.0 * 3.0 * 1e7) - 10.7
    assert abs(cat.Mw[0] - want_mw0) < 1e-12
    assert np.allclose(cat.recurrence, [100.0])
    c = compare(cat, cat)
    assert c["compared"] == 2 and c["recurrence"] == 0 and c["coseismic_slip"] == 0 and c["hypocentre_depth"] == 0


@pytest.mark.parametrize("cfg", [reference_config(res=1), preset("dz40")], ids=["ref-res1", "dz40"])
def test_damage_evolution_restatement(oracle_mod, cfg):
    """damageEvol.jl in the oracle: the damage zone of Assemble.jl:25-35 (the host setup gives
    the same elements), W of those elements scaled by the factor, K assembled again; the
    assembled and the element-wise apply still agree, and K changes only through those
    elements (K' x - K x = (f - 1) K_D x, K_D the damaged elements' part, which is zero for x
    supported away from the damage zone)."""
    from eqcycle_gb300 import set_parameters
    P = set_parameters(cfg)
    o = oracle_mod.Oracle(cfg)
    di = o.get("damage_idx")
    assert len(di) > 0 and np.array_equal(di, P.extra["damage_idx"])
    W0 = o.get("W").copy()
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, o.nglob)
    y0 = o.apply_K_csr(x)
    o.set_damage(di, 0.95)
    o.damage_evolve()
    assert o.scalar("damage_count") == 1
    W1 = o.get("W")
    mask = np.zeros(W0.shape[2], bool)
    mask[di - 1] = True
    assert np.array_equal(W1[:, :, ~mask], W0[:, :, ~mask])
    assert np.allclose(W1[:, :, mask], 0.95 * W0[:, :, mask], rtol=1e-15, atol=0)
    y1 = o.apply_K_csr(x)
    assert np.max(np.abs(y1 - o.apply_K_elem(x))) <= 1e-13 * np.max(np.abs(y1))
    # nodes of undamaged elements only: K x unchanged there
    ig = o.get("iglob") - 1
    touched = np.zeros(o.nglob, bool)
    touched[np.unique(ig[:, :, mask])] = True
    assert np.array_equal(y1[~touched], y0[~touched])
    assert np.max(np.abs(y1[touched] - y0[touched])) > 0
