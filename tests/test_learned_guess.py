"""Learned initial guess: the network's GPU forward/backward kernels against the CPU
restatement (oracle/guessnet.py), training on pairs the time loop logs, and what the trained
network gains over the previous-step guess.  CG always runs to the same tolerance, so the
guess may change iteration counts, never the converged answer."""
import numpy as np
import pytest

from eqcycle_gb300 import (EQC_GUESS_LEARNED, EQC_GUESS_PREVIOUS, EQC_MIXED, EQC_PC_AMG, Solver, preset,
                           set_parameters)

pytestmark = pytest.mark.gpu

SMALL = preset("homog48").replace(NelX=12, NelY=16, LX=6e3, LY=8e3, creep_depth=6e3)


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_guess_network_gradient_matches_oracle(eqclib):
    from oracle import guessnet as gn
    P = set_parameters(SMALL)
    with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG) as s:
        nin, nout, npar = s.guess_shape()
        Nf = P.int_.FltNglob
        assert nin == 2 * Nf and nout == gn.GX * gn.GY and npar == gn.shapes(Nf)[3]
        rng = np.random.default_rng(3)
        p = (rng.uniform(-1, 1, npar) * 0.2).astype(np.float32)
        s.set_guess_params(p)
        x0 = rng.uniform(-1, 1, (3, nin)).astype(np.float32)
        tgt = rng.uniform(-1, 1, (3, nout)).astype(np.float32)
        g_gpu, loss_gpu = s.guess_grad(x0, tgt)
        mse, out_gpu = s.guess_eval(x0, tgt, outputs=True)
    loss, g_ref, out_ref = gn.loss_and_grad(p.astype(np.float64), x0, tgt)
    assert rel(out_gpu, out_ref) <= 1e-5
    assert abs(loss_gpu - loss) <= 1e-5 * loss and abs(mse - loss) <= 1e-5 * loss
    _, _, offs, _ = gn.shapes(Nf)
    for name, (o, shp) in offs.items():   # every parameter block
        k = int(np.prod(shp))
        assert rel(g_gpu[o:o + k], g_ref[o:o + k]) <= 1e-4, name


def _collect(P, cfg, steps, seed_shift=0.0):
    """Pairs logged by the plain method's quasi-static steps (first solve of every step)."""
    with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=EQC_GUESS_PREVIOUS) as s:
        s.guess_log(steps)
        s.init(cfg.V_init)
        s.run(steps)
        return s.guess_pairs()


def test_learned_guess_trains_and_runs_in_the_time_loop(eqclib):
    cfg = SMALL.replace(V_init=1e-9)   # slow creep: quasi-static steps throughout
    P = set_parameters(cfg)
    xin, tgt = _collect(P, cfg, 80)
    assert len(xin) >= 60
    train, held = slice(0, 60), slice(60, None)
    with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=EQC_GUESS_LEARNED) as s:
        s.guess_init(7)
        losses = s.guess_train(xin[train], tgt[train], epochs=20, lr=1e-3, batch=16, seed=1)
        assert np.all(np.isfinite(losses)) and losses[-1] < losses[0]
        mse_held = s.guess_eval(xin[held], tgt[held])
        params = s.guess_params()
    zero_mse = float(np.mean(tgt[held].astype(np.float64) ** 2))   # the previous-step guess predicts 0
    print(f"held-out MSE: network {mse_held:.3e}, previous-step guess {zero_mse:.3e}")
    assert mse_held < zero_mse
    # time loop with the trained network: same converged state as the plain guess
    out = {}
    for mode, graphs in ((EQC_GUESS_PREVIOUS, 1), (EQC_GUESS_LEARNED, 1), (EQC_GUESS_LEARNED, 0)):
        with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=mode, cg_tol=1e-10, use_graphs=graphs) as s:
            if mode == EQC_GUESS_LEARNED:
                s.set_guess_params(params)
            s.init(cfg.V_init)
            st = s.run(20)
            out[(mode, graphs)] = (st, {k: s.state(k) for k in ("d", "v", "psi")})
    (st_p, x_p), (st_l, x_l), (st_e, x_e) = out[(0, 1)], out[(1, 1)], out[(1, 0)]
    print(f"CG iterations per solve: previous {st_p['cg_iters'] / st_p['qs_solves']:.2f}, "
          f"learned {st_l['cg_iters'] / st_l['qs_solves']:.2f}")
    assert st_l["qs_steps"] == st_p["qs_steps"] == 20
    for k in x_p:
        assert rel(x_l[k], x_p[k]) <= 1e-6, k
        assert np.array_equal(x_l[k], x_e[k]), k        # graph replay == host-driven step
    assert st_l["cg_iters"] == st_e["cg_iters"]


def test_learned_guess_gain_on_held_out_seeds(eqclib):
    """The network trained on pairs logged on six seeds of the 12 x 16 element model (seeded state
    noise, slow creep: quasi-static steps throughout) lowers the CG iterations of the first solve
    of each step on two held-out seeds, against the previous-step guess, at the same tolerance;
    the on-device check keeps increments only where they lower the residual."""
    base = SMALL.replace(V_init=1e-9, noise_amp=0.05)
    xs, ys = [], []
    for seed in range(1, 7):
        cfg = base.replace(seed=seed)
        x, y = _collect(set_parameters(cfg), cfg, 80)
        xs.append(x)
        ys.append(y)
    xin, tgt = np.concatenate(xs), np.concatenate(ys)
    P0 = set_parameters(base.replace(seed=1))
    with Solver(P0, precision=EQC_MIXED, precond=EQC_PC_AMG) as s:
        s.guess_init(7)
        losses = s.guess_train(xin, tgt, epochs=30, lr=1e-3, batch=32, seed=1)
        params = s.guess_params()
    assert losses[-1] < losses[0]
    iters = {EQC_GUESS_PREVIOUS: 0, EQC_GUESS_LEARNED: 0}
    solves = {EQC_GUESS_PREVIOUS: 0, EQC_GUESS_LEARNED: 0}
    kept = 0
    for seed in (7, 8):
        cfg = base.replace(seed=seed)
        P = set_parameters(cfg)
        for mode in (EQC_GUESS_PREVIOUS, EQC_GUESS_LEARNED):
            with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=mode, cg_tol=1e-10) as s:
                if mode == EQC_GUESS_LEARNED:
                    s.set_guess_params(params)
                s.init(cfg.V_init)
                st = s.run(30)
                iters[mode] += st["cg_iters"]
                solves[mode] += st["qs_solves"]
                if mode == EQC_GUESS_LEARNED:
                    kept += s.scalar("guess_kept")
    prev = iters[EQC_GUESS_PREVIOUS] / solves[EQC_GUESS_PREVIOUS]
    learned = iters[EQC_GUESS_LEARNED] / solves[EQC_GUESS_LEARNED]
    print(f"held-out seeds: CG iterations per solve previous {prev:.3f}, learned {learned:.3f}, kept {kept}")
    assert kept > 0
    assert learned < 0.97 * prev
