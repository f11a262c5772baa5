"""FP32 stiffness-apply kernels against each other and against the FP64 apply.

The element-per-lane kernels (one CTA per tile of 4, 6, 8 or 12 element rows, and the TMA-fed
walk up the strips) share their arithmetic and the order in which neighbouring contributions are added, so
their outputs must agree bit for bit on every mesh shape: strips that end inside the mesh,
walks of one and of several tiles, and the virtual last element row and column.  Against the
FP64 apply the FP32 result agrees to FP32 rounding (1e-5 of the largest entry), as does that of
the node-line kernels (apply variants 1-3: one TMA tile per CTA, plain tile loads, the persistent
TMA pipeline), which sum the two element rows of a shared node row before contracting.
"""
import ctypes as C

import numpy as np
import pytest

from eqcycle_gb300 import EQC_PC_JACOBI, Solver, preset, set_parameters
from eqcycle_gb300 import _lib as L

pytestmark = pytest.mark.gpu

MESHES = {
    "homog48": preset("homog48"),                                   # 2 strips, walks of 1 tile
    "odd37x23": preset("homog48").replace(NelX=37, NelY=23, LX=18.5e3, LY=11.5e3, creep_depth=18e3),
    "dz480": preset("dz480"),                                       # walks of 2 tiles
    "wide600x300": preset("dz480").replace(NelX=600, NelY=300),     # walks of 3 tiles
}


def _apply(s, torch, x, dtype):
    xd = x.cuda()
    yd = torch.zeros_like(xd)
    s._chk(L.lib().eqc_apply_K_device(s.h, C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), dtype))
    s._chk(L.lib().eqc_sync(s.h))
    return yd.cpu().numpy()


@pytest.mark.parametrize("name", list(MESHES))
def test_fp32_apply_kernels_agree(eqclib, name):
    torch = pytest.importorskip("torch")
    P = set_parameters(MESHES[name])
    out = {}
    for variant in (0, 4, 5, 6, 7, 8, 1, 2, 3):
        with Solver(P, precond=EQC_PC_JACOBI, apply_variant=variant) as s:
            nx, ny, ld = s.layout()
            g = torch.Generator().manual_seed(7)
            x = torch.zeros(ny, ld, dtype=torch.float32)
            x[:, :nx] = torch.rand(ny, nx, generator=g) - 0.5
            out[variant] = _apply(s, torch, x, 1)
            if variant == 0:
                out["f64"] = _apply(s, torch, x.double(), 0)
            assert np.array_equal(_apply(s, torch, x, 1), out[variant])   # deterministic
    for v in (4, 5, 6, 7, 8):            # element per lane: row tiles of 4-12 rows, the TMA walk
        assert np.array_equal(out[0], out[v]), v
    y64 = out["f64"][:, :nx]
    for v in (0, 1, 2, 3):               # and the node-line kernels: one TMA tile, plain loads, pipeline
        y32 = out[v][:, :nx].astype(np.float64)
        assert np.max(np.abs(y32 - y64)) <= 1e-5 * np.max(np.abs(y64)), v
        assert not np.any(out[v][:, nx:]), v   # row padding untouched


@pytest.mark.parametrize("variant", [0, 8])
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_fused_vcycle_equals_separate_kernels(eqclib, monkeypatch, variant, precision):
    """The V-cycle's residuals, Chebyshev steps and first coarse smoothing steps fused into the
    operator and restriction kernels give the same bits as the separate vector kernels
    (EQC_NO_FUSE), through quasi-static steps of the damage-zone model."""
    from eqcycle_gb300 import EQC_FP64, EQC_MIXED, EQC_PC_AMG
    cfg = preset("dz40")
    P = set_parameters(cfg)
    prec = EQC_MIXED if precision == "mixed" else EQC_FP64
    out = []
    for no_fuse in (False, True):
        if no_fuse:
            monkeypatch.setenv("EQC_NO_FUSE", "1")
        else:
            monkeypatch.delenv("EQC_NO_FUSE", raising=False)
        with Solver(P, precision=prec, precond=EQC_PC_AMG, guess=2, apply_variant=variant, mg_degree=4,
                    mg_degree_coarse=3) as s:
            s.init(cfg.V_init)
            st = s.run(8)
            out.append((st["cg_iters"], {k: s.state(k) for k in ("d", "psi", "tau")}))
    assert out[0][0] == out[1][0]
    for k in out[0][1]:
        assert np.array_equal(out[0][1][k], out[1][1][k]), k



@pytest.mark.parametrize("name", ["homog48", "odd37x23", "dz480"])
def test_double_float_apply_matches_fp64(eqclib, name):
    """The double-float apply of the mixed solver's true residuals against the FP64 apply: on
    random x to 1e-12 of max |K x|, and on a smooth field (K x small against |K| |x|, the
    cancellation a residual has) to 1e-12 of the random case's scale."""
    torch = pytest.importorskip("torch")
    P = set_parameters(MESHES[name])
    with Solver(P, precond=EQC_PC_JACOBI) as s:
        nx, ny, ld = s.layout()
        g = torch.Generator().manual_seed(11)
        x = torch.zeros(ny, ld, dtype=torch.float64)
        x[:, :nx] = torch.rand(ny, nx, generator=g, dtype=torch.float64) - 0.5
        y64, ydf = _apply(s, torch, x, 0), _apply(s, torch, x, 2)
        scale = np.max(np.abs(y64))
        assert np.max(np.abs(ydf - y64)) <= 1e-12 * scale
        xs = torch.zeros(ny, ld, dtype=torch.float64)
        ix = torch.arange(nx, dtype=torch.float64)[None, :]
        iy = torch.arange(ny, dtype=torch.float64)[:, None]
        xs[:, :nx] = 0.3 + 1e-3 * ix + 2e-3 * iy + 1e-4 * torch.sin(0.05 * ix) * torch.cos(0.03 * iy)
        z64, zdf = _apply(s, torch, xs, 0), _apply(s, torch, xs, 2)
        assert np.max(np.abs(zdf - z64)) <= 1e-12 * scale * float(xs.abs().max()) / 0.5


@pytest.mark.parametrize("variant", [0, 8])
def test_mixed_newmark_step_variants(eqclib, monkeypatch, variant):
    """The mixed method's dynamic step in its four-kernel form (predictor with the step counter;
    FP32 apply of the increment and one vector kernel ending the step off the fault row; the
    fault row -- its element row's apply, friction, end of step and control -- on a second stream
    beside them) replayed from its CUDA graph gives the same bits as the same kernels launched one
    by one, through 300 steps of fast slip that include a refresh of K d in FP64.  Against the
    plain FP64 step its error in every field stays within 1.5 times that of the seven-kernel form
    (EQC_NO_NM_FUSE: predictor, apply, force, boundary, fault, correction and control kernels) plus
    1e-7 of the field's scale.  This bound decides: a fault-row apply whose FP32 rounding differed
    from the bulk apply's made the displacement error ten times that of the seven-kernel form."""
    from eqcycle_gb300 import EQC_FP64, EQC_MIXED, EQC_PC_AMG
    cfg = preset("dz40").replace(V_init=5e-2)
    P = set_parameters(cfg)
    fields = ("d", "v", "a", "psi", "tau")
    out = []
    for env, graphs, prec in ((None, 1, EQC_MIXED), (None, 0, EQC_MIXED), ("EQC_NO_NM_FUSE", 1, EQC_MIXED),
                              (None, 1, EQC_FP64)):
        monkeypatch.delenv("EQC_NO_NM_FUSE", raising=False)
        if env:
            monkeypatch.setenv(env, "1")
        with Solver(P, precision=prec, precond=EQC_PC_AMG, apply_variant=variant, use_graphs=graphs) as s:
            s.init(cfg.V_init)
            st = s.run(300)                       # 300 > 256: one refresh of K d inside the phase
            out.append((st["dyn_steps"], {k: s.state(k) for k in fields}, s.results().Vfmax))
    assert out[0][0] >= 270, out[0][0]
    assert np.array_equal(out[0][2], out[1][2])
    ref = out[3][1]
    errs = {}
    for k in fields:
        assert np.array_equal(out[0][1][k], out[1][1][k]), k
        scale = np.max(np.abs(ref[k]))
        errs[k] = (float(np.max(np.abs(out[0][1][k] - ref[k])) / scale),
                   float(np.max(np.abs(out[2][1][k] - ref[k])) / scale))
    print({k: f"{a:.2e} / {b:.2e}" for k, (a, b) in errs.items()})
    for k, (fused, seven) in errs.items():
        assert seven <= 1e-3, (k, seven)
        assert fused <= 1.5 * seven + 1e-7, (k, fused, seven)


@pytest.mark.parametrize("name", ["homog48", "dz480"])
def test_double_float_intermediate_updates(eqclib, monkeypatch, name):
    """The mixed CG's intermediate reliable updates as r -= K dx with the double-float apply of the
    correction since the previous update, against every update recomputing b - K x in FP64
    (EQC_NO_DF_UPDATE): through quasi-static steps the CG iteration count stays within one per
    solve and the displacement and state agree to the solver tolerance's scale (1e-6 relative),
    every solve still certified on an FP64 residual (the run reports no CG failure)."""
    from eqcycle_gb300 import EQC_GUESS_EXTRAPOLATE, EQC_MIXED, EQC_PC_AMG
    cfg = preset(name)
    P = set_parameters(cfg)
    steps = 12 if name == "dz480" else 40
    out = []
    for env in (None, "EQC_NO_DF_UPDATE"):
        monkeypatch.delenv("EQC_NO_DF_UPDATE", raising=False)
        if env:
            monkeypatch.setenv(env, "1")
        with Solver(P, precision=EQC_MIXED, precond=EQC_PC_AMG, guess=EQC_GUESS_EXTRAPOLATE, cg_tol=1e-8) as s:
            s.init(cfg.V_init)
            st = s.run(steps)
            assert st["qs_steps"] == steps
            out.append((st["cg_iters"], st["qs_solves"], {k: s.state(k) for k in ("d", "psi", "tau")}))
    (it_df, solves, a), (it_64, _, b) = out
    assert abs(it_df - it_64) <= solves, (it_df, it_64)
    for k in a:
        assert np.max(np.abs(a[k] - b[k])) <= 1e-6 * np.max(np.abs(b[k])), k
