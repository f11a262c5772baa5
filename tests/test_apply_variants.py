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
