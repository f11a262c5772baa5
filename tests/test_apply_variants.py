"""FP32 stiffness-apply kernels against each other and against the FP64 apply.

The element-per-lane kernels (one CTA per tile of element rows, and the TMA-fed walk up the
strips) share their arithmetic and the order in which neighbouring contributions are added, so
their outputs must agree bit for bit on every mesh shape: strips that end inside the mesh,
walks of one and of several tiles, and the virtual last element row and column.  Against the
FP64 apply the FP32 result agrees to FP32 rounding (1e-5 of the largest entry).
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
    for variant in (0, 8):
        with Solver(P, precond=EQC_PC_JACOBI, apply_variant=variant) as s:
            nx, ny, ld = s.layout()
            g = torch.Generator().manual_seed(7)
            x = torch.zeros(ny, ld, dtype=torch.float32)
            x[:, :nx] = torch.rand(ny, nx, generator=g) - 0.5
            out[variant] = _apply(s, torch, x, 1)
            if variant == 0:
                out["f64"] = _apply(s, torch, x.double(), 0)
            assert np.array_equal(_apply(s, torch, x, 1), out[variant])   # deterministic
    assert np.array_equal(out[0], out[8])
    y32, y64 = out[8][:, :nx].astype(np.float64), out["f64"][:, :nx]
    assert np.max(np.abs(y32 - y64)) <= 1e-5 * np.max(np.abs(y64))
    assert not np.any(out[8][:, nx:])   # row padding untouched
