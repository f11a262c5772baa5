"""Setup on the device (eqc_create_structured): the model built by kernels from the material
rule equals, bit for bit, the one eqc_create builds from the host setup's arrays: same
stiffness apply, and the same state after quasi-static and dynamic steps."""
import numpy as np
import pytest

from eqcycle_gb300 import (EQC_FP64, EQC_MIXED, EQC_PC_AMG, Solver, preset, reference_config, set_parameters,
                           structured_parameters)

pytestmark = pytest.mark.gpu

CFGS = {"homog48": preset("homog48"), "dz40": preset("dz40"), "ref-res1": reference_config(res=1)}


@pytest.mark.parametrize("name", list(CFGS))
@pytest.mark.parametrize("precision", [EQC_FP64, EQC_MIXED])
def test_device_setup_equals_host_setup(eqclib, name, precision):
    cfg = CFGS[name]
    out = []
    for P in (set_parameters(cfg), structured_parameters(cfg)):
        with Solver(P, precision=precision, precond=EQC_PC_AMG, guess=2) as s:
            x = np.random.default_rng(2).uniform(-1e-3, 1e-3, P.int_.nglob)
            y = s.apply_K(x)
            s.init(cfg.V_init)
            st = s.run(6)
            s.set_scalar("isolver", 2)   # a few dynamic steps from there
            s.run(4)
            out.append((y, st, {k: s.state(k) for k in ("d", "v", "a", "psi", "tau")},
                        s.scalar("setup_ms_hierarchy")))
    (y0, st0, x0, _), (y1, st1, x1, hier) = out
    assert np.array_equal(y0, y1)
    assert st0["cg_iters"] == st1["cg_iters"]
    for k in x0:
        assert np.array_equal(x0[k], x1[k]), k
    assert hier > 0
