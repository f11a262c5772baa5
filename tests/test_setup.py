"""The product's host setup (eqcycle_gb300.params, the par.jl mirror) against the oracle's."""
import numpy as np
import pytest

from eqcycle_gb300.config import preset, reference_config
from eqcycle_gb300.params import set_parameters, gll

CFGS = [reference_config(res=1), reference_config(res=2), preset("homog48"), preset("dz40"),
        preset("homog48", seed=3).replace(NelX=10, NelY=30, LY=72e3)]


@pytest.mark.parametrize("cfg", CFGS, ids=["ref-res1", "ref-res2", "homog48", "dz40", "rect"])
def test_setup_bitwise_equal_to_oracle(oracle_mod, cfg):
    P = set_parameters(cfg)
    o = oracle_mod.Oracle(cfg)
    m, fa, ia = P.mesh, P.farray, P.iarray
    pairs = [("iglob", m.iglob), ("x", m.x), ("y", m.y), ("W", m.W), ("H", m.H)]
    pairs += [(n, getattr(fa, n)) for n in ("fo", "Vo", "xLf", "M", "BcLC", "BcTC", "FltB", "FltZ", "FltX", "cca",
                                            "ccb", "Seff", "tauo", "XiLf", "xout", "yout")]
    pairs += [(n, getattr(ia, n)) for n in ("iFlt", "iBcL", "iBcT", "FltIglobBC", "FltNI", "out_seis")]
    for name, a in pairs:
        b = o.get(name)
        assert np.asarray(a).shape == b.shape, name
        assert np.array_equal(np.asarray(a), b), name
    assert P.float_.dt0 == o.scalar("dt0")


def test_reference_creeping_nodes_match_par_jl_rule():
    """par.jl:214-217: FltIglobBC = fault nodes deeper than 24 km, listed element by element
    (shared element-edge nodes appear twice)."""
    P = set_parameters(reference_config(res=1))
    FltX = P.farray.FltX
    deep = P.iarray.iFlt[np.abs(FltX) > 24e3]
    assert set(P.iarray.FltIglobBC.tolist()) == set(deep.tolist())
    assert len(P.iarray.FltIglobBC) == len(deep) + (len(deep) - 1) // 4


def test_gll_symmetry():
    x, w, H = gll(5)
    assert np.allclose(x, -x[::-1], atol=0) and np.allclose(w, w[::-1], atol=0)
    assert np.allclose(H, -H[::-1, ::-1], atol=1e-13)
