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


@pytest.mark.parametrize("name", ["homog48", "dz40", "ref-res1", "ref-res2", "ens"])
def test_structured_parameters_equal_the_full_setup(name):
    """structured_parameters (the host part of the setup on the device: O(NelX + NelY) nodes)
    returns bitwise the arrays set_parameters builds over the whole mesh."""
    from eqcycle_gb300 import set_parameters, structured_parameters
    from eqcycle_gb300.config import ensemble_members, preset, reference_config
    cfg = {"homog48": preset("homog48"), "dz40": preset("dz40"), "ref-res1": reference_config(res=1),
           "ref-res2": reference_config(res=2), "ens": ensemble_members(4)[3]}[name]
    A, B = set_parameters(cfg), structured_parameters(cfg)
    for f in ("fo", "Vo", "xLf", "BcLC", "BcTC", "FltB", "FltZ", "FltX", "cca", "ccb", "Seff", "tauo", "XiLf",
              "xout", "yout"):
        assert np.array_equal(getattr(A.farray, f), getattr(B.farray, f)), f
    for f in ("iFlt", "iBcL", "iBcT", "FltIglobBC", "out_seis"):
        assert np.array_equal(getattr(A.iarray, f), getattr(B.iarray, f)), f
    assert A.float_.dt0 == B.float_.dt0 and A.mesh.muMax == B.mesh.muMax
    assert np.array_equal(A.extra["damage_idx"], B.extra["damage_idx"])
    assert np.array_equal(A.farray.M[A.iarray.iFlt - 1], B.extra["Mf"])
    assert B.mesh.W is None and B.farray.M is None and B.iarray.FltNI is None
