"""Model configuration: the inputs of the reference's ``setParameters`` (par.jl:15-231).

The reference hard-codes its model in par.jl and src/initialConditions/defaultInitialConditions.jl;
``ModelConfig`` names those inputs so that both the reference's own default
(``reference_config``) and the benchmark workloads (``preset``) can be built by the same
setup code (``eqcycle_gb300.params.set_parameters``).

Axis convention follows the reference: x is depth (NelX elements, LX metres, the fault is
the line y = 0 with x in [-LX, 0]) and y is the fault-normal distance (NelY elements, LY
metres).  A workload string "W x H" with the fault-normal size first therefore maps to
NelY = W and NelX = H.
"""
from __future__ import annotations

import dataclasses
import math
from dataclasses import dataclass, field
from typing import List

YR2SEC = 365 * 24 * 60 * 60


@dataclass
class ModelConfig:
    profile: int = 1          # 0: reference depth profiles; 1: uniform a / tapered b / uniform sigma
    damage: int = 0           # 0 none; 1 rectangle per element (par.jl rule); 2 trapezoid per GLL node
    NelX: int = 48            # elements along depth
    NelY: int = 48            # elements along the fault normal
    LX: float = 24e3
    LY: float = 24e3
    rho1: float = 2670.0
    vs1: float = 3464.0
    rho2: float = 2670.0
    vs2: float = 3464.0
    ThickX: float = 0.0
    ThickY: float = 0.0
    trap_w0: float = 0.0
    trap_w1: float = 0.0
    trap_z1: float = 1.0
    fo: float = 0.6
    Vo: float = 1e-6
    Dc: float = 0.008
    a0: float = 0.015
    b0: float = 0.019
    b1: float = 0.011
    zb0: float = 12e3
    zb1: float = 15e3
    sigma: float = 50e6
    V_init: float = 35e-3 / YR2SEC
    noise_amp: float = 0.01
    seed: int = 0
    Vpl: float = 35e-3 / YR2SEC
    creep_depth: float = 24e3
    creep_inclusive: int = 1
    CFL: float = 0.6
    total_years: float = 300.0
    Vthres: float = 0.001
    rec_x: List[float] = field(default_factory=list)
    rec_y: List[float] = field(default_factory=list)

    @property
    def FltNglob(self) -> int:
        return 4 * self.NelX + 1

    @property
    def nglob(self) -> int:
        return (4 * self.NelX + 1) * (4 * self.NelY + 1)

    def replace(self, **kw) -> "ModelConfig":
        return dataclasses.replace(self, **kw)


def reference_config(FZdepth: float = 24e3, res: int = 20) -> ModelConfig:
    """The reference's own model, ``setParameters(FZdepth, res)`` (par.jl:15-231, run.jl:28)."""
    LX, LY = 48e3, 30e3
    NelX, NelY = 30 * res, 20 * res
    dxe, dye = LX / NelX, LY / NelY
    vs1 = 3464.0
    return ModelConfig(
        profile=0, damage=1, NelX=NelX, NelY=NelY, LX=LX, LY=LY,
        rho1=2670.0, vs1=vs1, rho2=2500.0, vs2=0.60 * vs1,
        ThickX=LX - math.ceil(FZdepth / dxe) * dxe,
        ThickY=math.ceil(68 * 1 / dye) * dye,
        fo=0.6, Vo=1e-6, Dc=0.008,
        V_init=2 * 0.5e-3, noise_amp=0.0, seed=0,
        Vpl=35e-3 / YR2SEC, creep_depth=24e3, creep_inclusive=0,
        CFL=0.6, total_years=1000.0, Vthres=0.001,
        rec_x=[-48.0e3, -48.0e3, -48.0e3, -46.0e3, -44.0e3, -40.0e3],
        rec_y=[0.0, 150.0, 300.0, 0.0, 0.0, 0.0],
    )


def _receivers(LX: float):
    # Same placement relative to the domain bottom as the reference's par.jl:118-119.
    return ([-LX, -LX, -LX, -LX + 2e3, -LX + 4e3, -LX + 8e3], [0.0, 150.0, 300.0, 0.0, 0.0, 0.0])


def preset(name: str, seed: int = 0) -> ModelConfig:
    """Workload presets.

    ``homog48``   48x48 elements, 24 km x 24 km, homogeneous, 300 yr (CPU-runnable case).
    ``dz480``     480 (fault-normal) x 240 (depth) elements, 48 km x 24 km, trapezoidal
                  damage zone 0.5 km wide at the surface narrowing to 0.2 km at 10 km depth
                  with vs reduced 40 %, 1000 yr (1.85M nodes, 961 fault nodes).
    ``dz960``     the same model refined to 960 x 480 elements (7.4M nodes, 1921 fault nodes).
    ``dz<N>``     the damage-zone model with N fault-normal elements (N/2 along depth).
    Common physics: rho 2670, vs 3464, f0 0.6, V0 1e-6, a 0.015, b 0.019 to 12 km tapering
    linearly to 0.011 at 15 km and below, Dc 8 mm, sigma 50 MPa, Vpl 35 mm/yr creep imposed
    at the bottom of the fault (depth >= 24 km), V = Vpl initially with
    theta = Dc/Vpl * (1 + 0.01 U(-1,1)) seeded, Vthres 1 mm/s.
    """
    base = ModelConfig(seed=seed)
    if name == "homog48":
        rx, ry = _receivers(24e3)
        return base.replace(NelX=48, NelY=48, LX=24e3, LY=24e3, total_years=300.0, rec_x=rx, rec_y=ry)
    if name.startswith("dz"):
        nnormal = int(name[2:])
        ndepth = nnormal // 2
        rx, ry = _receivers(24e3)
        years = {480: 1000.0, 960: 500.0}.get(nnormal, 1000.0)
        return base.replace(
            NelX=ndepth, NelY=nnormal, LX=24e3, LY=48e3, damage=2,
            rho2=2670.0, vs2=0.6 * 3464.0, trap_w0=500.0, trap_w1=200.0, trap_z1=10e3,
            total_years=years, rec_x=rx, rec_y=ry)
    raise ValueError(f"unknown preset {name!r}")


def ensemble_members(n: int = 64, seed: int = 0, nmin: int = 120, nmax: int = 480):
    """The batched-ensemble workload: ``n`` damage-zone fault models with uneven meshes and seeded
    parameters (one ``ModelConfig`` each).

    Mesh: fault-normal elements N drawn uniformly from multiples of 8 in [nmin, nmax], N/2 along
    depth (120 x 60 to 480 x 240 elements over the same 48 km x 24 km domain).  Per model, drawn
    from one seeded stream: damage-zone width uniform in [0, 2] km at the surface (narrowing to 40 %
    of it at 10 km depth, the shape of the dz presets), vs reduction uniform in [0, 60] %, Dc
    log-uniform in [4, 16] mm, a - b uniform in [-0.006, -0.002] in the seismogenic zone (a = 0.015,
    b below 15 km unchanged), and the theta noise seed.
    """
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        N = int(8 * rng.integers(nmin // 8, nmax // 8 + 1))
        w = float(rng.uniform(0.0, 2000.0))
        red = float(rng.uniform(0.0, 0.6))
        Dc = float(np.exp(rng.uniform(np.log(4e-3), np.log(16e-3))))
        amb = float(rng.uniform(-0.006, -0.002))
        cfg = preset(f"dz{N}", seed=1000 + k).replace(
            trap_w0=w, trap_w1=0.4 * w, vs2=(1.0 - red) * 3464.0, Dc=Dc, b0=0.015 - amb, total_years=500.0)
        out.append(cfg)
    return out


def shard_members(cfgs, rank: int, world: int):
    """Indices (ascending) of the ensemble members that rank ``rank`` of ``world`` runs.  The
    members are independent models, so they split across GPUs with no exchange: largest first,
    each to the rank with the fewest nodes so far (ties to the lower rank); every member lands on
    exactly one rank and the node counts of the ranks differ by at most one member's."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    nodes = [(4 * c.NelX + 1) * (4 * c.NelY + 1) for c in cfgs]
    load = [0] * world
    own = [[] for _ in range(world)]
    for k in sorted(range(len(cfgs)), key=lambda k: (-nodes[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        load[r] += nodes[k]
        own[r].append(k)
    return sorted(own[rank])
