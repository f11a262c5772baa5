"""Host-side model setup: the Python counterpart of ``setParameters`` (par.jl:15-231).

Builds, with vectorised numpy, the same arrays the reference's setup builds -- the tuple
``(params_int, params_float, params_farray, params_iarray)`` of par.jl:227-230 in the
reference's node numbering (src/MeshBox.jl:27-88, indices 1-based as in Julia) -- plus the
element data (iglob, W, H) that the matrix-free stiffness apply consumes in place of the
assembled ``Ksparse``.  Setup runs once per model and is not on the hot path.

Cited reference pieces: GetGLL.jl:17-28 (GLL tables), MeshBox.jl:27-88 (numbering and
coordinates), Assemble.jl:7-71 (mass, dt, muMax), MaterialProperties.jl:3-21 / 77-101 (W),
BoundaryMatrix.jl:7-61, FindNearestNode.jl:3-19, defaultInitialConditions.jl:9-84
(depth profiles), par.jl:304-339 (XiLf).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, Optional

import numpy as np

from .config import ModelConfig, YR2SEC


# --------------------------------------------------------------------------- GLL
def _legendre(N: int, x: float):
    P = [1.0, x]
    for k in range(2, N + 1):
        P.append(((2.0 * k - 1.0) * x * P[k - 1] - (k - 1.0) * P[k - 2]) / k)
    return P


def gll(ngll: int = 5):
    """GLL nodes x, weights w and H[i, j] = h'_i(x_j) (the table GetGLL.jl reads)."""
    N = ngll - 1
    x = [-math.cos(math.pi * i / N) for i in range(ngll)]
    for i in range(1, N):
        for _ in range(100):
            P = _legendre(N, x[i])
            dx = (x[i] * P[N] - P[N - 1]) / ((N + 1) * P[N])
            x[i] -= dx
            if abs(dx) < 1e-17:
                break
    for i in range(ngll // 2):
        x[N - i] = -x[i]
    if N % 2 == 0:
        x[N // 2] = 0.0
    PN = [_legendre(N, xi)[N] for xi in x]
    w = [2.0 / (N * (N + 1.0) * p * p) for p in PN]
    H = np.zeros((ngll, ngll))
    for j in range(ngll):
        for i in range(ngll):
            if i != j:
                H[i, j] = PN[j] / (PN[i] * (x[j] - x[i]))
            elif i == 0:
                H[i, j] = -N * (N + 1.0) / 4.0
            elif i == N:
                H[i, j] = N * (N + 1.0) / 4.0
    return np.array(x), np.array(w), H


# --------------------------------------------------------------------------- seeded noise
_M64 = (1 << 64) - 1


def splitmix_uniform_pm1(seed: int, n: int) -> np.ndarray:
    """n draws of U(-1, 1) from the splitmix64 stream seeded with ``seed``."""
    s = seed & _M64
    out = np.empty(n)
    for k in range(n):
        s = (s + 0x9E3779B97F4A7C15) & _M64
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        z = z ^ (z >> 31)
        out[k] = float(z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0
    return out


# --------------------------------------------------------------------------- containers
@dataclass
class ParamsInt:          # par.jl:236-249
    Nel: int
    FltNglob: int
    yr2sec: int
    Total_time: float
    IDstate: int
    nglob: int


@dataclass
class ParamsFloat:        # par.jl:251-266
    ETA: float
    Vpl: float
    Vthres: float
    Vevne: float
    dt0: float


@dataclass
class ParamsFarray:       # par.jl:268-292
    fo: np.ndarray
    Vo: np.ndarray
    xLf: np.ndarray
    M: np.ndarray
    BcLC: np.ndarray
    BcTC: np.ndarray
    FltB: np.ndarray
    FltZ: np.ndarray
    FltX: np.ndarray
    cca: np.ndarray
    ccb: np.ndarray
    Seff: np.ndarray
    tauo: np.ndarray
    XiLf: np.ndarray
    xout: np.ndarray
    yout: np.ndarray


@dataclass
class ParamsIarray:       # par.jl:294-301 (1-based node indices)
    iFlt: np.ndarray
    iBcL: np.ndarray
    iBcT: np.ndarray
    FltIglobBC: np.ndarray
    FltNI: np.ndarray
    out_seis: np.ndarray


@dataclass
class Mesh:
    NelX: int
    NelY: int
    NGLL: int
    dxe: float
    dye: float
    iglob: np.ndarray     # [5, 5, Nel] Fortran-ordered, 1-based
    W: np.ndarray         # [5, 5, Nel] Fortran-ordered
    H: np.ndarray         # [5, 5]
    xgll: np.ndarray
    wgll: np.ndarray
    x: np.ndarray
    y: np.ndarray
    muMax: float


@dataclass
class Params:
    """The tuple of par.jl:227-230 plus the element data of the matrix-free apply."""
    int_: ParamsInt
    float_: ParamsFloat
    farray: ParamsFarray
    iarray: ParamsIarray
    mesh: Mesh
    cfg: ModelConfig
    extra: Dict[str, object] = field(default_factory=dict)

    def __getitem__(self, k):  # P[1]..P[4] as in main.jl
        return (None, self.int_, self.float_, self.farray, self.iarray)[k]


# --------------------------------------------------------------------------- setup
def _int1d(p1v, p1z, p2v, p2z, val):
    # Int1D, defaultInitialConditions.jl:2-5
    return p1v + ((p2v - p1v) / (p2z - p1z)) * (val - p1z)


def _mesh_numbering(NelX: int, NelY: int):
    """Reference node id (0-based) of every lexicographic node (ix, iy), MeshBox.jl:27-88.

    Node (ix, iy) is created by the first element (in element order) that contains it; its id
    is that element's first new id plus its rank among the element's new nodes."""
    nx, ny = 4 * NelX + 1, 4 * NelY + 1
    Nf = nx
    ix = np.arange(nx)
    iy = np.arange(ny)
    exc = np.where(ix == 0, 0, (ix - 1) // 4)
    i = ix - 4 * exc
    eyc = np.where(iy == 0, 0, (iy - 1) // 4)
    j = iy - 4 * eyc
    EXC, EYC = np.meshgrid(exc, eyc, indexing="xy")   # [ny, nx]
    I, J = np.meshgrid(i, j, indexing="xy")
    rowstart = np.where(EYC == 0, 0, 5 * Nf + (EYC - 1) * 4 * Nf)
    ids = np.empty((ny, nx), dtype=np.int64)
    m00 = (EYC == 0) & (EXC == 0)
    m10 = (EYC == 0) & (EXC >= 1)
    m01 = (EYC >= 1) & (EXC == 0)
    m11 = (EYC >= 1) & (EXC >= 1)
    ids[m00] = (I + 5 * J)[m00]
    ids[m10] = (25 + 20 * (EXC - 1) + (I - 1) + 4 * J)[m10]
    ids[m01] = (rowstart + I + 5 * (J - 1))[m01]
    ids[m11] = (rowstart + 20 + 16 * (EXC - 1) + (I - 1) + 4 * (J - 1))[m11]
    return ids  # [iy, ix]


def _fault_profiles(cfg: ModelConfig, FltX: np.ndarray, muMax: float, LX: float):
    """Friction parameters and initial stress along the fault (defaultInitialConditions.jl, or the
    workloads' uniform a / tapered b / seeded theta) and XiLf (par.jl:304-339)."""
    Nf = len(FltX)
    fo = np.full(Nf, cfg.fo)
    Vo = np.full(Nf, cfg.Vo)
    xLf = np.full(Nf, cfg.Dc)
    if cfg.profile == 0:
        X = FltX
        z = np.abs(X)
        ab = np.full(Nf, 0.015 - 0.019)
        ab = np.where(z <= 2e3, _int1d(0.012, 0e3, -0.0041, -2e3, X), ab)
        ab = np.where((z > 2e3) & (z <= 12e3), _int1d(-0.0041, -2e3, -0.0041, -12e3, X), ab)
        ab = np.where((z > 12e3) & (z <= 17e3), _int1d(-0.0041, -12e3, 0.015, -17e3, X), ab)
        ab = np.where((z > 17e3) & (z <= 24e3), _int1d(0.015, -17e3, 0.024, -24e3, X), ab)
        ab = np.where(z > 24e3, 0.0047, ab)
        ccb = np.full(Nf, 0.019)
        cca = ccb + ab
        Seff = np.where(z <= 2e3, _int1d(10e6, 0, 50e6, -2e3, X), 50e6)
        t0 = np.full(Nf, 22.5e6)
        t0 = np.where(z <= 2e3, _int1d(0.01e6, 0, 30e6, -2e3, X), t0)
        t0 = np.where((z > 2e3) & (z <= 12e3), _int1d(30e6, -2e3, 30e6, -12e3, X), t0)
        t0 = np.where((z > 12e3) & (z <= 17e3), _int1d(30e6, -12e3, 22.5e6, -17e3, X), t0)
        t0 = np.where((z > 17e3) & (z <= 24e3), _int1d(22.5e6, -17e3, 22.5e6, -24e3, X), t0)
        tauo = t0
    else:
        z = np.abs(FltX)
        b = np.where(z <= cfg.zb0, cfg.b0,
                     np.where(z >= cfg.zb1, cfg.b1, cfg.b0 + (cfg.b1 - cfg.b0) * ((z - cfg.zb0) / (cfg.zb1 - cfg.zb0))))
        cca = np.full(Nf, cfg.a0)
        ccb = b.astype(np.float64)
        Seff = np.full(Nf, cfg.sigma)
        u = splitmix_uniform_pm1(cfg.seed, Nf)
        theta = (cfg.Dc / cfg.Vpl) * (1.0 + cfg.noise_amp * u)
        psi0 = np.log(cfg.Vo * theta / cfg.Dc)
        tauo = Seff * (cfg.fo + ccb * psi0 + cca * np.log(cfg.V_init / cfg.Vo))

    # ---- XiLf (par.jl:304-339) ----
    hcell = LX / (Nf - 1)
    gamma_ = math.pi / 4.0
    expr1 = -(cca - ccb) / cca
    expr2 = gamma_ * muMax / hcell * xLf / (cca * Seff)
    ro = expr2 - expr1
    Xith = np.where(0.25 * ro * ro - expr2 >= 0, 1.0 / ro, 1.0 - expr1 / expr2)
    XiLf = np.where(1.0 * Xith > 0.5, 0.5 * xLf, 1.0 * Xith * xLf)

    return fo, Vo, xLf, cca, ccb, Seff, tauo, XiLf


def set_parameters(cfg: ModelConfig) -> Params:
    """Build the model of ``cfg`` exactly as par.jl:setParameters does."""
    NGLL = 5
    NelX, NelY = int(cfg.NelX), int(cfg.NelY)
    LX, LY = float(cfg.LX), float(cfg.LY)
    dxe, dye = LX / NelX, LY / NelY
    Nel = NelX * NelY
    FltNglob = NelX * (NGLL - 1) + 1
    dx_dxi, dy_deta = 0.5 * dxe, 0.5 * dye
    jac = dx_dxi * dy_deta
    yr2sec = YR2SEC
    Total_time = cfg.total_years * yr2sec
    xgll, wgll, H = gll(NGLL)
    nx, ny = 4 * NelX + 1, 4 * NelY + 1
    nglob = nx * ny

    # ---- numbering and coordinates (MeshBox.jl) ----
    ids = _mesh_numbering(NelX, NelY)                 # [ny, nx] -> ref id
    li = np.arange(5)
    I4 = 4 * np.arange(NelX)[None, :] + li[:, None]               # [i, ex] -> ix
    J4 = 4 * np.arange(NelY)[None, :] + li[:, None]               # [j, ey] -> iy
    ig = ids[J4[None, :, :, None], I4[:, None, None, :]]          # [i, j, ey, ex]
    iglob0 = np.ascontiguousarray(ig.reshape(5, 5, Nel))          # e = ey*NelX + ex
    # coordinates: last writing element (max ey, then max ex) defines the value
    ixs = np.arange(nx)
    exw = np.minimum(ixs // 4, NelX - 1)
    iw = ixs - 4 * exw
    iys = np.arange(ny)
    eyw = np.minimum(iys // 4, NelY - 1)
    jw = iys - 4 * eyw
    xcol = dxe * exw.astype(np.float64) + dxe * (0.5 * (1.0 + xgll[iw]))
    ycol = dye * eyw.astype(np.float64) + dye * (0.5 * (1.0 + xgll[jw]))
    x = np.empty(nglob)
    y = np.empty(nglob)
    x[ids] = np.broadcast_to(xcol[None, :], (ny, nx))
    y[ids] = np.broadcast_to(ycol[:, None], (ny, nx))
    x = x - LX

    # ---- material: rho, mu at every (i, j, e) ----
    wg2 = wgll[:, None] * wgll[None, :]
    if cfg.damage == 2:
        z = -x
        inside = z <= cfg.trap_z1
        wdt = cfg.trap_w0 + (cfg.trap_w1 - cfg.trap_w0) * (z / cfg.trap_z1)
        dmg = inside & (y <= wdt)
        rho_n = np.where(dmg, cfg.rho2, cfg.rho1)
        vs_n = np.where(dmg, cfg.vs2, cfg.vs1)
        mu_n = rho_n * (vs_n * vs_n)
        rho_e = rho_n[iglob0]
        mu_e = mu_n[iglob0]
    else:
        exx = (np.arange(Nel) % NelX) + 1
        eyy = (np.arange(Nel) // NelX) + 1
        if cfg.damage == 1:
            dm = (exx * dxe >= cfg.ThickX) & ((dye <= eyy * dye) & (eyy * dye <= cfg.ThickY))
        else:
            dm = np.zeros(Nel, dtype=bool)
        r_el = np.where(dm, cfg.rho2, cfg.rho1)
        m_el = np.where(dm, cfg.rho2 * (cfg.vs2 * cfg.vs2), cfg.rho1 * (cfg.vs1 * cfg.vs1))
        rho_e = np.broadcast_to(r_el[None, None, :], (5, 5, Nel))
        mu_e = np.broadcast_to(m_el[None, None, :], (5, 5, Nel))
    muMax = float(mu_e.max())
    # elements of the damage zone (Assemble.jl:25-35 returns them as damage_idx): the rectangle
    # rule, or, for the per-node trapezoid, every element holding a damaged node
    mu1 = cfg.rho1 * (cfg.vs1 * cfg.vs1)
    damage_idx = (np.nonzero(np.any(mu_e.reshape(25, Nel) != mu1, axis=0))[0] + 1 if cfg.damage
                  else np.zeros(0, dtype=np.int64)).astype(np.int64)
    W = wg2[:, :, None] * mu_e
    W = np.asfortranarray(W)
    # lumped mass, accumulated element by element (Assemble.jl:165)
    M = np.zeros(nglob)
    np.add.at(M, iglob0.reshape(-1, order="F"), ((wg2[:, :, None] * rho_e) * jac).reshape(-1, order="F"))
    # CFL dt (Assemble.jl:171-182)
    vso = np.sqrt(mu_e / rho_e)
    dxg = np.diff(xgll)
    if dxe < dye:
        vs = np.maximum(vso[:-1, :, :], vso[1:, :, :])            # [4, 5, Nel]
        dx = (dxg * 0.5 * dxe)[:, None, None]
    else:
        vs = np.transpose(np.maximum(vso[:, :-1, :], vso[:, 1:, :]), (1, 0, 2))
        dx = (dxg * 0.5 * dye)[:, None, None]
    dt = float(np.min(dx / vs))
    dt = cfg.CFL * dt
    half_dt = 0.5 * dt

    # ---- boundary matrices (BoundaryMatrix.jl) ----
    def boundary(side):
        if side == "L":
            eB = np.arange(NelY) * NelX
            nodes = lambda e, k: iglob0[0, k, e]
            jac1D, imp = dy_deta, cfg.rho1 * cfg.vs1
        elif side == "T":
            eB = (NelY - 1) * NelX + np.arange(NelX)
            nodes = lambda e, k: iglob0[k, 4, e]
            jac1D, imp = dx_dxi, cfg.rho1 * cfg.vs1
        else:
            eB = np.arange(NelX)
            nodes = lambda e, k: iglob0[k, 0, e]
            jac1D, imp = dx_dxi, 1.0
        ng = len(eB) * 4 + 1
        iB = np.zeros(ng, dtype=np.int64)
        B = np.zeros(ng)
        for k in range(5):
            ip = 4 * np.arange(len(eB)) + k
            iB[ip] = nodes(eB, k)
        contrib = (jac1D * wgll) * imp
        for k in range(5):   # element order: first element's k-th node, ...
            ip = 4 * np.arange(len(eB)) + k
            np.add.at(B, ip, contrib[k])
        return B, iB

    # B accumulates element by element in the reference; node contributions from two
    # elements meet only at element ends, where both orders give the same two-term sum.
    BcLC, iBcL = boundary("L")
    BcTC, iBcT = boundary("T")
    M[iBcL] = M[iBcL] + half_dt * BcLC
    M[iBcT] = M[iBcT] + half_dt * BcTC
    FltB, iFlt = boundary("B")
    FltZ = ((M[iFlt] / FltB) / half_dt) * 0.5
    FltX = x[iFlt]

    # ---- friction and profiles, XiLf ----
    fo, Vo, xLf, cca, ccb, Seff, tauo, XiLf = _fault_profiles(cfg, FltX, muMax, LX)

    # ---- FltNI, FltIglobBC, receivers ----
    mask = np.ones(nglob, dtype=bool)
    mask[iFlt] = False
    FltNI = np.nonzero(mask)[0]
    creeps = (np.abs(FltX) >= cfg.creep_depth) if cfg.creep_inclusive else (np.abs(FltX) > cfg.creep_depth)
    FltIglobBC = np.zeros(0, dtype=np.int64)
    if creeps.any():
        last = iFlt[np.nonzero(creeps)[0][-1]]
        fbc = iglob0[:, 0, :].reshape(-1, order="F")           # iglob[:,1,:][:]
        idx = int(np.nonzero(fbc == last)[0][0])
        FltIglobBC = fbc[: idx + 1].astype(np.int64)
    out = []
    for xr, yr in zip(cfg.rec_x, cfg.rec_y):
        dd = (x - xr) ** 2 + (y - yr) ** 2
        out.append(int(np.argmin(dd)))
    out_seis = np.array(out, dtype=np.int64)

    iglob = np.asfortranarray(iglob0 + 1)
    return Params(
        int_=ParamsInt(Nel, FltNglob, yr2sec, Total_time, 2, nglob),
        float_=ParamsFloat(0.0, cfg.Vpl, cfg.Vthres, cfg.Vthres, dt),
        farray=ParamsFarray(fo, Vo, xLf, M, BcLC, BcTC, FltB, FltZ, FltX, cca, ccb, Seff, tauo, XiLf,
                            x[out_seis], y[out_seis]),
        iarray=ParamsIarray(iFlt + 1, iBcL + 1, iBcT + 1, FltIglobBC + 1, FltNI + 1, out_seis + 1),
        mesh=Mesh(NelX, NelY, NGLL, dxe, dye, iglob, W, H, xgll, wgll, x, y, muMax),
        cfg=cfg,
        extra={"damage_idx": damage_idx},
    )


# --------------------------------------------------------------------------- structured setup
def meshbox_ids(ix, iy, nx: int):
    """Reference node id (0-based) of lexicographic nodes (ix, iy) by MeshBox.jl's numbering
    (the rule of ``_mesh_numbering``, for given nodes only)."""
    ix = np.asarray(ix, dtype=np.int64)
    iy = np.asarray(iy, dtype=np.int64)
    exc = np.where(ix == 0, 0, (ix - 1) // 4)
    i = ix - 4 * exc
    eyc = np.where(iy == 0, 0, (iy - 1) // 4)
    j = iy - 4 * eyc
    rowstart = np.where(eyc == 0, 0, 5 * nx + (eyc - 1) * 4 * nx)
    return np.where((eyc == 0) & (exc == 0), i + 5 * j,
           np.where(eyc == 0, 25 + 20 * (exc - 1) + (i - 1) + 4 * j,
           np.where(exc == 0, rowstart + i + 5 * (j - 1),
                    rowstart + 20 + 16 * (exc - 1) + (i - 1) + 4 * (j - 1))))


def structured_parameters(cfg: ModelConfig) -> Params:
    """The parameters of ``cfg`` without the per-node and per-element arrays (iglob, W, M,
    FltNI, coordinates), for ``eqc_create_structured``, which builds those on the device.  Every
    array it returns is bitwise the one ``set_parameters`` returns; it touches O(NelX + NelY)
    nodes instead of O(nglob)."""
    NGLL = 5
    NelX, NelY = int(cfg.NelX), int(cfg.NelY)
    LX, LY = float(cfg.LX), float(cfg.LY)
    dxe, dye = LX / NelX, LY / NelY
    Nel = NelX * NelY
    FltNglob = NelX * (NGLL - 1) + 1
    dx_dxi, dy_deta = 0.5 * dxe, 0.5 * dye
    jac = dx_dxi * dy_deta
    Total_time = cfg.total_years * YR2SEC
    xgll, wgll, H = gll(NGLL)
    nx, ny = 4 * NelX + 1, 4 * NelY + 1
    nglob = nx * ny
    # axis coordinates (the last element writing a node defines it, MeshBox.jl)
    ixs, iys = np.arange(nx), np.arange(ny)
    exw = np.minimum(ixs // 4, NelX - 1)
    eyw = np.minimum(iys // 4, NelY - 1)
    X = (dxe * exw.astype(np.float64) + dxe * (0.5 * (1.0 + xgll[ixs - 4 * exw]))) - LX
    Y = dye * eyw.astype(np.float64) + dye * (0.5 * (1.0 + xgll[iys - 4 * eyw]))
    mu1, mu2 = cfg.rho1 * (cfg.vs1 * cfg.vs1), cfg.rho2 * (cfg.vs2 * cfg.vs2)

    def element_rho(ex, ey):
        """rho of elements under the rectangle rule (Assemble.jl:34-35) or the homogeneous one."""
        if cfg.damage == 1:
            dm = ((ex + 1) * dxe >= cfg.ThickX) & ((dye <= (ey + 1) * dye) & ((ey + 1) * dye <= cfg.ThickY))
        else:
            dm = np.zeros(np.shape(ex), dtype=bool)
        return np.where(dm, cfg.rho2, cfg.rho1)

    def trap(ix, iy):
        z = -X[ix]
        wdt = cfg.trap_w0 + (cfg.trap_w1 - cfg.trap_w0) * (z / cfg.trap_z1)
        return (z <= cfg.trap_z1) & (Y[iy] <= wdt)

    # damage zone elements, muMax, CFL time step
    if cfg.damage == 1:
        ex_ok = (np.arange(1, NelX + 1) * dxe >= cfg.ThickX)
        ey_ok = (dye <= np.arange(1, NelY + 1) * dye) & (np.arange(1, NelY + 1) * dye <= cfg.ThickY)
        dmg_el = (ey_ok[:, None] & ex_ok[None, :]).reshape(-1)
        damage_idx = np.nonzero(dmg_el)[0] + 1
        present = [(cfg.rho1, mu1)] + ([(cfg.rho2, mu2)] if dmg_el.any() else [])
        if dmg_el.all():
            present = [(cfg.rho2, mu2)]
    elif cfg.damage == 2:
        # damaged nodes lie within the widest width of the trapezoid from the fault
        wmax = max(cfg.trap_w0, cfg.trap_w1, 0.0)
        iy_max = int(np.nonzero(Y <= wmax)[0][-1]) if np.any(Y <= wmax) else 0
        ey_max = min(iy_max // 4, NelY - 1)
        hit = np.zeros((ey_max + 1, NelX), dtype=bool)
        for j in range(5):
            for i in range(5):
                ixe = 4 * np.arange(NelX) + i
                iye = 4 * np.arange(ey_max + 1) + j
                hit |= trap(ixe[None, :], iye[:, None])
        damage_idx = np.nonzero(hit.reshape(-1))[0] + 1      # e = ey*NelX + ex for ey <= ey_max
        present = [(cfg.rho1, mu1)] + ([(cfg.rho2, mu2)] if hit.any() else [])
    else:
        damage_idx = np.zeros(0, dtype=np.int64)
        present = [(cfg.rho1, mu1)]
    damage_idx = damage_idx.astype(np.int64)
    muMax = float(max(m for _, m in present))
    vmax = max(float(np.sqrt(m / r)) for r, m in present)
    dxg = np.diff(xgll)
    h = dxe if dxe < dye else dye
    dt = float(np.min((dxg * 0.5 * h) / vmax))
    dt = cfg.CFL * dt
    half_dt = 0.5 * dt

    # boundary matrices (BoundaryMatrix.jl) with MeshBox ids of their nodes
    def boundary(side):
        if side == "L":
            ne, jac1D, imp = NelY, dy_deta, cfg.rho1 * cfg.vs1
            ixn, iyn = np.zeros(4 * ne + 1, np.int64), np.arange(4 * ne + 1)
        elif side == "T":
            ne, jac1D, imp = NelX, dx_dxi, cfg.rho1 * cfg.vs1
            ixn, iyn = np.arange(4 * ne + 1), np.full(4 * ne + 1, ny - 1)
        else:
            ne, jac1D, imp = NelX, dx_dxi, 1.0
            ixn, iyn = np.arange(4 * ne + 1), np.zeros(4 * ne + 1, np.int64)
        B = np.zeros(4 * ne + 1)
        contrib = (jac1D * wgll) * imp
        for k in range(5):
            np.add.at(B, 4 * np.arange(ne) + k, contrib[k])
        return B, meshbox_ids(ixn, iyn, nx), ixn, iyn

    BcLC, iBcL, _, _ = boundary("L")
    BcTC, iBcT, _, _ = boundary("T")
    FltB, iFlt, fix, _ = boundary("B")
    # M at the fault nodes: element row 0's contributions in element order, then the boundary terms
    Mf = np.zeros(FltNglob)
    for ex in range(NelX):
        i = np.arange(5)
        ix = 4 * ex + i
        if cfg.damage == 2:
            rho = np.where(trap(ix, np.zeros(5, np.int64)), cfg.rho2, cfg.rho1)
        else:
            rho = element_rho(np.full(5, ex), np.zeros(5, np.int64))
        np.add.at(Mf, ix, ((wgll * wgll[0]) * rho) * jac)
    Mf[0] = Mf[0] + half_dt * BcLC[0]               # node (0, 0) is the left boundary's first
    FltZ = ((Mf / FltB) / half_dt) * 0.5
    FltX = X[fix]
    fo, Vo, xLf, cca, ccb, Seff, tauo, XiLf = _fault_profiles(cfg, FltX, muMax, LX)

    # creeping nodes (main.jl:185) and receivers (nearest node, smallest reference id on ties)
    creeps = (np.abs(FltX) >= cfg.creep_depth) if cfg.creep_inclusive else (np.abs(FltX) > cfg.creep_depth)
    FltIglobBC = np.zeros(0, dtype=np.int64)
    if creeps.any():
        last = iFlt[np.nonzero(creeps)[0][-1]]
        fbc = meshbox_ids((4 * np.arange(NelX)[:, None] + np.arange(5)[None, :]).reshape(-1),
                          np.zeros(5 * NelX, np.int64), nx)
        idx = int(np.nonzero(fbc == last)[0][0])
        FltIglobBC = fbc[: idx + 1].astype(np.int64)
    out, rx, ry = [], [], []
    for xr, yr in zip(cfg.rec_x, cfg.rec_y):
        dx2, dy2 = (X - xr) ** 2, (Y - yr) ** 2
        dmin = np.min(dx2 + np.min(dy2))       # the sum is monotonic in each term
        best = None
        for ix in np.nonzero(dx2 + np.min(dy2) == dmin)[0]:
            for iy in np.nonzero(dx2[ix] + dy2 == dmin)[0]:
                g = int(meshbox_ids(ix, iy, nx))
                if best is None or g < best[0]:
                    best = (g, ix, iy)
        out.append(best[0])
        rx.append(X[best[1]])
        ry.append(Y[best[2]])
    out_seis = np.array(out, dtype=np.int64)

    return Params(
        int_=ParamsInt(Nel, FltNglob, YR2SEC, Total_time, 2, nglob),
        float_=ParamsFloat(0.0, cfg.Vpl, cfg.Vthres, cfg.Vthres, dt),
        farray=ParamsFarray(fo, Vo, xLf, None, BcLC, BcTC, FltB, FltZ, FltX, cca, ccb, Seff, tauo, XiLf,
                            np.array(rx), np.array(ry)),
        iarray=ParamsIarray(iFlt + 1, iBcL + 1, iBcT + 1, FltIglobBC + 1, None, out_seis + 1),
        mesh=Mesh(NelX, NelY, NGLL, dxe, dye, None, None, H, xgll, wgll, None, None, muMax),
        cfg=cfg,
        extra={"damage_idx": damage_idx, "structured": True, "Mf": Mf},
    )
