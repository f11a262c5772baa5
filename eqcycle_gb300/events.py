"""Event statistics of a run and the serialized result format.

Restates the reference's post-processing of ``main(P)``'s results (post/earthquake_cycles.jl):
``Coslip`` (per-event coseismic slip, stress drop, start/end times, hypocentre) and
``moment_magnitude_new`` (rupture area, moment magnitude, average stress drop and slip over the
part of the fault that slipped more than 1 % of the event's maximum), plus the quantities the
event-statistics comparison of two runs uses: recurrence interval, coseismic slip and hypocentre
depth.  ``save_results`` / ``load_results`` keep the ``results`` record of src/main.jl:479-498 in
one ``.npz`` file (the reference writes it with JLD2, output.jl:5-24).
"""
from __future__ import annotations

from dataclasses import dataclass, fields
from typing import Dict

import numpy as np

from .solver import Results


@dataclass
class EventCatalogue:
    tStart: np.ndarray        # [nev] s
    tEnd: np.ndarray          # [nev] s (events that ended)
    hypo: np.ndarray          # [nev] hypocentre position FltX (m, negative down)
    slip: np.ndarray          # [Nf, nev] coseismic slip delfafter
    stress_drop: np.ndarray   # [Nf, nev] taubefore - tauafter (MPa)
    Mw: np.ndarray            # [nev] moment magnitude
    mean_slip: np.ndarray     # [nev] average slip over the rupture (m)
    mean_drop: np.ndarray     # [nev] average stress drop over the rupture (MPa)
    max_slip: np.ndarray      # [nev] maximum coseismic slip (m)

    @property
    def recurrence(self) -> np.ndarray:
        """Intervals between consecutive event starts (s)."""
        return np.diff(self.tStart)

    def summary(self) -> Dict[str, float]:
        yr = 365 * 24 * 3600.0
        rec = self.recurrence
        return {"events": int(len(self.tStart)),
                "recurrence_yr": float(np.mean(rec) / yr) if len(rec) else float("nan"),
                "max_slip_m": float(np.mean(self.max_slip)) if len(self.max_slip) else float("nan"),
                "mean_slip_m": float(np.mean(self.mean_slip)) if len(self.mean_slip) else float("nan"),
                "hypo_depth_m": float(np.mean(-self.hypo)) if len(self.hypo) else float("nan"),
                "Mw": float(np.mean(self.Mw)) if len(self.Mw) else float("nan")}


def moment_magnitude(mu: float, FltX: np.ndarray, delfafter: np.ndarray, stressdrops: np.ndarray):
    """post/earthquake_cycles.jl:moment_magnitude_new: per event, over the fault nodes whose slip
    is at least 1 % of the event's maximum, area = sum slip * dx, zdim = sum dx,
    M0 = mu * area * zdim, Mw = 2/3 log10(M0 * 1e7) - 10.7, average stress drop and slip per zdim.
    dx[j] = FltX[j] - FltX[j-1]; the deepest node (no interval below it) contributes nothing."""
    nev = delfafter.shape[1]
    dx = np.diff(FltX)
    Mw, drop, slip = np.zeros(nev), np.zeros(nev), np.zeros(nev)
    for i in range(nev):
        d = delfafter[:, i]
        thres = 0.01 * d.max()
        sel = np.nonzero(d[1:] >= thres)[0] + 1          # nodes j >= 1 with dx[j-1]
        area = float(np.sum(d[sel] * dx[sel - 1]))
        zdim = float(np.sum(dx[sel - 1]))
        m0 = mu * area * zdim
        Mw[i] = (2.0 / 3.0) * np.log10(m0 * 1e7) - 10.7 if m0 > 0 else float("nan")
        drop[i] = float(np.sum(stressdrops[sel, i] * dx[sel - 1]) / zdim) if zdim > 0 else 0.0
        slip[i] = float(np.sum(d[sel]) / zdim) if zdim > 0 else 0.0
    return Mw, drop, slip


def catalogue(res: Results, FltX: np.ndarray, mu: float) -> EventCatalogue:
    """Event catalogue of a run (the events main.jl:361-380 records, Coslip's quantities)."""
    Nf = len(FltX)
    nev_end = len(res.tEnd)
    slip = np.asarray(res.delfafter).reshape(Nf, -1, order="F")[:, :nev_end] if nev_end else np.zeros((Nf, 0))
    tb = np.asarray(res.taubefore).reshape(Nf, -1, order="F")[:, :nev_end] if nev_end else np.zeros((Nf, 0))
    ta = np.asarray(res.tauafter).reshape(Nf, -1, order="F")[:, :nev_end] if nev_end else np.zeros((Nf, 0))
    drops = tb - ta
    Mw, mdrop, mslip = moment_magnitude(mu, FltX, slip, drops) if nev_end else (np.zeros(0),) * 3
    return EventCatalogue(tStart=np.asarray(res.tStart), tEnd=np.asarray(res.tEnd), hypo=np.asarray(res.hypo),
                          slip=slip, stress_drop=drops, Mw=Mw, mean_slip=mslip, mean_drop=mdrop,
                          max_slip=slip.max(axis=0) if nev_end else np.zeros(0))


def compare(a: EventCatalogue, b: EventCatalogue) -> Dict[str, float]:
    """Relative differences of the event statistics of two runs (b against a): mean recurrence
    interval, mean maximum coseismic slip, mean hypocentre depth, over the events both recorded."""
    n = min(len(a.tEnd), len(b.tEnd))
    out = {"events_a": int(len(a.tStart)), "events_b": int(len(b.tStart)), "compared": n}
    if n == 0:
        return out

    def rel(x, y):
        return float(abs(y - x) / max(abs(x), 1e-300))
    ra, rb = np.diff(a.tStart[:n]), np.diff(b.tStart[:n])
    if len(ra):
        out["recurrence"] = rel(np.mean(ra), np.mean(rb))
    out["coseismic_slip"] = rel(np.mean(a.max_slip[:n]), np.mean(b.max_slip[:n]))
    out["hypocentre_depth"] = rel(np.mean(-a.hypo[:n]), np.mean(-b.hypo[:n]))
    return out


def save_results(path: str, res: Results) -> None:
    np.savez_compressed(path, **{f.name: np.asarray(getattr(res, f.name)) for f in fields(res)})


def load_results(path: str) -> Results:
    z = np.load(path)
    return Results(**{f.name: z[f.name] for f in fields(Results)})
