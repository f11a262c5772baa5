"""The reference-facing API: ``main(P)`` and the operator entry points.

``main(P, ...)`` mirrors src/main.jl:67-477: it takes the setup tuple (``set_parameters``)
and returns the ``results`` record of main.jl:479-498, computed by libeqc on the GPU.
``Solver`` exposes the per-operator calls a caller of the hot path uses (the stiffness
apply that replaces ``Ksparse*x``, the quasi-static solve that replaces ``cg!``,
``slrFunc!``, ``FBC!``, ``dtevol!``) on host arrays in the reference numbering.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, Optional

import numpy as np

from . import _lib as L
from .params import Params


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


@dataclass
class Results:
    """main.jl:479-498 (``index_eq`` is never filled by the reference and stays empty)."""
    seismic_stress: np.ndarray
    seismic_slipvel: np.ndarray
    seismic_slip: np.ndarray
    index_eq: np.ndarray
    is_stress: np.ndarray
    is_slipvel: np.ndarray
    is_slip: np.ndarray
    dSeis: np.ndarray
    vSeis: np.ndarray
    aSeis: np.ndarray
    tStart: np.ndarray
    tEnd: np.ndarray
    taubefore: np.ndarray
    tauafter: np.ndarray
    delfafter: np.ndarray
    hypo: np.ndarray
    time_: np.ndarray
    Vfmax: np.ndarray


_FAULT_MATS = ("seismic_stress", "seismic_slipvel", "seismic_slip", "is_stress", "is_slipvel", "is_slip",
               "taubefore", "tauafter", "delfafter")
_SEIS_MATS = ("dSeis", "vSeis", "aSeis")


class Solver:
    """One fault model resident on one GPU (an ``eqc_handle``)."""

    def __init__(self, P: Params, precision: int = L.EQC_FP64, precond: int = L.EQC_PC_AMG,
                 guess: int = L.EQC_GUESS_PREVIOUS, cg_tol: float = 1e-8, cg_maxit: int = 0,
                 tol_rule: int = L.EQC_TOL_RHS, device: int = 0, use_graphs: int = 1, verbose: int = 0,
                 reliable_delta: float = 0.0, mg_degree: int = 0, mg_coarse_max: int = 0,
                 apply_variant: int = 0, mg_degree_coarse: int = 0, step_batch: int = 0):
        self.P = P
        lib = L.lib()
        fa, ia, m = P.farray, P.iarray, P.mesh
        keep = {}

        def d(name, a):
            keep[name] = _c(a, np.float64)
            return L.dptr(keep[name])

        def i(name, a):
            keep[name] = _c(a, np.int64)
            return L.iptr(keep[name])

        mod = L.EqcModel()
        mod.Nel, mod.FltNglob, mod.yr2sec = P.int_.Nel, P.int_.FltNglob, int(P.int_.yr2sec)
        mod.IDstate, mod.nglob, mod.Total_time = P.int_.IDstate, P.int_.nglob, float(P.int_.Total_time)
        mod.ETA, mod.Vpl, mod.Vthres, mod.Vevne, mod.dt0 = (P.float_.ETA, P.float_.Vpl, P.float_.Vthres,
                                                          P.float_.Vevne, P.float_.dt0)
        mod.NelX, mod.NelY, mod.NGLL, mod.dxe, mod.dye = m.NelX, m.NelY, m.NGLL, m.dxe, m.dye
        structured = bool(P.extra.get("structured"))   # element data built on the device
        if not structured:
            mod.iglob = i("iglob", np.asarray(m.iglob).reshape(-1, order="F"))
            mod.W = d("W", np.asarray(m.W).reshape(-1, order="F"))
        mod.H = d("H", np.asarray(m.H).reshape(-1, order="F"))
        for name in ("fo", "Vo", "xLf", "M", "BcLC", "BcTC", "FltB", "FltZ", "FltX", "cca", "ccb", "Seff", "tauo",
                     "XiLf"):
            if getattr(fa, name) is not None:
                setattr(mod, name, d(name, getattr(fa, name)))
        for name in ("iFlt", "iBcL", "iBcT", "FltIglobBC", "FltNI", "out_seis"):
            if getattr(ia, name) is not None:
                setattr(mod, name, i(name, getattr(ia, name)))
        mod.n_iBcL, mod.n_iBcT = len(ia.iBcL), len(ia.iBcT)
        mod.n_FltIglobBC, mod.n_out_seis = len(ia.FltIglobBC), len(ia.out_seis)
        mod.n_FltNI = 0 if ia.FltNI is None else len(ia.FltNI)
        self.options = L.default_options(precision=precision, precond=precond, guess=guess, cg_tol=cg_tol,
                                         cg_maxit=cg_maxit, tol_rule=tol_rule, device=device,
                                         use_graphs=use_graphs, verbose=verbose, reliable_delta=reliable_delta,
                                         mg_degree=mg_degree, mg_coarse_max=mg_coarse_max,
                                         apply_variant=apply_variant,
                                         mg_degree_coarse=mg_degree_coarse, step_batch=step_batch)
        h = C.c_void_p()
        if structured:
            cfg = P.cfg
            mat = L.EqcMaterial(rule=int(cfg.damage), rho1=cfg.rho1, vs1=cfg.vs1, rho2=cfg.rho2, vs2=cfg.vs2,
                                ThickX=cfg.ThickX, ThickY=cfg.ThickY, trap_w0=cfg.trap_w0, trap_w1=cfg.trap_w1,
                                trap_z1=cfg.trap_z1, LX=float(cfg.LX), xgll=d("xgll", m.xgll), wgll=d("wgll", m.wgll))
            L.check(lib.eqc_create_structured(C.byref(mod), C.byref(mat), C.byref(self.options), C.byref(h)), None)
        else:
            L.check(lib.eqc_create(C.byref(mod), C.byref(self.options), C.byref(h)), None)
        self.h = h
        self.nglob = P.int_.nglob
        self.Nf = P.int_.FltNglob
        self.nseis = len(ia.out_seis)

    # -- lifetime
    def close(self):
        if getattr(self, "h", None):
            L.lib().eqc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _chk(self, st):
        L.check(st, self.h)

    # -- operators (host arrays, reference numbering)
    def apply_K(self, x: np.ndarray) -> np.ndarray:
        x = _c(x, np.float64)
        y = np.zeros(self.nglob)
        self._chk(L.lib().eqc_apply_K(self.h, L.dptr(x), L.dptr(y)))
        return y

    def qs_solve(self, F_fault, d, tol: float = 1e-8, maxit: int = 0):
        F_fault = _c(F_fault, np.float64)
        dd = np.array(d, dtype=np.float64, copy=True)
        it = C.c_int32(0)
        rr = C.c_double(0)
        self._chk(L.lib().eqc_qs_solve(self.h, L.dptr(F_fault), L.dptr(dd), tol, maxit, C.byref(it), C.byref(rr)))
        return dd, it.value, rr.value

    def slrFunc(self, psi, psi1, Vf, Vf1, tau1, dt):
        psi1 = np.array(psi1, dtype=np.float64, copy=True)
        Vf1 = np.array(Vf1, dtype=np.float64, copy=True)
        self._chk(L.lib().eqc_slrFunc(self.h, L.dptr(_c(psi, np.float64)), L.dptr(psi1), L.dptr(_c(Vf, np.float64)),
                                      L.dptr(Vf1), L.dptr(_c(tau1, np.float64)), dt))
        return psi1, Vf1

    def FBC(self, psi1, Vf1, tau1, psi2, Vf2, tau2, psi, Vf, FltVfree, dt):
        outs = [np.array(a, dtype=np.float64, copy=True) for a in (psi1, Vf1, tau1, psi2, Vf2, tau2)]
        fail = C.c_int64(0)
        st = L.lib().eqc_FBC(self.h, *[L.dptr(a) for a in outs], L.dptr(_c(psi, np.float64)),
                             L.dptr(_c(Vf, np.float64)), L.dptr(_c(FltVfree, np.float64)), dt, C.byref(fail))
        if st == 3:
            raise L.EqcError(st, f"NR SEARCH FAILED at fault node {fail.value}")
        self._chk(st)
        return tuple(outs)

    def dtevol(self, dt, dtmin, Vf, isolver):
        out = C.c_double(0)
        self._chk(L.lib().eqc_dtevol(self.h, dt, dtmin, L.dptr(_c(Vf, np.float64)), isolver, C.byref(out)))
        return out.value

    # -- time loop
    def init(self, V_init: float):
        self._chk(L.lib().eqc_init(self.h, V_init))

    def run(self, max_steps: int, t_end: Optional[float] = None) -> Dict[str, float]:
        t_end = self.P.int_.Total_time if t_end is None else t_end
        st = L.EqcRunStats()
        self._chk(L.lib().eqc_run(self.h, int(max_steps), float(t_end), C.byref(st)))
        return st.as_dict()

    def state(self, name: str, out: np.ndarray = None) -> np.ndarray:
        """A state field in the reference numbering, into out when given (a C-contiguous float64
        array of the field's length, e.g. in pinned host memory) or a new array."""
        n = self.nglob if name in ("d", "v", "a") else self.Nf
        if out is None:
            out = np.zeros(n)
        elif out.dtype != np.float64 or out.shape != (n,) or not out.flags.c_contiguous:
            raise ValueError(f"state {name}: out must be a contiguous float64 array of length {n}")
        self._chk(L.lib().eqc_get_state(self.h, name.encode(), L.dptr(out)))
        return out

    def set_state(self, name: str, value: np.ndarray):
        self._chk(L.lib().eqc_set_state(self.h, name.encode(), L.dptr(_c(value, np.float64))))

    def autotune(self, reps: int = 2):
        """Choose the multigrid smoothing degrees and, in mixed precision, the FP32 apply kernel
        and the reliable-update factor by timed trial solves (state unchanged)."""
        dg, dc, ms = C.c_int32(0), C.c_int32(0), C.c_double(0)
        self._chk(L.lib().eqc_autotune(self.h, reps, C.byref(dg), C.byref(dc), C.byref(ms)))
        return {"mg_degree": dg.value, "mg_degree_coarse": dc.value, "solve_ms": ms.value,
                "apply_variant": int(self.scalar("apply_variant")),
                "reliable_delta": self.scalar("reliable_delta")}

    # -- learned initial guess
    def guess_shape(self):
        nin, nout, npar = C.c_int32(0), C.c_int32(0), C.c_int64(0)
        self._chk(L.lib().eqc_guess_shape(self.h, C.byref(nin), C.byref(nout), C.byref(npar)))
        return nin.value, nout.value, npar.value

    def guess_init(self, seed: int):
        self._chk(L.lib().eqc_guess_init(self.h, int(seed)))

    def guess_params(self) -> np.ndarray:
        p = np.zeros(self.guess_shape()[2], dtype=np.float32)
        self._chk(L.lib().eqc_guess_get_params(self.h, L.fptr(p)))
        return p

    def set_guess_params(self, p: np.ndarray):
        p = _c(p, np.float32)
        self._chk(L.lib().eqc_guess_set_params(self.h, L.fptr(p)))

    def guess_log(self, capacity: int):
        self._chk(L.lib().eqc_guess_log(self.h, int(capacity)))

    def guess_pairs(self):
        nin, nout, _ = self.guess_shape()
        n = C.c_int64(0)
        self._chk(L.lib().eqc_guess_pairs(self.h, None, None, C.byref(n)))
        xin = np.zeros((n.value, nin), dtype=np.float32)
        tgt = np.zeros((n.value, nout), dtype=np.float32)
        self._chk(L.lib().eqc_guess_pairs(self.h, L.fptr(xin), L.fptr(tgt), C.byref(n)))
        return xin, tgt

    def guess_train(self, xin, tgt, epochs: int = 20, lr: float = 1e-3, batch: int = 256, seed: int = 0):
        xin, tgt = _c(xin, np.float32), _c(tgt, np.float32)
        loss = np.zeros(epochs)
        self._chk(L.lib().eqc_guess_train(self.h, L.fptr(xin), L.fptr(tgt), len(xin), epochs, lr, batch, int(seed),
                                          L.dptr(loss)))
        return loss

    def guess_eval(self, xin, tgt, outputs: bool = False):
        xin, tgt = _c(xin, np.float32), _c(tgt, np.float32)
        mse = C.c_double(0)
        out = np.zeros(tgt.shape, dtype=np.float32) if outputs else None
        self._chk(L.lib().eqc_guess_eval(self.h, L.fptr(xin), L.fptr(tgt), len(xin), C.byref(mse), L.fptr(out)))
        return (mse.value, out) if outputs else mse.value

    def guess_grad(self, xin, tgt):
        xin, tgt = _c(xin, np.float32), _c(tgt, np.float32)
        g = np.zeros(self.guess_shape()[2], dtype=np.float32)
        loss = C.c_double(0)
        self._chk(L.lib().eqc_guess_grad(self.h, L.fptr(xin), L.fptr(tgt), len(xin), L.fptr(g), C.byref(loss)))
        return g, loss.value

    def scalar(self, name: str) -> float:
        out = C.c_double(0)
        self._chk(L.lib().eqc_get_scalar(self.h, name.encode(), C.byref(out)))
        return out.value

    def set_scalar(self, name: str, value: float):
        self._chk(L.lib().eqc_set_scalar(self.h, name.encode(), float(value)))

    def result(self, field: str) -> np.ndarray:
        n = L.lib().eqc_result_size(self.h, field.encode())
        if n < 0:
            raise KeyError(field)
        out = np.zeros(n)
        if n:
            self._chk(L.lib().eqc_get_result(self.h, field.encode(), L.dptr(out)))
        if field in _FAULT_MATS:
            return out.reshape(self.Nf, -1, order="F") if n else np.zeros((self.Nf, 0))
        if field in _SEIS_MATS:
            return out.reshape(-1, self.nseis, order="F") if n else np.zeros((0, self.nseis))
        return out

    def results(self) -> Results:
        kw = {f: self.result(f) for f in Results.__dataclass_fields__ if f != "index_eq"}
        return Results(index_eq=np.zeros(0), **kw)

    # -- damage evolution (damageEvol.jl)
    def set_damage(self, damage_idx=None, factor: float = 0.95):
        """Scale W of these elements (1-based; default: the model's damage zone) by ``factor`` at
        the end of every event."""
        idx = self.P.extra.get("damage_idx", np.zeros(0, np.int64)) if damage_idx is None else damage_idx
        a = np.ascontiguousarray(idx, dtype=np.int64)
        self._chk(L.lib().eqc_set_damage(self.h, a.ctypes.data_as(C.POINTER(C.c_int64)), len(a), float(factor)))

    def damage_evolve(self):
        self._chk(L.lib().eqc_damage_evolve(self.h))

    def time_apply(self, dtype: int = 0, nrep: int = 20, flush_l2: bool = True) -> float:
        ms = C.c_double(0)
        self._chk(L.lib().eqc_time_apply(self.h, dtype, nrep, int(flush_l2), C.byref(ms)))
        return ms.value

    def time_apply_stream(self, dtype: int = 1, nrep: int = 60, ncopies: int = 6) -> float:
        """Mean duration (ms) of back-to-back applies rotating over ncopies working-set replicas."""
        ms = C.c_double(0)
        self._chk(L.lib().eqc_time_apply_stream(self.h, dtype, nrep, ncopies, C.byref(ms)))
        return ms.value

    def launches(self) -> int:
        return int(L.lib().eqc_launch_count(self.h))

    def layout(self):
        nx, ny, ld = C.c_int64(), C.c_int64(), C.c_int64()
        self._chk(L.lib().eqc_layout(self.h, C.byref(nx), C.byref(ny), C.byref(ld)))
        return nx.value, ny.value, ld.value


def main(P: Params, V_init: Optional[float] = None, max_steps: int = 1 << 62, **solver_kw) -> Results:
    """src/main.jl:67-477 on the GPU: run the whole simulation and return ``results``."""
    V_init = P.cfg.V_init if V_init is None else V_init
    with Solver(P, **solver_kw) as s:
        s.init(V_init)
        s.run(max_steps)
        return s.results()


class Ensemble:
    """Independent fault models (``Solver`` objects on one GPU) advanced by one CUDA-graph launch
    per time step, each member in its own regime (``eqc_ensemble_*``)."""

    def __init__(self, members):
        self.members = list(members)
        arr = (C.c_void_p * len(self.members))(*[m.h.value for m in self.members])
        h = C.c_void_p()
        st = L.lib().eqc_ensemble_create(arr, len(self.members), C.byref(h))
        L.check(st, None)
        self.h = h

    def run(self, steps: int):
        """Advance every member by ``steps`` steps; returns ([stats dict per member], gpu_ms)."""
        n = len(self.members)
        stats = (L.EqcRunStats * n)()
        ms = C.c_double(0)
        st = L.lib().eqc_ensemble_run(self.h, int(steps), stats, C.byref(ms))
        if st != L.EQC_OK:
            msg = L.lib().eqc_ensemble_last_error(self.h)
            raise L.EqcError(st, msg.decode() if msg else "")
        return [stats[i].as_dict() for i in range(n)], ms.value

    def close(self):
        if getattr(self, "h", None):
            L.lib().eqc_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
