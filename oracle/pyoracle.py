"""ctypes wrapper of the CPU oracle (oracle/build/liboracle.so) -- TEST INFRASTRUCTURE ONLY.

Used by tests/, ``__graft_entry__.smoke()`` and the CPU legs of bench.py as the checker of
the GPU product.  The oracle restates the Julia reference (see orc_api.h for what is pinned
and what is not).  Node-index arrays come back 1-based like the reference's Julia arrays.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "build", "liboracle.so")
_lib: Optional[C.CDLL] = None


class OrcConfig(C.Structure):
    _fields_ = [
        ("profile", C.c_int32), ("damage", C.c_int32), ("NelX", C.c_int32), ("NelY", C.c_int32),
        ("LX", C.c_double), ("LY", C.c_double),
        ("rho1", C.c_double), ("vs1", C.c_double), ("rho2", C.c_double), ("vs2", C.c_double),
        ("ThickX", C.c_double), ("ThickY", C.c_double),
        ("trap_w0", C.c_double), ("trap_w1", C.c_double), ("trap_z1", C.c_double),
        ("fo", C.c_double), ("Vo", C.c_double), ("Dc", C.c_double),
        ("a0", C.c_double), ("b0", C.c_double), ("b1", C.c_double), ("zb0", C.c_double), ("zb1", C.c_double),
        ("sigma", C.c_double), ("V_init", C.c_double), ("noise_amp", C.c_double), ("seed", C.c_uint64),
        ("Vpl", C.c_double), ("creep_depth", C.c_double), ("creep_inclusive", C.c_int32),
        ("nrec", C.c_int32), ("CFL", C.c_double), ("total_years", C.c_double), ("Vthres", C.c_double),
        ("rec_x", C.c_double * 8), ("rec_y", C.c_double * 8),
    ]


def _wrong_machine() -> bool:
    import platform
    try:
        with open(_LIB_PATH, "rb") as f:
            hdr = f.read(20)
    except OSError:
        return True
    want = {"x86_64": 62, "aarch64": 183}.get(platform.machine())
    return want is not None and int.from_bytes(hdr[18:20], "little") != want


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ + OpenMP)."""
    if not force and os.path.exists(_LIB_PATH) and _wrong_machine():
        force = True
    if force:
        subprocess.run(["make", "-s", "-C", _HERE, "clean"], check=True)
    if force or not os.path.exists(_LIB_PATH) or _stale():
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(_LIB_PATH)
    for f in os.listdir(_HERE):
        if f.endswith((".cpp", ".h")) and os.path.getmtime(os.path.join(_HERE, f)) > t:
            return True
    return False


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        P, D, I64, I = C.c_void_p, C.c_double, C.c_int64, C.c_int
        dp = C.POINTER(C.c_double)
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.POINTER(OrcConfig)]
        L.orc_destroy.argtypes = [P]
        L.orc_size.restype = I64
        L.orc_size.argtypes = [P, C.c_char_p]
        L.orc_get.argtypes = [P, C.c_char_p, P]
        L.orc_scalar.restype = D
        L.orc_scalar.argtypes = [P, C.c_char_p]
        L.orc_gll.argtypes = [I, dp, dp, dp]
        L.orc_apply_K_csr.argtypes = [P, dp, dp]
        L.orc_apply_K_elem.argtypes = [P, dp, dp]
        L.orc_qs_solve.argtypes = [P, dp, dp, D, I, I, dp]
        L.orc_IDS.restype = D
        L.orc_IDS.argtypes = [D, D, D, D, D, D]
        L.orc_IDS2.restype = D
        L.orc_IDS2.argtypes = [D] * 7
        L.orc_NR.argtypes = [D] * 10 + [dp, dp]
        L.orc_NR_q.argtypes = [D] * 10 + [dp, dp]
        L.orc_slrFunc.argtypes = [P, dp, dp, dp, dp, dp, D]
        L.orc_FBC.argtypes = [P] + [dp] * 9 + [D]
        L.orc_dtevol.restype = D
        L.orc_dtevol.argtypes = [P, D, D, dp, I]
        L.orc_run.restype = I64
        L.orc_run.argtypes = [P, I64, D, I, D, I]
        L.orc_reset.argtypes = [P]
        L.orc_state.argtypes = [P, C.c_char_p, P]
        L.orc_set_state.argtypes = [P, C.c_char_p, P]
        L.orc_set_damage.restype = I
        L.orc_set_damage.argtypes = [P, C.POINTER(C.c_int64), I64, D]
        L.orc_damage_evolve.argtypes = [P]
        L.orc_set_threads.argtypes = [I]
        L.orc_get_threads.restype = I
        _lib = L
    return _lib


def _dp(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def to_struct(cfg) -> OrcConfig:
    s = OrcConfig()
    for name, _ in OrcConfig._fields_:
        if name in ("rec_x", "rec_y", "nrec"):
            continue
        setattr(s, name, getattr(cfg, name))
    s.nrec = len(cfg.rec_x)
    for k, (xr, yr) in enumerate(zip(cfg.rec_x, cfg.rec_y)):
        s.rec_x[k] = xr
        s.rec_y[k] = yr
    return s


def gll(ngll: int):
    x = np.zeros(ngll)
    w = np.zeros(ngll)
    H = np.zeros(ngll * ngll)
    lib().orc_gll(ngll, _dp(x), _dp(w), _dp(H))
    return x, w, H.reshape(ngll, ngll, order="F")


_INT_ARRAYS = {"iglob", "iFlt", "iBcL", "iBcT", "FltIglobBC", "FltNI", "out_seis", "K_ptr", "K_col",
               "regime", "cg_iters", "damage_idx"}
_COL_ARRAYS = {"seismic_stress", "seismic_slipvel", "seismic_slip", "is_stress", "is_slipvel", "is_slip",
               "taubefore", "tauafter", "delfafter"}
_ROW_ARRAYS = {"dSeis", "vSeis", "aSeis"}


class Oracle:
    """One oracle model built from a ``ModelConfig``."""

    def __init__(self, cfg):
        self.cfg = cfg
        self._s = to_struct(cfg)
        self.h = lib().orc_create(C.byref(self._s))
        self.nglob = int(self.scalar("nglob"))
        self.Nf = int(self.scalar("FltNglob"))

    def close(self):
        if self.h:
            lib().orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def scalar(self, name: str) -> float:
        return lib().orc_scalar(self.h, name.encode())

    def get(self, name: str) -> np.ndarray:
        n = lib().orc_size(self.h, name.encode())
        if n < 0:
            raise KeyError(name)
        dt = np.int64 if name in _INT_ARRAYS else np.float64
        out = np.zeros(n, dtype=dt)
        if n:
            lib().orc_get(self.h, name.encode(), out.ctypes.data_as(C.c_void_p))
        if name in _COL_ARRAYS and n:
            out = out.reshape(-1, self.Nf).T
        if name in _ROW_ARRAYS and n:
            out = out.reshape(-1, len(self.cfg.rec_x))
        if name in ("iglob", "W"):
            out = out.reshape(5, 5, -1, order="F")
        if name == "H":
            out = out.reshape(5, 5, order="F")
        return out

    def csr(self):
        import scipy.sparse as sp
        ptr, col, val = self.get("K_ptr"), self.get("K_col"), self.get("K_val")
        return sp.csr_matrix((val, col, ptr), shape=(self.nglob, self.nglob))

    def apply_K_csr(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.nglob)
        lib().orc_apply_K_csr(self.h, _dp(x), _dp(y))
        return y

    def apply_K_elem(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.nglob)
        lib().orc_apply_K_elem(self.h, _dp(x), _dp(y))
        return y

    def qs_solve(self, F_fault, d_full, tol=1e-8, mode=0, maxit=0):
        F_fault = np.ascontiguousarray(F_fault, dtype=np.float64)
        d = np.array(d_full, dtype=np.float64, copy=True)
        rr = C.c_double(0)
        it = lib().orc_qs_solve(self.h, _dp(F_fault), _dp(d), tol, mode, maxit, C.byref(rr))
        return d, it, rr.value

    def run(self, nsteps: int, t_end: Optional[float] = None, qs_mode: int = 0, qs_tol: float = 1e-8,
            qs_maxit: int = 0) -> int:
        t_end = self.scalar("Total_time") if t_end is None else t_end
        return lib().orc_run(self.h, nsteps, t_end, qs_mode, qs_tol, qs_maxit)

    def set_damage(self, idx, factor: float = 0.95):
        """Elements (1-based) whose W is scaled by ``factor`` at every event end (damageEvol.jl)."""
        a = np.ascontiguousarray(idx, dtype=np.int64)
        if lib().orc_set_damage(self.h, a.ctypes.data_as(C.POINTER(C.c_int64)), len(a), float(factor)) != 0:
            raise ValueError("damage element out of range")

    def damage_evolve(self):
        lib().orc_damage_evolve(self.h)

    def reset(self):
        lib().orc_reset(self.h)

    def state(self, name: str) -> np.ndarray:
        return self.get(name)

    def set_state(self, name: str, value):
        if np.ndim(value) == 0:
            v = C.c_double(float(value))
            lib().orc_set_state(self.h, name.encode(), C.byref(v))
        else:
            a = np.ascontiguousarray(value, dtype=np.float64)
            lib().orc_set_state(self.h, name.encode(), a.ctypes.data_as(C.c_void_p))


# scalar friction kernels
def IDS(xLf, Vo, psi, dt, Vf, cnd):
    return lib().orc_IDS(xLf, Vo, psi, dt, Vf, cnd)


def IDS2(xLf, Vo, psi, psi1, dt, Vf, Vf1):
    return lib().orc_IDS2(xLf, Vo, psi, psi1, dt, Vf, Vf1)


def NR(fo, Vo, cca, ccb, Seff, tau, tauo, psi, FltZ, FltVfree, quad=False):
    V, T = C.c_double(0), C.c_double(0)
    f = lib().orc_NR_q if quad else lib().orc_NR
    st = f(fo, Vo, cca, ccb, Seff, tau, tauo, psi, FltZ, FltVfree, C.byref(V), C.byref(T))
    return V.value, T.value, st


def set_threads(n: int):
    lib().orc_set_threads(int(n))


def get_threads() -> int:
    return lib().orc_get_threads()
