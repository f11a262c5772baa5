"""ctypes binding of libeqc.so (include/eqc.h).

The library is the only compute path: there is no CPU fallback.  If libeqc.so is missing
or cannot be loaded, ``lib()`` raises.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libeqc.so")

EQC_OK = 0
STATUS = {0: "EQC_OK", 1: "EQC_E_ARG", 2: "EQC_E_CUDA", 3: "EQC_E_NR", 4: "EQC_E_CG", 5: "EQC_E_NAN",
          6: "EQC_E_CAPACITY", 7: "EQC_E_TIMEOUT", 8: "EQC_E_NOMEM", 9: "EQC_E_STATE", 10: "EQC_E_NOGPU"}
EQC_FP64, EQC_MIXED = 0, 1
EQC_PC_AMG, EQC_PC_JACOBI = 0, 1
EQC_GUESS_PREVIOUS, EQC_GUESS_LEARNED, EQC_GUESS_EXTRAPOLATE = 0, 1, 2
EQC_TOL_RHS, EQC_TOL_R0 = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int64)


class EqcModel(C.Structure):
    _fields_ = [
        ("Nel", C.c_int64), ("FltNglob", C.c_int64), ("yr2sec", C.c_int64), ("IDstate", C.c_int64),
        ("nglob", C.c_int64), ("Total_time", C.c_double),
        ("ETA", C.c_double), ("Vpl", C.c_double), ("Vthres", C.c_double), ("Vevne", C.c_double), ("dt0", C.c_double),
        ("NelX", C.c_int64), ("NelY", C.c_int64), ("NGLL", C.c_int64), ("dxe", C.c_double), ("dye", C.c_double),
        ("iglob", _ip), ("W", _dp), ("H", _dp),
        ("fo", _dp), ("Vo", _dp), ("xLf", _dp), ("M", _dp), ("BcLC", _dp), ("BcTC", _dp),
        ("FltB", _dp), ("FltZ", _dp), ("FltX", _dp), ("cca", _dp), ("ccb", _dp), ("Seff", _dp), ("tauo", _dp),
        ("XiLf", _dp),
        ("iFlt", _ip), ("iBcL", _ip), ("iBcT", _ip), ("FltIglobBC", _ip), ("FltNI", _ip), ("out_seis", _ip),
        ("n_iBcL", C.c_int64), ("n_iBcT", C.c_int64), ("n_FltIglobBC", C.c_int64), ("n_FltNI", C.c_int64),
        ("n_out_seis", C.c_int64),
    ]


class EqcMaterial(C.Structure):
    _fields_ = [("rule", C.c_int32), ("rho1", C.c_double), ("vs1", C.c_double), ("rho2", C.c_double),
                ("vs2", C.c_double), ("ThickX", C.c_double), ("ThickY", C.c_double), ("trap_w0", C.c_double),
                ("trap_w1", C.c_double), ("trap_z1", C.c_double), ("LX", C.c_double), ("xgll", _dp), ("wgll", _dp)]


class EqcOptions(C.Structure):
    _fields_ = [("precision", C.c_int32), ("precond", C.c_int32), ("guess", C.c_int32), ("tol_rule", C.c_int32),
                ("cg_tol", C.c_double), ("cg_maxit", C.c_int32), ("device", C.c_int32),
                ("use_graphs", C.c_int32), ("verbose", C.c_int32),
                ("reliable_delta", C.c_double), ("mg_degree", C.c_int32), ("mg_coarse_max", C.c_int32),
                ("apply_variant", C.c_int32), ("mg_degree_coarse", C.c_int32),
                ("step_batch", C.c_int32)]


class EqcRunStats(C.Structure):
    _fields_ = [("steps", C.c_int64), ("qs_steps", C.c_int64), ("dyn_steps", C.c_int64), ("cg_iters", C.c_int64),
                ("qs_solves", C.c_int64), ("t", C.c_double), ("dt", C.c_double), ("isolver", C.c_int32),
                ("events", C.c_int32), ("wall_s", C.c_double), ("gpu_ms", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib: Optional[C.CDLL] = None

# Every symbol include/eqc.h declares (checked by the CPU test suite).
EXPORTS = ["eqc_default_options", "eqc_create", "eqc_destroy", "eqc_last_error", "eqc_apply_K", "eqc_qs_solve",
           "eqc_slrFunc", "eqc_FBC", "eqc_dtevol", "eqc_dtevol_noalloc", "eqc_init", "eqc_run", "eqc_get_state", "eqc_set_state",
           "eqc_get_scalar", "eqc_set_scalar", "eqc_result_size", "eqc_get_result", "eqc_layout", "eqc_apply_K_device",
           "eqc_time_apply", "eqc_time_apply_stream", "eqc_launch_count", "eqc_sync", "eqc_set_damage", "eqc_damage_evolve", "eqc_create_structured", "eqc_guess_shape", "eqc_guess_init",
           "eqc_guess_get_params", "eqc_guess_set_params", "eqc_guess_log", "eqc_guess_pairs", "eqc_guess_train",
           "eqc_guess_eval", "eqc_guess_grad", "eqc_autotune", "eqc_ensemble_create", "eqc_ensemble_run",
           "eqc_ensemble_destroy", "eqc_ensemble_last_error"]


def lib() -> C.CDLL:
    """Load libeqc.so (built by ``eqcycle_gb300.build``).  Raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m eqcycle_gb300.build` "
                           "(this package has no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    P, D, I32, I64 = C.c_void_p, C.c_double, C.c_int32, C.c_int64
    L.eqc_default_options.argtypes = [C.POINTER(EqcOptions)]
    L.eqc_create.argtypes = [C.POINTER(EqcModel), C.POINTER(EqcOptions), C.POINTER(P)]
    L.eqc_destroy.argtypes = [P]
    L.eqc_last_error.restype = C.c_char_p
    L.eqc_last_error.argtypes = [P]
    L.eqc_apply_K.argtypes = [P, _dp, _dp]
    L.eqc_qs_solve.argtypes = [P, _dp, _dp, D, I32, C.POINTER(I32), _dp]
    L.eqc_slrFunc.argtypes = [P, _dp, _dp, _dp, _dp, _dp, D]
    L.eqc_FBC.argtypes = [P] + [_dp] * 9 + [D, _ip]
    L.eqc_dtevol.argtypes = [P, D, D, _dp, I32, _dp]
    L.eqc_dtevol_noalloc.argtypes = [P, P, I64, I64, D, D, I32, P, P]
    L.eqc_init.argtypes = [P, D]
    L.eqc_run.argtypes = [P, I64, D, C.POINTER(EqcRunStats)]
    L.eqc_get_state.argtypes = [P, C.c_char_p, _dp]
    L.eqc_set_state.argtypes = [P, C.c_char_p, _dp]
    L.eqc_get_scalar.argtypes = [P, C.c_char_p, _dp]
    L.eqc_set_scalar.argtypes = [P, C.c_char_p, D]
    L.eqc_result_size.restype = I64
    L.eqc_result_size.argtypes = [P, C.c_char_p]
    L.eqc_get_result.argtypes = [P, C.c_char_p, _dp]
    L.eqc_layout.argtypes = [P, _ip, _ip, _ip]
    L.eqc_apply_K_device.argtypes = [P, P, P, I32]
    L.eqc_time_apply.argtypes = [P, I32, I32, I32, _dp]
    L.eqc_time_apply_stream.argtypes = [P, I32, I32, I32, _dp]
    L.eqc_launch_count.restype = I64
    L.eqc_launch_count.argtypes = [P]
    L.eqc_sync.argtypes = [P]
    L.eqc_set_damage.argtypes = [P, C.POINTER(C.c_int64), C.c_int64, C.c_double]
    L.eqc_damage_evolve.argtypes = [P]
    L.eqc_create_structured.argtypes = [C.POINTER(EqcModel), C.POINTER(EqcMaterial), C.POINTER(EqcOptions),
                                        C.POINTER(P)]
    _fp = C.POINTER(C.c_float)
    U64 = C.c_uint64
    L.eqc_guess_shape.argtypes = [P, C.POINTER(I32), C.POINTER(I32), C.POINTER(I64)]
    L.eqc_guess_init.argtypes = [P, U64]
    L.eqc_guess_get_params.argtypes = [P, _fp]
    L.eqc_guess_set_params.argtypes = [P, _fp]
    L.eqc_guess_log.argtypes = [P, I64]
    L.eqc_guess_pairs.argtypes = [P, _fp, _fp, C.POINTER(I64)]
    L.eqc_guess_train.argtypes = [P, _fp, _fp, I64, I32, D, I32, U64, _dp]
    L.eqc_guess_eval.argtypes = [P, _fp, _fp, I64, _dp, _fp]
    L.eqc_guess_grad.argtypes = [P, _fp, _fp, I64, _fp, _dp]
    L.eqc_autotune.argtypes = [P, I32, C.POINTER(I32), C.POINTER(I32), _dp]
    L.eqc_ensemble_create.argtypes = [C.POINTER(P), I32, C.POINTER(P)]
    L.eqc_ensemble_run.argtypes = [P, I64, C.POINTER(EqcRunStats), _dp]
    L.eqc_ensemble_destroy.argtypes = [P]
    L.eqc_ensemble_last_error.restype = C.c_char_p
    L.eqc_ensemble_last_error.argtypes = [P]
    for name in EXPORTS:
        getattr(L, name)
    _lib = L
    return L


def fptr(a):
    """float* of a float32 array (None -> NULL)."""
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(C.c_float))


def dptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


class EqcError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


def check(status: int, handle=None):
    if status != EQC_OK:
        msg = lib().eqc_last_error(handle)
        raise EqcError(status, msg.decode() if msg else "")


def default_options(**kw) -> EqcOptions:
    o = EqcOptions()
    lib().eqc_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o
