"""The C ABI: libeqc.so builds, loads on a machine without a GPU, and exports every symbol
include/eqc.h declares.  No compute call is made here."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "eqc.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(eqc_[A-Za-z0-9_]+)\s*\(", src)))


def test_header_symbols_exported(eqclib):
    names = _declared()
    assert "eqc_create" in names and len(names) >= 15
    missing = [n for n in names if not hasattr(eqclib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from eqcycle_gb300 import _lib
    assert sorted(_lib.EXPORTS) == _declared()


def test_create_without_gpu_reports_status(eqclib):
    import ctypes as C
    import torch
    if torch.cuda.is_available():
        return
    from eqcycle_gb300 import _lib
    h = C.c_void_p()
    st = eqclib.eqc_create(C.byref(_lib.EqcModel()), None, C.byref(h))
    assert st == 10 and not h.value   # EQC_E_NOGPU, no handle
