"""The C-ABI library: builds, loads, exports every declared symbol; host-only
argument checks return status codes (no GPU work is started here)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np

from tk_gb300 import _abi

HEADER = Path(__file__).resolve().parent.parent / "include" / "tk_heff.h"


def declared():
    txt = HEADER.read_text()
    return sorted(set(re.findall(r"^\s*(?:tk_status|void|const char\*|int32_t)\s+(tk_[a-z0-9_]+)\s*\(", txt, re.M)))


def test_exports_every_declared_symbol(lib_built):
    lib = _abi.load()
    names = declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    bound = {s[0] for s in _abi.SIGNATURES}
    assert set(names) <= bound


def test_version_and_error_string(lib_built):
    lib = _abi.load()
    assert lib.tk_version() >= 1
    assert isinstance(lib.tk_last_error(), bytes)


def test_null_arguments_rejected(lib_built):
    lib = _abi.load()
    assert lib.tk_heff2_plan_create(None, None, None, None, None, None, 0, None) == 1
    assert lib.tk_heff2_dims(None, None, None, None) == 1
    cfg = _abi.tk_lanczos_cfg(20, 0, 1e-10, 0)
    assert lib.tk_lanczos_lowest(None, C.byref(cfg), None, None, None, None) == 1
    assert b"null" in lib.tk_last_error()


def test_gemm_shape_mismatch_rejected(lib_built):
    lib = _abi.load()
    buf = np.zeros(16)
    a = _abi.tk_mat(buf.ctypes.data, 2, 3, 3, 1, 0)
    b = _abi.tk_mat(buf.ctypes.data, 2, 2, 2, 1, 0)
    c = _abi.tk_mat_mut(buf.ctypes.data, 2, 2, 2, 1)
    assert lib.tk_gemm_f64(None, 1.0, C.byref(a), C.byref(b), 0.0, C.byref(c), None) == 1
