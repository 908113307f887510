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
    dcfg = _abi.tk_davidson_cfg(60, 1000, 1e-10, None, 0)
    assert lib.tk_davidson_lowest(None, C.byref(dcfg), None, None, None, None) == 1
    assert b"tk_davidson_lowest" in lib.tk_last_error()


def test_gemm_shape_mismatch_rejected(lib_built):
    lib = _abi.load()
    buf = np.zeros(16)
    a = _abi.tk_mat(buf.ctypes.data, 2, 3, 3, 1, 0)
    b = _abi.tk_mat(buf.ctypes.data, 2, 2, 2, 1, 0)
    c = _abi.tk_mat_mut(buf.ctypes.data, 2, 2, 2, 1)
    assert lib.tk_gemm_f64(None, 1.0, C.byref(a), C.byref(b), 0.0, C.byref(c), None) == 1


def _plan_status(prob, all_sectors=False):
    """Runs tk_heff2_plan_create up to its first CUDA call with a fake context:
    the host tables are built and self-checked; on a machine without a GPU the
    call then stops at cudaSetDevice with TK_ERR_CUDA."""
    from tk_gb300.heff import _Marshal

    lib = _abi.load()
    m = _Marshal()
    el, er = m.env(prob.env_l), m.env(prob.env_r)
    bi, bj = m.bst(prob.w_i), m.bst(prob.w_j)
    fl = None
    if not all_sectors:
        farr = np.array(list(prob.flux) + [0], dtype=np.int32)
        m.keep.append(farr)
        fl = _abi.i32ptr(farr)
    fake_ctx = np.zeros(4, dtype=np.int32)  # struct tk_ctx { int device = 0; }
    h = C.c_void_p()
    st = lib.tk_heff2_plan_create(fake_ctx.ctypes.data, C.byref(el), C.byref(er), C.byref(bi), C.byref(bj), fl, 0,
                                  C.byref(h))
    return st, lib.tk_last_error().decode()


def test_host_tables_self_check_cpu(lib_built):
    import torch
    from helpers import small_problem

    if torch.cuda.is_available():
        import pytest

        pytest.skip("CPU-only check (a GPU would create a real plan)")
    # the larger cases build tall stage-1 stacks (split copy) and psi halves
    for name, D in [("heisenberg", 40), ("hubbard", 48), ("cylinder", 96), ("cylinder", 512), ("hubbard", 256)]:
        for all_sectors in (False, True):
            st, msg = _plan_status(small_problem(name, D), all_sectors)
            assert st == 4 and "cudaSetDevice" in msg, (name, st, msg)


def test_sector_mismatch_cpu(lib_built):
    import torch
    from helpers import small_problem
    from tk_gb300 import models

    if torch.cuda.is_available():
        import pytest

        pytest.skip("CPU-only check")
    p = small_problem("heisenberg", 12)
    p.w_i = models.hubbard().bulk  # different quantum-number kind
    st, msg = _plan_status(p)
    assert st == 1 and "kinds" in msg
    p = small_problem("heisenberg", 12)
    p.w_j = models.cylinder_j1(4).bulk  # bond QIndex differs from the environment's
    st, msg = _plan_status(p)
    assert st == 2, (st, msg)


def test_empty_two_site_space_cpu(lib_built):
    """A flux no sector combination reaches: the host tables build (on a
    machine without a GPU the call then stops at cudaSetDevice) and the
    restatement's space is empty."""
    import torch
    from helpers import oracle_bs, small_problem

    if torch.cuda.is_available():
        import pytest

        pytest.skip("CPU-only check")
    p = small_problem("heisenberg", 12)
    p.flux = (40,)
    st, msg = _plan_status(p)
    assert st == 4 and "cudaSetDevice" in msg, (st, msg)
    bs = oracle_bs(p)
    assert bs.total == 0 and bs.n_blocks == 0 and bs.flops() == 0.0
    assert bs.apply(np.zeros(0)).shape == (0,)


def test_header_is_plain_c(tmp_path):
    """include/tk_heff.h compiles as ISO C11 on its own (no CUDA or C++ types),
    which is what bindgen or cgo read."""
    import shutil
    import subprocess
    from pathlib import Path

    import pytest

    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    inc = Path(__file__).resolve().parents[1] / "include"
    src = tmp_path / "c_check.c"
    src.write_text('#include "tk_heff.h"\nint main(void) { return (int)sizeof(tk_bst) + TK_OK; }\n')
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only",
                        "-I", str(inc), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
