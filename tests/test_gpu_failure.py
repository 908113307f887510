"""Failure paths on the GPU, in forms that fault and hang nothing:

* the tensor-core kernels report a bounded wait that ran out through a device
  error word; the host plants that word (tk_heff2_inject_error_word) and the
  calls that read it back must return TK_ERR_TIMEOUT and clear it;
* a device allocation that fails while a plan is made (tk_debug_fail_device_alloc)
  returns TK_ERR_OOM and leaves the library usable;
* the eigensolvers stop at the caller's cancel flag with TK_ERR_CANCELLED, and a
  sweep raises SweepCancelled (DmrgError::Cancelled, tk-dmrg/src/sweep/mod.rs:287-289)."""
import threading
import time

import numpy as np
import pytest

from helpers import oracle_bs, rel_err, small_problem
from tk_gb300 import PREC_BF16X3, PREC_FP64, TkError, _abi

pytestmark = pytest.mark.gpu
TK_ERR_OOM, TK_ERR_TIMEOUT, TK_ERR_CANCELLED = 3, 5, 6


def test_error_word_read_back_is_timeout(lib_built):
    import torch

    p = small_problem("hubbard", 48)
    plan = p.plan(precision=PREC_BF16X3)
    x = np.random.default_rng(1).standard_normal(plan.block_dim)
    hx = torch.from_numpy(x).pin_memory()
    hy = torch.zeros_like(hx).pin_memory()
    plan.apply_host_flat_ptr(hx.data_ptr(), hy.data_ptr())  # the cached graph path, clean
    good = hy.numpy().copy()
    _abi.check(_abi.load().tk_heff2_inject_error_word(plan.handle, 2))
    with pytest.raises(TkError) as ei:
        plan.apply_host_flat_ptr(hx.data_ptr(), hy.data_ptr())
    assert ei.value.status == TK_ERR_TIMEOUT and "bounded wait" in str(ei.value)
    # the word was cleared: the next call is clean and gives the same bits
    plan.apply_host_flat_ptr(hx.data_ptr(), hy.data_ptr())
    assert np.array_equal(hy.numpy(), good)
    # the eigensolvers read it back too
    _abi.check(_abi.load().tk_heff2_inject_error_word(plan.handle, 1))
    with pytest.raises(TkError) as ei:
        plan.lanczos(krylov_dim=10, max_restarts=0, tol=1e-8)
    assert ei.value.status == TK_ERR_TIMEOUT
    r = plan.lanczos(krylov_dim=30, max_restarts=20, tol=1e-8, refine=10)
    assert r.converged
    # an FP64 plan has no tensor-core word
    p64 = p.plan(precision=PREC_FP64)
    with pytest.raises(TkError) as ei:
        _abi.check(_abi.load().tk_heff2_inject_error_word(p64.handle, 1))
    assert ei.value.status == 7


@pytest.mark.parametrize("countdown", [1, 3, 6])
def test_device_allocation_failure_is_oom(lib_built, countdown):
    lib = _abi.load()
    p = small_problem("hubbard", 48)
    try:
        lib.tk_debug_fail_device_alloc(countdown)
        with pytest.raises(TkError) as ei:
            p.plan(precision=PREC_FP64)
        assert ei.value.status == TK_ERR_OOM
    finally:
        lib.tk_debug_fail_device_alloc(0)
    plan = p.plan(precision=PREC_FP64)
    # the split operands allocate on switching precision
    try:
        lib.tk_debug_fail_device_alloc(countdown)
        with pytest.raises(TkError) as ei:
            plan.set_precision(PREC_BF16X3)
        assert ei.value.status == TK_ERR_OOM
    finally:
        lib.tk_debug_fail_device_alloc(0)
    x = np.random.default_rng(2).standard_normal(plan.block_dim)
    y = np.zeros_like(x)
    plan.apply_host_flat(x, y)  # still the FP64 plan, still exact
    assert rel_err(y, oracle_bs(p).apply(x)) < 1e-12
    plan.set_precision(PREC_BF16X3)
    plan.apply_host_flat(x, y)
    assert rel_err(y, oracle_bs(p).apply(x)) < 2e-4


def test_cancel_flag_stops_the_eigensolvers(lib_built):
    p = small_problem("heisenberg", 300)
    plan = p.plan(precision=PREC_FP64)
    flag = np.zeros(1, dtype=np.int32)
    plan.set_cancel_flag(flag)
    flag[0] = 1
    for solve in (lambda: plan.lanczos(krylov_dim=20, max_restarts=5, tol=1e-12),
                  lambda: plan.davidson(max_subspace=30, max_iter=100, tol=1e-12)):
        with pytest.raises(TkError) as ei:
            solve()
        assert ei.value.status == TK_ERR_CANCELLED and "cancelled" in str(ei.value)
    # set from another thread while Lanczos restarts (tol 0 is never met: without
    # the flag it would run all 10^6 restarts)
    flag[0] = 0
    t = threading.Timer(0.3, lambda: flag.__setitem__(0, 1))
    t0 = time.perf_counter()
    t.start()
    with pytest.raises(TkError) as ei:
        plan.lanczos(krylov_dim=20, max_restarts=10 ** 6, tol=0.0)
    assert ei.value.status == TK_ERR_CANCELLED
    assert time.perf_counter() - t0 < 30.0
    t.join()
    # detached, the plan solves as before
    plan.set_cancel_flag(None)
    r = plan.lanczos(krylov_dim=40, max_restarts=30, tol=1e-9)
    assert r.converged


def test_sweep_cancel(lib_built):
    from tk_gb300 import models, sweep

    m = models.heisenberg()
    sites, bonds = sweep.random_site_tensors(m, 8, 16, (0,), np.random.default_rng(3))
    dm = sweep.DeviceDMRG(m, sites, bonds, precision=PREC_FP64, solver="davidson", tol=1e-10)
    flag = sweep.CancelFlag()
    t = threading.Timer(0.5, flag.set)
    t.start()
    with pytest.raises(sweep.SweepCancelled):
        dm.run(16, 10 ** 6, cancel=flag)
    t.join()
    # the MPS is the last completed step's: a plain run from it still converges
    flag.clear()
    rec = dm.run(16, 2, cancel=flag)
    assert np.isfinite(rec.energies[-1])
