"""Failure paths that need no GPU: a host allocation that fails inside the
plan-table builders comes back as TK_ERR_OOM (never an abort or an uncaught
exception across the C ABI), plan sizing runs without CUDA, and a sweep stops
at its cancel flag (DMRGEngine::run_with_cancel_flag,
tk-dmrg/src/sweep/mod.rs:273-289) with DmrgError::Cancelled."""
import ctypes as C

import numpy as np
import pytest

from helpers import oracle_bs, small_problem
from tk_gb300 import PREC_BF16X3, PREC_FP64, TkError, _abi
from tk_gb300.heff import plan_footprint

TK_ERR_OOM = 3


def _footprint(p, precision=PREC_FP64):
    return plan_footprint(p.env_l, p.env_r, p.w_i, p.w_j, p.flux, precision)


@pytest.mark.parametrize("name,D", [("heisenberg", 40), ("hubbard", 48), ("cylinder", 96)])
def test_footprint_without_gpu(lib_built, name, D):
    p = small_problem(name, D)
    bd, nb, b64 = _footprint(p)
    bs = oracle_bs(p)
    assert bd == bs.total and nb == bs.n_blocks
    _, _, b16 = _footprint(p, PREC_BF16X3)
    # the FP64 tables hold at least the block-sparse environments and two intermediates
    assert b64 >= 8 * bd and b16 > b64


def test_host_allocation_failure_is_oom(lib_built):
    lib = _abi.load()
    p = small_problem("hubbard", 48)
    want = _footprint(p, PREC_BF16X3)
    try:
        for k in range(1, 7):  # every checkpoint of the builder, split tables included
            lib.tk_debug_fail_host_alloc(k)
            with pytest.raises(TkError) as ei:
                _footprint(p, PREC_BF16X3)
            assert ei.value.status == TK_ERR_OOM, k
            assert "host allocation failed" in str(ei.value)
    finally:
        lib.tk_debug_fail_host_alloc(0)
    # nothing is left armed or half-built: the same call succeeds with the same answer
    assert _footprint(p, PREC_BF16X3) == want


def test_plan_create_host_oom_before_cuda(lib_built):
    """tk_heff2_plan_create builds its host tables before any CUDA call: an
    allocation failure there is TK_ERR_OOM on any machine."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("CPU-only check (a GPU would create a real plan)")
    from test_abi_cpu import _plan_status

    lib = _abi.load()
    try:
        lib.tk_debug_fail_host_alloc(2)
        st, msg = _plan_status(small_problem("heisenberg", 40))
    finally:
        lib.tk_debug_fail_host_alloc(0)
    assert st == TK_ERR_OOM and "host allocation failed" in msg, (st, msg)
    st, msg = _plan_status(small_problem("heisenberg", 40))
    assert st == 4 and "cudaSetDevice" in msg  # the normal CPU-machine stop


class _StubSweep:
    """DeviceDMRG.run's loop on stub steps: records which bonds ran."""

    def __init__(self, n, cancel_after, flag):
        from tk_gb300.sweep import DeviceDMRG

        self.dm = DeviceDMRG.__new__(DeviceDMRG)
        self.dm.n = n
        self.dm.bonds = [type("B", (), {"total_dim": 4})() for _ in range(n + 1)]
        self.calls = []

        def step(i, to_right, max_bond, cutoff, rec, min_bond=1, cancel=None):
            assert cancel is flag
            self.calls.append((i, to_right))
            if len(self.calls) == cancel_after:
                flag.set()  # another thread would do this; the next step must not start
            return -1.0 * len(self.calls), 0.0

        self.dm.step = step


def test_sweep_stops_at_the_cancel_flag():
    from tk_gb300.sweep import CancelFlag, SweepCancelled

    flag = CancelFlag()
    s = _StubSweep(6, 7, flag)
    with pytest.raises(SweepCancelled):
        s.dm.run(16, 3, cancel=flag)
    # one full left-to-right half sweep (5 bonds) and two steps of the way back
    assert s.calls == [(i, True) for i in range(5)] + [(4, False), (3, False)]
    assert len(s.dm.record.energies) == 1
    # a cleared flag runs to the end
    flag.clear()
    s2 = _StubSweep(6, 10 ** 9, flag)
    rec = s2.dm.run(16, 2, cancel=flag)
    assert len(s2.calls) == 2 * 2 * 5 and len(rec.energies) == 4


def test_cancel_flag_is_already_set():
    from tk_gb300.sweep import CancelFlag, SweepCancelled

    flag = CancelFlag()
    flag.set()
    s = _StubSweep(4, 10 ** 9, flag)
    with pytest.raises(SweepCancelled):
        s.dm.run(16, 1, cancel=flag)
    assert s.calls == []
