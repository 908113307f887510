"""tk_gemm_f64_noalloc against tk_gemm_f64, through the C ABI.

The no-allocation variant exists for callers that cannot allocate device
memory when they call the GEMM (arena-driven sweeps, graph-recorded work,
latency-bound loops); it keeps its tile tables in a fixed 1 MiB array inside
the library.  Its results must equal the allocating entry point's, call after
call, even though every call reuses (and overwrites) the same array.

This file is collected last on purpose, and must pass both on its own in a
fresh process (the first call then performs the array set-up) and after the
other tests."""
import ctypes as C

import numpy as np
import pytest

from tk_gb300 import _abi
from tk_gb300.heff import context

pytestmark = pytest.mark.gpu
TOL = 1e-12  # same kernel on both paths; relative max-norm


def _mats(torch, rng, M, K, N, ta, tb):
    A = rng.standard_normal((K, M) if ta else (M, K))
    B = rng.standard_normal((N, K) if tb else (K, N))
    Cm = rng.standard_normal((M, N))
    dA, dB = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    a = _abi.tk_mat(dA.data_ptr(), M, K, 1 if ta else K, M if ta else 1, 0)
    b = _abi.tk_mat(dB.data_ptr(), K, N, 1 if tb else N, K if tb else 1, 0)
    return dA, dB, a, b, Cm


def test_noalloc_gemm_matches_allocating_gemm_twice(lib_built):
    import torch

    lib = _abi.load()
    ctx = context(0)
    rng = np.random.default_rng(123)
    stream = torch.cuda.Stream()
    # two calls in a row, different shapes and layouts, so a stale table from
    # the first call would corrupt the second
    for (M, K, N, ta, tb, alpha, beta) in [(300, 77, 190, False, True, 1.5, -0.5), (65, 400, 129, True, False, 1.0, 0.0)]:
        dA, dB, a, b, Cm = _mats(torch, rng, M, K, N, ta, tb)
        c_ref = torch.from_numpy(Cm).cuda()
        c_new = torch.from_numpy(Cm).cuda()
        cr = _abi.tk_mat_mut(c_ref.data_ptr(), M, N, N, 1)
        cn = _abi.tk_mat_mut(c_new.data_ptr(), M, N, N, 1)
        torch.cuda.synchronize()
        _abi.check(lib.tk_gemm_f64(ctx, alpha, C.byref(a), C.byref(b), beta, C.byref(cr), None))
        _abi.check(lib.tk_gemm_f64_noalloc(ctx, alpha, C.byref(a), C.byref(b), beta, C.byref(cn),
                                           C.c_void_p(stream.cuda_stream)))
        stream.synchronize()
        ref = c_ref.cpu().numpy()
        got = c_new.cpu().numpy()
        assert np.abs(got - ref).max() <= TOL * max(1.0, np.abs(ref).max())
        want = alpha * ((dA.cpu().numpy().T if ta else dA.cpu().numpy()) @ (dB.cpu().numpy().T if tb else dB.cpu().numpy())) + beta * Cm
        assert np.abs(got - want).max() < 1e-10 * max(1.0, np.abs(want).max())


def test_noalloc_gemm_rejects_oversize(lib_built):
    lib = _abi.load()
    ctx = context(0)
    big = 70000 * 64  # more output tiles than the fixed array holds (no GPU work is started)
    dummy = 1 << 20
    a = _abi.tk_mat(dummy, big, 1, 1, 1, 0)
    b = _abi.tk_mat(dummy, 1, 64, 64, 1, 0)
    c = _abi.tk_mat_mut(dummy, big, 64, 64, 1)
    assert lib.tk_gemm_f64_noalloc(ctx, 1.0, C.byref(a), C.byref(b), 0.0, C.byref(c), None) == 1
    assert b"no-allocation scratch" in lib.tk_last_error()
