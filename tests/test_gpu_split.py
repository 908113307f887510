"""Split-precision (bf16x3 on tcgen05) matvec and refined Lanczos against FP64.

Tolerances: one bf16x3 product carries a relative error of about 2^-16
(the dropped lo*lo term and the bf16 rounding of lo), accumulated in fp32,
so the matvec is checked at 2e-4 relative 2-norm error against the FP64
oracle.  After FP64 refinement the Lanczos energy must agree with the FP64
solver to 1e-10 (absolute), the target the split path is built for."""
import numpy as np
import pytest

from helpers import exact_problem, models, oracle_bs, rel_err, small_problem
from tk_gb300 import PREC_BF16X3, PREC_FP64, TkError

pytestmark = pytest.mark.gpu
SPLIT_TOL = 2e-4


def _run(plan, x):
    import torch

    xd = torch.from_numpy(x).cuda()
    yd = torch.full_like(xd, float("nan"))
    plan.apply(xd, yd)
    torch.cuda.synchronize()
    return yd.cpu().numpy()


# cylinder at D=512 has stage-1 stacks taller than three row tiles (psi taken
# from the split copy) beside short ones (psi split inside the GEMM kernel)
@pytest.mark.parametrize("name,D", [("heisenberg", 40), ("hubbard", 48), ("cylinder", 96), ("heisenberg", 300),
                                    ("cylinder", 512)])
def test_split_matvec_small(lib_built, name, D):
    p = small_problem(name, D)
    plan = p.plan(precision=PREC_BF16X3)
    x = np.random.default_rng(2).standard_normal(plan.block_dim)
    y = _run(plan, x)
    assert np.isfinite(y).all()
    assert rel_err(y, oracle_bs(p).apply(x)) < SPLIT_TOL


# cylinder_d4096 runs the tall-stack stage 1 (split copy + TMA) on its large sectors
@pytest.mark.parametrize("name", ["heisenberg_d1024", "hubbard_d2048", "cylinder_d4096"])
def test_split_matvec_full(lib_built, name):
    p = models.workload(name)
    plan = p.plan(precision=PREC_BF16X3)
    x = np.random.default_rng(3).standard_normal(plan.block_dim)
    y = _run(plan, x)
    assert np.isfinite(y).all()
    ref = oracle_bs(p).apply(x)
    err = rel_err(y, ref)
    assert err < SPLIT_TOL, err
    # switching the same plan back to FP64 restores oracle parity
    plan.set_precision(PREC_FP64)
    assert rel_err(_run(plan, x), ref) < 1e-12


def test_split_host_paths(lib_built):
    p = small_problem("hubbard", 32)
    plan = p.plan(precision=PREC_BF16X3)
    x = np.random.default_rng(4).standard_normal(plan.block_dim)
    y = np.zeros_like(x)
    plan.apply_host_flat(x, y)
    assert rel_err(y, oracle_bs(p).apply(x)) < SPLIT_TOL


@pytest.mark.parametrize("name", ["heisenberg", "hubbard"])
def test_refined_energy_matches_fp64(lib_built, name):
    p = small_problem(name, 64)
    plan64 = p.plan(precision=PREC_FP64)
    r64 = plan64.lanczos(krylov_dim=40, max_restarts=30, tol=1e-10)
    assert r64.converged
    plan = p.plan(precision=PREC_BF16X3)
    r = plan.lanczos(krylov_dim=40, max_restarts=30, tol=1e-10, refine=20)
    assert abs(r.eigenvalue - r64.eigenvalue) < 1e-10, (r.eigenvalue, r64.eigenvalue, r.residual_norm)
    assert r.residual_norm < 1e-9


def test_refined_energy_exact_environment(lib_built):
    from helpers import ed_heisenberg

    p = exact_problem(models.heisenberg(), 10, 4, (0,))
    plan = p.plan(precision=PREC_BF16X3)
    r = plan.lanczos(krylov_dim=60, max_restarts=20, tol=1e-10, refine=20)
    assert abs(r.eigenvalue - ed_heisenberg(10)) < 1e-10


def test_integer_pipe_conversions_match_hardware(lib_built):
    """The split kernels' fp64 <-> fp32 conversions (integer pipes) equal the
    hardware conversions: random doubles over many magnitudes, ties, and edge
    patterns."""
    import ctypes as C

    import torch
    from tk_gb300 import _abi
    from tk_gb300.heff import context

    rng = np.random.default_rng(12)
    vals = [rng.standard_normal(200_000) * 10.0 ** rng.uniform(-30, 30, 200_000),
            rng.uniform(-1, 1, 100_000),
            # exact round-to-nearest-even ties and their neighbours at the fp32 boundary
            np.frombuffer((np.arange(50_000, dtype=np.uint64) * np.uint64(1 << 29)
                           | np.uint64(0x3FF0000010000000)).tobytes(), dtype=np.float64),
            np.array([0.0, -0.0, 1.0, -1.0, 3.4028234663852886e38, 1.1754943508222875e-38, 2.0 ** -149,
                      np.inf, -np.inf, 1e-300, 1e300, 65504.0, np.pi])]
    x = torch.from_numpy(np.concatenate(vals)).cuda()
    bad = C.c_uint64(99)
    _abi.check(_abi.load().tk_check_split_conversions(context(0), C.c_void_p(x.data_ptr()), x.numel(),
                                                      C.byref(bad)))
    assert bad.value == 0


# cylinder D=512 has tall stage-1 stacks (split copy); hubbard D=64 has none,
# so its staged psi copy runs in pieces overlapped with stage 1
@pytest.mark.parametrize("name,D", [("cylinder", 512), ("hubbard", 64), ("hubbard", 256)])
def test_host_io_direct_matches_staged(lib_built, name, D):
    """Split matvec from page-locked host buffers: the kernels reading psi and
    writing y over the CPU-GPU link give the same bits as the staged copies."""
    import torch

    from tk_gb300 import _abi

    p = small_problem(name, D)
    plan = p.plan(precision=PREC_BF16X3)
    x = np.random.default_rng(5).standard_normal(plan.block_dim)
    hx = torch.from_numpy(x).pin_memory()
    out = {}
    modes = (_abi.HOST_IO_STAGED, _abi.HOST_IO_DIRECT, _abi.HOST_IO_DIRECT_OUT, _abi.HOST_IO_AUTO)
    for mode in modes:
        plan.set_host_io(mode)
        hy = torch.full_like(hx, float("nan")).pin_memory()
        plan.apply_host_flat_ptr(hx.data_ptr(), hy.data_ptr())
        out[mode] = hy.numpy().copy()
    for mode in modes[1:]:
        assert np.array_equal(out[_abi.HOST_IO_STAGED], out[mode]), mode
    # psi copied in 1, 2, 4 or 8 pieces: the same bits (the cached graph is rebuilt per setting)
    for pieces in (1, 4, 8, 2):
        plan.set_psi_pieces(pieces)
        for mode in (_abi.HOST_IO_STAGED, _abi.HOST_IO_DIRECT_OUT):
            plan.set_host_io(mode)
            hy = torch.full_like(hx, float("nan")).pin_memory()
            plan.apply_host_flat_ptr(hx.data_ptr(), hy.data_ptr())
            assert np.array_equal(hy.numpy(), out[_abi.HOST_IO_STAGED]), (pieces, mode)
    with pytest.raises(TkError):
        plan.set_psi_pieces(3)
    assert rel_err(out[_abi.HOST_IO_AUTO], oracle_bs(p).apply(x)) < SPLIT_TOL
    # pageable buffers fall back to staged copies in every mode
    plan.set_host_io(_abi.HOST_IO_DIRECT)
    y = np.zeros_like(x)
    plan.apply_host_flat(x, y)
    assert np.array_equal(y, out[_abi.HOST_IO_STAGED])
    # and the device-buffer matvec gives the same bits
    assert np.array_equal(_run(plan, x), out[_abi.HOST_IO_STAGED])


def test_refined_eigenpair_full_hubbard(lib_built):
    """The metric's accuracy target at full size (Hubbard D=2048, 976 476
    block elements): split-precision Lanczos with FP64 Jacobi-Davidson
    refinement reaches the FP64 Lanczos eigenvalue to |dE| <= 1e-10, and its
    FP64 residual meets the tolerance."""
    p = models.workload("hubbard_d2048")
    plan = p.plan(precision=PREC_FP64)
    r64 = plan.lanczos(krylov_dim=30, max_restarts=40, tol=1e-9)
    assert r64.converged
    plan.set_precision(PREC_BF16X3)
    r = plan.lanczos(krylov_dim=30, max_restarts=40, tol=1e-9, refine=30)
    assert r.converged and r.residual_norm <= 1e-9
    assert abs(r.eigenvalue - r64.eigenvalue) <= 1e-10, (r.eigenvalue, r64.eigenvalue)
    # most matvecs ran in split precision
    assert r.fp64_matvec_count < r.matvec_count
