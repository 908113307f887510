"""Split-precision (bf16x3 on tcgen05) matvec and refined Lanczos against FP64.

Tolerances: one bf16x3 product carries a relative error of about 2^-16
(the dropped lo*lo term and the bf16 rounding of lo), accumulated in fp32,
so the matvec is checked at 2e-4 relative 2-norm error against the FP64
oracle.  After FP64 refinement the Lanczos energy must agree with the FP64
solver to 1e-10 (absolute), the target the split path is built for."""
import numpy as np
import pytest

from helpers import exact_problem, models, oracle_bs, rel_err, small_problem
from tk_gb300 import PREC_BF16X3, PREC_FP64

pytestmark = pytest.mark.gpu
SPLIT_TOL = 2e-4


def _run(plan, x):
    import torch

    xd = torch.from_numpy(x).cuda()
    yd = torch.full_like(xd, float("nan"))
    plan.apply(xd, yd)
    torch.cuda.synchronize()
    return yd.cpu().numpy()


@pytest.mark.parametrize("name,D", [("heisenberg", 40), ("hubbard", 48), ("cylinder", 96), ("heisenberg", 300)])
def test_split_matvec_small(lib_built, name, D):
    p = small_problem(name, D)
    plan = p.plan(precision=PREC_BF16X3)
    x = np.random.default_rng(2).standard_normal(plan.block_dim)
    y = _run(plan, x)
    assert np.isfinite(y).all()
    assert rel_err(y, oracle_bs(p).apply(x)) < SPLIT_TOL


@pytest.mark.parametrize("name", ["heisenberg_d1024", "hubbard_d2048"])
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
