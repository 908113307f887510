"""The stacked FP64 schedule (TK_SCHED_STACKED): the sector GEMMs regrouped
into the split path's operand stacks and computed in FP64.  Parity with the
block-sparse oracle at the FP64 tolerance, on the small problems of every
model and at the full Hubbard and cylinder sizes, through the device, host
and eigensolver entry points."""
import numpy as np
import pytest

from helpers import models, oracle_bs, rel_err, small_problem
from tk_gb300 import _abi

pytestmark = pytest.mark.gpu
TOL = 1e-12  # FP64 vs the FP64 oracle, relative 2-norm (the sums run in another order)


def _torch():
    import torch

    assert torch.cuda.is_available()
    return torch


@pytest.mark.parametrize("name,D", [("heisenberg", 96), ("hubbard", 96), ("cylinder", 128), ("hubbard", 24)])
def test_stacked_matches_oracle(lib_built, name, D):
    torch = _torch()
    p = small_problem(name, D)
    plan = p.plan()
    assert plan.schedule == _abi.SCHED_STACKED  # the default of real plans
    assert plan.launches() <= 3
    bs = oracle_bs(p)
    x = np.random.default_rng(5).standard_normal(plan.block_dim)
    xd = torch.from_numpy(x).cuda()
    yd = torch.full_like(xd, float("nan"))  # every output written
    plan.apply(xd, yd)
    torch.cuda.synchronize()
    y = yd.cpu().numpy()
    assert np.isfinite(y).all()
    assert rel_err(y, bs.apply(x)) < TOL
    # the host-buffer entry point runs the same launches
    y2 = np.zeros_like(x)
    plan.apply_host_flat(x, y2)
    assert np.array_equal(y2, y)
    # repeated applies are deterministic
    plan.apply(xd, yd)
    torch.cuda.synchronize()
    assert np.array_equal(yd.cpu().numpy(), y)


@pytest.mark.parametrize("name", ["hubbard_d2048", "cylinder_d4096"])
def test_stacked_full_size(lib_built, name):
    """Full sizes: oracle parity, linearity, and agreement with the grouped schedule."""
    torch = _torch()
    p = models.workload(name)
    plan = p.plan()
    rng = np.random.default_rng(11)
    n = plan.block_dim
    x, u = rng.standard_normal(n), rng.standard_normal(n)
    X = torch.from_numpy(np.stack([x, u, 2.0 * x - 3.0 * u])).cuda()
    Y = torch.empty_like(X)
    yg = torch.empty_like(X[0])
    plan.set_schedule(_abi.SCHED_GROUPED)
    plan.apply(X[0], yg)
    plan.set_schedule(_abi.SCHED_STACKED)
    for k in range(3):
        plan.apply(X[k], Y[k])
    torch.cuda.synchronize()
    Yh = Y.cpu().numpy()
    assert rel_err(Yh[2], 2.0 * Yh[0] - 3.0 * Yh[1]) < 1e-13
    assert rel_err(Yh[0], yg.cpu().numpy()) < 1e-13
    assert rel_err(Yh[0], oracle_bs(p).apply(x)) < TOL


def test_stacked_eigensolvers(lib_built):
    """Lanczos and Davidson on the stacked schedule reach the grouped schedule's eigenvalue."""
    _torch()
    p = small_problem("hubbard", 64)
    plan = p.plan()
    plan.set_schedule(_abi.SCHED_GROUPED)
    e_g = plan.lanczos(krylov_dim=40, max_restarts=20, tol=1e-11).eigenvalue
    plan.set_schedule(_abi.SCHED_STACKED)
    r = plan.lanczos(krylov_dim=40, max_restarts=20, tol=1e-11)
    assert abs(r.eigenvalue - e_g) < 1e-9 * max(1.0, abs(e_g))
    d = plan.davidson(max_subspace=40, max_iter=400, tol=1e-9)
    assert abs(d.eigenvalue - e_g) < 1e-8 * max(1.0, abs(e_g))
    # back to the grouped schedule: the cached Lanczos graph is rebuilt
    plan.set_schedule(_abi.SCHED_GROUPED)
    assert abs(plan.lanczos(krylov_dim=40, max_restarts=20, tol=1e-11).eigenvalue - e_g) < 1e-9 * max(1.0, abs(e_g))


def test_stacked_profile_and_switching(lib_built):
    torch = _torch()
    p = small_problem("cylinder", 96)
    plan = p.plan()
    x = torch.from_numpy(np.random.default_rng(2).standard_normal(plan.block_dim)).cuda()
    y1, y2, y3 = (torch.empty_like(x) for _ in range(3))
    plan.set_schedule(_abi.SCHED_GROUPED)
    plan.apply(x, y1)
    plan.set_schedule(_abi.SCHED_STACKED)
    ms, fl, by = plan.profile(x, y2, reps=2)
    assert all(m >= 0.0 for m in ms) and all(b > 0.0 for b in by)
    plan.set_schedule(_abi.SCHED_PER_BLOCK)
    plan.apply(x, y3)
    plan.set_schedule(_abi.SCHED_STACKED)  # the stacks are kept, not rebuilt
    plan.apply(x, y2)
    torch.cuda.synchronize()
    assert torch.equal(y1, y3)
    assert rel_err(y2.cpu().numpy(), y1.cpu().numpy()) < 1e-13


def test_stacked_complex_matches_grouped(lib_built):
    """Complex environments: the stacked schedule (the default of complex plans
    too) against the grouped one, and launches counted per schedule."""
    import torch

    from tk_gb300 import Heff2Plan, sweep

    p = small_problem("hubbard", 40)
    rng = np.random.default_rng(8)

    def cplx_env(e):
        im = rng.standard_normal(e.data.shape)
        return e.data + 0.3j * (im - np.transpose(im, (2, 1, 0)))

    dl = sweep.DeviceEnv.from_dense(p.kind, cplx_env(p.env_l), p.env_l.bra_idx, p.env_l.mpo_idx, p.env_l.ket_idx)
    dr = sweep.DeviceEnv.from_dense(p.kind, cplx_env(p.env_r), p.env_r.bra_idx, p.env_r.mpo_idx, p.env_r.ket_idx)
    plan = Heff2Plan.from_device_envs_complex(dl, dr, p.w_i, p.w_j, p.flux)
    assert plan.schedule == _abi.SCHED_STACKED
    n = plan.block_dim
    xr = torch.from_numpy(rng.standard_normal(n)).cuda()
    xi = torch.from_numpy(rng.standard_normal(n)).cuda()
    out = {}
    for sched in (_abi.SCHED_STACKED, _abi.SCHED_GROUPED):
        plan.set_schedule(sched)
        yr, yi = torch.full_like(xr, float("nan")), torch.full_like(xr, float("nan"))
        plan.apply_complex(xr, xi, yr, yi)
        torch.cuda.synchronize()
        out[sched] = yr.cpu().numpy() + 1j * yi.cpu().numpy()
        assert np.isfinite(out[sched]).all()
    a, b = out[_abi.SCHED_STACKED], out[_abi.SCHED_GROUPED]
    assert np.linalg.norm(a - b) < 1e-13 * np.linalg.norm(b)
    plan.set_schedule(_abi.SCHED_STACKED)
    assert plan.launches() <= 4
