"""GPU parity of the two-site H_eff (FP64) against the CPU oracle, through the C ABI."""
import ctypes as C

import numpy as np
import pytest

import oracle
from helpers import (exact_problem, models, oracle_bs, oracle_dense_literal, rel_err, small_problem)
from tk_gb300 import PREC_FP64, TkError, _abi
from tk_gb300.heff import Heff2Plan, build_heff_two_site

pytestmark = pytest.mark.gpu
TOL = 1e-12  # FP64 path vs the FP64 oracle, relative 2-norm


def _torch():
    import torch

    assert torch.cuda.is_available()
    return torch


def _oracle_keys(prob, bs):
    """Packed keys of the oracle's block list (its own enumerate + sort)."""
    sec, off = bs.blocks()
    legs = [prob.w_i.indices[0], prob.w_j.indices[0], prob.env_l.ket_idx, prob.env_r.ket_idx]
    keys = [oracle.key_pack(prob.kind, [legs[l].sectors[s[l]][0] for l in range(4)]) for s in sec]
    return np.array(keys, dtype=np.uint64), off


@pytest.mark.parametrize("name,D", [("heisenberg", 40), ("hubbard", 48), ("cylinder", 64)])
def test_block_layout_bit_exact(lib_built, name, D):
    p = small_problem(name, D)
    plan = p.plan()
    bs = oracle_bs(p)
    keys, offs = plan.blocks()
    okeys, ooffs = _oracle_keys(p, bs)
    assert np.array_equal(keys, okeys)
    assert np.array_equal(offs, ooffs)
    assert plan.block_dim == bs.total


@pytest.mark.parametrize("name,D", [("heisenberg", 12), ("hubbard", 10), ("cylinder", 16)])
def test_closure_matches_literal_dense(lib_built, name, D):
    """build_heff_two_site closure on dense host vectors == the reference's dense H."""
    p = small_problem(name, D)
    H = oracle_dense_literal(p)
    mpo = models.MPO([p.w_i, p.w_j], [p.w_i.indices[0].total_dim] * 2, p.flux)
    matvec, dim = build_heff_two_site(p.env_l, p.env_r, mpo, (0, 1))  # all sectors, like the reference
    assert dim == H.shape[0]
    rng = np.random.default_rng(3)
    for _ in range(3):
        x = rng.standard_normal(dim)
        y = np.zeros(dim)
        matvec(x, y)
        assert rel_err(y, H @ x) < TOL


@pytest.mark.parametrize("name,D", [("heisenberg", 96), ("hubbard", 96), ("cylinder", 128)])
def test_device_apply_matches_oracle(lib_built, name, D):
    torch = _torch()
    p = small_problem(name, D)
    plan = p.plan()
    bs = oracle_bs(p)
    rng = np.random.default_rng(5)
    x = rng.standard_normal(plan.block_dim)
    xd = torch.from_numpy(x).cuda()
    yd = torch.full_like(xd, float("nan"))  # output must be fully overwritten
    plan.apply(xd, yd)
    torch.cuda.synchronize()
    assert rel_err(yd.cpu().numpy(), bs.apply(x)) < TOL
    # host flat path gives the same numbers
    y2 = np.zeros_like(x)
    plan.apply_host_flat(x, y2)
    assert np.array_equal(y2, yd.cpu().numpy())


# cylinder_d4096: 41 heavy-tailed sectors up to 1535 (the uneven-block stress case)
@pytest.mark.parametrize("name", ["heisenberg_d1024", "hubbard_d2048", "cylinder_d4096"])
def test_full_size_against_oracle(lib_built, name):
    """Full workload sizes: parity with the block-sparse oracle + symmetry and linearity."""
    torch = _torch()
    p = models.workload(name)
    plan = p.plan()
    rng = np.random.default_rng(11)
    n = plan.block_dim
    x = rng.standard_normal(n)
    u = rng.standard_normal(n)
    X = torch.from_numpy(np.stack([x, u, 2.0 * x - 3.0 * u])).cuda()
    Y = torch.empty_like(X)
    for k in range(3):
        plan.apply(X[k], Y[k])
    torch.cuda.synchronize()
    Yh = Y.cpu().numpy()
    assert rel_err(Yh[2], 2.0 * Yh[0] - 3.0 * Yh[1]) < 1e-13      # linearity
    assert abs(u @ Yh[0] - x @ Yh[1]) < 1e-11 * np.linalg.norm(Yh[0]) * np.linalg.norm(u)  # symmetry
    bs = oracle_bs(p)
    assert bs.total == n
    assert rel_err(Yh[0], bs.apply(x)) < TOL


def test_exact_environments_ground_energy(lib_built):
    """Device Lanczos on exact environments reproduces exact diagonalisation."""
    from helpers import ed_heisenberg

    p = exact_problem(models.heisenberg(), 8, 3, (0,))
    plan = p.plan()
    r = plan.lanczos(krylov_dim=60, max_restarts=3, tol=1e-9)
    assert abs(r.eigenvalue - ed_heisenberg(8)) < 1e-9
    assert r.residual_norm < 1e-8


def test_empty_and_tiny(lib_built):
    """Boundary environments (1x1x1) and a single-sector bond."""
    p = exact_problem(models.heisenberg(), 2, 0, (0,))
    H = oracle_dense_literal(p)
    x = np.random.default_rng(0).standard_normal(H.shape[0])
    # all sectors: the reference's dense closure exactly
    plan_all = p.plan(all_sectors=True)
    assert plan_all.block_dim == 4
    y = np.zeros_like(x)
    plan_all.apply_host(x, y)
    assert rel_err(y, H @ x) < TOL
    # flux 0: the Sz = 0 sector |up,down>, |down,up> only (projected closure)
    plan = p.plan()
    assert plan.block_dim == 2
    sel = plan.flat_to_dense(np.ones(2)) != 0
    xs = np.where(sel, x, 0.0)
    plan.apply_host(x, y)
    assert rel_err(y, np.where(sel, H @ xs, 0.0)) < TOL


def test_sector_mismatch_reported(lib_built):
    p = small_problem("heisenberg", 12)
    q = small_problem("heisenberg", 14)
    env_r_bad = models.Environment(q.env_r.data, q.env_r.bra_idx, q.env_r.mpo_idx, q.env_r.ket_idx)
    wrong_w = models.hubbard().bulk
    with pytest.raises(TkError) as e:
        Heff2Plan(p.env_l, p.env_r, wrong_w, p.w_j)
    assert e.value.status in (1, 2)
    # bra/ket QIndex disagreement
    bad = models.Environment(np.zeros((12, 5, 12)), p.env_l.bra_idx, p.env_l.mpo_idx, p.env_l.ket_idx)
    bad.bra_idx = q.env_l.bra_idx
    with pytest.raises(TkError):
        Heff2Plan(bad, env_r_bad, p.w_i, p.w_j)


def test_per_block_schedule_matches_grouped(lib_built):
    """One launch per output block gives the same numbers as the grouped launch."""
    import torch
    from tk_gb300 import _abi

    p = small_problem("cylinder", 96)
    plan = p.plan()
    assert plan.schedule == _abi.SCHED_STACKED  # the default of real plans
    plan.set_schedule(_abi.SCHED_GROUPED)
    x = torch.from_numpy(np.random.default_rng(8).standard_normal(plan.block_dim)).cuda()
    y1, y2 = torch.empty_like(x), torch.empty_like(x)
    plan.apply(x, y1)
    plan.set_schedule(_abi.SCHED_PER_BLOCK)
    plan.apply(x, y2)
    torch.cuda.synchronize()
    assert torch.equal(y1, y2)
