"""Edge cases of the two-site matvec on the device: an empty two-site space (a
flux that no sector combination reaches), the smallest spaces (boundary
environments of dimension one), and bonds whose sectors all have dimension
one, in both precisions and in each stage-1 and combine form of the split
path."""
import numpy as np
import pytest

from helpers import exact_problem, models, oracle_bs, oracle_dense_literal, rel_err, small_problem
from tk_gb300 import PREC_BF16X3, PREC_FP64, TkError, _abi

pytestmark = pytest.mark.gpu
TOL = 1e-12  # FP64 against the FP64 oracle, relative 2-norm
SPLIT_TOL = 2e-4  # bf16x3 against the FP64 oracle
# (tall_max_mtiles, fuse_max_ntiles, combine_warps, stage1_persistent, stage1_narrow)
FORMS = [(3, 0, 0, 0, 0), (3, 0, 0, 0, 1), (3, 0, 3, 0, 1), (3, 0, 0, 1, 0), (3, 0, 2, 0, 0)]


def _dev(x):
    import torch

    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def test_empty_space(lib_built):
    """No valid sector: every matvec entry point returns without a launch and
    the eigensolvers refuse the empty space with TK_ERR_INVALID_ARG."""
    p = small_problem("heisenberg", 12)
    p.flux = (40,)
    for prec in (PREC_FP64, PREC_BF16X3):
        plan = p.plan(precision=prec)
        assert plan.block_dim == 0
        x, y = _dev(np.zeros(0)), _dev(np.zeros(0))
        plan.apply(x, y)
        plan.apply_host_flat(np.zeros(0), np.zeros(0))
        with pytest.raises(TkError) as e:
            plan.lanczos(krylov_dim=10, max_restarts=1, tol=1e-9)
        assert _abi.STATUS_NAMES[e.value.status] == "INVALID_ARG"


def test_smallest_space_split(lib_built):
    """Two sites with boundary environments (1 x 1 x 1): the split path's
    operand stacks are a few rows tall with K = 1, far inside one TMA box."""
    p = exact_problem(models.heisenberg(), 2, 0, (0,))
    H = oracle_dense_literal(p)
    x = np.random.default_rng(0).standard_normal(H.shape[0])
    plan = p.plan(precision=PREC_BF16X3)
    assert plan.block_dim == 2
    sel = plan.flat_to_dense(np.ones(2)) != 0
    ref = np.where(sel, H @ np.where(sel, x, 0.0), 0.0)
    ys = []
    for opts in FORMS:
        plan.set_tc_options(*opts)
        y = np.zeros_like(x)
        plan.apply_host(x, y)
        assert rel_err(y, ref) < SPLIT_TOL, opts
        ys.append(y)
    assert all(np.array_equal(ys[0], y) for y in ys[1:])


def _unit_problem(name):
    if name == "heisenberg":
        b = models.gaussian_bond_u1(5, 5, 100.0)
        return b, b, models.two_site_problem(models.heisenberg(), b, b, 3, name)
    bl = models.gaussian_bond_u1u1(5, 6, 50.0, 50.0, 1)
    br = models.gaussian_bond_u1u1(5, 8, 50.0, 50.0, 1)
    return bl, br, models.two_site_problem(models.hubbard(), bl, br, 3, name)


@pytest.mark.parametrize("name", ["heisenberg", "hubbard"])
def test_sectors_of_dimension_one(lib_built, name):
    """Every bond sector of dimension one: K = 1 for every stage-1 stack and
    one-column ψ blocks, through every FP64 schedule and split form."""
    import torch

    bl, br, p = _unit_problem(name)
    assert all(d == 1 for _, d in bl.sectors) and all(d == 1 for _, d in br.sectors)
    bs = oracle_bs(p)
    plan = p.plan()
    assert plan.block_dim > 0
    x = np.random.default_rng(4).standard_normal(plan.block_dim)
    ref = bs.apply(x)
    xd = _dev(x)
    for sched in (_abi.SCHED_STACKED, _abi.SCHED_GROUPED, _abi.SCHED_PER_BLOCK):
        plan.set_schedule(sched)
        yd = torch.full_like(xd, float("nan"))
        plan.apply(xd, yd)
        torch.cuda.synchronize()
        assert rel_err(yd.cpu().numpy(), ref) < TOL, sched
    plan.set_precision(PREC_BF16X3)
    ys = []
    for opts in FORMS:
        plan.set_tc_options(*opts)
        yd = torch.full_like(xd, float("nan"))
        plan.apply(xd, yd)
        torch.cuda.synchronize()
        y = yd.cpu().numpy()
        assert np.isfinite(y).all() and rel_err(y, ref) < SPLIT_TOL, opts
        ys.append(y)
    assert all(np.array_equal(ys[0], y) for y in ys[1:])
