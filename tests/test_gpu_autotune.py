"""The split-precision schedule options and the autotuner: every candidate
schedule (split copy for tall stage-1 stacks or not, the W_i W_j combine
fused into the stage-3 kernel or in one of its three separate forms) gives the same matvec to the split
tolerance (2e-4 relative against the FP64 oracle), and the autotuner keeps
the fastest timed candidate and caches it per sector-size histogram class."""
import numpy as np
import pytest

from helpers import models, oracle_bs, rel_err, small_problem
from tk_gb300 import PREC_BF16X3

pytestmark = pytest.mark.gpu
SPLIT_TOL = 2e-4
OPTIONS = [(3, 0, 0, 0), (3, 0, 1, 0), (3, 0, 2, 0), (3, 0, 3, 0), (3, 0, 0, 1), (3, 2, 0, 0), (1 << 30, 0, 1, 1), (1, 0, 0, 0),
           (1, 0, 2, 1), (3, 1, 1, 0), (1, 8, 0, 1)]


def _run(plan, x):
    import torch

    xd = torch.from_numpy(x).cuda()
    yd = torch.full_like(xd, float("nan"))
    plan.apply(xd, yd)
    torch.cuda.synchronize()
    return yd.cpu().numpy()


@pytest.mark.parametrize("name,D", [("cylinder", 512), ("hubbard", 256), ("heisenberg", 300)])
def test_every_schedule_matches_the_oracle(lib_built, name, D):
    p = small_problem(name, D)
    plan = p.plan(precision=PREC_BF16X3)
    x = np.random.default_rng(11).standard_normal(plan.block_dim)
    ref = oracle_bs(p).apply(x)
    ys = {}
    for tall, fuse, warps, pers in OPTIONS:
        plan.set_tc_options(tall, fuse, warps, pers)
        assert plan.tc_options() == {"tall_max_mtiles": tall, "fuse_max_ntiles": fuse, "combine_warps": warps,
                                     "stage1_persistent": pers}
        y = _run(plan, x)
        assert np.isfinite(y).all()
        assert rel_err(y, ref) < SPLIT_TOL, (tall, fuse, warps, pers)
        ys[(tall, fuse, warps, pers)] = y
    # the combine's four launch forms and both stage-1 kernels compute the same numbers, bit for bit
    assert np.array_equal(ys[(3, 0, 0, 0)], ys[(3, 0, 1, 0)])
    assert np.array_equal(ys[(3, 0, 0, 0)], ys[(3, 0, 2, 0)])
    assert np.array_equal(ys[(3, 0, 0, 0)], ys[(3, 0, 3, 0)])
    assert np.array_equal(ys[(3, 0, 0, 0)], ys[(3, 0, 0, 1)])


def test_fused_stage3_full_size(lib_built):
    """The fused combine + stage-3 kernel and the persistent-warp combine on the
    full Hubbard D=2048 workload."""
    p = models.workload("hubbard_d2048")
    plan = p.plan(precision=PREC_BF16X3)
    x = np.random.default_rng(3).standard_normal(plan.block_dim)
    ref = oracle_bs(p).apply(x)
    y0 = _run(plan, x)
    for opts in ((3, 2, 0, 0), (3, 0, 1, 0), (3, 0, 2, 0), (3, 0, 3, 0), (3, 0, 0, 1)):
        plan.set_tc_options(*opts)
        y = _run(plan, x)
        assert rel_err(y, ref) < SPLIT_TOL, opts
        if opts[1] == 0:
            assert np.array_equal(y, y0), opts  # every combine form writes the same T2


def test_autotune_keeps_the_fastest_and_caches(lib_built):
    p = small_problem("cylinder", 512)
    plan = p.plan(precision=PREC_BF16X3)
    r = plan.autotune(reps=3, use_cache=False)
    assert not r["from_cache"] and len(r["candidates"]) >= 2
    best = min(r["candidates"], key=lambda c: c["ms"])
    assert r["chosen"] == {k: best[k] for k in ("tall_max_mtiles", "fuse_max_ntiles", "combine_warps",
                                                "stage1_persistent")}
    assert plan.tc_options() == r["chosen"]
    # a second plan of the same histogram class takes the cached choice
    plan2 = p.plan(precision=PREC_BF16X3)
    r2 = plan2.autotune(reps=3, use_cache=True)
    assert r2["from_cache"] and r2["chosen"] == r["chosen"] and plan2.tc_options() == r["chosen"]
    # the tuned plan still solves (its cached graphs were rebuilt)
    x = np.random.default_rng(5).standard_normal(plan.block_dim)
    assert rel_err(_run(plan2, x), oracle_bs(p).apply(x)) < SPLIT_TOL
    e = plan2.lanczos(krylov_dim=30, max_restarts=30, tol=1e-8, refine=20)
    assert e.converged
