"""The split-precision schedule options and the autotuner: every candidate
schedule (split copy for tall stage-1 stacks or not, the W_i W_j combine
fused into the stage-3 kernel or in one of its three separate forms, stage 1
in 64- or 32-wide K chunks) gives the same matvec to the split
tolerance (2e-4 relative against the FP64 oracle), and the autotuner keeps
the fastest timed candidate and caches it per sector-size histogram class."""
import numpy as np
import pytest

from helpers import models, oracle_bs, rel_err, small_problem
from tk_gb300 import PREC_BF16X3

pytestmark = pytest.mark.gpu
SPLIT_TOL = 2e-4
OPTIONS = [(3, 0, 0, 0, 0), (3, 0, 1, 0, 0), (3, 0, 2, 0, 0), (3, 0, 3, 0, 0), (3, 0, 0, 1, 0), (3, 2, 0, 0, 0),
           (1 << 30, 0, 1, 1, 0), (1, 0, 0, 0, 0), (1, 0, 2, 1, 0), (3, 1, 1, 0, 0), (1, 8, 0, 1, 0), (3, 0, 0, 0, 1),
           (3, 0, 3, 0, 1), (1 << 30, 0, 0, 0, 1), (3, 2, 0, 0, 1)]
KEYS = ("tall_max_mtiles", "fuse_max_ntiles", "combine_warps", "stage1_persistent", "stage1_narrow")


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
    for opts in OPTIONS:
        plan.set_tc_options(*opts)
        assert plan.tc_options() == dict(zip(KEYS, opts))
        y = _run(plan, x)
        assert np.isfinite(y).all()
        assert rel_err(y, ref) < SPLIT_TOL, opts
        ys[opts] = y
    # the combine's four launch forms and the three stage-1 kernels (64- and
    # 32-wide K chunks, persistent) compute the same numbers, bit for bit
    base = ys[(3, 0, 0, 0, 0)]
    for opts in ((3, 0, 1, 0, 0), (3, 0, 2, 0, 0), (3, 0, 3, 0, 0), (3, 0, 0, 1, 0), (3, 0, 0, 0, 1), (3, 0, 3, 0, 1)):
        assert np.array_equal(base, ys[opts]), opts
    assert np.array_equal(ys[(1 << 30, 0, 0, 0, 1)], ys[(1 << 30, 0, 1, 1, 0)])
    assert np.array_equal(ys[(3, 2, 0, 0, 1)], ys[(3, 2, 0, 0, 0)])


def test_fused_stage3_full_size(lib_built):
    """The fused combine + stage-3 kernel and the persistent-warp combine on the
    full Hubbard D=2048 workload."""
    p = models.workload("hubbard_d2048")
    plan = p.plan(precision=PREC_BF16X3)
    x = np.random.default_rng(3).standard_normal(plan.block_dim)
    ref = oracle_bs(p).apply(x)
    y0 = _run(plan, x)
    for opts in ((3, 2, 0, 0, 0), (3, 0, 1, 0, 0), (3, 0, 2, 0, 0), (3, 0, 3, 0, 0), (3, 0, 0, 1, 0), (3, 0, 0, 0, 1),
                 (3, 0, 3, 0, 1)):
        plan.set_tc_options(*opts)
        y = _run(plan, x)
        assert rel_err(y, ref) < SPLIT_TOL, opts
        if opts[1] == 0:
            assert np.array_equal(y, y0), opts  # every combine form and stage-1 kernel writes the same bits
    # the host-buffer path with psi in pieces runs the narrow stage 1 per piece
    plan.set_tc_options(3, 0, 0, 0, 1)
    for pieces in (1, 2, 8):
        plan.set_psi_pieces(pieces)
        yh = np.zeros_like(x)
        plan.apply_host_flat(x, yh)
        assert np.array_equal(yh, y0), pieces


def test_autotune_keeps_the_fastest_and_caches(lib_built):
    p = small_problem("cylinder", 512)
    plan = p.plan(precision=PREC_BF16X3)
    r = plan.autotune(reps=3, use_cache=False)
    assert not r["from_cache"] and len(r["candidates"]) >= 2
    best = min(r["candidates"], key=lambda c: c["ms"])
    assert r["chosen"] == {k: best[k] for k in KEYS}
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
