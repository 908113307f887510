"""Device Davidson (tk_davidson_lowest) against the reference's Davidson known
answers, the numpy restatement of DavidsonSolver, and the FP64 Lanczos."""
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import oracle_bs, oracle_dense_literal, small_problem
from test_gpu_lanczos import matrix_plan
from tk_gb300 import PREC_BF16X3, PREC_FP64, DavidsonSolver

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


def test_davidson_defaults_match_reference():
    d = DavidsonSolver()
    case = KATS["davidson"][0]
    assert (d.max_subspace, d.tol, d.max_iter, d.restart_vectors, d.diagonal) == (case["max_subspace"], case["tol"],
                                                                                 1000, 5, None)


@pytest.mark.parametrize("case", [c for c in KATS["davidson"] if not c.get("defaults")],
                         ids=lambda c: c["source"].split(":")[-1])
def test_davidson_kats(lib_built, case):
    M = np.diag(np.array(case["diag"], float)) if case["matrix"] == "diag" else np.array(case["dense"], float)
    plan = matrix_plan(M)
    diag = _dev(case["diagonal"]) if case["diagonal"] is not None else None
    r = plan.davidson(tol=case["tol"], diagonal=diag)
    assert abs(r.eigenvalue - case["eigenvalue"]) < case["atol"]
    if case["converged"]:
        assert r.converged and r.residual_norm < case["tol"]


@pytest.mark.parametrize("max_subspace", [60, 6])
def test_davidson_follows_restatement(lib_built, max_subspace):
    """Same iterates as the numpy DavidsonSolver: eigenvalue, matvec count, eigenvector."""
    from oracle import davidson

    rng = np.random.default_rng(2)
    A = rng.standard_normal((48, 48))
    M = A + A.T
    plan = matrix_plan(M)
    r = plan.davidson(max_subspace=max_subspace, tol=1e-9)
    lam, x, conv, count, rn = davidson.lowest_eigenpair(lambda v: M @ v, 48, max_subspace=max_subspace, tol=1e-9)
    assert r.converged and conv
    assert abs(r.eigenvalue - lam) < 1e-10
    assert abs(r.eigenvalue - np.linalg.eigvalsh(M)[0]) < 1e-9
    assert abs(r.matvec_count - count) <= 1
    v = r.eigenvector.cpu().numpy()
    assert abs(abs(v @ x) - 1.0) < 1e-9


def test_davidson_preconditioned_heff(lib_built):
    """Diagonal preconditioner on a two-site H_eff, against the restatement on the oracle matvec."""
    from oracle import davidson

    p = small_problem("heisenberg", 16)
    plan = p.plan(all_sectors=True)
    H = oracle_dense_literal(p)
    diag = plan.dense_to_flat(np.diag(H).copy())
    assert plan.block_dim == H.shape[0]
    r = plan.davidson(tol=1e-9, diagonal=_dev(diag))
    bs = oracle_bs(p, all_sectors=True)
    lam, _, conv, count, _ = davidson.lowest_eigenpair(bs.apply, bs.total, tol=1e-9, diagonal=diag)
    assert r.converged and conv
    assert abs(r.eigenvalue - lam) < 1e-9
    assert abs(r.eigenvalue - np.linalg.eigvalsh(H)[0]) < 1e-9


@pytest.mark.parametrize("name,D", [("heisenberg", 64), ("hubbard", 64)])
def test_davidson_matches_lanczos_on_heff(lib_built, name, D):
    p = small_problem(name, D)
    plan = p.plan(precision=PREC_FP64)
    r = plan.davidson(tol=1e-9)
    r64 = plan.lanczos(krylov_dim=40, max_restarts=30, tol=1e-10)
    assert r.converged and r64.converged
    assert abs(r.eigenvalue - r64.eigenvalue) < 1e-9
    assert r.fp64_matvec_count == r.matvec_count


def test_split_jacobi_davidson_matches_fp64(lib_built):
    """Split-precision plan, corrections from split-precision CG: FP64 energy, fewer FP64 matvecs."""
    p = small_problem("hubbard", 64)
    r64 = p.plan(precision=PREC_FP64).davidson(tol=1e-9)
    plan = p.plan(precision=PREC_BF16X3)
    r = plan.davidson(tol=1e-9, inner=12)
    assert r.converged and r.residual_norm < 1e-9
    assert abs(r.eigenvalue - r64.eigenvalue) < 1e-10
    assert r.fp64_matvec_count < r64.fp64_matvec_count
    # inner = 0 on a split plan is the reference's Davidson in FP64
    r0 = plan.davidson(tol=1e-9, inner=0)
    assert r0.matvec_count == r0.fp64_matvec_count
    assert abs(r0.eigenvalue - r64.eigenvalue) < 1e-10
