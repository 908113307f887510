"""Device Krylov exponential (tk_expm_krylov) against the reference's
exp_krylov_f64 known answers, the numpy restatement and scipy's expm, and
imaginary-time two-site TDVP sweeps against exact diagonalisation."""
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import ed_heisenberg, models, oracle_dense_literal, small_problem
from test_gpu_lanczos import matrix_plan
from tk_gb300 import PREC_FP64, sweep

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("case", KATS["exp_krylov"], ids=lambda c: c["source"].split("(")[-1][:-1])
def test_expm_kats(lib_built, case):
    M = np.diag(case["diag"]).astype(float) if case["matrix"] == "diag" else np.array(case["dense"], float)
    plan = matrix_plan(M)
    v = np.array(case["v"], float)
    out, _, used, _ = plan.expm(case["alpha"], _dev(v), krylov_dim=case["krylov"], tol=case["tol"])
    from scipy.linalg import expm

    assert np.allclose(out.cpu().numpy(), expm(case["alpha"] * M) @ v, atol=case["atol"], rtol=0)


def test_expm_follows_restatement_and_breakdown(lib_built):
    """Same result as the numpy exp_krylov_f64 with a truncated Krylov space; the
    breakdown cut on a 3-dimensional invariant space."""
    from oracle import krylov_exp

    rng = np.random.default_rng(9)
    A = rng.standard_normal((40, 40))
    M = (A + A.T) / 2
    plan = matrix_plan(M)
    v = rng.standard_normal(40)
    for k in (8, 20):
        out, _, used, mv = plan.expm(-0.2, _dev(v), krylov_dim=k, tol=1e-12)
        ref = krylov_exp.exp_krylov(lambda x: M @ x, v, -0.2, 40, k, 1e-12)
        assert used == k and mv == k
        assert np.allclose(out.cpu().numpy(), ref, atol=1e-10 * np.linalg.norm(ref), rtol=0)
    D = np.diag([1.0] * 10 + [2.0] * 10 + [5.0] * 20)
    out, _, used, _ = matrix_plan(D).expm(-0.1, _dev(np.ones(40)), krylov_dim=30, tol=1e-10)
    assert used == 3
    assert np.allclose(out.cpu().numpy(), np.exp(-0.1 * np.diag(D)), atol=1e-12, rtol=0)


@pytest.mark.parametrize("alpha,cplx", [(-0.3, False), (-0.7j, False), (-0.7j, True), (0.1 - 0.4j, True)])
def test_expm_heff_matches_scipy(lib_built, alpha, cplx):
    """exp(alpha H_eff) v on a two-site H_eff (all sectors), real and complex alpha and v."""
    from scipy.linalg import expm

    p = small_problem("heisenberg", 10)
    plan = p.plan(all_sectors=True)
    H = oracle_dense_literal(p)
    rng = np.random.default_rng(3)
    vr, vi = rng.standard_normal(H.shape[0]), rng.standard_normal(H.shape[0]) if cplx else None
    v = vr + (1j * vi if cplx else 0)
    ref = expm(alpha * H) @ v
    out_re, out_im, _, _ = plan.expm(alpha, _dev(plan.dense_to_flat(vr)),
                                     _dev(plan.dense_to_flat(vi)) if cplx else None, krylov_dim=40, tol=1e-12)
    got = plan.flat_to_dense(out_re.cpu().numpy()) + (1j * plan.flat_to_dense(out_im.cpu().numpy())
                                                       if out_im is not None else 0)
    assert np.linalg.norm(got - ref) < 1e-10 * np.linalg.norm(ref)


def test_imaginary_time_tdvp_reaches_ground_state(lib_built):
    """exp(-tau H) by two-site TDVP from a random MPS: the energy falls to exact diagonalisation."""
    m = models.heisenberg()
    sites, bonds = sweep.random_site_tensors(m, 10, 32, (0,), np.random.default_rng(3))
    d = sweep.DeviceDMRG(m, sites, bonds, precision=PREC_FP64, krylov=20)
    rec = sweep.SweepRecord()
    energies = [d.tdvp_step(1.5, 32, rec) for _ in range(30)]
    assert all(b <= a + 1e-9 for a, b in zip(energies[5:], energies[6:]))
    assert abs(energies[-1] - ed_heisenberg(10)) < 1e-8
