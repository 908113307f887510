"""Device Lanczos against the reference's eigensolver known answers.

A dense symmetric M is embedded as H_eff = L (trivial physical legs, one
channel, R = [1]) so that the device solver runs on exactly M."""
import json
from pathlib import Path

import numpy as np
import pytest

from tk_gb300.heff import Environment, Heff2Plan
from tk_gb300.models import site_tensor
from tk_gb300.symmetry import U1, QIndex

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def matrix_plan(M: np.ndarray) -> Heff2Plan:
    n = M.shape[0]
    bond = QIndex(U1, [((0,), n)])
    one = QIndex(U1, [((0,), 1)])
    phys = QIndex(U1, [((0,), 1)])
    W, _, _ = site_tensor(U1, phys, [(0,)], [(0,)], [(0, 0, np.eye(1))])
    L = Environment(M.reshape(n, 1, n), bond, one, bond)
    R = Environment(np.ones((1, 1, 1)), one, one, one)
    return Heff2Plan(L, R, W, W, psi_flux=(0,))


@pytest.mark.parametrize("case", KATS["lanczos"], ids=lambda c: c["source"].split(":")[-1])
def test_lanczos_kats(lib_built, case):
    M = np.diag(np.array(case["diag"], float)) if case["matrix"] == "diag" else np.array(case["dense"], float)
    plan = matrix_plan(M)
    r = plan.lanczos(krylov_dim=case["krylov"], tol=1e-10)
    assert abs(r.eigenvalue - case["eigenvalue"]) < case["tol"]


def test_lanczos_random_diagonals(lib_built):
    rd = KATS["lanczos_random_diagonal"]
    for case in rd["cases"]:
        plan = matrix_plan(np.diag(case["diag"]))
        r = plan.lanczos(krylov_dim=100, tol=1e-10)
        assert abs(r.eigenvalue - case["eigenvalue"]) < rd["tol"], case


def test_lanczos_matches_restatement_and_eigenvector(lib_built):
    """Same Krylov sequence as the numpy restatement; the Ritz vector is a true eigenvector."""
    import torch
    from oracle import lanczos

    rng = np.random.default_rng(2)
    A = rng.standard_normal((40, 40))
    M = A + A.T
    plan = matrix_plan(M)
    r = plan.lanczos(krylov_dim=40, tol=1e-9)
    lam, x, _ = lanczos.lowest_eigenpair(lambda v: M @ v, 40, 40)
    assert abs(r.eigenvalue - lam) < 1e-9
    assert abs(r.eigenvalue - np.linalg.eigvalsh(M)[0]) < 1e-9
    v = r.eigenvector.cpu().numpy()
    assert np.linalg.norm(M @ v - r.eigenvalue * v) < 1e-8
    assert r.residual_norm < 1e-8
    torch.cuda.synchronize()


def test_lanczos_restart_and_graph_reuse(lib_built):
    rng = np.random.default_rng(4)
    d = np.sort(rng.uniform(-5, 5, 300))
    plan = matrix_plan(np.diag(d))
    r1 = plan.lanczos(krylov_dim=30, max_restarts=20, tol=1e-8)
    r2 = plan.lanczos(krylov_dim=30, max_restarts=20, tol=1e-8)  # cached graph
    assert abs(r1.eigenvalue - d[0]) < 1e-8 and abs(r2.eigenvalue - r1.eigenvalue) < 1e-12
    assert r1.restarts >= 1 and r1.converged
