"""The oracle's three matvec forms agree, and exact environments reproduce
exact diagonalisation (physics known answers for the H_eff conventions)."""
import numpy as np
import pytest

from helpers import (ed_heisenberg, ed_hubbard, exact_problem, models, oracle_bs, oracle_dense_factored,
                     oracle_dense_literal, rel_err, small_problem)


@pytest.mark.parametrize("name,D", [("heisenberg", 12), ("hubbard", 10), ("cylinder", 16)])
def test_literal_factored_blocksparse_agree(name, D):
    p = small_problem(name, D)
    H = oracle_dense_literal(p)
    assert np.abs(H - H.T).max() == 0.0  # synthetic environments are symmetrised
    rng = np.random.default_rng(1)
    x = rng.standard_normal(H.shape[0])
    y = H @ x
    assert rel_err(oracle_dense_factored(p, x), y) < 1e-13
    bs = oracle_bs(p, all_sectors=True)
    assert rel_err(bs.to_dense(bs.apply(bs.from_dense(x))), y) < 1e-13
    bsf = oracle_bs(p)
    xf = rng.standard_normal(bsf.total)
    assert rel_err(bsf.to_dense(bsf.apply(xf)), H @ bsf.to_dense(xf)) < 1e-13


def _lowest(bs):
    n = bs.total
    H = np.column_stack([bs.apply(np.eye(n)[:, k]) for k in range(n)])
    return np.linalg.eigvalsh(0.5 * (H + H.T))[0]


@pytest.mark.parametrize("n,i", [(6, 0), (6, 2), (8, 3)])
def test_exact_heisenberg_matches_ed(n, i):
    p = exact_problem(models.heisenberg(), n, i, (0,))
    assert abs(_lowest(oracle_bs(p)) - ed_heisenberg(n)) < 1e-10


def test_exact_hubbard_matches_ed():
    p = exact_problem(models.hubbard(), 4, 1, (4, 0))
    assert abs(_lowest(oracle_bs(p)) - ed_hubbard(4)) < 1e-10


def test_two_site_hubbard_textbook():
    # half-filled Hubbard dimer: E0 = (U - sqrt(U^2 + 16 t^2)) / 2
    assert abs(ed_hubbard(2, N=2) - (4 - np.sqrt(32)) / 2) < 1e-12
    p = exact_problem(models.hubbard(), 2, 0, (2, 0))
    assert abs(_lowest(oracle_bs(p)) - (4 - np.sqrt(32)) / 2) < 1e-12


def test_two_site_heisenberg_spectrum():
    # two spins: singlet -3/4, triplet +1/4 (all Sz sectors)
    p = exact_problem(models.heisenberg(), 2, 0, (0,))
    H = oracle_dense_literal(p)
    assert np.allclose(np.linalg.eigvalsh(H), [-0.75, 0.25, 0.25, 0.25])


def test_blocksparse_large_sectors():
    """Sectors taller than the restatement's 64-row task ranges and deeper than
    its 256-wide k panels, with dimensions that are not multiples of its 4 x 4
    register tiles (67, 301, 70), against a dense contraction in numpy:
    y[t,v,p,q] = sum L[p,w,a] W_i[s,t,w,m] W_j[u,v,m,r] R[q,r,b] x[s,u,a,b]
    (environments/mod.rs:540-578)."""
    from tk_gb300.symmetry import QIndex

    m = models.heisenberg()
    b = QIndex(m.kind, [((-2,), 67), ((0,), 301), ((2,), 70)])
    p = models.two_site_problem(m, b, b, 11, "heisenberg")
    bs = oracle_bs(p)
    x = np.random.default_rng(3).standard_normal(bs.total)
    D = b.total_dim
    xd = bs.to_dense(x).reshape(2, 2, D, D)
    Wi, Wj = p.w_i.to_dense(), p.w_j.to_dense()
    T = np.tensordot(xd, p.env_r.data, axes=([3], [2]))       # s u a q r
    T = np.tensordot(p.env_l.data, T, axes=([2], [2]))        # p w s u q r
    W2 = np.einsum("stwm,uvmr->suwrtv", Wi, Wj)
    y = np.tensordot(T, W2, axes=([2, 3, 1, 5], [0, 1, 2, 3]))  # p q t v
    assert rel_err(bs.to_dense(bs.apply(x)), y.transpose(2, 3, 0, 1).reshape(-1)) < 1e-13
