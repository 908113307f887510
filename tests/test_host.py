"""Host-side mirror: model MPOs, synthetic workloads, table invariants (no GPU)."""
import numpy as np

from helpers import models
from tk_gb300 import symmetry as sym


def test_qindex_sorts_and_rejects_duplicates():
    ix = sym.QIndex(sym.U1, [((1,), 4), ((-1,), 2), ((0,), 3)])
    assert [q for q, _ in ix.sectors] == [(-1,), (0,), (1,)]
    try:
        sym.QIndex(sym.U1, [((0,), 1), ((0,), 2)])
        raise AssertionError("duplicate sectors accepted")
    except ValueError:
        pass


def test_mpo_adjoint_symmetry():
    for m in (models.heisenberg(), models.hubbard(), models.cylinder_j1(4)):
        W = m.bulk.to_dense()
        pi = m.pi
        Wt = W.transpose(1, 0, 2, 3)[:, :, pi][:, :, :, pi]
        assert np.array_equal(W, Wt)
        assert m.bond.total_dim == W.shape[2]


def test_mpo_bond_dims():
    assert models.heisenberg().bond.total_dim == 5
    assert models.hubbard().bond.total_dim == 6
    assert models.cylinder_j1(4).bond.total_dim == 14


def test_workload_bonds():
    b = models.gaussian_bond_u1(1024, 15, 3.0)
    assert b.total_dim == 1024 and b.n_sectors == 15
    h = models.gaussian_bond_u1u1(2048, 30)
    assert h.total_dim == 2048
    for (n, s), _ in h.sectors:
        assert (n - 30 - s) % 2 == 0
    rng = np.random.default_rng(0)
    c = models.heavy_tailed_bond_u1(4096, 41, rng)
    dims = sorted((d for _, d in c.sectors), reverse=True)
    assert c.total_dim == 4096 and dims[0] > 500 and sum(d < 16 for d in dims) >= 8


def test_flatten_layout_is_key_sorted():
    t = models.hubbard().bulk
    keys, offs, data = t.flatten()
    assert np.all(np.diff(keys.astype(np.float64)) > 0)
    assert offs[0] == 0 and data.size == sum(b.size for b in t.blocks.values())


def _mpo_dense(mpo):
    """Contract an open-boundary MPO into its dense operator (site 0 most significant)."""
    Ws = [t.to_dense() for t in mpo.tensors]
    M = Ws[0][:, :, 0, :]  # (s_in, s_out, w)
    for W in Ws[1:]:
        M = np.einsum("abw,cdwv->acbdv", M, W).reshape(M.shape[0] * W.shape[0], M.shape[1] * W.shape[1], -1)
    return M[:, :, 0].T  # H[out, in]


def test_fermion_chain_mpo_matches_jordan_wigner():
    """models.fermion_chain contracted to a dense operator == the Jordan-Wigner H of the
    same couplings, and the uniform case is models.hubbard."""
    from helpers import fermion_chain_dense
    from tk_gb300 import models

    hop, U, eps = [0.4, -0.7], [3.0, 0.5, 0.0], [-1.5, 0.2, -0.1]
    H, _ = fermion_chain_dense(hop, U, eps)
    assert np.allclose(_mpo_dense(models.fermion_chain(hop, U, eps).chain(3)), H, atol=1e-12)
    uni = models.fermion_chain([-1.0, -1.0, -1.0], [4.0] * 4, [0.0] * 4).chain(4)
    ref = models.hubbard(1.0, 4.0).chain(4)
    assert np.allclose(_mpo_dense(uni), _mpo_dense(ref), atol=1e-12)
