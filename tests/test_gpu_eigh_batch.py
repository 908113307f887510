"""Batched device eigensolver (tk_eigh_batched_f64) and the two-site
truncation that uses it, against numpy's eigh and a dense SVD."""
import numpy as np
import pytest

from test_host_truncation import _case, _dense, _rebuild
from tk_gb300.sweep import eigh_batch_device, split_two_site

pytestmark = pytest.mark.gpu


def test_eigh_batch_matches_numpy(lib_built):
    rng = np.random.default_rng(11)
    mats = []
    for n in (1, 3, 16, 17, 40, 64, 100):
        X = rng.standard_normal((n, n + 5))
        mats.append(X @ X.T)  # positive semi-definite, like the truncation's density matrices
    out = eigh_batch_device(mats)
    for G, (w, Z) in zip(mats, out):
        w_ref = np.linalg.eigvalsh(G)
        scale = max(1.0, float(np.abs(w_ref).max()))
        assert np.allclose(w, w_ref, atol=1e-12 * scale)
        assert np.allclose(Z.T @ Z, np.eye(len(w)), atol=1e-12)
        assert np.allclose(G @ Z, Z * w, atol=1e-11 * scale)


def test_split_with_device_eigh_matches_host(lib_built):
    kind, P, QA, QB, keys, offs, qs, psi = _case()
    T = _dense(kind, psi, keys, offs, qs, P, QA, QB)
    for to_right in (True, False):
        for max_bond in (10_000, 9):
            host = split_two_site(kind, psi, keys, offs, [P, P, QA, QB], max_bond, 0.0, to_right)
            dev = split_two_site(kind, psi, keys, offs, [P, P, QA, QB], max_bond, 0.0, to_right,
                                 eigh_batch=eigh_batch_device)
            assert dev[2] == host[2]  # same kept bond charges and dimensions
            assert abs(dev[3] - host[3]) < 1e-13
            A, B = _rebuild(dev[0], dev[1], dev[2], P, QA, QB)
            Ah, Bh = _rebuild(host[0], host[1], host[2], P, QA, QB)
            # the kept two-site state is gauge-invariant
            assert np.allclose(np.einsum("sab,tbc->stac", A, B), np.einsum("sab,tbc->stac", Ah, Bh), atol=1e-12)
            if max_bond == 10_000:
                assert np.allclose(np.einsum("sab,tbc->stac", A, B), T, atol=1e-12)
