"""The two-site truncation on the device data path (split_two_site_device:
M_q gathered on the GPU, an SVD per bond charge on the host, the factors
scattered into the new site tensors on the GPU) against dense SVDs, the
reference's truncate_svd known answers (tk-dmrg/src/truncation/mod.rs:185-236)
and the host density-matrix split.  Tolerances: reconstructions and
isometries to 1e-12 (FP64), kept dimensions and discarded counts exact."""
import json
from pathlib import Path

import numpy as np
import pytest

from test_host_truncation import _case, _dense, _layout
from tk_gb300.sweep import split_two_site, split_two_site_device
from tk_gb300.symmetry import QIndex

pytestmark = pytest.mark.gpu


def _dev(psi):
    import torch

    return torch.from_numpy(np.ascontiguousarray(psi)).cuda()


def _product(Ai, Aj):
    return np.einsum("sab,tbc->stac", Ai.to_dense(), Aj.to_dense())


def test_full_rank_reconstructs_and_is_isometric(lib_built):
    kind, P, QA, QB, keys, offs, qs, psi = _case()
    T = _dense(kind, psi, keys, offs, qs, P, QA, QB)
    for to_right in (True, False):
        Ai, Aj, nb, disc = split_two_site_device(kind, _dev(psi), keys, offs, [P, P, QA, QB], 10_000, 0.0, to_right)
        assert disc < 1e-24
        assert np.allclose(_product(Ai, Aj), T, atol=1e-12)
        A, B = Ai.to_dense(), Aj.to_dense()
        if to_right:
            assert np.allclose(np.einsum("sab,sac->bc", A, A), np.eye(nb.total_dim), atol=1e-12)
        else:
            assert np.allclose(np.einsum("sab,scb->ac", B, B), np.eye(nb.total_dim), atol=1e-12)


def test_truncation_rule_and_weight(lib_built):
    kind, P, QA, QB, keys, offs, qs, psi = _case()
    T = _dense(kind, psi, keys, offs, qs, P, QA, QB)
    d = P.total_dim
    M = T.transpose(0, 2, 1, 3).reshape(d * QA.total_dim, d * QB.total_dim)
    sv = np.sort(np.linalg.svd(M, compute_uv=False))[::-1]
    for cutoff, max_bond in ((0.5, 100), (0.2, 5), (2.0, 100), (0.0, 9)):
        want = max(1, min(max_bond, int(np.sum(sv >= cutoff * sv[0]))))
        for to_right in (True, False):
            Ai, Aj, nb, disc = split_two_site_device(kind, _dev(3.0 * psi), keys, offs, [P, P, QA, QB], max_bond,
                                                     cutoff, to_right)
            assert nb.total_dim == want, (cutoff, max_bond)
            assert abs(disc - np.sum(sv[want:] ** 2) / np.sum(sv ** 2)) < 1e-12
            # the kept state is the normalised best rank-`want` approximation of 3T:
            # its overlap with 3T is the norm of the kept part, 3 sqrt(sum sigma^2)
            overlap = float(np.sum(_product(Ai, Aj) * 3.0 * T))
            assert abs(overlap - 3.0 * np.sqrt(np.sum(sv[:want] ** 2))) < 1e-10


def test_truncate_svd_known_answers(lib_built):
    kats = json.loads((Path(__file__).resolve().parent / "golden" / "reference_kats.json").read_text())
    kind = 1
    for case in kats["truncate_svd"]:
        rows, cols = case["rows"], case["cols"]
        P = QIndex(kind, [((0,), 1)])
        QA, QB = QIndex(kind, [((0,), rows)]), QIndex(kind, [((0,), cols)])
        keys, offs, _, total = _layout(kind, P, QA, QB)
        psi = np.array(case["data"], dtype=np.float64)
        Ai, Aj, nb, disc = split_two_site_device(kind, _dev(psi), keys, offs, [P, P, QA, QB], case["max_bond_dim"],
                                                 case["svd_cutoff"], True, min_bond=case["min_bond_dim"])
        k = nb.total_dim
        if "bond_dim_new_at_least" in case:
            assert k >= case["bond_dim_new_at_least"], case["source"]
            continue
        assert k == case["bond_dim_new"], case["source"]
        assert min(rows, cols) - k == case["n_discarded"], case["source"]
        assert abs(disc - case["truncation_error"]) < case["error_atol"], case["source"]
        if "singular_values" in case:
            B = Aj.to_dense()[0]  # (k, cols) = S V^T / norm of the kept part
            sv = np.linalg.norm(B, axis=1) * np.sqrt((1.0 - disc) * float(psi @ psi))
            assert np.allclose(sv, case["singular_values"], atol=case["sv_atol"]), case["source"]


def test_exact_rank_keeps_exactly_the_rank(lib_built):
    kind = 1
    P = QIndex(kind, [((0,), 1)])
    QA, QB = QIndex(kind, [((0,), 6)]), QIndex(kind, [((0,), 6)])
    keys, offs, _, total = _layout(kind, P, QA, QB)
    rng = np.random.default_rng(4)
    psi = np.outer(rng.standard_normal(6), rng.standard_normal(6)).reshape(-1)
    for to_right in (True, False):
        Ai, Aj, nb, disc = split_two_site_device(kind, _dev(psi), keys, offs, [P, P, QA, QB], 100, 1e-12, to_right)
        assert nb.total_dim == 1
        rec = _product(Ai, Aj).reshape(-1) * np.linalg.norm(psi)
        assert np.allclose(rec, psi, atol=1e-13)


def test_matches_the_host_split(lib_built):
    """A D=2048-class Hubbard bond (random two-site vector): the same bond
    (charges and kept dimensions), the same discarded weight and the same
    kept state as the host split."""
    import math

    from tk_gb300 import models
    from tk_gb300.symmetry import fuse

    m = models.hubbard()
    kind, P = m.kind, m.phys
    QA = models.gaussian_bond_u1u1(512, 30)
    QB = models.gaussian_bond_u1u1(512, 32)
    keys, offs, qs, total = _layout(kind, P, QA, QB)
    psi = np.random.default_rng(7).standard_normal(total)
    psi /= np.linalg.norm(psi)
    for to_right in (True, False):
        Ai, Aj, nb, disc = split_two_site_device(kind, _dev(psi), keys, offs, [P, P, QA, QB], 300, 1e-14, to_right)
        Hi, Hj, hb, hdisc = split_two_site(kind, psi, keys, offs, [P, P, QA, QB], 300, 1e-14, to_right)
        assert nb.sectors == hb.sectors
        assert abs(disc - hdisc) < 1e-12
        from tk_gb300.sweep import SiteTensor
        hi = SiteTensor.from_blocks(kind, [P, QA, hb], Hi, 0)
        hj = SiteTensor.from_blocks(kind, [P, hb, QB], Hj, 0)
        a, b = _product(Ai, Aj), _product(hi, hj)
        assert np.linalg.norm(a - b) < 1e-10 * np.linalg.norm(b)


def test_complex_vector_reconstructs_and_truncates(lib_built):
    """A complex two-site vector (real and imaginary parts on the device): full
    rank reconstructs T, the factor on the growing side is an isometry in the
    Hermitian sense, and a truncation keeps truncate_svd's count with the
    weight of the discarded singular values of the complex matrix."""
    kind, P, QA, QB, keys, offs, qs, psi = _case()
    rng = np.random.default_rng(9)
    psi_im = rng.standard_normal(psi.shape)
    scale = 1.0 / np.sqrt(np.sum(psi ** 2) + np.sum(psi_im ** 2))  # the split returns the normalised state
    psi, psi_im = psi * scale, psi_im * scale
    T = _dense(kind, psi, keys, offs, qs, P, QA, QB) + 1j * _dense(kind, psi_im, keys, offs, qs, P, QA, QB)
    d = P.total_dim
    M = T.transpose(0, 2, 1, 3).reshape(d * QA.total_dim, d * QB.total_dim)
    sv = np.sort(np.linalg.svd(M, compute_uv=False))[::-1]
    for to_right in (True, False):
        Ai, Aj, nb, disc = split_two_site_device(kind, (_dev(psi), _dev(psi_im)), keys, offs, [P, P, QA, QB],
                                                 10_000, 0.0, to_right)
        assert Ai.is_complex and Aj.is_complex
        A, B = Ai.to_dense(), Aj.to_dense()
        assert disc < 1e-24
        assert np.allclose(np.einsum("sab,tbc->stac", A, B), T, atol=1e-12)
        if to_right:
            assert np.allclose(np.einsum("sab,sac->bc", A.conj(), A), np.eye(nb.total_dim), atol=1e-12)
        else:
            assert np.allclose(np.einsum("sab,scb->ac", B, B.conj()), np.eye(nb.total_dim), atol=1e-12)
    for cutoff, max_bond in ((0.3, 100), (0.0, 6)):
        want = max(1, min(max_bond, int(np.sum(sv >= cutoff * sv[0]))))
        Ai, Aj, nb, disc = split_two_site_device(kind, (_dev(psi), _dev(psi_im)), keys, offs, [P, P, QA, QB],
                                                 max_bond, cutoff, True)
        assert nb.total_dim == want
        assert abs(disc - np.sum(sv[want:] ** 2) / np.sum(sv ** 2)) < 1e-12

