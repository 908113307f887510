"""Host side of the device sweeps: the two-site truncation (density-matrix
eigendecomposition per bond charge) against a dense SVD."""
import numpy as np

from tk_gb300 import models
from tk_gb300.sweep import split_two_site
from tk_gb300.symmetry import QIndex, fuse, key_pack


def _layout(kind, P, QA, QB):
    items = []
    for qi, di in P.sectors:
        for qj, dj in P.sectors:
            for qa, da in QA.sectors:
                qb = fuse(kind, fuse(kind, qi, qj), qa)
                if QB.offset_of(qb) is None:
                    continue
                items.append((key_pack(kind, [qi, qj, qa, qb]), (qi, qj, qa, qb), di * dj * da * QB.dim_of(qb)))
    items.sort()
    keys = np.array([k for k, _, _ in items], dtype=np.uint64)
    offs = np.zeros(len(items), dtype=np.int64)
    offs[1:] = np.cumsum([s for _, _, s in items])[:-1]
    return keys, offs, [q for _, q, _ in items], sum(s for _, _, s in items)


def _dense(kind, psi, keys, offs, qs, P, QA, QB):
    d = P.total_dim
    T = np.zeros((d, d, QA.total_dim, QB.total_dim))
    for off, (qi, qj, qa, qb) in zip(offs, qs):
        ni, nj, da, db = P.dim_of(qi), P.dim_of(qj), QA.dim_of(qa), QB.dim_of(qb)
        oi, oj, oa, ob = P.offset_of(qi), P.offset_of(qj), QA.offset_of(qa), QB.offset_of(qb)
        T[oi:oi + ni, oj:oj + nj, oa:oa + da, ob:ob + db] = psi[off:off + ni * nj * da * db].reshape(ni, nj, da, db)
    return T


def _rebuild(Ai, Aj, nb, P, QA, QB):
    d = P.total_dim
    A = np.zeros((d, QA.total_dim, nb.total_dim))
    B = np.zeros((d, nb.total_dim, QB.total_dim))
    for (qs, ql, qr), b in Ai.items():
        A[P.offset_of(qs):P.offset_of(qs) + b.shape[0], QA.offset_of(ql):QA.offset_of(ql) + b.shape[1],
          nb.offset_of(qr):nb.offset_of(qr) + b.shape[2]] = b
    for (qs, ql, qr), b in Aj.items():
        B[P.offset_of(qs):P.offset_of(qs) + b.shape[0], nb.offset_of(ql):nb.offset_of(ql) + b.shape[1],
          QB.offset_of(qr):QB.offset_of(qr) + b.shape[2]] = b
    return A, B


def _case():
    m = models.hubbard()
    kind, P = m.kind, m.phys
    QA = QIndex(kind, [((2, 0), 3), ((3, -1), 4), ((3, 1), 4), ((4, 0), 5)])
    QB = QIndex(kind, [((4, 0), 3), ((5, -1), 5), ((5, 1), 5), ((6, 0), 6), ((6, 2), 2), ((6, -2), 2)])
    keys, offs, qs, total = _layout(kind, P, QA, QB)
    psi = np.random.default_rng(0).standard_normal(total)
    psi /= np.linalg.norm(psi)
    return kind, P, QA, QB, keys, offs, qs, psi


def test_full_rank_reconstructs_and_is_isometric():
    kind, P, QA, QB, keys, offs, qs, psi = _case()
    T = _dense(kind, psi, keys, offs, qs, P, QA, QB)
    for to_right in (True, False):
        Ai, Aj, nb, disc = split_two_site(kind, psi, keys, offs, [P, P, QA, QB], 10_000, 0.0, to_right)
        A, B = _rebuild(Ai, Aj, nb, P, QA, QB)
        assert disc < 1e-24
        assert np.allclose(np.einsum("sab,tbc->stac", A, B), T, atol=1e-12)
        if to_right:
            assert np.allclose(np.einsum("sab,sac->bc", A, A), np.eye(nb.total_dim), atol=1e-12)
        else:
            assert np.allclose(np.einsum("sab,scb->ac", B, B), np.eye(nb.total_dim), atol=1e-12)


def test_truncation_keeps_the_largest_singular_values():
    kind, P, QA, QB, keys, offs, qs, psi = _case()
    T = _dense(kind, psi, keys, offs, qs, P, QA, QB)
    d = P.total_dim
    M = T.transpose(0, 2, 1, 3).reshape(d * QA.total_dim, d * QB.total_dim)
    sv = np.sort(np.linalg.svd(M, compute_uv=False))[::-1]  # block structure: same singular values
    D = 9
    Ai, Aj, nb, disc = split_two_site(kind, psi, keys, offs, [P, P, QA, QB], D, 0.0, True)
    assert nb.total_dim == D
    assert abs(disc - np.sum(sv[D:] ** 2)) < 1e-12
    A, B = _rebuild(Ai, Aj, nb, P, QA, QB)
    kept = np.einsum("sab,tbc->stac", A, B) * np.sqrt(np.sum(sv[:D] ** 2))  # undo the normalisation
    # the kept state is the best rank-D approximation: its overlap with T is the kept weight
    assert abs(np.sum(kept * T) - np.sum(sv[:D] ** 2)) < 1e-12


def test_truncation_rule_of_truncate_svd():
    """sigma >= cutoff * sigma_max, at most max_bond, at least one; relative discarded weight
    (truncation/mod.rs:71-99)."""
    kind, P, QA, QB, keys, offs, qs, psi = _case()
    T = _dense(kind, psi, keys, offs, qs, P, QA, QB)
    d = P.total_dim
    M = T.transpose(0, 2, 1, 3).reshape(d * QA.total_dim, d * QB.total_dim)
    sv = np.sort(np.linalg.svd(M, compute_uv=False))[::-1]
    for cutoff, max_bond in ((0.5, 100), (0.2, 5), (2.0, 100)):
        want = max(1, min(max_bond, int(np.sum(sv >= cutoff * sv[0]))))
        _, _, nb, disc = split_two_site(kind, psi * 3.0, keys, offs, [P, P, QA, QB], max_bond, cutoff, True)
        assert nb.total_dim == want, (cutoff, max_bond)
        assert abs(disc - np.sum(sv[want:] ** 2) / np.sum(sv ** 2)) < 1e-12


def test_complex_full_rank_reconstructs_and_is_isometric():
    """Complex two-site vectors (real-time TDVP): the same per-charge
    truncation with Hermitian density matrices."""
    kind, P, QA, QB, keys, offs, qs, psi_r = _case()
    psi = psi_r + 1j * np.random.default_rng(1).standard_normal(psi_r.shape)
    psi /= np.linalg.norm(psi)
    d = P.total_dim
    T = np.zeros((d, d, QA.total_dim, QB.total_dim), dtype=complex)
    for off, (qi, qj, qa, qb) in zip(offs, qs):
        ni, nj, da, db = P.dim_of(qi), P.dim_of(qj), QA.dim_of(qa), QB.dim_of(qb)
        oi, oj, oa, ob = P.offset_of(qi), P.offset_of(qj), QA.offset_of(qa), QB.offset_of(qb)
        T[oi:oi + ni, oj:oj + nj, oa:oa + da, ob:ob + db] = psi[off:off + ni * nj * da * db].reshape(ni, nj, da, db)
    for to_right in (True, False):
        Ai, Aj, nb, disc = split_two_site(kind, psi, keys, offs, [P, P, QA, QB], 10_000, 0.0, to_right)
        A = np.zeros((d, QA.total_dim, nb.total_dim), dtype=complex)
        B = np.zeros((d, nb.total_dim, QB.total_dim), dtype=complex)
        for (s, ql, qr), b in Ai.items():
            A[P.offset_of(s):P.offset_of(s) + b.shape[0], QA.offset_of(ql):QA.offset_of(ql) + b.shape[1],
              nb.offset_of(qr):nb.offset_of(qr) + b.shape[2]] = b
        for (s, ql, qr), b in Aj.items():
            B[P.offset_of(s):P.offset_of(s) + b.shape[0], nb.offset_of(ql):nb.offset_of(ql) + b.shape[1],
              QB.offset_of(qr):QB.offset_of(qr) + b.shape[2]] = b
        assert disc < 1e-24
        assert np.allclose(np.einsum("sab,tbc->stac", A, B), T, atol=1e-12)
        if to_right:
            assert np.allclose(np.einsum("sab,sac->bc", A.conj(), A), np.eye(nb.total_dim), atol=1e-12)
        else:
            assert np.allclose(np.einsum("sab,scb->ac", B, B.conj()), np.eye(nb.total_dim), atol=1e-12)


def test_tied_singular_values_keep_the_charges_that_sort_first():
    """The deterministic sector assignment: every bond charge gets exactly one
    singular value 1.0 (one unit entry in its block), so all of them tie, and
    a bond of D states keeps the D charges that come first in charge order."""
    kind, P, QA, QB, keys, offs, qs, psi0 = _case()
    psi = np.zeros_like(psi0)
    seen = []
    for off, (qi, qj, qa, qb) in zip(offs, qs):
        q = fuse(kind, qi, qa)
        if q not in seen:
            psi[off] = 1.0
            seen.append(q)
    assert len(seen) >= 4
    for to_right in (True, False):
        for D in (1, 2, 3):
            Ai, Aj, nb, disc = split_two_site(kind, psi, keys, offs, [P, P, QA, QB], D, 0.5, to_right)
            assert {q for q, _ in nb.sectors} == set(sorted(seen)[:D]), (to_right, D)
            assert all(d == 1 for _, d in nb.sectors)
            assert abs(disc - (len(seen) - D) / len(seen)) < 1e-14


def test_truncate_svd_known_answers():
    """The reference's truncate_svd tests (truncation/mod.rs:185-236, in
    tests/golden/reference_kats.json) on a two-site vector with one charge
    and one-dimensional physical legs, so that its single block is the
    test's matrix: kept dimension, discarded count and error, and the kept
    singular values (row norms of the right factor, rescaled)."""
    import json
    from pathlib import Path

    kats = json.loads((Path(__file__).resolve().parent / "golden" / "reference_kats.json").read_text())
    kind = 1  # U(1)
    for case in kats["truncate_svd"]:
        rows, cols = case["rows"], case["cols"]
        P = QIndex(kind, [((0,), 1)])
        QA, QB = QIndex(kind, [((0,), rows)]), QIndex(kind, [((0,), cols)])
        keys, offs, _, total = _layout(kind, P, QA, QB)
        assert total == rows * cols
        psi = np.array(case["data"], dtype=np.float64)
        Ai, Aj, nb, disc = split_two_site(kind, psi, keys, offs, [P, P, QA, QB], case["max_bond_dim"],
                                          case["svd_cutoff"], True, min_bond=case["min_bond_dim"])
        k = nb.total_dim
        if "bond_dim_new_at_least" in case:
            assert k >= case["bond_dim_new_at_least"], case["source"]
            continue
        assert k == case["bond_dim_new"], case["source"]
        assert min(rows, cols) - k == case["n_discarded"], case["source"]
        assert abs(disc - case["truncation_error"]) < case["error_atol"], case["source"]
        if "singular_values" in case:
            B = Aj[((0,), (0,), (0,))][0]  # (k, cols): sigma_r v_r^T / norm of the kept part
            kept = np.sqrt((1.0 - disc) * float(psi @ psi))
            sv = np.linalg.norm(B, axis=1) * kept
            assert np.allclose(sv, case["singular_values"], atol=case["sv_atol"]), (sv, case["source"])


def test_exact_rank_keeps_exactly_the_rank():
    """A rank-1 6 x 6 block with cutoff 1e-12: truncate_svd's SVD gives one
    singular value and five at rounding level (< 1e-15 sigma_max), so it keeps
    one state.  The density matrix alone resolves sigma only to ~1e-7 sigma_max,
    which would keep noise states; the split takes those charges by SVD."""
    kind = 1
    P = QIndex(kind, [((0,), 1)])
    QA, QB = QIndex(kind, [((0,), 6)]), QIndex(kind, [((0,), 6)])
    keys, offs, _, total = _layout(kind, P, QA, QB)
    rng = np.random.default_rng(4)
    u, v = rng.standard_normal(6), rng.standard_normal(6)
    psi = np.outer(u, v).reshape(-1)
    for to_right in (True, False):
        Ai, Aj, nb, disc = split_two_site(kind, psi, keys, offs, [P, P, QA, QB], 100, 1e-12, to_right)
        assert nb.total_dim == 1, to_right
        assert disc < 1e-28
        A, B = _rebuild(Ai, Aj, nb, P, QA, QB)
        rec = np.einsum("sab,tbc->stac", A, B).reshape(-1) * np.linalg.norm(psi)
        assert np.allclose(rec, psi, atol=1e-13)


def test_rank_deficient_charges_match_a_dense_svd():
    """Several charges, each of a known rank below its size, cutoff 1e-12 and no
    max_bond limit: the kept dimension per charge is that rank (what an SVD of
    each charge block keeps), and the product of the factors is the state."""
    kind, P, QA, QB, keys, offs, qs, _ = _case()
    rng = np.random.default_rng(9)
    psi = np.zeros(sum(int(np.prod([P.dim_of(a), P.dim_of(b), QA.dim_of(c), QB.dim_of(d)])) for a, b, c, d in qs))
    T = np.zeros((P.total_dim, P.total_dim, QA.total_dim, QB.total_dim))
    d = P.total_dim
    # M = X Y with X (rows x 2), Y (2 x cols): every charge block has rank <= 2
    X = rng.standard_normal((d * QA.total_dim, 2))
    Y = rng.standard_normal((2, d * QB.total_dim))
    Md = (X @ Y).reshape(d, QA.total_dim, d, QB.total_dim).transpose(0, 2, 1, 3)
    for off, (qi, qj, qa, qb) in zip(offs, qs):
        ni, nj, da, db = P.dim_of(qi), P.dim_of(qj), QA.dim_of(qa), QB.dim_of(qb)
        oi, oj, oa, ob = P.offset_of(qi), P.offset_of(qj), QA.offset_of(qa), QB.offset_of(qb)
        blk = Md[oi:oi + ni, oj:oj + nj, oa:oa + da, ob:ob + db]
        psi[off:off + blk.size] = blk.reshape(-1)
        T[oi:oi + ni, oj:oj + nj, oa:oa + da, ob:ob + db] = blk
    for to_right in (True, False):
        Ai, Aj, nb, disc = split_two_site(kind, psi, keys, offs, [P, P, QA, QB], 10_000, 1e-12, to_right)
        assert all(k <= 2 for _, k in nb.sectors), nb.sectors
        A, B = _rebuild(Ai, Aj, nb, P, QA, QB)
        rec = np.einsum("sab,tbc->stac", A, B) * np.linalg.norm(psi)
        assert np.allclose(rec, T, atol=1e-12)


def test_threads_for_the_largest_block():
    """The largest factorisation of a truncation gets several BLAS threads only
    when it would otherwise set the wall time alone."""
    from tk_gb300.sweep import _big_block_threads

    assert _big_block_threads([100.0] + [1.0] * 30, 16) > 0  # one dominant block
    assert _big_block_threads([1.0] * 40, 16) == 0  # balanced: every block on one thread
    assert _big_block_threads([100.0, 1.0], 4) == 0  # too few cores to share
    assert _big_block_threads([5.0], 16) == 0


def test_factor_blocks_matches_numpy():
    """_factor_blocks: every block's thin SVD, whichever BLAS and thread count
    factor it (the dominant block through scipy.linalg on several threads)."""
    from tk_gb300 import sweep

    rng = np.random.default_rng(3)
    shapes = [(160, 150)] + [(rng.integers(2, 30), rng.integers(2, 30)) for _ in range(12)] + [(1, 5), (7, 1)]
    blocks = [rng.standard_normal(s) for s in shapes]
    for workers in (1, 8, 16):
        saved = sweep._pool_size
        sweep._pool_size = lambda w=workers: w
        try:
            cost = [m * n * min(m, n) for m, n in shapes]
            order = sorted(range(len(blocks)), key=lambda i: -cost[i])
            out = sweep._factor_blocks(lambda i: blocks[i], order, [cost[i] for i in order])
        finally:
            sweep._pool_size = saved
        assert sorted(out) == list(range(len(blocks)))
        for i, (U, s, Vt) in out.items():
            ref = np.linalg.svd(blocks[i], compute_uv=False)
            assert np.allclose(s, ref, rtol=1e-12, atol=1e-13)
            assert np.allclose((U * s) @ Vt, blocks[i], atol=1e-12)
            k = len(s)
            assert np.allclose(U.T @ U, np.eye(k), atol=1e-12) and np.allclose(Vt @ Vt.T, np.eye(k), atol=1e-12)
