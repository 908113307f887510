"""Host side of the MPS canonicalisation (per-charge thin QR / LQ) on random
block-sparse MPS: isometries on either side of the centre, the represented
state unchanged."""
import numpy as np

from tk_gb300 import models
from tk_gb300.sweep import canonicalize_blocks
from tk_gb300.symmetry import QIndex, fuse


def _random_mps(rng):
    m = models.hubbard()
    kind, P = m.kind, m.phys
    bonds = [QIndex(kind, [((0, 0), 1)])]
    for i in range(4):  # bonds grow by the physical charges, capped dims
        secs = {}
        for q, d in bonds[-1].sectors:
            for qs, _ in P.sectors:
                qr = fuse(kind, qs, q)
                secs[qr] = min(secs.get(qr, 0) + d, 5)
        bonds.append(QIndex(kind, sorted(secs.items())))
    blocks = []
    for i in range(4):
        b = {}
        for qs, ds in P.sectors:
            for ql, dl in bonds[i].sectors:
                qr = fuse(kind, qs, ql)
                dr = bonds[i + 1].dim_of(qr)
                if dr is not None:
                    b[(qs, ql, qr)] = rng.standard_normal((ds, dl, dr)) * rng.uniform(0.5, 2.0)
        blocks.append(b)
    return kind, P, bonds, blocks


def _dense(P, bonds, blocks):
    """The full state as a dense array over (s_0, ..., s_3) and the last bond."""
    v = np.ones((1, 1))
    for i, b in enumerate(blocks):
        A = np.zeros((P.total_dim, bonds[i].total_dim, bonds[i + 1].total_dim))
        for (qs, ql, qr), blk in b.items():
            A[P.offset_of(qs):P.offset_of(qs) + blk.shape[0], bonds[i].offset_of(ql):bonds[i].offset_of(ql) + blk.shape[1],
              bonds[i + 1].offset_of(qr):bonds[i + 1].offset_of(qr) + blk.shape[2]] = blk
        v = np.einsum("xa,sab->xsb", v, A).reshape(-1, A.shape[2])
    return v


def _site_dense(P, bl, br, b):
    A = np.zeros((P.total_dim, bl.total_dim, br.total_dim))
    for (qs, ql, qr), blk in b.items():
        A[P.offset_of(qs):P.offset_of(qs) + blk.shape[0], bl.offset_of(ql):bl.offset_of(ql) + blk.shape[1],
          br.offset_of(qr):br.offset_of(qr) + blk.shape[2]] = blk
    return A


def test_canonicalize_blocks_mixed():
    rng = np.random.default_rng(3)
    kind, P, bonds, blocks = _random_mps(rng)
    ref = _dense(P, bonds, blocks)
    for center in (3, 0, 1, 2):
        out, nb = canonicalize_blocks(kind, blocks, bonds, center)
        assert np.allclose(_dense(P, nb, out), ref, atol=1e-12 * np.abs(ref).max())
        for i, b in enumerate(out):
            A = _site_dense(P, nb[i], nb[i + 1], b)
            if i < center:
                G = np.einsum("sab,sac->bc", A, A)
                assert np.allclose(G, np.eye(G.shape[0]), atol=1e-12), (center, i)
            elif i > center:
                G = np.einsum("sab,scb->ac", A, A)
                assert np.allclose(G, np.eye(G.shape[0]), atol=1e-12), (center, i)
