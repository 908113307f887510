"""Environment growth restatement (numpy) -- TEST INFRASTRUCTURE ONLY.

contract_left_environment (tk-dmrg/src/environments/mod.rs:221-355) and
contract_right_environment (:357-483) sum, over every (ket block, bra block,
MPO block) triple of the site tensors, the products
  L'[b', v, b] += conj(A[s', a', b']) L[a', w, a] W[s, s', w, v] A[s, a, b]
  R'[a', w, a] += conj(A[s', a', b']) R[b', v, b] W[s, s', w, v] A[s, a, b]
into a dense (bra, w, ket) array, with W's s_in pairing the ket and s_out the
bra (:285-289).  On dense (zero-padded) site tensors that is one einsum each.
"""
from __future__ import annotations

import numpy as np

# pairwise contraction order with intermediates allowed to exceed the inputs (numpy's
# default limit, the largest operand, falls back to one nested loop over every index)
_PATH = ("greedy", 2 ** 34)


def grow_left(L, A, W):
    """L: (Da, w, Da); A: (d, Da, Db); W: (d, d, w, v) -> (Db, v, Db)."""
    return np.einsum("tpx,pwa,stwv,sab->xvb", A.conj(), L, W, A, optimize=_PATH)


def grow_right(R, A, W):
    """R: (Db, v, Db); A: (d, Da, Db); W: (d, d, w, v) -> (Da, w, Da)."""
    return np.einsum("txp,pvb,stwv,sab->xwa", A.conj(), R, W, A, optimize=_PATH)


def heff_single_site_dense(L, W, R):
    """Dense single-site H_eff of build_heff_single_site (environments/mod.rs:603-678):
    H[(s', a', b'), (s, a, b)] = sum L[a', w, a] W[s, s', w, v] R[b', v, b],
    rows and columns in the (s, a_L, a_R) row-major layout."""
    d, Da, Db = W.shape[0], L.shape[0], R.shape[0]
    H = np.einsum("pwa,stwv,qvb->tpqsab", L, W, R, optimize=_PATH)
    return H.reshape(d * Da * Db, d * Da * Db)
