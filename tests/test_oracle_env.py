"""The environment-growth restatement against the reference's literal sums
(contract_left/right_environment, tk-dmrg/src/environments/mod.rs:221-483)."""
import numpy as np

from oracle import environments as oe


def _literal_left(L, A, W):
    d, Da, Db = A.shape
    out = np.zeros((Db, W.shape[3], Db))
    for si in range(d):
        for so in range(d):
            for ab in range(Da):
                for w in range(W.shape[2]):
                    for ak in range(Da):
                        for wp in range(W.shape[3]):
                            c = L[ab, w, ak] * W[si, so, w, wp]
                            for apk in range(Db):
                                for apb in range(Db):
                                    out[apb, wp, apk] += A[so, ab, apb] * c * A[si, ak, apk]
    return out


def _literal_right(R, A, W):
    d, Da, Db = A.shape
    out = np.zeros((Da, W.shape[2], Da))
    for si in range(d):
        for so in range(d):
            for apb in range(Db):
                for wp in range(W.shape[3]):
                    for apk in range(Db):
                        for w in range(W.shape[2]):
                            c = R[apb, wp, apk] * W[si, so, w, wp]
                            for ak in range(Da):
                                for ab in range(Da):
                                    out[ab, w, ak] += A[so, ab, apb] * c * A[si, ak, apk]
    return out


def test_growth_restatement_matches_literal_sums():
    rng = np.random.default_rng(3)
    A = rng.standard_normal((2, 3, 4))
    W = rng.standard_normal((2, 2, 2, 3))
    L = rng.standard_normal((3, 2, 3))
    R = rng.standard_normal((4, 3, 4))
    assert np.allclose(oe.grow_left(L, A, W), _literal_left(L, A, W), rtol=0, atol=1e-12)
    assert np.allclose(oe.grow_right(R, A, W), _literal_right(R, A, W), rtol=0, atol=1e-12)


def test_single_site_restatement_matches_literal_loops():
    """heff_single_site_dense against the reference's element loops (environments/mod.rs:619-664)."""
    rng = np.random.default_rng(5)
    d, Da, Db, w, v = 2, 3, 4, 2, 3
    L = rng.standard_normal((Da, w, Da))
    R = rng.standard_normal((Db, v, Db))
    W = rng.standard_normal((d, d, w, v))
    dim = d * Da * Db
    H = np.zeros((dim, dim))
    for s_in in range(d):
        for s_out in range(d):
            for wl in range(w):
                for wr in range(v):
                    for a_l in range(Da):
                        for ap_l in range(Da):
                            lw = L[ap_l, wl, a_l] * W[s_in, s_out, wl, wr]
                            for a_r in range(Db):
                                for ap_r in range(Db):
                                    H[(s_out * Da + ap_l) * Db + ap_r, (s_in * Da + a_l) * Db + a_r] += \
                                        lw * R[ap_r, wr, a_r]
    assert np.allclose(oe.heff_single_site_dense(L, W, R), H, atol=1e-12, rtol=0)
