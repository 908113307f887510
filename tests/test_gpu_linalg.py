"""LinAlgBackend::gemm and SparseLinAlgBackend::{block_gemm, spmv} on the device."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from tk_gb300 import _abi
from tk_gb300.heff import _Marshal, context
from tk_gb300.symmetry import U1, BlockSparseTensor, QIndex, key_pack

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def _bst(spec):
    rows = QIndex(U1, [((q,), d) for q, d in spec["rows"]])
    cols = QIndex(U1, [((q,), d) for q, d in spec["cols"]])
    t = BlockSparseTensor([rows, cols], (0,), [0, 1])
    for blk in spec["blocks"]:
        t.set_block([(blk["qns"][0],), (blk["qns"][1],)], np.array(blk["data"]).reshape(blk["shape"]))
    return t


def test_block_gemm_golden(lib_built):
    g = KATS["block_gemm"]
    a, b = _bst(g["a"]), _bst(g["b"])
    m = _Marshal()
    ba, bb = m.bst(a), m.bst(b)
    out = _abi.tk_bst_out()
    lib = _abi.load()
    _abi.check(lib.tk_block_gemm_f64(context(0), C.byref(ba), C.byref(bb), C.byref(out)))
    try:
        keys = [out.keys[i] for i in range(out.n_blocks)]
        assert keys == sorted(keys)
        offs = [out.block_offsets[i] for i in range(out.n_blocks)]
        data = np.array([out.data[i] for i in range(out.total)])
        res = BlockSparseTensor([a.indices[0], b.indices[1]], (0,), [0, 1])
        for k, o in zip(keys, offs):
            from tk_gb300.symmetry import key_unpack
            qns = key_unpack(U1, k, 2)
            shp = res.block_shape(qns)
            res.set_block(qns, data[o:o + shp[0] * shp[1]].reshape(shp))
        dense = res.to_dense()
        want = np.array(g["dense_product"]).reshape(g["shape"])
        assert np.abs(dense - want).max() < g["tol"]
    finally:
        lib.tk_bst_free(C.byref(out))


def test_spmv_matches_dense(lib_built):
    g = KATS["block_gemm"]
    a = _bst(g["a"])
    x = np.random.default_rng(0).standard_normal(a.indices[1].total_dim)
    y = np.full(a.indices[0].total_dim, np.nan)
    m = _Marshal()
    ba = m.bst(a)
    _abi.check(_abi.load().tk_spmv_f64(context(0), C.byref(ba), _abi.dptr(x), _abi.dptr(y)))
    assert np.abs(y - a.to_dense() @ x).max() < 1e-12


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_gemm_strided(lib_built, ta, tb):
    import torch

    rng = np.random.default_rng(1)
    M, K, N = 70, 45, 130
    A = rng.standard_normal((K, M) if ta else (M, K))
    B = rng.standard_normal((N, K) if tb else (K, N))
    Cm = rng.standard_normal((M, N))
    dA, dB, dC = (torch.from_numpy(v).cuda() for v in (A, B, Cm))
    a = _abi.tk_mat(dA.data_ptr(), M, K, 1 if ta else K, M if ta else 1, 0)
    b = _abi.tk_mat(dB.data_ptr(), K, N, 1 if tb else N, K if tb else 1, 0)
    c = _abi.tk_mat_mut(dC.data_ptr(), M, N, N, 1)
    _abi.check(_abi.load().tk_gemm_f64(context(0), 0.5, C.byref(a), C.byref(b), 2.0, C.byref(c), None))
    want = 0.5 * ((A.T if ta else A) @ (B.T if tb else B)) + 2.0 * Cm
    assert np.abs(dC.cpu().numpy() - want).max() < 1e-11


def _mat(t, rows, cols, rs, cs):
    return _abi.tk_mat(C.c_void_p(t.data_ptr()), rows, cols, rs, cs, 0)


@pytest.mark.parametrize("m,n,transposed", [(40, 25, False), (25, 40, False), (33, 33, True)])
def test_svd_truncated_matches_numpy(lib_built, m, n, transposed):
    """svd_truncated (traits.rs:63-104): singular values descending, the faer
    truncation rule (device/faer.rs:127-179), U and Vt row-major; strided input."""
    import torch

    rng = np.random.default_rng(m + n)
    A = rng.standard_normal((m, n)) @ np.diag(np.logspace(0, -6, n)) if m >= n else \
        np.diag(np.logspace(0, -6, m)) @ rng.standard_normal((m, n))
    src = torch.from_numpy(np.ascontiguousarray(A.T if transposed else A)).cuda()
    mat = _mat(src, m, n, 1 if transposed else n, m if transposed else 1)
    k = min(m, n)
    sv_ref = np.linalg.svd(A, compute_uv=False)
    for max_rank, cutoff in ((k, 0.0), (10, 0.0), (k, 1e-3)):
        u = torch.empty(m * k, dtype=torch.float64).cuda()
        vt = torch.empty(k * n, dtype=torch.float64).cuda()
        s = np.zeros(k)
        rank, err = C.c_int64(), C.c_double()
        _abi.check(_abi.load().tk_svd_truncated_f64(context(0), C.byref(mat), max_rank, cutoff,
                                                    C.c_void_p(u.data_ptr()), _abi.dptr(s),
                                                    C.c_void_p(vt.data_ptr()), C.byref(rank), C.byref(err), None))
        r = rank.value
        want = int(min(max_rank, np.sum(sv_ref >= cutoff * sv_ref[0])))
        assert r == want
        assert np.allclose(s[:r], sv_ref[:r], rtol=1e-12, atol=1e-14)
        assert abs(err.value - np.sum(sv_ref[r:] ** 2)) < 1e-12
        U = u.cpu().numpy()[:m * r].reshape(m, r)
        Vt = vt.cpu().numpy()[:r * n].reshape(r, n)
        assert np.allclose(U.T @ U, np.eye(r), atol=1e-11)
        assert np.allclose(Vt @ Vt.T, np.eye(r), atol=1e-11)
        approx = U @ np.diag(s[:r]) @ Vt
        assert np.linalg.norm(A - approx) ** 2 - np.sum(sv_ref[r:] ** 2) < 1e-10


def test_eigh_lowest_and_qr(lib_built):
    import torch

    rng = np.random.default_rng(3)
    B = rng.standard_normal((30, 30))
    S = (B + B.T) / 2
    st = torch.from_numpy(S).cuda()
    ev = np.zeros(5)
    vecs = torch.empty(30 * 5, dtype=torch.float64).cuda()
    lib = _abi.load()
    _abi.check(lib.tk_eigh_lowest_f64(context(0), C.byref(_mat(st, 30, 30, 30, 1)), 5, _abi.dptr(ev),
                                      C.c_void_p(vecs.data_ptr()), None))
    w = np.linalg.eigvalsh(S)
    assert np.allclose(ev, w[:5], atol=1e-12)
    V = vecs.cpu().numpy().reshape(30, 5)
    assert np.allclose(S @ V, V * ev[None, :], atol=1e-10)
    assert lib.tk_eigh_lowest_f64(context(0), C.byref(_mat(st, 30, 30, 30, 1)), 31, _abi.dptr(np.zeros(31)),
                                  C.c_void_p(vecs.data_ptr()), None) == 1  # EighKTooLarge
    for m, n in ((20, 12), (12, 20)):
        A = rng.standard_normal((m, n))
        at = torch.from_numpy(A).cuda()
        k = min(m, n)
        q = torch.empty(m * k, dtype=torch.float64).cuda()
        r = torch.empty(k * n, dtype=torch.float64).cuda()
        _abi.check(lib.tk_qr_f64(context(0), C.byref(_mat(at, m, n, n, 1)), C.c_void_p(q.data_ptr()),
                                 C.c_void_p(r.data_ptr()), None))
        Q, R = q.cpu().numpy().reshape(m, k), r.cpu().numpy().reshape(k, n)
        assert np.allclose(Q.T @ Q, np.eye(k), atol=1e-12)
        assert np.allclose(np.tril(R, -1), 0.0)
        assert np.allclose(Q @ R, A, atol=1e-12)


def _cmat(re, im, rows, cols, rs, cs, conj=0):
    return _abi.tk_cmat(re.data_ptr(), im.data_ptr(), rows, cols, rs, cs, conj)


@pytest.mark.parametrize("m,n,transposed,conj", [(30, 18, False, 0), (18, 30, False, 1), (24, 24, True, 0)])
def test_complex_svd_truncated_matches_numpy(lib_built, m, n, transposed, conj):
    """svd_truncated for C64 (planar): A = U S V^H with the real version's rank rule;
    strided and conjugated inputs."""
    import torch

    rng = np.random.default_rng(m * n + conj)
    A = (rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))) @ np.diag(np.logspace(0, -6, n))
    stored = np.ascontiguousarray(A.T if transposed else A)
    if conj:
        stored = stored.conj()  # the matrix handed over is conj(A), flagged as conjugated
    re = torch.from_numpy(stored.real.copy()).cuda()
    im = torch.from_numpy(stored.imag.copy()).cuda()
    mat = _cmat(re, im, m, n, 1 if transposed else n, m if transposed else 1, conj)
    k = min(m, n)
    sv_ref = np.linalg.svd(A, compute_uv=False)
    for max_rank, cutoff in ((k, 0.0), (7, 0.0), (k, 1e-3)):
        ur, ui = (torch.empty(m * k, dtype=torch.float64).cuda() for _ in range(2))
        vr, vi = (torch.empty(k * n, dtype=torch.float64).cuda() for _ in range(2))
        s = np.zeros(k)
        rank, err = C.c_int64(), C.c_double()
        _abi.check(_abi.load().tk_svd_truncated_c64(context(0), C.byref(mat), max_rank, cutoff,
                                                    C.c_void_p(ur.data_ptr()), C.c_void_p(ui.data_ptr()),
                                                    _abi.dptr(s), C.c_void_p(vr.data_ptr()),
                                                    C.c_void_p(vi.data_ptr()), C.byref(rank), C.byref(err), None))
        r = rank.value
        assert r == int(min(max_rank, np.sum(sv_ref >= cutoff * sv_ref[0])))
        assert np.allclose(s[:r], sv_ref[:r], rtol=1e-12, atol=1e-14)
        assert abs(err.value - np.sum(sv_ref[r:] ** 2)) < 1e-12
        U = (ur.cpu().numpy() + 1j * ui.cpu().numpy())[:m * r].reshape(m, r)
        Vt = (vr.cpu().numpy() + 1j * vi.cpu().numpy())[:r * n].reshape(r, n)
        assert np.allclose(U.conj().T @ U, np.eye(r), atol=1e-11)
        assert np.allclose(Vt @ Vt.conj().T, np.eye(r), atol=1e-11)
        assert np.linalg.norm(A - U @ np.diag(s[:r]) @ Vt) ** 2 - np.sum(sv_ref[r:] ** 2) < 1e-10


def test_complex_eigh_lowest_and_qr(lib_built):
    import torch

    rng = np.random.default_rng(4)
    B = rng.standard_normal((26, 26)) + 1j * rng.standard_normal((26, 26))
    H = (B + B.conj().T) / 2
    hr, hi = torch.from_numpy(H.real.copy()).cuda(), torch.from_numpy(H.imag.copy()).cuda()
    lib = _abi.load()
    ev = np.zeros(4)
    vr, vi = (torch.empty(26 * 4, dtype=torch.float64).cuda() for _ in range(2))
    _abi.check(lib.tk_eigh_lowest_c64(context(0), C.byref(_cmat(hr, hi, 26, 26, 26, 1)), 4, _abi.dptr(ev),
                                      C.c_void_p(vr.data_ptr()), C.c_void_p(vi.data_ptr()), None))
    assert np.allclose(ev, np.linalg.eigvalsh(H)[:4], atol=1e-12)
    V = (vr.cpu().numpy() + 1j * vi.cpu().numpy()).reshape(26, 4)
    assert np.allclose(H @ V, V * ev[None, :], atol=1e-10)
    assert lib.tk_eigh_lowest_c64(context(0), C.byref(_cmat(hr, hi, 26, 26, 26, 1)), 27, _abi.dptr(np.zeros(27)),
                                  C.c_void_p(vr.data_ptr()), C.c_void_p(vi.data_ptr()), None) == 1
    for m, n in ((20, 12), (12, 20)):
        A = rng.standard_normal((m, n)) + 1j * rng.standard_normal((m, n))
        ar, ai = torch.from_numpy(A.real.copy()).cuda(), torch.from_numpy(A.imag.copy()).cuda()
        k = min(m, n)
        qr_, qi = (torch.empty(m * k, dtype=torch.float64).cuda() for _ in range(2))
        rr, ri = (torch.empty(k * n, dtype=torch.float64).cuda() for _ in range(2))
        _abi.check(lib.tk_qr_c64(context(0), C.byref(_cmat(ar, ai, m, n, n, 1)), C.c_void_p(qr_.data_ptr()),
                                 C.c_void_p(qi.data_ptr()), C.c_void_p(rr.data_ptr()), C.c_void_p(ri.data_ptr()),
                                 None))
        Q = (qr_.cpu().numpy() + 1j * qi.cpu().numpy()).reshape(m, k)
        R = (rr.cpu().numpy() + 1j * ri.cpu().numpy()).reshape(k, n)
        assert np.allclose(Q.conj().T @ Q, np.eye(k), atol=1e-12)
        assert np.allclose(np.tril(R, -1), 0.0)
        assert np.allclose(Q @ R, A, atol=1e-12)
