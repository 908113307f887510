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
