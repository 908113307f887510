"""Block-sparse contraction and the rank-2 backend calls on the device.

contract_pairwise mirrors SparseContractionExecutor::execute_pairwise_sparse
(tk-contract/src/sparse.rs:124-265): permute, fuse the free and the
contracted legs of each operand, block_gemm; the work runs in
tk_contract_pairwise_f64.  block_gemm mirrors SparseLinAlgBackend::block_gemm
(tk-linalg/src/traits.rs:200-204) through tk_block_gemm_f64.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import check
from .heff import _Marshal, context
from .symmetry import BlockSparseTensor, QIndex, key_unpack, ncomp


def _from_out(res: _abi.tk_bst_out) -> BlockSparseTensor:
    kind = res.qn_kind
    nc = ncomp(kind)
    legs = []
    for l in range(2):
        q = res.legs[l]
        ch = [tuple(q.charges[s * nc + k] for k in range(nc)) for s in range(q.n_sectors)]
        legs.append(QIndex(kind, [(c, int(q.dims[s])) for s, c in enumerate(ch)]))
    t = BlockSparseTensor(legs, tuple(res.flux[k] for k in range(nc)), [int(res.leg_dirs[0]), int(res.leg_dirs[1])])
    n = res.n_blocks
    keys = np.ctypeslib.as_array(res.keys, shape=(n,)).copy() if n else np.zeros(0, dtype=np.uint64)
    offs = np.ctypeslib.as_array(res.block_offsets, shape=(n,)).copy() if n else np.zeros(0, dtype=np.int64)
    data = np.ctypeslib.as_array(res.data, shape=(res.total,)).copy() if res.total else np.zeros(0)
    for k, o in zip(keys, offs):
        qns = key_unpack(kind, int(k), 2)
        shape = t.block_shape(qns)
        t.blocks[int(k)] = data[o:o + shape[0] * shape[1]].reshape(shape)
    return t


def contract_pairwise(a: BlockSparseTensor, a_legs, b: BlockSparseTensor, b_legs, device: int = 0) -> BlockSparseTensor:
    """Contract legs a_legs of `a` with legs b_legs of `b`; the rank-2 result has
    the fused free legs of `a` as rows and those of `b` as columns."""
    lib = _abi.load()
    m = _Marshal()
    ba, bb = m.bst(a), m.bst(b)
    la = np.ascontiguousarray(a_legs, dtype=np.int32)
    lb = np.ascontiguousarray(b_legs, dtype=np.int32)
    res = _abi.tk_bst_out()
    check(lib.tk_contract_pairwise_f64(context(device), C.byref(ba), _abi.i32ptr(la), len(la), C.byref(bb),
                                       _abi.i32ptr(lb), len(lb), C.byref(res)))
    try:
        return _from_out(res)
    finally:
        lib.tk_bst_free(C.byref(res))


def block_gemm(a: BlockSparseTensor, b: BlockSparseTensor, device: int = 0) -> BlockSparseTensor:
    """Rank-2 C = A B (host tensors)."""
    lib = _abi.load()
    m = _Marshal()
    ba, bb = m.bst(a), m.bst(b)
    res = _abi.tk_bst_out()
    check(lib.tk_block_gemm_f64(context(device), C.byref(ba), C.byref(bb), C.byref(res)))
    try:
        return _from_out(res)
    finally:
        lib.tk_bst_free(C.byref(res))
