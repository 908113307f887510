"""tk_contract_pairwise_f64 (SparseContractionExecutor::execute_pairwise_sparse,
tk-contract/src/sparse.rs:124-265) against the CPU restatement in
oracle/contract.py.

CPU: the restatement itself -- fuse_legs keeps every element once, and for
rank-2 operands block_gemm equals the dense product.  GPU (through the C ABI):
random block-sparse tensors of ranks 2 to 4 with U(1) and U(1)xU(1) charges,
mixed leg directions and several contracted-leg choices, the proptest pattern
of tk-contract/tests/proptest_contract.rs; the fused legs, packed keys and
block offsets must be identical to the restatement's and the values within
1e-12 relative (FP64)."""
import itertools

import numpy as np
import pytest

import oracle
from oracle import contract as oc
from tk_gb300.symmetry import U1, U1U1, BlockSparseTensor, QIndex, enumerate_valid_sectors, key_pack

TOL = 1e-12


def _random_leg(kind, rng, n, dmax):
    if kind == U1:
        qs = sorted(rng.choice(np.arange(-4, 5), size=n, replace=False).tolist())
        return QIndex(kind, [((int(q),), int(rng.integers(1, dmax + 1))) for q in qs])
    pool = [(a, b) for a in range(0, 4) for b in range(-2, 3)]
    sel = sorted(pool[i] for i in rng.choice(len(pool), size=n, replace=False))
    return QIndex(kind, [(q, int(rng.integers(1, dmax + 1))) for q in sel])


def _random_tensor(kind, legs, dirs, flux, rng):
    t = BlockSparseTensor(list(legs), tuple(flux), list(dirs))
    for qns in enumerate_valid_sectors(legs, flux, dirs):
        if rng.random() < 0.85:
            t.set_block(qns, rng.standard_normal(t.block_shape(qns)))
    return t


def _to_oracle(t: BlockSparseTensor):
    return {"kind": t.kind, "legs": [list(ix.sectors) for ix in t.indices], "dirs": list(t.dirs),
            "flux": tuple(t.flux), "blocks": {tuple(tuple(q) for q in qns): blk for qns, blk in t.iter_blocks()}}


def _case(kind, seed, ranks, n_contract):
    """Two tensors whose contracted legs share QIndex (A's contracted legs in
    ascending order meet B's in ascending order) with opposite directions."""
    rng = np.random.default_rng(seed)
    ra, rb = ranks
    shared = [_random_leg(kind, rng, int(rng.integers(2, 4)), 4) for _ in range(n_contract)]
    ca = sorted(rng.choice(ra, size=n_contract, replace=False).tolist())
    cb = sorted(rng.choice(rb, size=n_contract, replace=False).tolist())
    legs_a, dirs_a, legs_b, dirs_b = [], [], [], []
    k = 0
    for l in range(ra):
        if l in ca:
            legs_a.append(shared[k]); dirs_a.append(1); k += 1
        else:
            legs_a.append(_random_leg(kind, rng, int(rng.integers(1, 4)), 4)); dirs_a.append(int(rng.integers(0, 2)))
    k = 0
    for l in range(rb):
        if l in cb:
            legs_b.append(shared[k]); dirs_b.append(0); k += 1
        else:
            legs_b.append(_random_leg(kind, rng, int(rng.integers(1, 4)), 4)); dirs_b.append(int(rng.integers(0, 2)))
    zero = (0,) if kind == U1 else (0, 0)
    a = _random_tensor(kind, legs_a, dirs_a, zero, rng)
    b = _random_tensor(kind, legs_b, dirs_b, zero, rng)
    return a, ca, b, cb


def _oracle_result(a, ca, b, cb):
    return oc.execute_pairwise_sparse(_to_oracle(a), ca, _to_oracle(b), cb, oracle.key_pack)


def test_oracle_fuse_keeps_every_element():
    a, ca, b, cb = _case(U1, 3, (4, 3), 2)
    t = _to_oracle(a)
    for start, end in ((0, 2), (1, 3), (0, 4), (2, 4)):
        f = oc.fuse_legs(t, start, end)
        v0 = np.sort(np.concatenate([x.reshape(-1) for x in t["blocks"].values()]))
        v1 = np.concatenate([x.reshape(-1) for x in f["blocks"].values()])
        v1 = np.sort(v1[v1 != 0.0])
        assert np.array_equal(v0[v0 != 0.0], v1)
        assert sum(d for _, d in f["legs"][start]) == int(np.prod([sum(d for _, d in t["legs"][l])
                                                                     for l in range(start, end)]))


def test_oracle_block_gemm_rank2_is_the_dense_product():
    rng = np.random.default_rng(1)
    leg = _random_leg(U1, rng, 3, 5)
    a = _random_tensor(U1, [leg, leg], [0, 1], (0,), rng)
    b = _random_tensor(U1, [leg, leg], [0, 1], (0,), rng)
    res, order = oc.block_gemm(_to_oracle(a), _to_oracle(b), oracle.key_pack)
    dense = np.zeros((leg.total_dim, leg.total_dim))
    for (qr, qc), blk in res["blocks"].items():
        dense[leg.offset_of(qr):leg.offset_of(qr) + blk.shape[0], leg.offset_of(qc):leg.offset_of(qc) + blk.shape[1]] = blk
    assert np.allclose(dense, a.to_dense() @ b.to_dense(), atol=1e-12)
    assert order == sorted(order, key=lambda q: oracle.key_pack(U1, list(q)))


CASES = [(kind, seed, ranks, nc) for kind in (U1, U1U1) for seed, ranks, nc in
         [(0, (2, 2), 1), (1, (3, 2), 1), (2, (3, 3), 2), (3, (4, 3), 2), (4, (4, 4), 2), (5, (3, 4), 1),
          (6, (4, 4), 3)]]


@pytest.mark.gpu
@pytest.mark.parametrize("kind,seed,ranks,nc", CASES)
def test_contract_pairwise_matches_restatement(lib_built, kind, seed, ranks, nc):
    from tk_gb300.contract import contract_pairwise

    a, ca, b, cb = _case(kind, seed, ranks, nc)
    ref, order = _oracle_result(a, ca, b, cb)
    got = contract_pairwise(a, ca, b, cb)
    # fused legs and directions identical
    assert [list(ix.sectors) for ix in got.indices] == [list(leg) for leg in ref["legs"]]
    assert got.dirs == ref["dirs"] and tuple(got.flux) == tuple(ref["flux"])
    # identical block list in the same (ascending key) order and layout
    keys, offs, data = got.flatten()
    want_keys = [oracle.key_pack(kind, list(q)) for q in order]
    assert keys.tolist() == want_keys
    want = np.concatenate([ref["blocks"][q].reshape(-1) for q in order]) if order else np.zeros(0)
    assert data.shape == want.shape
    if want.size:
        assert np.linalg.norm(data - want) <= TOL * np.linalg.norm(want)


@pytest.mark.gpu
def test_contract_pairwise_repeats_without_growth(lib_built):
    """Repeated calls reuse the context scratch and give the same bits."""
    from tk_gb300.contract import contract_pairwise

    a, ca, b, cb = _case(U1, 11, (4, 3), 2)
    first = contract_pairwise(a, ca, b, cb).flatten()[2]
    for _ in range(3):
        assert np.array_equal(contract_pairwise(a, ca, b, cb).flatten()[2], first)


@pytest.mark.gpu
def test_contract_pairwise_rejects_degenerate(lib_built):
    from tk_gb300 import TkError
    from tk_gb300.contract import contract_pairwise

    a, ca, b, cb = _case(U1, 12, (2, 2), 1)
    with pytest.raises(TkError) as e:
        contract_pairwise(a, [0, 1], b, [0, 1])  # no free leg left
    assert e.value.status == 7
    with pytest.raises(TkError) as e:
        contract_pairwise(a, [0], b, [0, 1])
    assert e.value.status == 1


@pytest.mark.gpu
def test_block_gemm_dev_matches_host(lib_built):
    """tk_block_gemm_f64_dev (device operands, two-call sizing) equals the
    host-buffer call bit for bit."""
    import ctypes as C

    import torch
    from tk_gb300 import _abi
    from tk_gb300.contract import block_gemm
    from tk_gb300.heff import _Marshal, context

    rng = np.random.default_rng(2)
    leg = _random_leg(U1, rng, 5, 40)
    a = _random_tensor(U1, [leg, leg], [0, 1], (0,), rng)
    b = _random_tensor(U1, [leg, leg], [0, 1], (0,), rng)
    host = block_gemm(a, b).flatten()
    m = _Marshal()
    ba, bb = m.bst(a), m.bst(b)
    da = torch.from_numpy(a.flatten()[2]).cuda()
    db = torch.from_numpy(b.flatten()[2]).cuda()
    ba.data = C.cast(C.c_void_p(da.data_ptr()), C.POINTER(C.c_double))
    bb.data = C.cast(C.c_void_p(db.data_ptr()), C.POINTER(C.c_double))
    lib = _abi.load()
    res = _abi.tk_bst_out()
    _abi.check(lib.tk_block_gemm_f64_dev(context(0), C.byref(ba), C.byref(bb), C.byref(res), None, None))
    total = res.total
    keys = np.ctypeslib.as_array(res.keys, shape=(res.n_blocks,)).copy()
    lib.tk_bst_free(C.byref(res))
    dc = torch.empty(total, dtype=torch.float64, device="cuda")
    _abi.check(lib.tk_block_gemm_f64_dev(context(0), C.byref(ba), C.byref(bb), C.byref(res),
                                         C.c_void_p(dc.data_ptr()), None))
    lib.tk_bst_free(C.byref(res))
    assert np.array_equal(keys, host[0])
    assert np.array_equal(dc.cpu().numpy(), host[2])
