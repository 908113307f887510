"""The host BlockSparseTensor's leg operations (tk-symmetry/src/block_sparse.rs):
permute (:400-431), fuse_legs (:444-611), split_leg (:622-793) and get_block
(:284-290), on random U(1) and U(1)xU(1) tensors of ranks 2 to 4 with mixed
leg directions (the proptest pattern of the reference's tests).  fuse_legs is
checked against the CPU restatement in oracle/contract.py (fused QIndex,
keys and blocks identical), permute against the dense transpose, and
split_leg as the exact inverse of fuse_legs."""
import numpy as np
import pytest

from oracle import contract as oc
from test_contract import _random_leg, _random_tensor, _to_oracle
from tk_gb300.symmetry import U1, U1U1, BlockSparseTensor, key_pack

CASES = [(kind, rank, seed) for kind in (U1, U1U1) for rank in (2, 3, 4) for seed in range(3)]


def _tensor(kind, rank, seed):
    rng = np.random.default_rng(100 * kind + 10 * rank + seed)
    legs = [_random_leg(kind, rng, int(rng.integers(1, 4)), 3) for _ in range(rank)]
    dirs = [int(rng.integers(0, 2)) for _ in range(rank)]
    flux = (0,) if kind == U1 else (0, 0)
    return _random_tensor(kind, legs, dirs, flux, rng), rng


def _same(a: BlockSparseTensor, b: BlockSparseTensor):
    assert [ix.sectors for ix in a.indices] == [ix.sectors for ix in b.indices]
    assert list(a.dirs) == list(b.dirs) and tuple(a.flux) == tuple(b.flux)
    assert a.sorted_keys() == b.sorted_keys()
    for k in a.sorted_keys():
        assert a.blocks[k].shape == b.blocks[k].shape and np.array_equal(a.blocks[k], b.blocks[k])


@pytest.mark.parametrize("kind,rank,seed", CASES)
def test_permute_is_the_dense_transpose(kind, rank, seed):
    t, rng = _tensor(kind, rank, seed)
    perm = [int(p) for p in rng.permutation(rank)]
    p = t.permute(perm)
    assert np.array_equal(p.to_dense(), np.transpose(t.to_dense(), perm))
    assert all(a < b for a, b in zip(p.sorted_keys(), p.sorted_keys()[1:]))
    _same(p.permute([perm.index(i) for i in range(rank)]), t)


@pytest.mark.parametrize("kind,rank,seed", CASES)
def test_fuse_legs_matches_the_restatement_and_split_leg_inverts_it(kind, rank, seed):
    t, _ = _tensor(kind, rank, seed)
    for start in range(rank):
        for end in range(start + 1, rank + 1):
            f = t.fuse_legs(start, end)
            ref = oc.fuse_legs(_to_oracle(t), start, end)
            assert [list(ix.sectors) for ix in f.indices] == [list(l) for l in ref["legs"]]
            assert list(f.dirs) == list(ref["dirs"])
            assert sorted(f.blocks) == sorted(key_pack(kind, q) for q in ref["blocks"])
            for q, blk in ref["blocks"].items():
                assert np.array_equal(f.get_block(q), blk)
            # every element kept once, and split_leg gives the tensor back
            assert np.isclose(sum(float(np.sum(b * b)) for b in f.blocks.values()),
                              sum(float(np.sum(b * b)) for b in t.blocks.values()), rtol=0, atol=1e-12)
            s = f.split_leg(start, t.indices[start:end], t.dirs[start:end])
            assert [ix.sectors for ix in s.indices] == [ix.sectors for ix in t.indices]
            assert list(s.dirs) == list(t.dirs)
            for k in s.sorted_keys():
                want = t.blocks.get(k)
                if want is None:  # a sub-sector combination t leaves empty
                    assert not np.any(s.blocks[k])
                else:
                    assert np.array_equal(s.blocks[k], want)
            assert set(t.blocks) <= set(s.blocks)


def test_get_block_and_argument_checks():
    t, _ = _tensor(U1, 3, 0)
    qns, blk = next(t.iter_blocks())
    assert t.get_block(qns) is blk
    assert t.get_block([(99,), (0,), (0,)]) is None
    with pytest.raises(ValueError):
        t.permute([0, 0, 1])
    with pytest.raises(ValueError):
        t.fuse_legs(2, 2)
    with pytest.raises(ValueError):
        t.split_leg(3, [], [])
    with pytest.raises(ValueError):
        t.split_leg(0, t.indices[:2], [0])
