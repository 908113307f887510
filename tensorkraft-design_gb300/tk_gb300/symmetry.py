"""Host-side block-sparse tensors in tensorkraft's formats.

Mirrors (kyungminlee/tensorkraft-design):
  tk-symmetry/src/builtins.rs:12-152     U1 / Z2 / U1Z2 / U1Wide quantum numbers
  tk-symmetry/src/sector_key.rs:18-148   PackedSectorKey, QIndex
  tk-symmetry/src/flux.rs:9-234          check_flux_rule, enumerate_valid_sectors
  tk-symmetry/src/block_sparse.rs:21-159 BlockSparseTensor (sorted keys + blocks)
  tk-symmetry/src/flat_storage.rs:14-167 FlatBlockStorage (contiguous blocks)

Quantum numbers are tuples of ints (one entry per component); U1U1 is the
(N, 2Sz) pair the Hubbard models need, 8 bits per component, 16 per leg.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

U1, Z2, U1Z2, U1WIDE, U1U1 = 1, 2, 3, 4, 5
INCOMING, OUTGOING = 0, 1

_NCOMP = {U1: 1, Z2: 1, U1Z2: 2, U1WIDE: 1, U1U1: 2}
_BITS = {U1: 8, Z2: 1, U1Z2: 9, U1WIDE: 16, U1U1: 16}


def ncomp(kind: int) -> int:
    return _NCOMP[kind]


def bit_width(kind: int) -> int:
    return _BITS[kind]


def fuse(kind: int, a: tuple, b: tuple) -> tuple:
    if kind == Z2:
        return (a[0] ^ b[0],)
    if kind == U1Z2:
        return (a[0] + b[0], a[1] ^ b[1])
    return tuple(x + y for x, y in zip(a, b))


def dual(kind: int, a: tuple) -> tuple:
    if kind == Z2:
        return (a[0],)
    if kind == U1Z2:
        return (-a[0], a[1])
    return tuple(-x for x in a)


def identity(kind: int) -> tuple:
    return (0,) * ncomp(kind)


def qn_pack(kind: int, q: tuple) -> int:
    if kind == U1:
        return q[0] & 0xFF
    if kind == Z2:
        return int(q[0] != 0)
    if kind == U1Z2:
        return (q[0] & 0xFF) | (int(q[1] != 0) << 8)
    if kind == U1WIDE:
        return q[0] & 0xFFFF
    if kind == U1U1:
        return (q[0] & 0xFF) | ((q[1] & 0xFF) << 8)
    raise ValueError(kind)


def _sext(v: int, bits: int) -> int:
    v &= (1 << bits) - 1
    return v - (1 << bits) if v >> (bits - 1) else v


def qn_unpack(kind: int, bits: int) -> tuple:
    if kind == U1:
        return (_sext(bits, 8),)
    if kind == Z2:
        return (bits & 1,)
    if kind == U1Z2:
        return (_sext(bits, 8), (bits >> 8) & 1)
    if kind == U1WIDE:
        return (_sext(bits, 16),)
    if kind == U1U1:
        return (_sext(bits, 8), _sext(bits >> 8, 8))
    raise ValueError(kind)


def key_pack(kind: int, qns) -> int:
    bw = bit_width(kind)
    if len(qns) * bw > 64:
        raise ValueError("sector key exceeds 64 bits")
    key = 0
    for i, q in enumerate(qns):
        key |= (qn_pack(kind, q) & ((1 << bw) - 1)) << (i * bw)
    return key


def key_unpack(kind: int, key: int, rank: int) -> list:
    bw = bit_width(kind)
    return [qn_unpack(kind, (key >> (i * bw)) & ((1 << bw) - 1)) for i in range(rank)]


@dataclass
class QIndex:
    """Per-leg basis: sectors sorted by quantum number (QIndex::new sorts)."""

    kind: int
    sectors: list  # [(q tuple, dim)]

    def __post_init__(self):
        self.sectors = sorted(((tuple(q), int(d)) for q, d in self.sectors), key=lambda s: s[0])
        for i in range(1, len(self.sectors)):
            if not self.sectors[i - 1][0] < self.sectors[i][0]:
                raise ValueError("QIndex sectors must be strictly sorted / unique")
        if any(d <= 0 for _, d in self.sectors):
            raise ValueError("QIndex sector dims must be positive")

    @property
    def total_dim(self) -> int:
        return sum(d for _, d in self.sectors)

    @property
    def n_sectors(self) -> int:
        return len(self.sectors)

    def _lookup(self) -> dict:
        # {charge: (offset, dim)}, rebuilt when the sector list object changes
        cache = self.__dict__.get("_lookup_cache")
        if cache is None or cache[0] is not self.sectors or cache[1] != len(self.sectors):
            table, off = {}, 0
            for sq, d in self.sectors:
                table[sq] = (off, d)
                off += d
            cache = (self.sectors, len(self.sectors), table)
            self.__dict__["_lookup_cache"] = cache
        return cache[2]

    def offset_of(self, q):
        hit = self._lookup().get(tuple(q))
        return None if hit is None else hit[0]

    def dim_of(self, q):
        hit = self._lookup().get(tuple(q))
        return None if hit is None else hit[1]

    def charges(self) -> np.ndarray:
        return np.array([list(q) for q, _ in self.sectors], dtype=np.int32).reshape(-1)

    def dims(self) -> np.ndarray:
        return np.array([d for _, d in self.sectors], dtype=np.int64)

    def state_charges(self) -> list:
        out = []
        for q, d in self.sectors:
            out.extend([q] * d)
        return out

    def __eq__(self, other) -> bool:
        return isinstance(other, QIndex) and self.kind == other.kind and self.sectors == other.sectors


def check_flux_rule(kind: int, qns, flux, dirs) -> bool:
    acc = identity(kind)
    for q, d in zip(qns, dirs):
        acc = fuse(kind, acc, tuple(q) if d == INCOMING else dual(kind, tuple(q)))
    return acc == tuple(flux)


def enumerate_valid_sectors(indices, flux, dirs) -> list:
    """DFS over legs in QIndex order, last leg solved (flux.rs:43-234)."""
    kind = indices[0].kind
    rank = len(indices)
    out = []

    def rec(cur):
        depth = len(cur)
        if depth == rank - 1:
            acc = identity(kind)
            for q, d in zip(cur, dirs):
                acc = fuse(kind, acc, q if d == INCOMING else dual(kind, q))
            req = fuse(kind, tuple(flux), dual(kind, acc))
            if dirs[depth] == OUTGOING:
                req = dual(kind, req)
            if indices[depth].dim_of(req) is not None:
                out.append(cur + [req])
            return
        for q, _ in indices[depth].sectors:
            rec(cur + [q])

    rec([])
    return out


@dataclass
class BlockSparseTensor:
    """Sorted packed keys + dense row-major blocks (block_sparse.rs:21-34)."""

    indices: list
    flux: tuple
    dirs: list
    blocks: dict = field(default_factory=dict)  # key -> ndarray

    @property
    def kind(self) -> int:
        return self.indices[0].kind

    @property
    def rank(self) -> int:
        return len(self.indices)

    def block_shape(self, qns) -> tuple:
        return tuple(ix.dim_of(q) for ix, q in zip(self.indices, qns))

    @classmethod
    def zeros(cls, indices, flux, dirs):
        t = cls(list(indices), tuple(flux), list(dirs))
        for qns in enumerate_valid_sectors(indices, flux, dirs):
            t.blocks[key_pack(t.kind, qns)] = np.zeros(t.block_shape(qns))
        return t

    def set_block(self, qns, data: np.ndarray):
        shape = self.block_shape(qns)
        data = np.asarray(data, dtype=np.float64)
        if data.shape != shape:
            raise ValueError(f"block shape {data.shape} != {shape}")
        self.blocks[key_pack(self.kind, qns)] = data

    def sorted_keys(self) -> list:
        return sorted(self.blocks)

    def iter_blocks(self):
        for k in self.sorted_keys():
            yield key_unpack(self.kind, k, self.rank), self.blocks[k]

    def flatten(self):
        """FlatBlockStorage: (keys u64, offsets i64, data f64) in key order."""
        keys = self.sorted_keys()
        offs, parts, off = [], [], 0
        for k in keys:
            b = np.ascontiguousarray(self.blocks[k], dtype=np.float64).reshape(-1)
            offs.append(off)
            parts.append(b)
            off += b.size
        data = np.concatenate(parts) if parts else np.zeros(0)
        return (np.array(keys, dtype=np.uint64), np.array(offs, dtype=np.int64), data)

    def to_dense(self) -> np.ndarray:
        out = np.zeros([ix.total_dim for ix in self.indices])
        for qns, blk in self.iter_blocks():
            sl = tuple(slice(ix.offset_of(q), ix.offset_of(q) + ix.dim_of(q)) for ix, q in zip(self.indices, qns))
            out[sl] += blk
        return out

    def get_block(self, qns):
        """The block of sector `qns`, or None when the tensor stores none
        (block_sparse.rs:284-290)."""
        return self.blocks.get(key_pack(self.kind, qns))

    def permute(self, perm) -> "BlockSparseTensor":
        """Legs, directions and every block's axes reordered by `perm`, keys
        re-packed (block_sparse.rs:400-431).  Blocks are copied."""
        perm = [int(p) for p in perm]
        if sorted(perm) != list(range(self.rank)):
            raise ValueError(f"permute: {perm} is not a permutation of {self.rank} legs")
        out = BlockSparseTensor([self.indices[i] for i in perm], self.flux, [self.dirs[i] for i in perm])
        for qns, blk in self.iter_blocks():
            out.blocks[key_pack(self.kind, [qns[i] for i in perm])] = np.ascontiguousarray(blk.transpose(perm))
        return out

    def fuse_legs(self, start: int, end: int) -> "BlockSparseTensor":
        """Legs [start, end) fused into one Incoming leg (block_sparse.rs:444-611):
        its sectors are the fused charges of the sub-legs' sector combinations
        (each leg's charge dualised when Outgoing), ascending, and within one
        fused charge the combinations lie back to back in product order (first
        sub-leg slowest).  A block's fused axis takes the row-major merge of
        its sub-axes at the combination's offset."""
        if not 0 <= start < end <= self.rank:
            raise ValueError(f"fuse_legs: invalid range {start}..{end} for a rank-{self.rank} tensor")
        if end - start == 1:
            out = BlockSparseTensor(list(self.indices), self.flux, list(self.dirs))
            out.blocks = {k: b.copy() for k, b in self.blocks.items()}
            return out
        fused, where = fuse_map(self.kind, self.indices[start:end], self.dirs[start:end])
        out = BlockSparseTensor(self.indices[:start] + [fused] + self.indices[end:], self.flux,
                                self.dirs[:start] + [INCOMING] + self.dirs[end:])
        for qns, blk in self.iter_blocks():
            fq, off = where[tuple(qns[start:end])]
            new_q = list(qns[:start]) + [fq] + list(qns[end:])
            key = key_pack(self.kind, new_q)
            dst = out.blocks.get(key)
            if dst is None:
                dst = out.blocks[key] = np.zeros(out.block_shape(new_q))
            d = blk.shape
            width = int(np.prod(d[start:end]))
            dst[(slice(None),) * start + (slice(off, off + width),)] = blk.reshape(d[:start] + (width,) + d[end:])
        return out

    def split_leg(self, leg: int, original_indices, original_dirs) -> "BlockSparseTensor":
        """The inverse of fuse_legs (block_sparse.rs:622-793): leg `leg` split
        back into sub-legs with these QIndices and directions; every
        combination of sub-sectors that fuses to a stored block's charge
        becomes a block of its own (zero where the fused block held zeros)."""
        if not 0 <= leg < self.rank:
            raise ValueError(f"split_leg: leg {leg} out of range")
        original_indices, original_dirs = list(original_indices), list(original_dirs)
        if len(original_indices) != len(original_dirs):
            raise ValueError("split_leg: indices and directions length mismatch")
        if len(original_indices) <= 1:
            out = BlockSparseTensor(list(self.indices), self.flux, list(self.dirs))
            out.blocks = {k: b.copy() for k, b in self.blocks.items()}
            return out
        _, where = fuse_map(self.kind, original_indices, original_dirs)
        parts = {}
        for sub, (fq, off) in where.items():
            parts.setdefault(fq, []).append((sub, off))
        out = BlockSparseTensor(self.indices[:leg] + original_indices + self.indices[leg + 1:], self.flux,
                                self.dirs[:leg] + original_dirs + self.dirs[leg + 1:])
        for qns, blk in self.iter_blocks():
            for sub, off in parts.get(tuple(qns[leg]), []):
                dims = tuple(ix.dim_of(q) for ix, q in zip(original_indices, sub))
                width = int(np.prod(dims))
                piece = blk[(slice(None),) * leg + (slice(off, off + width),)]
                new_q = list(qns[:leg]) + list(sub) + list(qns[leg + 1:])
                out.blocks[key_pack(self.kind, new_q)] = np.ascontiguousarray(piece).reshape(
                    blk.shape[:leg] + dims + blk.shape[leg + 1:])
        return out


def fuse_map(kind: int, indices, dirs):
    """The fused leg of `indices` (with their directions) and where each
    combination of sub-sector charges lands in it: (QIndex, {charges tuple:
    (fused charge, offset)}), the layout fuse_legs and split_leg share."""
    combos = [((), identity(kind), 1)]
    for ix, d in zip(indices, dirs):
        combos = [(qs + (q,), fuse(kind, part, q if d == INCOMING else dual(kind, q)), dim * n)
                  for qs, part, dim in combos for q, n in ix.sectors]
    groups = {}
    for qs, fq, dim in combos:
        groups.setdefault(fq, []).append((qs, dim))
    sectors, where = [], {}
    for fq in sorted(groups):
        off = 0
        for qs, dim in groups[fq]:
            where[qs] = (fq, off)
            off += dim
        sectors.append((fq, off))
    return QIndex(kind, sectors), where
