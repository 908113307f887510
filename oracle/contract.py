"""CPU restatement of one pairwise block-sparse contraction step -- TEST
INFRASTRUCTURE ONLY (the checker of tk_contract_pairwise_f64).

Follows, step by step, kyungminlee/tensorkraft-design:
  tk-contract/src/sparse.rs:124-265     execute_pairwise_sparse / reshape_for_gemm
  tk-symmetry/src/block_sparse.rs:400-431  BlockSparseTensor::permute
  tk-symmetry/src/block_sparse.rs:444-611  BlockSparseTensor::fuse_legs
  tk-linalg/src/tasks.rs:36-81,180-188    compute_fusion_rule / compute_output_indices
  tk-linalg/src/device/faer.rs:390-575    DeviceFaer::block_gemm (accumulate per
                                          output key, output keys ascending)

A tensor here is a plain dict: kind, legs (list of [(charge tuple, dim), ...]
sorted by charge), dirs (0 Incoming / 1 Outgoing), flux (tuple) and blocks
({charge-tuple per leg: ndarray}).  Charges fuse as the reference's built-in
quantum numbers: U(1) components add, Z2 components xor.
"""
from __future__ import annotations

import numpy as np

U1, Z2, U1Z2, U1WIDE, U1U1 = 1, 2, 3, 4, 5


def _fuse(kind, a, b):
    if kind == Z2:
        return (a[0] ^ b[0],)
    if kind == U1Z2:
        return (a[0] + b[0], a[1] ^ b[1])
    if kind == U1U1:
        return (a[0] + b[0], a[1] + b[1])
    return (a[0] + b[0],)


def _dual(kind, a):
    if kind == Z2:
        return (a[0],)
    if kind == U1Z2:
        return (-a[0], a[1])
    if kind == U1U1:
        return (-a[0], -a[1])
    return (-a[0],)


def _identity(kind):
    return (0, 0) if kind in (U1Z2, U1U1) else (0,)


def _dim(leg, q):
    for c, d in leg:
        if c == q:
            return d
    raise KeyError(q)


def permute(t, perm):
    """block_sparse.rs:400-431: legs, directions and every block's axes reordered."""
    return {"kind": t["kind"], "legs": [t["legs"][i] for i in perm], "dirs": [t["dirs"][i] for i in perm],
            "flux": t["flux"],
            "blocks": {tuple(q[i] for i in perm): np.ascontiguousarray(np.transpose(b, perm))
                       for q, b in t["blocks"].items()}}


def fuse_legs(t, start, end):
    """block_sparse.rs:444-611: legs [start, end) into one Incoming leg whose
    sectors are the fused charges (BTreeMap order, i.e. ascending) of the
    Cartesian product of the sub-legs' sectors, combinations in product order."""
    kind = t["kind"]
    if end - start == 1:
        return {**t, "blocks": {q: b.copy() for q, b in t["blocks"].items()}}
    combos = [((), _identity(kind), 1)]
    for l in range(start, end):
        new = []
        for qns, part, dim in combos:
            for q, d in t["legs"][l]:
                eff = q if t["dirs"][l] == 0 else _dual(kind, q)
                new.append((qns + (q,), _fuse(kind, part, eff), dim * d))
        combos = new
    groups = {}
    for qns, fq, dim in combos:
        groups.setdefault(fq, []).append((qns, dim))
    fused_leg, offset_map = [], {}
    for fq in sorted(groups):
        off = 0
        for qns, dim in groups[fq]:
            offset_map[qns] = (fq, off)
            off += dim
        fused_leg.append((fq, off))
    legs = t["legs"][:start] + [fused_leg] + t["legs"][end:]
    dirs = t["dirs"][:start] + [0] + t["dirs"][end:]
    blocks = {}
    for qns, blk in t["blocks"].items():
        fq, foff = offset_map[tuple(qns[start:end])]
        new_q = tuple(qns[:start]) + (fq,) + tuple(qns[end:])
        dims = blk.shape
        ftot = _dim(fused_leg, fq)
        new_dims = dims[:start] + (ftot,) + dims[end:]
        nb = blocks.setdefault(new_q, np.zeros(new_dims))
        outer = int(np.prod(dims[:start])) if start > 0 else 1
        trail = int(np.prod(dims[end:])) if end < len(dims) else 1
        fdim = int(np.prod(dims[start:end]))
        src, dst = blk.reshape(-1), nb.reshape(-1)
        for o in range(outer):
            s0 = o * fdim * trail
            d0 = o * ftot * trail + foff * trail
            dst[d0:d0 + fdim * trail] = src[s0:s0 + fdim * trail]
    return {"kind": kind, "legs": legs, "dirs": dirs, "flux": t["flux"], "blocks": blocks}


def reshape_for_gemm(t, contracted, contracted_trailing):
    """sparse.rs:172-265."""
    rank = len(t["legs"])
    if rank == 2 and len(contracted) == 1:
        leg = contracted[0]
        if (contracted_trailing and leg == 1) or (not contracted_trailing and leg == 0):
            return t
    free = [i for i in range(rank) if i not in contracted]
    cont = [i for i in range(rank) if i in contracted]
    perm = free + cont if contracted_trailing else cont + free
    p = t if perm == list(range(rank)) else permute(t, perm)
    nc, nf = len(contracted), rank - len(contracted)
    if contracted_trailing:
        s1 = fuse_legs(p, 0, nf) if nf > 1 else p
        return fuse_legs(s1, 1, 1 + nc) if nc > 1 else s1
    s1 = fuse_legs(p, 0, nc) if nc > 1 else p
    return fuse_legs(s1, 1, 1 + nf) if nf > 1 else s1


def block_gemm(a, b, key_pack):
    """faer.rs:390-575 with tasks.rs:36-81: pairs with A's column charge ==
    B's row charge whose output (row, col) satisfies row (+) dual(col) ==
    flux_a (+) flux_b; same-key products summed; output in ascending packed
    key order.  Returns (tensor, ordered output keys)."""
    kind = a["kind"]
    target = _fuse(kind, a["flux"], b["flux"])
    out = {}
    for qa, ba in a["blocks"].items():
        for qb, bb in b["blocks"].items():
            if qa[1] != qb[0]:
                continue
            oq = (qa[0], qb[1])
            if _fuse(kind, oq[0], _dual(kind, oq[1])) != target:
                continue
            prod = ba @ bb
            out[oq] = out[oq] + prod if oq in out else prod
    order = sorted(out, key=lambda q: key_pack(kind, list(q)))
    return ({"kind": kind, "legs": [a["legs"][0], b["legs"][1]], "dirs": [a["dirs"][0], b["dirs"][1]],
             "flux": target, "blocks": out}, order)


def execute_pairwise_sparse(a, a_legs, b, b_legs, key_pack):
    """sparse.rs:124-163: reshape both operands, then block_gemm."""
    return block_gemm(reshape_for_gemm(a, list(a_legs), True), reshape_for_gemm(b, list(b_legs), False), key_pack)
