"""MPOs and synthetic two-site workloads.

The reference's MPO compiler is a stub (tk-dmrg/src/mpo/mod.rs:126-145), so
the Heisenberg (bond 5), Hubbard (bond 6, Jordan-Wigner) and J1-cylinder
(bond 14) MPOs are written out as site tensors in the reference's layout
(s_in, s_out, w_L, w_R), W[s_in, s_out, wl, wr] = <s_out| op |s_in>.

MPO-bond charges follow q(w_R) = q(w_L) + q(s_out) - q(s_in); environments
then satisfy q(a') = q(a) + q(w) for L(a', w, a) and R(a', w, a), and the
two-site blocks satisfy q(s_i) + q(s_j) + q(a_L) = q(a_R) + flux.

Every channel c has an adjoint partner pi(c) (S+ <-> S-, c^dag F <-> F c)
with W[s_out, s_in, pi wl, pi wr] = W[s_in, s_out, wl, wr]; environments
built with L_pi(w) = L_w^T make H_eff symmetric.

Synthetic inputs use a seeded numpy Generator (PCG64) -- N(0,1) blocks.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .heff import Environment, MPO
from .symmetry import INCOMING, OUTGOING, U1, U1U1, BlockSparseTensor, QIndex, key_pack

# ----------------------------------------------------------------------------
# generic site tensor from channel lists
# ----------------------------------------------------------------------------


def channel_qindex(kind, charges):
    """QIndex of an MPO bond + map channel -> global (sorted, stable) index."""
    order = sorted(range(len(charges)), key=lambda c: tuple(charges[c]))
    glob = {c: g for g, c in enumerate(order)}
    sectors = {}
    for c in order:
        q = tuple(charges[c])
        sectors[q] = sectors.get(q, 0) + 1
    return QIndex(kind, list(sectors.items())), glob


def dense_to_bst(kind, dense, legs, dirs, flux):
    """Cuts a dense tensor into the blocks of `legs` that hold non-zeros."""
    t = BlockSparseTensor(list(legs), tuple(flux), list(dirs))
    offs = []
    for ix in legs:
        o, lst = 0, []
        for q, d in ix.sectors:
            lst.append((q, o, d))
            o += d
        offs.append(lst)
    import itertools

    for combo in itertools.product(*offs):
        sl = tuple(slice(o, o + d) for (_, o, d) in combo)
        blk = dense[sl]
        if np.any(blk != 0.0):
            t.blocks[key_pack(kind, [q for (q, _, _) in combo])] = np.array(blk, dtype=np.float64)
    return t


def site_tensor(kind, phys: QIndex, wl_charges, wr_charges, entries):
    """entries: list of (wl channel, wr channel, matrix[out, in]) in sorted physical order."""
    wlq, wlg = channel_qindex(kind, wl_charges)
    wrq, wrg = channel_qindex(kind, wr_charges)
    d = phys.total_dim
    W = np.zeros((d, d, wlq.total_dim, wrq.total_dim))
    for wl, wr, m in entries:
        W[:, :, wlg[wl], wrg[wr]] += np.asarray(m, dtype=np.float64).T  # W[s_in, s_out] = m[s_out, s_in]
    zero = (0,) * (2 if kind == U1U1 else 1)
    t = dense_to_bst(kind, W, [phys, phys, wlq, wrq], [INCOMING, OUTGOING, OUTGOING, INCOMING], zero)
    return t, wlg, wrg


@dataclass
class ModelMPO:
    kind: int
    phys: QIndex
    bulk: BlockSparseTensor          # W with full bonds on both sides
    first: BlockSparseTensor         # left edge (w_L = start channel only)
    last: BlockSparseTensor          # right edge (w_R = end channel only)
    pi: np.ndarray                   # adjoint involution on the sorted bond index
    bond: QIndex                     # MPO bond QIndex

    def chain(self, n_sites: int) -> MPO:
        ts = [self.first] + [self.bulk] * (n_sites - 2) + [self.last]
        return MPO(ts, [self.phys.total_dim] * n_sites, (0,) * (2 if self.kind == U1U1 else 1))


def _model(kind, phys, charges, entries, start, end, partner):
    bulk, wlg, _ = site_tensor(kind, phys, charges, charges, entries)
    first, _, _ = site_tensor(kind, phys, [charges[start]], charges,
                              [(0, wr, m) for (wl, wr, m) in entries if wl == start])
    last, _, _ = site_tensor(kind, phys, charges, [charges[end]],
                             [(wl, 0, m) for (wl, wr, m) in entries if wr == end])
    bond, _ = channel_qindex(kind, charges)
    pi = np.zeros(len(charges), dtype=np.int64)
    for c in range(len(charges)):
        pi[wlg[c]] = wlg[partner.get(c, c)]
    return ModelMPO(kind, phys, bulk, first, last, pi, bond)


# ----------------------------------------------------------------------------
# spin-1/2 Heisenberg, U(1) 2Sz, bond 5
# ----------------------------------------------------------------------------


def heisenberg(J: float = 1.0) -> ModelMPO:
    phys = QIndex(U1, [((-1,), 1), ((1,), 1)])  # states: down, up
    I = np.eye(2)
    Sz = np.diag([-0.5, 0.5])
    Sp = np.array([[0.0, 0.0], [1.0, 0.0]])  # |up><down|
    Sm = Sp.T
    # channels: 0 start, 1 after S+, 2 after S-, 3 after Sz, 4 end
    charges = [(0,), (2,), (-2,), (0,), (0,)]
    entries = [(0, 0, I), (0, 1, 0.5 * J * Sp), (0, 2, 0.5 * J * Sm), (0, 3, J * Sz),
               (1, 4, Sm), (2, 4, Sp), (3, 4, Sz), (4, 4, I)]
    return _model(U1, phys, charges, entries, 0, 4, {1: 2, 2: 1})


# ----------------------------------------------------------------------------
# Fermi-Hubbard, U(1)xU(1) (N, 2Sz), bond 6, Jordan-Wigner
# ----------------------------------------------------------------------------


def hubbard_local():
    """Local operators in the sorted basis [0, dn, up, updn] ((N,2Sz) ascending)."""
    # standard order [0, up, dn, updn], |updn> = c+_up c+_dn |0>
    cdu = np.zeros((4, 4))
    cdu[1, 0] = 1.0   # |0> -> |up>
    cdu[3, 2] = 1.0   # |dn> -> |updn>
    cdd = np.zeros((4, 4))
    cdd[2, 0] = 1.0   # |0> -> |dn>
    cdd[3, 1] = -1.0  # |up> -> -|updn>
    F = np.diag([1.0, -1.0, -1.0, 1.0])
    nu = np.diag([0.0, 1.0, 0.0, 1.0])
    nd = np.diag([0.0, 0.0, 1.0, 1.0])
    perm = [0, 2, 1, 3]  # sorted index -> standard index
    P = np.eye(4)[perm]
    tr = lambda m: P @ m @ P.T
    return {k: tr(v) for k, v in dict(cdu=cdu, cdd=cdd, F=F, nu=nu, nd=nd, I=np.eye(4)).items()}


def hubbard(t: float = 1.0, U: float = 4.0) -> ModelMPO:
    phys = QIndex(U1U1, [((0, 0), 1), ((1, -1), 1), ((1, 1), 1), ((2, 0), 1)])
    o = hubbard_local()
    cdu, cdd, F, I = o["cdu"], o["cdd"], o["F"], o["I"]
    cu, cd = cdu.T, cdd.T
    # channels: 0 start, 1 after c+up F, 2 after F cup, 3 after c+dn F, 4 after F cdn, 5 end
    charges = [(0, 0), (1, 1), (-1, -1), (1, -1), (-1, 1), (0, 0)]
    entries = [(0, 0, I), (0, 1, -t * (cdu @ F)), (0, 2, -t * (F @ cu)), (0, 3, -t * (cdd @ F)),
               (0, 4, -t * (F @ cd)), (1, 5, cu), (2, 5, cdu), (3, 5, cd), (4, 5, cdd),
               (0, 5, U * (o["nu"] @ o["nd"])), (5, 5, I)]
    return _model(U1U1, phys, charges, entries, 0, 5, {1: 2, 2: 1, 3: 4, 4: 3})


# ----------------------------------------------------------------------------
# Fermion chains with site-dependent couplings (Anderson impurity, chain geometry)
# ----------------------------------------------------------------------------


@dataclass
class ChainModel:
    """A chain MPO with its own tensor on every site (same interface as ModelMPO.chain)."""

    kind: int
    phys: QIndex
    tensors: list

    def chain(self, n_sites: int) -> MPO:
        if n_sites != len(self.tensors):
            raise ValueError("ChainModel has a fixed length")
        return MPO(list(self.tensors), [self.phys.total_dim] * n_sites, (0,) * (2 if self.kind == U1U1 else 1))


def fermion_chain(hop, U, eps) -> ChainModel:
    """H = sum_i hop[i] sum_s (c+_{i s} c_{i+1 s} + h.c.) + sum_i U[i] n_{i up} n_{i dn}
    + sum_i eps[i] (n_{i up} + n_{i dn}); (N, 2Sz) charges, Jordan-Wigner strings as in
    `hubbard` (which is the uniform case hop = -t)."""
    n = len(U)
    if len(eps) != n or len(hop) != n - 1:
        raise ValueError("need n on-site terms and n-1 hoppings")
    phys = QIndex(U1U1, [((0, 0), 1), ((1, -1), 1), ((1, 1), 1), ((2, 0), 1)])
    o = hubbard_local()
    cdu, cdd, F, I = o["cdu"], o["cdd"], o["F"], o["I"]
    cu, cd = cdu.T, cdd.T
    charges = [(0, 0), (1, 1), (-1, -1), (1, -1), (-1, 1), (0, 0)]
    tensors = []
    for i in range(n):
        onsite = U[i] * (o["nu"] @ o["nd"]) + eps[i] * (o["nu"] + o["nd"])
        t = hop[i] if i < n - 1 else 0.0
        entries = [(0, 0, I), (0, 1, t * (cdu @ F)), (0, 2, t * (F @ cu)), (0, 3, t * (cdd @ F)),
                   (0, 4, t * (F @ cd)), (1, 5, cu), (2, 5, cdu), (3, 5, cd), (4, 5, cdd), (0, 5, onsite),
                   (5, 5, I)]
        if i == 0:
            w, _, _ = site_tensor(U1U1, phys, [charges[0]], charges, [(0, wr, m) for (wl, wr, m) in entries if wl == 0])
        elif i == n - 1:
            w, _, _ = site_tensor(U1U1, phys, charges, [charges[5]], [(wl, 0, m) for (wl, wr, m) in entries if wr == 5])
        else:
            w, _, _ = site_tensor(U1U1, phys, charges, charges, entries)
        tensors.append(w)
    return ChainModel(U1U1, phys, tensors)


def anderson_chain(n: int, U: float = 3.0, seed: int = 5, v: float = 0.5) -> ChainModel:
    """Single-impurity Anderson model in chain geometry (impurity = site 0, n-1 bath
    sites): U on the impurity at half filling (eps_d = -U/2), impurity-bath hopping v,
    seeded bath on-site energies eps_k ~ 0.1 N(0,1) and chain hoppings 0.5 (1 + 0.1 N(0,1))."""
    rng = np.random.default_rng(seed)
    hop = [v] + list(0.5 * (1.0 + 0.1 * rng.standard_normal(n - 2)))
    eps = [-0.5 * U] + list(0.1 * rng.standard_normal(n - 1))
    Us = [U] + [0.0] * (n - 1)
    return fermion_chain(hop, Us, eps)


# ----------------------------------------------------------------------------
# J1 Heisenberg on a width-W cylinder, column-major (snake) ordering, bond 2+3W
# ----------------------------------------------------------------------------


def cylinder_j1(width: int = 4, J: float = 1.0) -> ModelMPO:
    """Nearest-neighbour couplings reach at most `width` sites along the chain;
    the MPO keeps 3 operator channels per open distance (bond 2 + 3*width).
    Bulk tensor: every coupling distance a column-major site can have --
    1 (rung), width-1 (periodic rung) and width (leg) -- carries J."""
    phys = QIndex(U1, [((-1,), 1), ((1,), 1)])
    I = np.eye(2)
    Sz = np.diag([-0.5, 0.5])
    Sp = np.array([[0.0, 0.0], [1.0, 0.0]])
    Sm = Sp.T
    W = width
    # channels: 0 start, then (op, distance r) for r = 1..W as 1 + 3*(r-1) + {0:S+,1:S-,2:Sz}, end = 1 + 3W
    end = 1 + 3 * W
    charges = [(0,)] + [q for _ in range(W) for q in ((2,), (-2,), (0,))] + [(0,)]
    ch = lambda op, r: 1 + 3 * (r - 1) + op
    couple = {1: J, W - 1: J, W: J}  # rung, periodic rung, leg
    entries = [(0, 0, I), (end, end, I)]
    for op, m in ((0, 0.5 * Sp), (1, 0.5 * Sm), (2, Sz)):
        entries.append((0, ch(op, 1), m))
        for r in range(1, W):
            entries.append((ch(op, r), ch(op, r + 1), I))
        closing = {0: Sm, 1: Sp, 2: Sz}[op]
        for r, c in couple.items():
            entries.append((ch(op, r), end, c * closing))
    partner = {}
    for r in range(1, W + 1):
        partner[ch(0, r)] = ch(1, r)
        partner[ch(1, r)] = ch(0, r)
    return _model(U1, phys, charges, entries, 0, end, partner)


# ----------------------------------------------------------------------------
# synthetic bonds, environments and two-site vectors
# ----------------------------------------------------------------------------


def largest_remainder(weights, total):
    w = np.asarray(weights, dtype=np.float64)
    raw = w / w.sum() * total
    base = np.floor(raw).astype(np.int64)
    rem = total - base.sum()
    order = np.argsort(-(raw - base), kind="stable")
    base[order[:rem]] += 1
    return base


def gaussian_bond_u1(D: int, n_sectors: int = 15, s: float = 3.0, step: int = 2, center: int = 0) -> QIndex:
    """Sz sectors k = -(n-1)/2 .. (n-1)/2 (charge step*k + center), dims ~ exp(-k^2/2s^2), sum D."""
    h = (n_sectors - 1) // 2
    ks = np.arange(-h, h + 1)
    dims = largest_remainder(np.exp(-ks.astype(float) ** 2 / (2 * s * s)), D)
    return QIndex(U1, [((int(step * k + center),), int(d)) for k, d in zip(ks, dims) if d > 0])


def gaussian_bond_u1u1(D: int, n0: int, sn: float = 3.5, ss: float = 3.0, kmax: int = 10) -> QIndex:
    """(N, 2Sz) sectors around (n0, 0), N = n0 + dn with dn = 2Sz (mod 2); dims ~ Gaussian, sum D."""
    pts, ws = [], []
    for dn in range(-kmax, kmax + 1):
        for sz in range(-kmax, kmax + 1):
            if (dn - sz) % 2:
                continue
            pts.append((n0 + dn, sz))
            ws.append(np.exp(-dn * dn / (2 * sn * sn) - sz * sz / (2 * ss * ss)))
    dims = largest_remainder(ws, D)
    return QIndex(U1U1, [(p, int(d)) for p, d in zip(pts, dims) if d > 0])


def heavy_tailed_bond_u1(D: int, n_sectors: int, rng: np.random.Generator, alpha: float = 1.3,
                         step: int = 2) -> QIndex:
    """~n_sectors Sz sectors with power-law dims (a few large, many small), sum D.

    The r-th largest weight is r^-alpha times a seeded +-20% jitter, so for
    D=4096, 41 sectors, alpha=1.3 a few sectors exceed 500 and about a
    quarter stay below 16."""
    h = (n_sectors - 1) // 2
    ks = np.arange(-h, h + 1)
    w = (np.arange(1, len(ks) + 1, dtype=float) ** -alpha) * rng.uniform(0.8, 1.2, size=len(ks))
    w = np.sort(w)[::-1]
    # largest weights near Sz = 0, alternating sides
    order = sorted(range(len(ks)), key=lambda i: (abs(ks[i]), ks[i]))
    ww = np.zeros(len(ks))
    for rank, i in enumerate(order):
        ww[i] = w[rank]
    dims = largest_remainder(ww, D)
    dims = np.maximum(dims, 1)
    while dims.sum() > D:
        dims[np.argmax(dims)] -= 1
    return QIndex(U1, [((int(step * k),), int(d)) for k, d in zip(ks, dims) if d > 0])


def random_environment(bond: QIndex, wq: QIndex, pi: np.ndarray, rng: np.random.Generator) -> Environment:
    """N(0,1) on every block with q(a') = q(a) + q(w); L_pi(w) = L_w^T."""
    from .symmetry import fuse

    kind = bond.kind
    D, nw = bond.total_dim, wq.total_dim
    data = np.zeros((D, nw, D))
    wch = wq.state_charges()
    offs = []
    o = 0
    for q, d in bond.sectors:
        offs.append((q, o, d))
        o += d
    for w in range(nw):
        if pi[w] < w:
            continue
        for (qa, oa, da) in offs:
            qb = fuse(kind, qa, wch[w])
            ob = bond.offset_of(qb)
            if ob is None:
                continue
            db = bond.dim_of(qb)
            data[ob:ob + db, w, oa:oa + da] = rng.standard_normal((db, da))
        M = data[:, w, :]
        if pi[w] == w:
            data[:, w, :] = 0.5 * (M + M.T)
        else:
            data[:, pi[w], :] = M.T
    return Environment(data, bond, wq, bond)


@dataclass
class TwoSiteProblem:
    kind: int
    env_l: Environment
    env_r: Environment
    w_i: BlockSparseTensor
    w_j: BlockSparseTensor
    flux: tuple
    name: str

    def plan(self, precision=0, device=0, all_sectors=False):
        from .heff import Heff2Plan

        return Heff2Plan(self.env_l, self.env_r, self.w_i, self.w_j,
                         psi_flux=None if all_sectors else self.flux, precision=precision, device=device)


def two_site_problem(model: ModelMPO, bond_l: QIndex, bond_r: QIndex, seed: int, name: str = "",
                     flux=None) -> TwoSiteProblem:
    rng = np.random.default_rng(seed)
    env_l = random_environment(bond_l, model.bond, model.pi, rng)
    env_r = random_environment(bond_r, model.bond, model.pi, rng)
    if flux is None:
        flux = (0,) * (2 if model.kind == U1U1 else 1)
    return TwoSiteProblem(model.kind, env_l, env_r, model.bulk, model.bulk, tuple(flux), name)


def workload(name: str, seed: int = 1234, scale: float = 1.0) -> TwoSiteProblem:
    """The named synthetic workloads; `scale` shrinks D for quick checks."""
    if name == "heisenberg_d1024":
        D = max(16, int(1024 * scale))
        b = gaussian_bond_u1(D, 15, 3.0)
        return two_site_problem(heisenberg(), b, b, seed, name)
    if name == "hubbard_d2048":
        D = max(32, int(2048 * scale))
        bl = gaussian_bond_u1u1(D, 30)
        br = gaussian_bond_u1u1(D, 32)
        return two_site_problem(hubbard(), bl, br, seed, name)
    if name == "cylinder_d4096":
        D = max(64, int(4096 * scale))
        rng = np.random.default_rng(seed + 7)
        b = heavy_tailed_bond_u1(D, 41, rng)
        return two_site_problem(cylinder_j1(4), b, b, seed, name)
    raise KeyError(name)
