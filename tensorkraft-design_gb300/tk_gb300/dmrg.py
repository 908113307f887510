"""Two-site DMRG sweeps around the device H_eff (the reference's caller).

Mirrors DMRGEngine::dmrg_step_two_site (tk-dmrg/src/sweep/mod.rs:348-448)
and the sweep schedule (sweep/mod.rs:72-81: left-to-right over bonds 0..N-2,
then right-to-left), with the pieces the reference leaves out done properly:
the right environment of bond (i, i+1) covers sites i+2.. (the reference
passes right(site+1) = sites site+3.., mod.rs:169-172), the Lanczos Ritz
vector is solved for, and the truncated SVD is written back into the MPS
(sweep/mod.rs:420-437 only reads the truncation error).

Environment growth follows contract_left/right_environment
(tk-dmrg/src/environments/mod.rs:225-483) on dense (bra, w, ket) blocks.
Truncation: block SVD per bond charge, ranked over all sectors (ties broken
by the sector's charge order so the kept set is deterministic) and cut by the
rule of truncate_svd (truncation/mod.rs:56-127: sigma >= cutoff * sigma_max,
at most max_bond, at least one), which does one dense SVD and assigns no
sectors.

The eigen-solver is pluggable: anything with
`solve(env_l, env_r, w_i, w_j, flux, theta_dense) -> (energy, vector)`;
`GpuSolver` runs Heff2Plan + tk_lanczos_lowest (FP64 or split precision).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .heff import Environment, Heff2Plan
from .models import ModelMPO
from .symmetry import QIndex, dual, fuse, identity


@dataclass
class DenseMPS:
    """MPS with dense site tensors A[s, aL, aR] (zeros outside charge blocks)
    and a charge-sorted QIndex per bond: bonds[i] is the bond left of site i
    (bonds[0] the left vacuum, bonds[n] the total charge).  Bond charges are
    cumulative from the left: q(s) + q(aL) = q(aR)."""

    kind: int
    phys: QIndex
    bonds: list        # n+1 QIndex
    tensors: list      # n arrays (d, DL, DR)

    @property
    def n(self):
        return len(self.tensors)


def _binom(n, k):
    return math.comb(n, k) if 0 <= k <= n else 0


def random_mps_u1(model: ModelMPO, n: int, max_bond: int, total, rng: np.random.Generator) -> DenseMPS:
    """Random U(1) MPS for spin-1/2 (2Sz charges +-1): every reachable bond
    charge gets a share of max_bond capped by its exact Hilbert-space count;
    blocks N(0,1); then right-canonicalised and normalised."""
    kind = model.kind
    tot = total[0]
    bonds = [QIndex(kind, [((0,), 1)])]
    for i in range(1, n):
        nl, nr = i, n - i
        sec = []
        for q in range(-nl, nl + 1, 2):
            cl = _binom(nl, (nl + q) // 2)
            cr = _binom(nr, (nr + (tot - q)) // 2) if (nr + tot - q) % 2 == 0 else 0
            cap = min(cl, cr)
            if cap > 0:
                sec.append((q, cap))
        w = np.array([math.exp(-(q * q) / (2.0 * max(1.0, 0.35 * math.sqrt(n)) ** 2)) for q, _ in sec])
        alloc = np.maximum(1, np.floor(w / w.sum() * max_bond)).astype(int)
        dims = [min(int(a), cap) for a, (_, cap) in zip(alloc, sec)]
        bonds.append(QIndex(kind, [((q,), d) for (q, _), d in zip(sec, dims) if d > 0]))
    bonds.append(QIndex(kind, [((tot,), 1)]))
    tensors = []
    pq = model.phys.state_charges()
    for i in range(n):
        bl, br = bonds[i], bonds[i + 1]
        A = np.zeros((model.phys.total_dim, bl.total_dim, br.total_dim))
        for s, qs in enumerate(pq):
            ol = 0
            for ql, dl in bl.sectors:
                qr = fuse(kind, ql, qs)
                orr = br.offset_of(qr)
                if orr is not None:
                    A[s, ol:ol + dl, orr:orr + br.dim_of(qr)] = rng.standard_normal((dl, br.dim_of(qr)))
                ol += dl
        tensors.append(A)
    mps = DenseMPS(kind, model.phys, bonds, tensors)
    right_canonicalize(mps)
    return mps


def _charge_counts(pq, kind, n):
    """Number of basis states of n sites per total charge (dict), by convolution."""
    counts = [{identity(kind): 1}]
    for _ in range(n):
        nxt = {}
        for q, c in counts[-1].items():
            for qs in pq:
                r = fuse(kind, q, qs)
                nxt[r] = nxt.get(r, 0) + c
        counts.append(nxt)
    return counts


def random_mps(model: ModelMPO, n: int, max_bond: int, total, rng: np.random.Generator, width: float = 0.35) -> DenseMPS:
    """Random MPS for any abelian model: bond i gets every charge q reachable
    from the left with total - q reachable from the right, weighted by a
    Gaussian in q around the uniform filling i/n * total (width
    width*sqrt(i(n-i)/n) per component), max_bond shared out by floor(weight
    share) capped by the state count (sectors rounding to 0 dropped); blocks
    N(0,1); then right-canonicalised and normalised."""
    kind = model.kind
    total = tuple(total)
    pq = model.phys.state_charges()
    cl = _charge_counts(pq, kind, n)
    bonds = [QIndex(kind, [(identity(kind), 1)])]
    for i in range(1, n):
        sec = []
        for q, c in cl[i].items():
            rest = fuse(kind, total, dual(kind, q))
            cr = cl[n - i].get(rest, 0)
            if cr > 0:
                sec.append((q, min(c, cr)))
        sig = max(0.5, width * math.sqrt(i * (n - i) / n))
        mean = [i / n * t for t in total]
        w = np.array([math.exp(-sum((qc - m) ** 2 for qc, m in zip(q, mean)) / (2 * sig * sig)) for q, _ in sec])
        share = np.floor(w / w.sum() * max_bond).astype(int)
        if share.max() == 0:
            share[int(np.argmax(w))] = 1
        secs = sorted((q, int(min(a, cap))) for (q, cap), a in zip(sec, share) if min(a, cap) > 0)
        bonds.append(QIndex(kind, secs))
    bonds.append(QIndex(kind, [(total, 1)]))
    tensors = []
    for i in range(n):
        bl, br = bonds[i], bonds[i + 1]
        A = np.zeros((model.phys.total_dim, bl.total_dim, br.total_dim))
        for s, qs in enumerate(pq):
            ol = 0
            for ql, dl in bl.sectors:
                qr = fuse(kind, ql, qs)
                orr = br.offset_of(qr)
                if orr is not None:
                    A[s, ol:ol + dl, orr:orr + br.dim_of(qr)] = rng.standard_normal((dl, br.dim_of(qr)))
                ol += dl
        tensors.append(A)
    mps = DenseMPS(kind, model.phys, bonds, tensors)
    right_canonicalize(mps)
    return mps


def _block_svd(M, row_q, col_q, kind):
    """SVD of M restricted to equal row/column charge; returns per-charge (q, U, S, Vt, rows, cols)."""
    out = []
    for q in sorted(set(row_q) & set(col_q)):
        r = np.array([i for i, x in enumerate(row_q) if x == q])
        c = np.array([j for j, x in enumerate(col_q) if x == q])
        U, S, Vt = np.linalg.svd(M[np.ix_(r, c)], full_matrices=False)
        out.append((q, U, S, Vt, r, c))
    return out


def right_canonicalize(mps: DenseMPS):
    """Sweeps right to left: A_i -> (LQ) so every A_i for i >= 1 is right-isometric."""
    kind = mps.kind
    pq = mps.phys.state_charges()
    for i in range(mps.n - 1, 0, -1):
        A = mps.tensors[i]
        d, DL, DR = A.shape
        M = A.transpose(1, 0, 2).reshape(DL, d * DR)
        row_q = [q for q, dd in mps.bonds[i].sectors for _ in range(dd)]
        col_q = [dual(kind, fuse(kind, qs, dual(kind, qr)))  # q(aL) = q(aR) - q(s)
                 for qs in pq for qr, dd in mps.bonds[i + 1].sectors for _ in range(dd)]
        blocks = _block_svd(M, row_q, col_q, kind)
        new_sec, Unew, Vnew = [], [], []
        for q, U, S, Vt, r, c in blocks:
            k = int(np.sum(S > 1e-14 * max(1.0, S[0]))) if S.size else 0
            if k == 0:
                continue
            new_sec.append((q, k))
            Unew.append((r, U[:, :k] * S[:k]))
            Vnew.append((c, Vt[:k]))
        nb = QIndex(kind, new_sec)
        Dn = nb.total_dim
        Us = np.zeros((DL, Dn))
        Vs = np.zeros((Dn, d * DR))
        for (q, k), (r, Uk), (c, Vk) in zip(new_sec, Unew, Vnew):
            o = nb.offset_of(q)
            Us[np.ix_(r, np.arange(o, o + k))] = Uk
            Vs[np.ix_(np.arange(o, o + k), c)] = Vk
        mps.tensors[i] = Vs.reshape(Dn, d, DR).transpose(1, 0, 2)
        mps.tensors[i - 1] = np.einsum("sab,bc->sac", mps.tensors[i - 1], Us)
        mps.bonds[i] = nb
    nrm = np.linalg.norm(mps.tensors[0])
    mps.tensors[0] /= nrm


def grow_left(L: np.ndarray, A: np.ndarray, W: np.ndarray) -> np.ndarray:
    """contract_left_environment (environments/mod.rs:223-355): L'[b', v, b]
    = sum conj(A[s', a', b']) L[a', w, a] W[s, s', w, v] A[s, a, b]."""
    t = np.einsum("pwa,sab->pwsb", L, A)
    t = np.einsum("pwsb,stwv->pvtb", t, W)
    return np.einsum("pvtb,tpc->cvb", t, A.conj())


def grow_right(R: np.ndarray, A: np.ndarray, W: np.ndarray) -> np.ndarray:
    """contract_right_environment (environments/mod.rs:357-483): R'[a', w, a]
    = sum conj(A[s', a', b']) R[b', v, b] W[s, s', w, v] A[s, a, b]."""
    t = np.einsum("pvb,sab->pvsa", R, A)
    t = np.einsum("pvsa,stwv->ptwa", t, W)
    return np.einsum("ptwa,tcp->cwa", t, A.conj())


class GpuSolver:
    """Device H_eff plan + device Lanczos (tk_heff2_plan_create + tk_lanczos_lowest)."""

    def __init__(self, precision: int = 0, krylov: int = 20, tol: float = 1e-12, restarts: int = 3, refine: int = 20,
                 device: int = 0):
        self.precision, self.krylov, self.tol, self.restarts, self.refine = precision, krylov, tol, restarts, refine
        self.device = device
        self.matvecs = 0

    def solve(self, env_l: Environment, env_r: Environment, wi, wj, flux, theta_dense: np.ndarray):
        import torch

        plan = Heff2Plan(env_l, env_r, wi, wj, psi_flux=flux, precision=self.precision, device=self.device)
        x0 = torch.from_numpy(plan.dense_to_flat(theta_dense.reshape(-1))).to(f"cuda:{self.device}")
        if float(torch.linalg.norm(x0)) == 0.0:
            x0 = None
        r = plan.lanczos(krylov_dim=self.krylov, max_restarts=self.restarts, tol=self.tol, refine=self.refine, x0=x0)
        self.matvecs += r.matvec_count
        vec = plan.flat_to_dense(r.eigenvector.cpu().numpy())
        plan.close()
        return r.eigenvalue, vec


@dataclass
class SweepStats:
    energies: list = field(default_factory=list)   # energy after each half sweep
    trunc: list = field(default_factory=list)      # max discarded weight per half sweep
    max_bond: list = field(default_factory=list)


def dmrg_two_site(model: ModelMPO, mps: DenseMPS, max_bond: int, sweeps: int, solver, total, cutoff: float = 1e-14):
    """Runs `sweeps` full (left-to-right + right-to-left) two-site sweeps in place."""
    kind, n = mps.kind, mps.n
    mpo = model.chain(n)
    Wd = [t.to_dense() for t in mpo.tensors]
    pq = mps.phys.state_charges()
    d = mps.phys.total_dim
    zero = identity(kind)
    # environments: Ls[i] covers sites < i, Rs[i] covers sites >= i
    Ls = [None] * (n + 1)
    Rs = [None] * (n + 1)
    Ls[0] = np.ones((1, 1, 1))
    Rs[n] = np.ones((1, 1, 1))
    for i in range(n - 1, 0, -1):
        Rs[i] = grow_right(Rs[i + 1], mps.tensors[i], Wd[i])
    stats = SweepStats()

    def env(data, bond, wq):
        return Environment(data, bond, wq, bond)

    def step(i, to_right):
        A, B = mps.tensors[i], mps.tensors[i + 1]
        theta = np.einsum("sab,tbc->stac", A, B)  # (s_i, s_j, aL, aR)
        bl, br = mps.bonds[i], mps.bonds[i + 2]
        wi, wj = mpo.tensors[i], mpo.tensors[i + 1]
        # bond charges are cumulative from the left, so the two-site flux is zero
        E, vec = solver.solve(env(Ls[i], bl, wi.indices[2]), env(Rs[i + 2], br, wj.indices[3]), wi, wj, zero,
                              theta)
        theta = vec.reshape(d, d, bl.total_dim, br.total_dim)
        # M[(s_i, aL), (s_j, aR)], row charge q(s_i)+q(aL), column charge q(aR)-q(s_j)
        M = theta.transpose(0, 2, 1, 3).reshape(d * bl.total_dim, d * br.total_dim)
        row_q = [fuse(kind, qs, ql) for qs in pq for ql, dd in bl.sectors for _ in range(dd)]
        col_q = [fuse(kind, qr, dual(kind, qs)) for qs in pq for qr, dd in br.sectors for _ in range(dd)]
        blocks = _block_svd(M, row_q, col_q, kind)
        allsv = [(s, bi) for bi, b in enumerate(blocks) for s in b[2]]
        allsv.sort(key=lambda t: (-t[0], t[1]))
        # truncate_svd (truncation/mod.rs:71-99): sigma >= cutoff * sigma_max, at most
        # max_bond, at least one; error = discarded share of sum sigma^2
        thr = cutoff * (allsv[0][0] if allsv else 0.0)
        nkeep = 0
        while nkeep < min(max_bond, len(allsv)) and not allsv[nkeep][0] < thr:
            nkeep += 1
        keep = allsv[:max(nkeep, min(1, len(allsv)))]
        kept = {}
        for s, bi in keep:
            kept[bi] = kept.get(bi, 0) + 1
        total_sq = sum(s * s for s, _ in allsv)
        disc = (sum(s * s for s, _ in allsv[len(keep):]) / total_sq) if total_sq > 0 else 0.0
        new_sec = [(blocks[bi][0], k) for bi, k in sorted(kept.items(), key=lambda t: blocks[t[0]][0])]
        nb = QIndex(kind, new_sec)
        Dn = nb.total_dim
        U = np.zeros((M.shape[0], Dn))
        V = np.zeros((Dn, M.shape[1]))
        for bi, k in kept.items():
            q, Ub, S, Vt, r, c = blocks[bi]
            o = nb.offset_of(q)
            cols = np.arange(o, o + k)
            if to_right:
                U[np.ix_(r, cols)] = Ub[:, :k]
                V[np.ix_(cols, c)] = S[:k, None] * Vt[:k]
            else:
                U[np.ix_(r, cols)] = Ub[:, :k] * S[:k]
                V[np.ix_(cols, c)] = Vt[:k]
        nrm = np.linalg.norm(V if to_right else U)
        if to_right:
            V /= nrm
        else:
            U /= nrm
        mps.tensors[i] = U.reshape(d, bl.total_dim, Dn)
        mps.tensors[i + 1] = V.reshape(Dn, d, br.total_dim).transpose(1, 0, 2)
        mps.bonds[i + 1] = nb
        if to_right:
            Ls[i + 1] = grow_left(Ls[i], mps.tensors[i], Wd[i])
        else:
            Rs[i + 1] = grow_right(Rs[i + 2], mps.tensors[i + 1], Wd[i + 1])
        return E, disc

    for _ in range(sweeps):
        for to_right, bonds in ((True, range(0, n - 1)), (False, range(n - 2, -1, -1))):
            e, tmax = None, 0.0
            for i in bonds:
                e, disc = step(i, to_right)
                tmax = max(tmax, disc)
            stats.energies.append(e)
            stats.trunc.append(tmax)
            stats.max_bond.append(max(b.total_dim for b in mps.bonds))
    return stats
