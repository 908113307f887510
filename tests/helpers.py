"""Shared test helpers: converts the product's host structures into oracle inputs."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "tensorkraft-design_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)

import oracle  # noqa: E402
from tk_gb300 import models  # noqa: E402
from tk_gb300.symmetry import QIndex  # noqa: E402


def qlegs(ix: QIndex):
    return ([list(q) for q, _ in ix.sectors], [d for _, d in ix.sectors])


def bst_legs(t):
    keys, offs, data = t.flatten()
    return ([qlegs(ix) for ix in t.indices], keys, offs, data)


def oracle_bs(prob, all_sectors=False):
    """Block-sparse oracle of a TwoSiteProblem."""
    Wi = prob.w_i.to_dense()
    Wj = prob.w_j.to_dense()
    return oracle.BlockSparseOracle(prob.kind, qlegs(prob.w_i.indices[0]), qlegs(prob.w_j.indices[0]),
                                    qlegs(prob.env_l.ket_idx), qlegs(prob.env_r.ket_idx),
                                    None if all_sectors else prob.flux, Wi, Wj, prob.env_l.data, prob.env_r.data)


def oracle_dense_factored(prob, x_dense):
    return oracle.heff_apply_dense(prob.w_i.to_dense(), prob.w_j.to_dense(), prob.env_l.data, prob.env_r.data,
                                   x_dense)


def oracle_dense_literal(prob):
    return oracle.heff_dense(prob.kind, bst_legs(prob.w_i), bst_legs(prob.w_j), prob.env_l.data, prob.env_r.data)


def small_problem(name: str, D: int, seed: int = 7):
    if name == "heisenberg":
        b = models.gaussian_bond_u1(D, 5, 1.5)
        return models.two_site_problem(models.heisenberg(), b, b, seed, "heisenberg")
    if name == "hubbard":
        bl = models.gaussian_bond_u1u1(D, 6, 1.5, 1.5, 4)
        br = models.gaussian_bond_u1u1(D, 8, 1.5, 1.5, 4)
        return models.two_site_problem(models.hubbard(), bl, br, seed, "hubbard")
    if name == "cylinder":
        rng = np.random.default_rng(seed)
        b = models.heavy_tailed_bond_u1(D, 9, rng)
        return models.two_site_problem(models.cylinder_j1(4), b, b, seed, "cylinder")
    raise KeyError(name)


def rel_err(a, b) -> float:
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _sorted_basis(charges):
    order = sorted(range(len(charges)), key=lambda k: charges[k])
    qs = [charges[k] for k in order]
    sectors = []
    for q in qs:
        if sectors and sectors[-1][0] == q:
            sectors[-1] = (q, sectors[-1][1] + 1)
        else:
            sectors.append((q, 1))
    return np.array(order), sectors


def exact_problem(model, n_sites: int, i: int, total):
    """Two-site problem on sites (i, i+1) of an n-site chain with L and R exact:
    the bond bases are the full product bases of the left/right blocks, so the
    lowest eigenvalue of H_eff in sector `total` is the exact ground energy."""
    from tk_gb300.heff import Environment
    from tk_gb300.symmetry import QIndex, fuse, dual

    kind = model.kind
    mpo = model.chain(n_sites)
    dense = [t.to_dense() for t in mpo.tensors]
    pq = model.phys.state_charges()
    zero = (0,) * len(total)
    # left block
    Lm = np.ones((1, 1, 1))
    qL = [zero]
    for k in range(i):
        W = dense[k]
        Lm = np.einsum("pwa,stwv->ptvas", Lm, W)
        p_, t_, v_, a_, s_ = Lm.shape
        Lm = Lm.reshape(p_ * t_, v_, a_ * s_)
        qL = [fuse(kind, qa, qs) for qa in qL for qs in pq]
    # right block
    Rm = np.ones((1, 1, 1))
    qR = [zero]
    for k in range(n_sites - 1, i + 1, -1):
        W = dense[k]
        Rm = np.einsum("stwv,pva->tpwsa", W, Rm)
        t_, p_, w_, s_, a_ = Rm.shape
        Rm = Rm.reshape(t_ * p_, w_, s_ * a_)
        qR = [fuse(kind, qs, qa) for qs in pq for qa in qR]
    labels_r = [dual(kind, q) for q in qR]
    oL, secL = _sorted_basis(qL)
    oR, secR = _sorted_basis(labels_r)
    Lm = Lm[np.ix_(oL, np.arange(Lm.shape[1]), oL)]
    Rm = Rm[np.ix_(oR, np.arange(Rm.shape[1]), oR)]
    wi, wj = mpo.tensors[i], mpo.tensors[i + 1]
    env_l = Environment(Lm, QIndex(kind, secL), wi.indices[2], QIndex(kind, secL))
    env_r = Environment(Rm, QIndex(kind, secR), wj.indices[3], QIndex(kind, secR))
    return models.TwoSiteProblem(kind, env_l, env_r, wi, wj, tuple(total), f"exact_{n_sites}_{i}")


def ed_heisenberg(n: int, J: float = 1.0) -> float:
    """Lowest energy in the Sz = 0 sector of the open Heisenberg chain."""
    Sz = np.diag([-0.5, 0.5])
    Sp = np.array([[0.0, 0.0], [1.0, 0.0]])
    Sm = Sp.T

    def op(m, k):
        out = np.array([[1.0]])
        for s in range(n):
            out = np.kron(out, m if s == k else np.eye(2))
        return out

    H = np.zeros((2 ** n, 2 ** n))
    for k in range(n - 1):
        H += J * (op(Sz, k) @ op(Sz, k + 1) + 0.5 * (op(Sp, k) @ op(Sm, k + 1) + op(Sm, k) @ op(Sp, k + 1)))
    sz = np.zeros(2 ** n)
    for idx in range(2 ** n):
        bits = [(idx >> (n - 1 - s)) & 1 for s in range(n)]
        sz[idx] = sum(1 if b else -1 for b in bits)
    sel = np.where(sz == 0)[0]
    return float(np.linalg.eigvalsh(H[np.ix_(sel, sel)])[0])


def ed_hubbard(n: int, t: float = 1.0, U: float = 4.0, N: int | None = None, sz2: int = 0) -> float:
    """Lowest energy of the open Hubbard chain in sector (N, 2Sz), from
    Jordan-Wigner fermion operators built independently of the MPO."""
    o = models.hubbard_local()
    a_up, a_dn, F = o["cdu"].T, o["cdd"].T, o["F"]
    N = n if N is None else N

    def site_op(m, k):
        out = np.array([[1.0]])
        for s in range(n):
            out = np.kron(out, m if s == k else (F if s < k else np.eye(4)))
        return out

    c = {(k, sg): site_op(a, k) for k in range(n) for sg, a in (("u", a_up), ("d", a_dn))}
    dim = 4 ** n
    H = np.zeros((dim, dim))
    for k in range(n - 1):
        for sg in "ud":
            hop = c[(k, sg)].T @ c[(k + 1, sg)]
            H += -t * (hop + hop.T)
    for k in range(n):
        H += U * (c[(k, "u")].T @ c[(k, "u")]) @ (c[(k, "d")].T @ c[(k, "d")])
    nt = sum(c[(k, s)].T @ c[(k, s)] for k in range(n) for s in "ud")
    s2 = sum(c[(k, "u")].T @ c[(k, "u")] - c[(k, "d")].T @ c[(k, "d")] for k in range(n))
    sel = np.where((np.abs(np.diag(nt) - N) < 1e-9) & (np.abs(np.diag(s2) - sz2) < 1e-9))[0]
    return float(np.linalg.eigvalsh(H[np.ix_(sel, sel)])[0])


def fermion_ops(n: int):
    """Jordan-Wigner annihilators c[(site, 'u'|'d')] on the 4^n Fock space (site 0 the
    most significant factor), in the sorted local basis of models.hubbard_local."""
    o = models.hubbard_local()
    a_up, a_dn, F = o["cdu"].T, o["cdd"].T, o["F"]

    def site_op(m, k):
        out = np.array([[1.0]])
        for s in range(n):
            out = np.kron(out, m if s == k else (F if s < k else np.eye(4)))
        return out

    return {(k, sg): site_op(a, k) for k in range(n) for sg, a in (("u", a_up), ("d", a_dn))}


def fermion_chain_dense(hop, U, eps):
    """Dense H of models.fermion_chain, built from fermion_ops (independently of the MPO)."""
    n = len(U)
    c = fermion_ops(n)
    H = np.zeros((4 ** n, 4 ** n))
    for k in range(n - 1):
        for sg in "ud":
            h = c[(k, sg)].T @ c[(k + 1, sg)]
            H += hop[k] * (h + h.T)
    for k in range(n):
        nu, nd = c[(k, "u")].T @ c[(k, "u")], c[(k, "d")].T @ c[(k, "d")]
        H += U[k] * nu @ nd + eps[k] * (nu + nd)
    return H, c


class CpuSolver:
    """DMRG eigen-solver on the CPU oracle: block-sparse FP64 matvec + numpy Lanczos."""

    def __init__(self, krylov=20, restarts=3, tol=1e-12):
        self.krylov, self.restarts, self.tol = krylov, restarts, tol

    def solve(self, env_l, env_r, wi, wj, flux, theta_dense):
        from oracle import lanczos

        orc = oracle.BlockSparseOracle(wi.kind, qlegs(wi.indices[0]), qlegs(wj.indices[0]), qlegs(env_l.ket_idx),
                                       qlegs(env_r.ket_idx), flux, wi.to_dense(), wj.to_dense(), env_l.data,
                                       env_r.data)
        x = orc.from_dense(theta_dense.reshape(-1))
        if np.linalg.norm(x) == 0:
            x = None
        for _ in range(self.restarts + 1):
            lam, x, _ = lanczos.lowest_eigenpair(orc.apply, orc.total, self.krylov, x0=x)
            r = orc.apply(x) - lam * x
            if np.linalg.norm(r) < self.tol:
                break
        return float(x @ orc.apply(x)), orc.to_dense(x)
