"""Davidson restatement (numpy) -- TEST INFRASTRUCTURE ONLY.

Follows DavidsonSolver::lowest_eigenpair (tk-dmrg/src/eigensolver/mod.rs:325-517)
step by step: deterministic start vector ((i*7+13)%97)/97-0.5 (:337-345),
max_sub = min(max_subspace, dim) (:332), projected matrix from basis_i . ab_j
on the upper triangle (:368-376), Jacobi eigen-solve of the small matrix
(symmetric_eigen_small, :532-601: largest off-diagonal pivot, angle
0.5*atan(2 a_pq / (a_pp - a_qq)), stop below 1e-15 or after 100 n^2 rotations),
Ritz vector and residual (:389-411), stop when |r| < tol (:413), optional
diagonal preconditioner r_i / (theta - d_i) where |theta - d_i| > 1e-14
(:427-437), one modified Gram-Schmidt pass (:440-446), raw-residual fallback
when the correction norm is below 1e-14 (:449-477), restart from the Ritz
vector with one matvec at max_sub (:485-500).
"""
from __future__ import annotations

import math

import numpy as np


def symmetric_eigen_small(mat, n):
    """Jacobi rotations with the largest off-diagonal pivot (mod.rs:532-601)."""
    a = np.array(mat, dtype=float).reshape(n, n).copy()
    v = np.eye(n)
    for _ in range(100 * n * n):
        max_val, p, q = 0.0, 0, 1
        for i in range(n):
            for j in range(i + 1, n):
                if abs(a[i, j]) > max_val:
                    max_val, p, q = abs(a[i, j]), i, j
        if max_val < 1e-15:
            break
        app, aqq, apq = a[p, p], a[q, q], a[p, q]
        theta = math.pi / 4 if abs(app - aqq) < 1e-30 else 0.5 * math.atan(2.0 * apq / (app - aqq))
        c, s = math.cos(theta), math.sin(theta)
        new = a.copy()
        for i in range(n):
            if i != p and i != q:
                new[i, p] = c * a[i, p] + s * a[i, q]
                new[p, i] = new[i, p]
                new[i, q] = -s * a[i, p] + c * a[i, q]
                new[q, i] = new[i, q]
        new[p, p] = c * c * app + 2.0 * s * c * apq + s * s * aqq
        new[q, q] = s * s * app - 2.0 * s * c * apq + c * c * aqq
        new[p, q] = new[q, p] = 0.0
        a = new
        vp, vq = v[:, p].copy(), v[:, q].copy()
        v[:, p] = c * vp + s * vq
        v[:, q] = -s * vp + c * vq
    return np.diag(a).copy(), v


def lowest_eigenpair(matvec, dim, max_subspace=60, max_iter=1000, tol=1e-10, diagonal=None, x0=None):
    """Returns (eigenvalue, eigenvector, converged, matvec_count, residual_norm)."""
    max_sub = min(max_subspace, dim)
    v0 = (np.array([((i * 7 + 13) % 97) / 97.0 - 0.5 for i in range(dim)]) if x0 is None
          else np.array(x0, dtype=float))
    nrm = np.linalg.norm(v0)
    if nrm > 0:
        v0 = v0 / nrm
    basis, ab = [v0], [matvec(v0)]
    count = 1
    eigenvalue, eigenvector, rnorm = 0.0, v0.copy(), math.inf
    for _ in range(max_iter):
        nsub = len(basis)
        h = np.zeros((nsub, nsub))
        for i in range(nsub):
            for j in range(i, nsub):
                h[i, j] = h[j, i] = basis[i] @ ab[j]
        evals, evecs = symmetric_eigen_small(h, nsub)
        k = int(np.argmin(evals))
        eigenvalue = float(evals[k])
        c = evecs[:, k]
        eigenvector = sum(ci * b for ci, b in zip(c, basis))
        residual = sum(ci * a for ci, a in zip(c, ab)) - eigenvalue * eigenvector
        rnorm = float(np.linalg.norm(residual))
        if rnorm < tol:
            return eigenvalue, eigenvector, True, count, rnorm
        corr = residual.copy()
        if diagonal is not None:
            den = eigenvalue - np.asarray(diagonal, dtype=float)
            big = np.abs(den) > 1e-14
            corr[big] = corr[big] / den[big]
        for b in basis:
            corr = corr - (b @ corr) * b
        cn = np.linalg.norm(corr)
        if cn < 1e-14:
            raw = residual.copy()
            for b in basis:
                raw = raw - (b @ raw) * b
            rn2 = np.linalg.norm(raw)
            if rn2 < 1e-14:
                break
            corr = raw / rn2
        else:
            corr = corr / cn
        if nsub >= max_sub:
            if nsub >= dim:
                break
            basis, ab = [eigenvector.copy()], [matvec(eigenvector)]
            count += 1
            continue
        basis.append(corr)
        ab.append(matvec(corr))
        count += 1
    return eigenvalue, eigenvector, rnorm < tol, count, rnorm
