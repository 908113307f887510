"""Lanczos restatement (numpy) -- TEST INFRASTRUCTURE ONLY.

Follows LanczosSolver::lowest_eigenpair (tk-dmrg/src/eigensolver/mod.rs:80-164):
deterministic start vector ((i*7+13)%97)/97-0.5 (:96-101), normalisation,
k = min(max_krylov_dim, dim) steps with full re-orthogonalisation (:121-161),
stop when beta < 1e-15 (:152), eigenvalue by 100 Sturm-bisection steps
(:210-233, :277-297).  The reference's Ritz vector is never solved (:236-257);
this restatement returns the true tridiagonal eigenvector (scipy) instead.
"""
from __future__ import annotations

import numpy as np


def _count_below(d, e, mu):
    n = len(d)
    count = 0
    dp = d[0] - mu
    if dp < 0.0:
        count += 1
    for i in range(1, n):
        q = e[i - 1] * e[i - 1] / (1e-30 if abs(dp) < 1e-30 else dp)
        dd = d[i] - mu - q
        if dd < 0.0:
            count += 1
        dp = dd
    return count


def bisect_lowest(d, e):
    lo = min(d) - sum(abs(x) for x in e)
    hi = max(d) + sum(abs(x) for x in e)
    for _ in range(100):
        mid = 0.5 * (lo + hi)
        if _count_below(d, e, mid) >= 1:
            hi = mid
        else:
            lo = mid
    return 0.5 * (lo + hi)


def lowest_eigenpair(matvec, dim, krylov=100, x0=None):
    k = min(krylov, dim)
    v = np.array([((i * 7 + 13) % 97) / 97.0 - 0.5 for i in range(dim)]) if x0 is None else np.array(x0, float)
    nrm = np.linalg.norm(v)
    if nrm > 0:
        v = v / nrm
    V = [v]
    alpha, beta = [], []
    for j in range(k):
        w = matvec(V[j])
        a = float(V[j] @ w)
        alpha.append(a)
        w = w - a * V[j]
        if j > 0:
            w = w - beta[j - 1] * V[j - 1]
        for p in V:
            w = w - (p @ w) * p
        b = float(np.linalg.norm(w))
        if b < 1e-15 or j + 1 >= k:
            break
        beta.append(b)
        V.append(w / b)
    m = len(alpha)
    lam = bisect_lowest(alpha, beta[:m - 1])
    if m == 1:
        z = np.array([1.0])
    else:
        from scipy.linalg import eigh_tridiagonal

        w_, Z = eigh_tridiagonal(np.array(alpha), np.array(beta[:m - 1]))
        z = Z[:, 0]
    x = sum(zi * vi for zi, vi in zip(z, V[:m]))
    x = x / np.linalg.norm(x)
    return lam, x, m
