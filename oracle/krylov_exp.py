"""Krylov exponential restatement (numpy) -- TEST INFRASTRUCTURE ONLY.

Follows exp_krylov_f64 (tk-dmrg/src/tdvp/mod.rs:197-270) step by step:
m = min(krylov_dim, dim); beta = |v|, zeros when beta < 1e-30; Arnoldi with
one modified Gram-Schmidt pass filling the (m+1) x m Hessenberg matrix;
happy breakdown when the new norm is below tol (actual_m = j + 1); then
mat_exp_times_vec (:274-382) on alpha * H_m: s = max(0, ceil(log2(mean |a_ij|
/ 0.5))) scalings, the Taylor series of the vector when s = 0, else the
Taylor series of the matrix (20 terms, stop below 1e-16) squared s times;
result = V_m times that vector.  Works for complex alpha as well (numpy
complex arithmetic), which the reference does not.
"""
from __future__ import annotations

import math

import numpy as np


def _mat_exp_times_vec(a, n, beta):
    if n == 0:
        return np.zeros(0)
    a = np.asarray(a).reshape(n, n)
    norm = float(np.sum(np.abs(a))) / n
    s = max(0, math.ceil(math.log2(norm / 0.5))) if norm > 0 else 0
    scale = 2.0 ** (-s)
    res = np.zeros(n, dtype=a.dtype)
    res[0] = beta
    term = res.copy()
    for k in range(1, 21):
        term = (a * scale) @ term / k
        res = res + term
        if np.linalg.norm(term) < 1e-16 * abs(beta):
            break
    if s > 0:
        e = np.eye(n, dtype=a.dtype)
        t = e.copy()
        for k in range(1, 21):
            t = (a * scale) @ t / k
            e = e + t
            if np.linalg.norm(t) < 1e-16:
                break
        for _ in range(s):
            e = e @ e
        res = e[:, 0] * beta
    return res


def exp_krylov(matvec, v, alpha, dim, krylov_dim, tol):
    m = min(krylov_dim, dim)
    v = np.asarray(v)
    if m == 0 or dim == 0:
        return v.copy()
    beta = float(np.linalg.norm(v))
    if beta < 1e-30:
        return np.zeros(dim, dtype=np.result_type(v, alpha))
    V = [v / beta]
    H = np.zeros((m + 1, m), dtype=v.dtype)
    actual = m
    for j in range(m):
        w = matvec(V[j])
        for i in range(j + 1):
            d = np.vdot(V[i], w)
            H[i, j] = d
            w = w - d * V[i]
        hn = float(np.linalg.norm(w))
        H[j + 1, j] = hn
        if hn < tol:
            actual = j + 1
            break
        V.append(w / hn)
    hm = alpha * H[:actual, :actual]
    c = _mat_exp_times_vec(hm, actual, beta)
    return sum(ci * V[i] for i, ci in enumerate(c))
