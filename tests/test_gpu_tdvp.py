"""Device Krylov exponential (tk_expm_krylov) against the reference's
exp_krylov_f64 known answers, the numpy restatement and scipy's expm, and
imaginary-time two-site TDVP sweeps against exact diagonalisation."""
import json
from pathlib import Path

import numpy as np
import pytest

from helpers import ed_heisenberg, models, oracle_dense_literal, small_problem
from test_gpu_lanczos import matrix_plan
from tk_gb300 import PREC_FP64, sweep

# pairwise contraction order with intermediates allowed to exceed the inputs (numpy's
# default limit, the largest operand, falls back to one nested loop over every index)
_PATH = ("greedy", 2 ** 34)

pytestmark = pytest.mark.gpu
KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float64)).cuda()


@pytest.mark.parametrize("case", KATS["exp_krylov"], ids=lambda c: c["source"].split("(")[-1][:-1])
def test_expm_kats(lib_built, case):
    M = np.diag(case["diag"]).astype(float) if case["matrix"] == "diag" else np.array(case["dense"], float)
    plan = matrix_plan(M)
    v = np.array(case["v"], float)
    out, _, used, _ = plan.expm(case["alpha"], _dev(v), krylov_dim=case["krylov"], tol=case["tol"])
    from scipy.linalg import expm

    assert np.allclose(out.cpu().numpy(), expm(case["alpha"] * M) @ v, atol=case["atol"], rtol=0)


def test_expm_follows_restatement_and_breakdown(lib_built):
    """Same result as the numpy exp_krylov_f64 with a truncated Krylov space; the
    breakdown cut on a 3-dimensional invariant space."""
    from oracle import krylov_exp

    rng = np.random.default_rng(9)
    A = rng.standard_normal((40, 40))
    M = (A + A.T) / 2
    plan = matrix_plan(M)
    v = rng.standard_normal(40)
    for k in (8, 20):
        out, _, used, mv = plan.expm(-0.2, _dev(v), krylov_dim=k, tol=1e-12)
        ref = krylov_exp.exp_krylov(lambda x: M @ x, v, -0.2, 40, k, 1e-12)
        assert used == k and mv == k
        assert np.allclose(out.cpu().numpy(), ref, atol=1e-10 * np.linalg.norm(ref), rtol=0)
    D = np.diag([1.0] * 10 + [2.0] * 10 + [5.0] * 20)
    out, _, used, _ = matrix_plan(D).expm(-0.1, _dev(np.ones(40)), krylov_dim=30, tol=1e-10)
    assert used == 3
    assert np.allclose(out.cpu().numpy(), np.exp(-0.1 * np.diag(D)), atol=1e-12, rtol=0)


@pytest.mark.parametrize("alpha,cplx", [(-0.3, False), (-0.7j, False), (-0.7j, True), (0.1 - 0.4j, True)])
def test_expm_heff_matches_scipy(lib_built, alpha, cplx):
    """exp(alpha H_eff) v on a two-site H_eff (all sectors), real and complex alpha and v."""
    from scipy.linalg import expm

    p = small_problem("heisenberg", 10)
    plan = p.plan(all_sectors=True)
    H = oracle_dense_literal(p)
    rng = np.random.default_rng(3)
    vr, vi = rng.standard_normal(H.shape[0]), rng.standard_normal(H.shape[0]) if cplx else None
    v = vr + (1j * vi if cplx else 0)
    ref = expm(alpha * H) @ v
    out_re, out_im, _, _ = plan.expm(alpha, _dev(plan.dense_to_flat(vr)),
                                     _dev(plan.dense_to_flat(vi)) if cplx else None, krylov_dim=40, tol=1e-12)
    got = plan.flat_to_dense(out_re.cpu().numpy()) + (1j * plan.flat_to_dense(out_im.cpu().numpy())
                                                       if out_im is not None else 0)
    assert np.linalg.norm(got - ref) < 1e-10 * np.linalg.norm(ref)


def test_imaginary_time_tdvp_reaches_ground_state(lib_built):
    """exp(-tau H) by two-site TDVP from a random MPS: the energy falls to exact diagonalisation."""
    m = models.heisenberg()
    sites, bonds = sweep.random_site_tensors(m, 10, 32, (0,), np.random.default_rng(3))
    d = sweep.DeviceDMRG(m, sites, bonds, precision=PREC_FP64, krylov=20)
    rec = sweep.SweepRecord()
    energies = [d.tdvp_step(1.5, 32, rec) for _ in range(30)]
    assert all(b <= a + 1e-9 for a, b in zip(energies[5:], energies[6:]))
    assert abs(energies[-1] - ed_heisenberg(10)) < 1e-8


@pytest.mark.parametrize("name,D", [("heisenberg", 12), ("hubbard", 10)])
def test_single_site_closure_matches_dense(lib_built, name, D):
    """build_heff_single_site (a two-site plan with a dummy second site) == the reference's dense H."""
    from oracle import environments as oe
    from tk_gb300.heff import MPO, build_heff_single_site

    p = small_problem(name, D)
    mpo = MPO([p.w_i], [p.w_i.indices[0].total_dim], p.flux)
    matvec, dim = build_heff_single_site(p.env_l, p.env_r, mpo, 0)
    H = oe.heff_single_site_dense(p.env_l.data, p.w_i.to_dense(), p.env_r.data)
    assert dim == H.shape[0]
    rng = np.random.default_rng(2)
    for _ in range(2):
        x = rng.standard_normal(dim)
        y = np.zeros(dim)
        matvec(x, y)
        assert np.linalg.norm(y - H @ x) < 1e-12 * np.linalg.norm(H @ x)


def _dense_state(sites):
    v = np.ones((1,), dtype=complex)
    for t in sites:
        A = t.to_dense()
        v = np.einsum("xa,sab->xsb", v.reshape(-1, A.shape[1]), A).reshape(-1, A.shape[2])
    return v.reshape(-1)


def _heisenberg_dense(n):
    sz = np.diag([-0.5, 0.5])
    sp = np.array([[0.0, 0.0], [1.0, 0.0]])
    eye = np.eye(2)

    def site(o, k):
        out = np.ones((1, 1))
        for j in range(n):
            out = np.kron(out, o if j == k else eye)
        return out

    H = np.zeros((2 ** n, 2 ** n))
    for k in range(n - 1):
        H += site(sz, k) @ site(sz, k + 1)
        H += 0.5 * (site(sp, k) @ site(sp.T, k + 1) + site(sp.T, k) @ site(sp, k + 1))
    return H


def test_complex_plan_matches_dense(lib_built):
    """Complex environments: tk_heff2_apply_complex against the dense complex H_eff."""
    import torch

    p = small_problem("heisenberg", 10)
    rng = np.random.default_rng(8)
    # Hermitian complex environments: real part from the problem, imaginary part antisymmetric in (bra, ket)
    def cplx_env(e):
        im = rng.standard_normal(e.data.shape)
        im = im - np.transpose(im, (2, 1, 0))
        return e.data + 0.3j * im

    Lc, Rc = cplx_env(p.env_l), cplx_env(p.env_r)
    # keep only the charge-allowed blocks (the canonical layout's support)
    dl = sweep.DeviceEnv.from_dense(p.kind, Lc, p.env_l.bra_idx, p.env_l.mpo_idx, p.env_l.ket_idx)
    dr = sweep.DeviceEnv.from_dense(p.kind, Rc, p.env_r.bra_idx, p.env_r.mpo_idx, p.env_r.ket_idx)
    plan = __import__("tk_gb300").Heff2Plan.from_device_envs_complex(dl, dr, p.w_i, p.w_j, p.flux)
    Lm, Rm = dl.to_dense(), dr.to_dense()
    Wi, Wj = p.w_i.to_dense(), p.w_j.to_dense()
    x = rng.standard_normal(plan.block_dim) + 1j * rng.standard_normal(plan.block_dim)
    xd = plan.flat_to_dense(x.real) + 1j * plan.flat_to_dense(x.imag)
    d = Wi.shape[0]
    X = xd.reshape(d, d, Lm.shape[0], Rm.shape[0])
    Y = np.einsum("pwa,stwv,uxvz,qzb,suab->txpq", Lm, Wi, Wj, Rm, X, optimize=_PATH)
    yr, yi = torch.empty(plan.block_dim, dtype=torch.float64).cuda(), torch.empty(plan.block_dim,
                                                                                 dtype=torch.float64).cuda()
    plan.apply_complex(_dev(x.real), _dev(x.imag), yr, yi)
    got = yr.cpu().numpy() + 1j * yi.cpu().numpy()
    want = plan.dense_to_flat(Y.reshape(-1).real) + 1j * plan.dense_to_flat(Y.reshape(-1).imag)
    assert np.linalg.norm(got - want) < 1e-12 * np.linalg.norm(want)


def test_real_time_tdvp_matches_exact_evolution(lib_built):
    """G(t) = <phi| exp(-i H t) |phi>, phi = S+_0 |ground state>, by real-time two-site
    TDVP with complex environments, against dense evolution (Heisenberg chain, 8 sites,
    exact bond dimension)."""
    from scipy.linalg import expm

    from tk_gb300 import dmrg

    m = models.heisenberg()
    n, D = 8, 16
    mps = dmrg.random_mps_u1(m, n, D, (0,), np.random.default_rng(4))
    dev = sweep.DeviceDMRG.from_dense_mps(m, mps, precision=PREC_FP64, solver="davidson", tol=1e-11)
    rec = dev.run(D, 3)
    H = _heisenberg_dense(n)
    assert abs(rec.energies[-1] - np.linalg.eigvalsh(H)[0]) < 1e-9
    dev.apply_site_operator(0, np.array([[0.0, 0.0], [1.0, 0.0]]), (2,))
    phi = _dense_state(dev.sites)
    phi /= np.linalg.norm(phi)
    rec2 = sweep.SweepRecord()
    dt = 0.1
    for step in range(1, 9):
        dev.tdvp_step(dt, D, rec2, real_time=True)
        phit = _dense_state(dev.sites)
        g = np.vdot(phi, phit)
        g_ref = np.vdot(phi, expm(-1j * H * dt * step) @ phi)
        assert abs(g - g_ref) < 1e-8, (step, g, g_ref)


def test_anderson_impurity_greens_function(lib_built):
    """Impurity G(t) ~ <phi| exp(-i H t) |phi>, phi = c+_{0 up} |ground state>, of the
    Anderson chain (4 sites, exact bond dimension) by real-time TDVP, against the dense
    Jordan-Wigner evolution."""
    from scipy.linalg import expm

    from helpers import fermion_chain_dense
    from tk_gb300 import dmrg

    n, D = 4, 16
    U = 3.0
    rng = np.random.default_rng(5)
    hop = [0.5] + list(0.5 * (1.0 + 0.1 * rng.standard_normal(n - 2)))
    eps = [-0.5 * U] + list(0.1 * rng.standard_normal(n - 1))
    Us = [U] + [0.0] * (n - 1)
    m = models.fermion_chain(hop, Us, eps)
    H, c = fermion_chain_dense(hop, Us, eps)
    mps = dmrg.random_mps(m, n, D, (n, 0), np.random.default_rng(3))
    dev = sweep.DeviceDMRG.from_dense_mps(m, mps, precision=PREC_FP64, solver="davidson", tol=1e-11)
    rec = dev.run(D, 3)
    nt = sum(c[(k, s)].T @ c[(k, s)] for k in range(n) for s in "ud")
    s2 = sum(c[(k, "u")].T @ c[(k, "u")] - c[(k, "d")].T @ c[(k, "d")] for k in range(n))
    sel = np.where((np.abs(np.diag(nt) - n) < 1e-9) & (np.abs(np.diag(s2)) < 1e-9))[0]
    w, V = np.linalg.eigh(H[np.ix_(sel, sel)])
    assert abs(rec.energies[-1] - w[0]) < 1e-9
    cdu = models.hubbard_local()["cdu"]
    dev.apply_site_operator(0, cdu, (1, 1))
    phi_sites = [t.clone() for t in dev.sites]
    phi_norm2 = sweep.mps_overlap(phi_sites, phi_sites).real
    phi = _dense_state(dev.sites)
    assert abs(np.vdot(phi, phi).real - phi_norm2) < 1e-12
    phi /= np.linalg.norm(phi)
    rec2 = sweep.SweepRecord()
    dt = 0.1
    for step in range(1, 7):
        dev.tdvp_step(dt, D, rec2, real_time=True)
        g = np.vdot(phi, _dense_state(dev.sites))
        g_ref = np.vdot(phi, expm(-1j * H * dt * step) @ phi)
        assert abs(g - g_ref) < 1e-8, (step, g, g_ref)
        # the block-sparse overlap gives the same amplitude
        assert abs(sweep.mps_overlap(phi_sites, dev.sites) / np.sqrt(phi_norm2) - g) < 1e-10
