"""Device-resident sweeps: block-sparse environments grown on the device
(tk_env_grow_left/right) against the numpy restatement of
contract_left/right_environment, plans over device environments against plans
over dense ones, the two-site start vector, and whole sweeps against the
dense-host DMRG driver and exact diagonalisation."""
import numpy as np
import pytest

from helpers import ed_heisenberg, ed_hubbard, models, rel_err
from oracle import environments as oe
from tk_gb300 import PREC_BF16X3, PREC_FP64, dmrg, sweep
from tk_gb300.heff import Environment, Heff2Plan
from tk_gb300.symmetry import fuse, key_unpack

pytestmark = pytest.mark.gpu


def _chain(name, n, D, seed=3):
    if name == "heisenberg":
        m = models.heisenberg()
        mps = dmrg.random_mps_u1(m, n, D, (0,), np.random.default_rng(seed))
    elif name == "hubbard":
        m = models.hubbard()
        mps = dmrg.random_mps(m, n, D, (n, 0), np.random.default_rng(seed))
    else:
        m = models.cylinder_j1(4)
        mps = dmrg.random_mps(m, n, D, (0,), np.random.default_rng(seed))
    return m, mps


def _sites(m, mps):
    return [sweep.SiteTensor.from_dense(m.kind, [mps.phys, mps.bonds[i], mps.bonds[i + 1]], mps.tensors[i])
            for i in range(mps.n)]


def test_env_layout_is_canonical(lib_built):
    m = models.hubbard()
    _, mps = _chain("hubbard", 6, 16)
    bond, wq = mps.bonds[3], m.chain(6).tensors[3].indices[2]
    keys, offs, total = sweep.env_layout(m.kind, bond, wq, bond)
    assert np.all(np.diff(keys.astype(np.int64)) > 0) or len(keys) < 2
    want = []
    for qb, db in bond.sectors:
        for qw, dw in wq.sectors:
            for qk, dk in bond.sectors:
                if fuse(m.kind, qk, qw) == qb:
                    want.append((qb, qw, qk, db * dw * dk))
    assert len(want) == len(keys)
    got = [tuple(tuple(q) for q in key_unpack(m.kind, int(k), 3)) for k in keys]
    assert sorted(got) == sorted((a, b, c) for a, b, c, _ in want)
    sizes = np.diff(np.append(offs, total))
    size_of = {(a, b, c): s for a, b, c, s in want}
    assert [size_of[g] for g in got] == list(sizes)


@pytest.mark.parametrize("name,n,D", [("heisenberg", 8, 12), ("hubbard", 6, 16), ("cylinder", 6, 10)])
def test_env_growth_matches_restatement(lib_built, name, n, D):
    m, mps = _chain(name, n, D)
    W = m.chain(n).tensors
    Wd = [w.to_dense() for w in W]
    sites = _sites(m, mps)
    L = np.ones((1, 1, 1))
    for i in range(n - 1):
        Ld = sweep.DeviceEnv.from_dense(m.kind, L, mps.bonds[i], W[i].indices[2], mps.bonds[i])
        L = oe.grow_left(L, mps.tensors[i], Wd[i])
        got = sweep.grow_left(Ld, sites[i], W[i]).to_dense()
        assert rel_err(got, L) < 1e-12, i
    R = np.ones((1, 1, 1))
    for i in range(n - 1, 0, -1):
        Rd = sweep.DeviceEnv.from_dense(m.kind, R, mps.bonds[i + 1], W[i].indices[3], mps.bonds[i + 1])
        R = oe.grow_right(R, mps.tensors[i], Wd[i])
        got = sweep.grow_right(Rd, sites[i], W[i]).to_dense()
        assert rel_err(got, R) < 1e-12, i


@pytest.mark.parametrize("name,n,D,prec,tol", [("heisenberg", 10, 24, PREC_FP64, 1e-13),
                                                ("hubbard", 6, 24, PREC_FP64, 1e-13),
                                                ("hubbard", 6, 24, PREC_BF16X3, 2e-4)])
def test_plan_over_device_envs_matches_dense(lib_built, name, n, D, prec, tol):
    import torch

    m, mps = _chain(name, n, D)
    W = m.chain(n).tensors
    Wd = [w.to_dense() for w in W]
    i = n // 2 - 1
    L = np.ones((1, 1, 1))
    for k in range(i):
        L = oe.grow_left(L, mps.tensors[k], Wd[k])
    R = np.ones((1, 1, 1))
    for k in range(n - 1, i + 1, -1):
        R = oe.grow_right(R, mps.tensors[k], Wd[k])
    bl, br = mps.bonds[i], mps.bonds[i + 2]
    zero = (0,) * len(mps.bonds[0].sectors[0][0])
    dense = Heff2Plan(Environment(L, bl, W[i].indices[2], bl), Environment(R, br, W[i + 1].indices[3], br),
                      W[i], W[i + 1], psi_flux=zero, precision=prec)
    dev = Heff2Plan.from_device_envs(sweep.DeviceEnv.from_dense(m.kind, L, bl, W[i].indices[2], bl),
                                     sweep.DeviceEnv.from_dense(m.kind, R, br, W[i + 1].indices[3], br),
                                     W[i], W[i + 1], zero, precision=prec)
    assert np.array_equal(dense.blocks()[0], dev.blocks()[0])
    x = torch.from_numpy(np.random.default_rng(1).standard_normal(dense.block_dim)).cuda()
    y1, y2 = torch.empty_like(x), torch.empty_like(x)
    dense.apply(x, y1)
    dev.apply(x, y2)
    torch.cuda.synchronize()
    assert rel_err(y2.cpu().numpy(), y1.cpu().numpy()) < tol
    # the two-site start vector
    psi = sweep.two_site_product(dev, *_sites(m, mps)[i:i + 2]).cpu().numpy()
    theta = np.einsum("sab,tbc->stac", mps.tensors[i], mps.tensors[i + 1])
    assert rel_err(psi, dev.dense_to_flat(theta.reshape(-1))) < 1e-13


def test_random_site_tensors_right_canonical(lib_built):
    m = models.hubbard()
    sites, bonds = sweep.random_site_tensors(m, 8, 40, (8, 0), np.random.default_rng(4))
    for i in range(1, 8):
        A = sites[i].to_dense()
        G = np.einsum("sab,scb->ac", A, A)
        assert np.allclose(G, np.eye(G.shape[0]), atol=1e-12), i
        assert A.shape[1] == bonds[i].total_dim
    A0 = sites[0].to_dense()
    assert abs(np.sum(A0 * A0) - 1.0) < 1e-12


def test_canonicalize_mixed(lib_built):
    """Per-charge QR / LQ canonicalisation (mps/mod.rs:346-419): left
    isometries left of the centre, right isometries right of it, the state
    unchanged (overlaps with the original), the bonds in the form the charges
    allow."""
    m = models.hubbard()
    rng = np.random.default_rng(9)
    sites, bonds = sweep.random_site_tensors(m, 6, 24, (6, 0), rng)
    # break the canonical form: scale every block of each site by random factors
    mixed = []
    for t in sites:
        blocks = {k: v * rng.uniform(0.5, 2.0) for k, v in t.blocks_host().items()}
        mixed.append(sweep.SiteTensor.from_blocks(t.kind, t.legs, blocks))
    ref = sweep.mps_overlap(mixed, mixed).real
    for center in (5, 0, 2):
        out, nb = sweep.canonicalize(mixed, bonds, center)
        assert abs(sweep.mps_overlap(out, out).real - ref) < 1e-10 * ref
        assert abs(sweep.mps_overlap(mixed, out).real - ref) < 1e-10 * ref
        for i, t in enumerate(out):
            A = t.to_dense()
            assert A.shape[1] == nb[i].total_dim and A.shape[2] == nb[i + 1].total_dim
            if i < center:
                G = np.einsum("sab,sac->bc", A, A)
                assert np.allclose(G, np.eye(G.shape[0]), atol=1e-12), (center, i)
            elif i > center:
                G = np.einsum("sab,scb->ac", A, A)
                assert np.allclose(G, np.eye(G.shape[0]), atol=1e-12), (center, i)


def test_device_sweeps_match_dense_driver(lib_built):
    m, mps = _chain("heisenberg", 12, 16, seed=5)
    mps2 = dmrg.DenseMPS(mps.kind, mps.phys, list(mps.bonds), [t.copy() for t in mps.tensors])
    ref = dmrg.dmrg_two_site(m, mps2, 16, 2, dmrg.GpuSolver(PREC_FP64, krylov=20, restarts=8, tol=1e-11), (0,))
    dev = sweep.DeviceDMRG.from_dense_mps(m, mps, precision=PREC_FP64, solver="lanczos", krylov=20, restarts=8,
                                          tol=1e-11)
    rec = dev.run(16, 2)
    assert np.allclose(rec.energies, ref.energies, atol=1e-9, rtol=0)
    assert rec.max_bond == ref.max_bond


def test_device_sweeps_exact_hubbard(lib_built):
    """Open Hubbard chain at half filling: Davidson sweeps reach exact diagonalisation."""
    n = 6
    m, mps = _chain("hubbard", n, 64, seed=2)
    dev = sweep.DeviceDMRG.from_dense_mps(m, mps, precision=PREC_FP64, solver="davidson", tol=1e-10)
    rec = dev.run(64, 3)
    assert abs(rec.energies[-1] - ed_hubbard(n, N=n, sz2=0)) < 1e-9


def test_device_sweeps_split_matches_fp64(lib_built):
    """Split-precision Jacobi-Davidson sweeps reach the FP64 sweeps' energy; at
    D = 2^(n/2) the chain is exact."""
    m = models.heisenberg()
    sites, bonds = sweep.random_site_tensors(m, 10, 32, (0,), np.random.default_rng(7))
    e = {}
    for prec in (PREC_FP64, PREC_BF16X3):
        s2 = [sweep.SiteTensor(t.kind, t.legs, t.keys, t.offs, t.data.clone()) for t in sites]
        rec = sweep.DeviceDMRG(m, s2, list(bonds), precision=prec, solver="davidson", tol=1e-10).run(32, 2)
        e[prec] = rec.energies[-1]
        if prec == PREC_BF16X3:
            assert rec.fp64_matvecs < rec.matvecs
    assert abs(e[PREC_FP64] - e[PREC_BF16X3]) < 1e-10
    assert abs(e[PREC_FP64] - ed_heisenberg(10)) < 1e-9


def test_mps_energy_matches_the_dense_contraction_and_the_sweep(lib_built):
    """mps_energy (mps/mod.rs:277-337) on device site tensors: against the
    dense host transfer (dmrg.grow_left over dense tensors) for a random
    MPS, and equal to the last two-site eigenvalue after an untruncated
    FP64 sweep (the state is then the normalised ground-state estimate)."""
    n = 8
    m, mps = _chain("heisenberg", n, 16, seed=6)
    sites = _sites(m, mps)
    W = m.chain(n).tensors
    L = np.ones((1, 1, 1))
    for i in range(n):
        L = dmrg.grow_left(L, mps.tensors[i], W[i].to_dense())
    e = sweep.mps_energy(m, sites, mps.bonds)
    assert isinstance(e, float)
    assert abs(e - float(L[0, 0, 0])) < 1e-12 * max(1.0, abs(float(L[0, 0, 0])))
    dev = sweep.DeviceDMRG.from_dense_mps(m, mps, precision=PREC_FP64, solver="davidson", tol=1e-11)
    rec = dev.run(16, 1)
    assert abs(sweep.mps_energy(m, dev.sites, dev.bonds) - rec.energies[-1]) < 1e-9
