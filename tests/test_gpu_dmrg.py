"""Two-site DMRG sweeps driven by the device H_eff and Lanczos, against the
CPU oracle solver and exact diagonalisation (Heisenberg chains, U(1) 2Sz)."""
import numpy as np
import pytest

from helpers import CpuSolver, ed_heisenberg, models
from tk_gb300 import PREC_BF16X3, PREC_FP64, dmrg

pytestmark = pytest.mark.gpu


def _run(n, D, sweeps, solver, seed=5):
    m = models.heisenberg()
    mps = dmrg.random_mps_u1(m, n, D, (0,), np.random.default_rng(seed))
    return dmrg.dmrg_two_site(m, mps, D, sweeps, solver, (0,))


def test_dmrg_exact_small_chain(lib_built):
    st = _run(10, 32, 2, dmrg.GpuSolver(PREC_FP64, krylov=20, restarts=5, tol=1e-11))
    assert abs(st.energies[-1] - ed_heisenberg(10)) < 1e-10


def test_dmrg_fp64_matches_cpu_oracle(lib_built):
    gpu = _run(16, 24, 2, dmrg.GpuSolver(PREC_FP64, krylov=20, restarts=5, tol=1e-11))
    cpu = _run(16, 24, 2, CpuSolver(krylov=20, restarts=5, tol=1e-11))
    assert np.allclose(gpu.energies, cpu.energies, atol=1e-9, rtol=0)
    assert gpu.max_bond == cpu.max_bond


def test_dmrg_split_refined_matches_fp64(lib_built):
    fp64 = _run(14, 24, 2, dmrg.GpuSolver(PREC_FP64, krylov=20, restarts=5, tol=1e-11))
    split = _run(14, 24, 2, dmrg.GpuSolver(PREC_BF16X3, krylov=20, restarts=5, tol=1e-11, refine=20))
    assert abs(split.energies[-1] - fp64.energies[-1]) < 1e-10


class _CheckedSolver(dmrg.GpuSolver):
    """GpuSolver that also checks the closure against the reference's literal
    dense H (oracle/heff_oracle.c, the 11-deep loop of environments/mod.rs:540-590)
    at every step whose dense dimension is at most `dense_max`."""

    def __init__(self, dense_max=2048, **kw):
        super().__init__(**kw)
        self.dense_max, self.checked = dense_max, 0

    def solve(self, env_l, env_r, wi, wj, flux, theta_dense):
        from helpers import oracle_dense_literal, rel_err
        from tk_gb300.heff import MPO, build_heff_two_site

        dim = theta_dense.size
        if dim <= self.dense_max:
            prob = models.TwoSiteProblem(wi.kind, env_l, env_r, wi, wj, tuple(flux), "cfg1_step")
            H = oracle_dense_literal(prob)
            mpo = MPO([wi, wj], [wi.indices[0].total_dim] * 2, flux)
            matvec, n = build_heff_two_site(env_l, env_r, mpo, (0, 1))
            x = np.random.default_rng(dim).standard_normal(n)
            y = np.zeros(n)
            matvec(x, y)
            assert rel_err(y, H @ x) < 1e-12
            self.checked += 1
        return super().solve(env_l, env_r, wi, wj, flux, theta_dense)


def test_cfg1_exact_configuration(lib_built):
    """Heisenberg OBC L=32, J=1, U(1) 2Sz, MPO bond 5, D=64, random seeded MPS,
    4 two-site sweeps, Lanczos with Krylov dimension 20 and tol 1e-12: the device
    FP64 run against the CPU oracle solver (block-sparse FP64 matvec + the
    reference's Lanczos restated) at every half sweep, the per-matvec closure
    against the literal dense H at the small bonds near both ends, and the
    split-precision + FP64-refinement run against FP64."""
    kw = dict(krylov=20, restarts=4, tol=1e-12)
    gpu_solver = _CheckedSolver(precision=PREC_FP64, **kw)
    gpu = _run(32, 64, 4, gpu_solver, seed=2024)
    assert gpu_solver.checked >= 8
    cpu = _run(32, 64, 4, CpuSolver(**kw), seed=2024)
    assert len(gpu.energies) == len(cpu.energies) == 8
    assert np.allclose(gpu.energies, cpu.energies, atol=1e-9, rtol=0), (gpu.energies, cpu.energies)
    assert gpu.max_bond == cpu.max_bond and gpu.max_bond[-1] == 64
    split = _run(32, 64, 4, dmrg.GpuSolver(PREC_BF16X3, refine=20, **kw), seed=2024)
    assert abs(split.energies[-1] - gpu.energies[-1]) <= 1e-10
    # converged to the known L=32 open-chain value within the truncation at D=64
    assert -13.9974 < gpu.energies[-1] < -13.9972
