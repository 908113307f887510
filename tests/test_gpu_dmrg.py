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
