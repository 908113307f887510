"""Writes tests/golden/reference_kats.json: the known answers of the reference's
own tests for this path, restated as data (kyungminlee/tensorkraft-design).

The reference is a Rust workspace that cannot be built here, so these values
are transcribed from its test sources (cited per entry) and, where a test
generates data, regenerated with a restatement of its generator:

  lcg_next (tk-linalg/tests/block_gemm_realistic.rs:12-15):
      state = state*6364136223846793005 + 1 (mod 2^64);
      value = ((state >> 33) as i32 as f64) / 2^30

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "reference_kats.json"
M64 = (1 << 64) - 1


def lcg_values(seed: int, n: int) -> list:
    s = seed
    out = []
    for _ in range(n):
        s = (s * 6364136223846793005 + 1) & M64
        v = (s >> 33) & 0xFFFFFFFF
        if v >= 1 << 31:
            v -= 1 << 32
        out.append(v / float(1 << 30))
    return out


def block_gemm_case():
    """block_gemm_matches_dense_reference (block_gemm_realistic.rs:90-...)."""
    row = [(-1, 4), (0, 8), (1, 4)]
    col = [(-1, 3), (0, 6), (1, 3)]

    def build(rs, cs, seed):
        s = seed
        blocks = []
        for rq, rd in rs:  # QIndex order (sorted by charge)
            for cq, cd in cs:
                if rq - cq != 0:  # flux rule rq (+) dual(cq) == 0
                    continue
                vals = []
                for _ in range(rd * cd):
                    s = (s * 6364136223846793005 + 1) & M64
                    v = (s >> 33) & 0xFFFFFFFF
                    if v >= 1 << 31:
                        v -= 1 << 32
                    vals.append(v / float(1 << 30))
                blocks.append({"qns": [rq, cq], "shape": [rd, cd], "data": vals})
        return {"rows": rs, "cols": cs, "blocks": blocks}

    a = build(row, col, 42)
    b = build(col, row, 137)

    def dense(t):
        ro = {q: o for (q, o) in zip([q for q, _ in t["rows"]], np.cumsum([0] + [d for _, d in t["rows"]])[:-1])}
        co = {q: o for (q, o) in zip([q for q, _ in t["cols"]], np.cumsum([0] + [d for _, d in t["cols"]])[:-1])}
        m = np.zeros((sum(d for _, d in t["rows"]), sum(d for _, d in t["cols"])))
        for blk in t["blocks"]:
            r, c = blk["qns"]
            m[ro[r]:ro[r] + blk["shape"][0], co[c]:co[c] + blk["shape"][1]] = np.array(blk["data"]).reshape(blk["shape"])
        return m

    c = dense(a) @ dense(b)
    return {"source": "tk-linalg/tests/block_gemm_realistic.rs:90-196", "a": a, "b": b,
            "dense_product": c.reshape(-1).tolist(), "shape": list(c.shape), "tol": 1e-10}


def main():
    kats = {
        "enumerate_valid_sectors": [
            {"source": "tk-symmetry/src/flux.rs:527-550", "legs": [[[-1, 0, 1], [1, 1, 1]]] * 3,
             "dirs": [0, 0, 1], "flux": [0], "count": 7},
            {"source": "tk-symmetry/src/flux.rs:553-577", "legs": [[[-1, 0, 1], [1, 1, 1]]] * 6,
             "dirs": [0] * 6, "flux": [0], "count": 141},
            {"source": "tk-symmetry/src/flux.rs:580-597", "legs": [[[-1, 0, 1], [1, 1, 1]]] * 5,
             "dirs": [0] * 5, "flux": [0], "count": 51},
        ],
        "check_flux_rule": [
            {"source": "tk-symmetry/src/flux.rs:510-524", "qns": [1, 2, 3], "dirs": [0, 0, 1], "flux": [0], "ok": True},
            {"source": "tk-symmetry/src/flux.rs:510-524", "qns": [1, 2, 4], "dirs": [0, 0, 1], "flux": [0], "ok": False},
        ],
        "qindex_offset_of": {"source": "tk-symmetry/src/sector_key.rs:245-254",
                             "sectors": [[-1, 2], [0, 3], [1, 4]],
                             "offsets": {"-1": 0, "0": 2, "1": 5, "2": None}, "total_dim": 9},
        "packed_key_round_trip": [
            {"source": "tk-symmetry/src/sector_key.rs:228-234", "kind": 1, "qns": [[3], [-2], [0]]},
            {"source": "tk-symmetry/src/sector_key.rs:256-263 (u64 form)", "kind": 4,
             "qns": [[1000], [-500], [0]]},
        ],
        "packed_key_wrap": {"source": "tk-symmetry/src/sector_key.rs:209-226",
                            "comment": "U1(-1) packs to 255, so raw u64 order differs from Q order",
                            "kind": 1, "q": [-1], "bits": 255},
        "qn_round_trip_ranges": {"source": "tk-symmetry/src/builtins.rs:172-213",
                                 "u1": [-128, 127], "u1wide": [-32768, -1, 0, 1, 127, 128, 32767]},
        "lanczos": [
            {"source": "tk-dmrg/src/eigensolver/mod.rs:660-680", "matrix": "diag", "diag": [3, 1, 4, 1, 5],
             "krylov": 100, "eigenvalue": 1.0, "tol": 1e-6},
            {"source": "tk-dmrg/src/eigensolver/mod.rs:682-700", "matrix": "dense",
             "dense": [[2, -1], [-1, 2]], "krylov": 10, "eigenvalue": 1.0, "tol": 1e-6},
            {"source": "tk-dmrg/src/eigensolver/mod.rs:780-801 (symmetric_eigen_small)", "matrix": "dense",
             "dense": [[2, -1, 0], [-1, 2, -1], [0, -1, 2]], "krylov": 10, "eigenvalue": 2 - 2 ** 0.5,
             "tol": 1e-10},
        ],
        "davidson": [
            {"source": "tk-dmrg/src/eigensolver/mod.rs:702-707 (defaults)", "defaults": True,
             "max_subspace": 60, "tol": 1e-10},
            {"source": "tk-dmrg/src/eigensolver/mod.rs:709-732", "matrix": "diag", "diag": [3, 1, 4, 1, 5],
             "diagonal": [3, 1, 4, 1, 5], "tol": 1e-10, "eigenvalue": 1.0, "atol": 1e-6, "converged": True},
            {"source": "tk-dmrg/src/eigensolver/mod.rs:734-755", "matrix": "dense", "dense": [[2, -1], [-1, 2]],
             "diagonal": [2, 2], "tol": 1e-8, "eigenvalue": 1.0, "atol": 1e-6, "converged": True},
            {"source": "tk-dmrg/src/eigensolver/mod.rs:757-778", "matrix": "diag", "diag": [5, 2, 8, 1, 3],
             "diagonal": None, "tol": 1e-8, "eigenvalue": 1.0, "atol": 1e-6, "converged": None},
        ],
        "exp_krylov": [
            {"source": "tk-dmrg/src/tdvp/mod.rs:411-433 (identity)", "matrix": "diag", "diag": [1, 1, 1, 1, 1],
             "v": [1, 0, 0, 0, 0], "alpha": 0.5, "krylov": 10, "tol": 1e-12, "atol": 1e-8},
            {"source": "tk-dmrg/src/tdvp/mod.rs:435-460 (diagonal)", "matrix": "diag", "diag": [1, 2, 3],
             "v": [1, 1, 1], "alpha": -0.1, "krylov": 10, "tol": 1e-12, "atol": 1e-6},
            {"source": "tk-dmrg/src/tdvp/mod.rs:462-484 (zero time)", "matrix": "dense",
             "dense": [[2, -1, 0, 0], [-1, 2, -1, 0], [0, -1, 2, -1], [0, 0, -1, 2]],
             "v": [1, 2, 3, 4], "alpha": 0.0, "krylov": 10, "tol": 1e-12, "atol": 1e-10},
        ],
        "lanczos_random_diagonal": {
            "source": "tk-dmrg/tests/proptest_dmrg.rs:18-49 (+ regression seed dim=4, seed=0)",
            "cases": [{"dim": d, "seed": s, "diag": lcg_values(s + 42, d), "eigenvalue": min(lcg_values(s + 42, d))}
                      for d, s in [(4, 0), (3, 1), (7, 99), (12, 4242), (20, 9999), (16, 31337)]],
            "tol": 1e-6},
        "block_gemm": block_gemm_case(),
        "truncate_svd": [
            {"source": "tk-dmrg/src/truncation/mod.rs:185-202 (basic)", "rows": 3, "cols": 2,
             "data": [3.0, 0.0, 0.0, 2.0, 0.0, 0.0], "max_bond_dim": 200, "svd_cutoff": 1e-12, "min_bond_dim": 1,
             "bond_dim_new": 2, "n_discarded": 0, "truncation_error": 0.0, "error_atol": 1e-14,
             "singular_values": [3.0, 2.0], "sv_atol": 1e-10},
            {"source": "tk-dmrg/src/truncation/mod.rs:204-220 (with truncation)", "rows": 3, "cols": 3,
             "data": [3.0, 0.0, 0.0, 0.0, 2.0, 0.0, 0.0, 0.0, 1.0], "max_bond_dim": 2, "svd_cutoff": 1e-12,
             "min_bond_dim": 1, "bond_dim_new": 2, "n_discarded": 1, "truncation_error": 1.0 / 14.0,
             "error_atol": 1e-10},
            {"source": "tk-dmrg/src/truncation/mod.rs:222-236 (min_bond_dim)", "rows": 2, "cols": 2,
             "data": [10.0, 0.0, 0.0, 1e-15], "max_bond_dim": 200, "svd_cutoff": 1e-10, "min_bond_dim": 2,
             "bond_dim_new_at_least": 2},
        ],
    }
    OUT.write_text(json.dumps(kats, indent=1))
    print(f"wrote {OUT}")


if __name__ == "__main__":
    main()
