"""bench.py's CPU-baseline leg (the oracle timed on the host cores) without a GPU."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def test_cpu_baseline_leg():
    sys.path.insert(0, str(ROOT))
    import bench
    import oracle
    from tk_gb300 import models

    prob = models.workload("heisenberg_d1024", scale=0.25)
    cores = oracle.num_threads(timed=True)
    d = bench.cpu_baseline(prob, "heisenberg_d1024", 0.2, 2.0)
    assert d["value"] > 0 and d["unit"] == "matvec/s" and d["kind"] == "port" and d["cores"] == cores
    assert "heisenberg_d1024" in d["sample"] and "ffp-contract=fast" in d["build"]
    assert d["one_core"]["value"] > 0 and d["one_core"]["unit"] == "matvec/s"
    assert oracle.num_threads(timed=True) == cores  # the thread count is restored
    assert "one_core" not in bench.cpu_baseline(prob, "heisenberg_d1024", 0.1, 0.0)


def test_timed_build_agrees_with_the_checker():
    """The FMA build that is timed computes the checker's matvec to rounding
    (contraction changes the last bits only)."""
    sys.path.insert(0, str(ROOT))
    import bench
    from tk_gb300 import models

    prob = models.workload("hubbard_d2048", scale=0.125)
    a, b = bench.oracle_for(prob), bench.oracle_for(prob, timed=True)
    x = np.random.default_rng(3).standard_normal(a.total)
    ya, yb = a.apply(x), b.apply(x)
    assert np.linalg.norm(ya - yb) <= 1e-13 * np.linalg.norm(ya)


def test_cpu_child_process_line():
    """The GPU arm times the CPU in a child process (no torch, no CUDA); the
    child prints one JSON line with the baseline."""
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--cpu-child", "--workload", "heisenberg_d1024",
                        "--cpu-seconds", "0.2", "--cpu-one-core-seconds", "0"], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    assert d["value"] > 0 and d["kind"] == "port" and "matvecs of heisenberg_d1024" in d["sample"]


def test_traffic_table_covers_the_default_bench():
    """The default bench line (Hubbard D=2048, split precision) finds the ncu
    DRAM traffic of every stage it can name as the dominant one."""
    sys.path.insert(0, str(ROOT))
    import bench

    for stage in bench.STAGES:
        t = bench.traffic_for("hubbard_d2048", "bf16x3", stage)
        assert isinstance(t, int) and t > 0, stage
    assert bench.traffic_for("hubbard_d2048", "bf16x3", "no_such_kernel") is None
    assert "stored" in bench.TRAFFIC_SOURCE
