"""bench.py's CPU-baseline leg (the oracle timed on the host cores) without a GPU."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_cpu_baseline_leg():
    sys.path.insert(0, str(ROOT))
    import bench
    import oracle
    from tk_gb300 import models

    prob = models.workload("heisenberg_d1024", scale=0.25)
    cores = oracle.num_threads()
    d = bench.cpu_baseline(prob, "heisenberg_d1024", 0.2, 2.0)
    assert d["value"] > 0 and d["unit"] == "matvec/s" and d["kind"] == "port" and d["cores"] == cores
    assert "heisenberg_d1024" in d["sample"]
    assert d["one_core"]["value"] > 0 and d["one_core"]["unit"] == "matvec/s"
    assert oracle.num_threads() == cores  # the thread count is restored
    assert "one_core" not in bench.cpu_baseline(prob, "heisenberg_d1024", 0.1, 0.0)


def test_traffic_table_covers_the_default_bench():
    """The default bench line (Hubbard D=2048, split precision) finds the ncu
    DRAM traffic of every stage it can name as the dominant one."""
    sys.path.insert(0, str(ROOT))
    import bench

    for stage in bench.STAGES:
        t = bench.traffic_for("hubbard_d2048", "bf16x3", stage)
        assert isinstance(t, int) and t > 0, stage
    assert bench.traffic_for("hubbard_d2048", "bf16x3", "no_such_kernel") is None
