#!/usr/bin/env python
"""Two-site DMRG H_eff matvec throughput on GB300.

One step = one matvec y = H_eff x of the named two-site workload (synthetic,
seeded; inputs resident in HBM for `value`, L2 flushed between steps).
`--impl reference` times the CPU restatement of the reference's matvec (the
Rust reference cannot be built here) on the host cores instead.  With N ranks
every rank runs an independent replica (the matvec does not shard across
GPUs: replicas only); value = matvecs of all ranks / max-over-ranks time.

Besides matvec/s the line reports the time to the lowest eigenpair of the same
H_eff with the FP64 path and with the split-precision path + FP64 refinement,
and |dE| between them (the metric's "at |dE| <= 1e-10").

Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "tensorkraft-design_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "H_eff matvec/s (two-site, D=2048 Hubbard U(1)xU(1))"
# the metric and data description of each matvec workload (the first is the headline)
WORKLOADS = {
    "hubbard_d2048": (METRIC, "synthetic (seeded N(0,1) environments, Gaussian (N,2Sz) sector dims)"),
    "heisenberg_d1024": ("H_eff matvec/s (two-site, D=1024 Heisenberg chain U(1))",
                         "synthetic (seeded N(0,1) environments, Gaussian Sz sector dims)"),
    "cylinder_d4096": ("H_eff matvec/s (two-site, D=4096 width-4 J1 cylinder U(1))",
                       "synthetic (seeded N(0,1) environments, heavy-tailed Sz sector dims)"),
}
UNIT = "matvec/s"
L2_BYTES = 129 * 1024 * 1024
STAGES = ["stage1_L_psi", "stage2_wij_combine", "stage3_R"]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hubbard_d2048")
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "bf16x3"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--cpu-one-core-seconds", type=float, default=5.0,
                    help="budget of the one-thread CPU timing beside the all-threads baseline (0: skip)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-lanczos", action="store_true")
    ap.add_argument("--dmrg", action="store_true",
                    help="also run the Heisenberg L=32, D=64, 4-sweep two-site DMRG (FP64 and split precision)")
    ap.add_argument("--dmrg-cpu", action="store_true", help="with --dmrg: also run it on the CPU oracle solver")
    ap.add_argument("--sweeps", type=int, default=1, metavar="K",
                    help="time K device-resident two-site sweeps of the Hubbard chain (FP64 Davidson and "
                         "split-precision Jacobi-Davidson from the same MPS, after --sweep-warmup split sweeps); "
                         "0 skips them")
    ap.add_argument("--sweep-sites", type=int, default=64)
    ap.add_argument("--sweep-bond", type=int, default=2048)
    ap.add_argument("--sweep-warmup", type=int, default=1)
    ap.add_argument("--ref-seconds", type=float, default=8.0,
                    help="--impl reference: time at least this long (and at least --steps matvecs)")
    ap.add_argument("--cpu-child", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--autotune", type=int, default=1,
                    help="1: time the split-precision schedule candidates and keep the fastest; 0: the default "
                         "schedule (for profiler launch lists)")
    ap.add_argument("--tc-options", default=None, metavar="T,F,W,P,N",
                    help="with --autotune 0: this split-precision schedule (tk_tc_options: tall_max_mtiles, "
                         "fuse_max_ntiles, combine_warps, stage1_persistent, stage1_narrow), e.g. the autotuner's "
                         "choice for a profiler launch list")
    ap.add_argument("--tdvp-steps", type=int, default=0, metavar="K",
                    help="also time K real-time TDVP steps of the impurity Green's function (Anderson chain, "
                         "16 sites, D=1024, dt=0.05, Krylov 16) after a split-precision DMRG ground state")
    ap.add_argument("--rows", action="store_true",
                    help="also time environment growth, the dense GEMM and the block GEMM beside CPU restatements")
    ap.add_argument("--fp64-schedule", default="stacked", choices=["grouped", "stacked"],
                    help="launch schedule of the FP64 matvec (the fp64 line and the fp64 comparison)")
    ap.add_argument("--compare-schedules", type=int, default=0, metavar="STEPS",
                    help="also time STEPS FP64 matvecs with one grouped launch per stage, with one launch "
                         "per sector block and on operand stacks")
    return ap.parse_args()


def compare_schedules(plan, x, y, torch, dev, steps: int, flush):
    """FP64 matvec/s with the grouped launch, with one launch per output block
    and on operand stacks."""
    from tk_gb300 import PREC_BF16X3, PREC_FP64, _abi

    prec = plan.precision
    sched_before = plan.schedule
    plan.set_precision(PREC_FP64)
    out = {}
    for name, sched in (("fp64_grouped", _abi.SCHED_GROUPED), ("fp64_per_block", _abi.SCHED_PER_BLOCK),
                        ("fp64_stacked", _abi.SCHED_STACKED)):
        plan.set_schedule(sched)
        plan.apply(x, y)
        torch.cuda.synchronize(dev)
        tot = 0.0
        for _ in range(steps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            plan.apply(x, y)
            e.record()
            e.synchronize()
            tot += s.elapsed_time(e) / 1e3
        out[name] = steps / tot
    plan.set_schedule(sched_before)
    plan.set_precision(prec)
    out["grouped_speedup"] = out["fp64_grouped"] / out["fp64_per_block"]
    out["stacked_speedup"] = out["fp64_stacked"] / out["fp64_grouped"]
    return out


def dmrg_cfg1(torch, with_cpu: bool):
    """Heisenberg OBC L=32, J=1, U(1) 2Sz, MPO bond 5, D=64, random seeded MPS,
    4 two-site sweeps, Lanczos krylov 20, tol 1e-12: energy per sweep and time."""
    from tk_gb300 import PREC_BF16X3, PREC_FP64, dmrg, models

    out = {"config": "heisenberg L=32 D=64 4 sweeps krylov=20 tol=1e-12 seed=2024"}
    runs = [("gpu_fp64", lambda: dmrg.GpuSolver(PREC_FP64, krylov=20, restarts=4, tol=1e-12)),
            ("gpu_bf16x3_refined", lambda: dmrg.GpuSolver(PREC_BF16X3, krylov=20, restarts=4, tol=1e-12, refine=20))]
    if with_cpu:
        sys.path.insert(0, str(ROOT / "tests"))
        from helpers import CpuSolver

        runs.append(("cpu_oracle_fp64", lambda: CpuSolver(krylov=20, restarts=4, tol=1e-12)))
    m = models.heisenberg()
    for name, mk in runs:
        mps = dmrg.random_mps_u1(m, 32, 64, (0,), np.random.default_rng(2024))
        solver = mk()
        t0 = time.perf_counter()
        st = dmrg.dmrg_two_site(m, mps, 64, 4, solver, (0,))
        torch.cuda.synchronize()
        out[name] = {"energies": st.energies, "seconds": time.perf_counter() - t0,
                     "max_bond": st.max_bond[-1], "discarded_weight": st.trunc[-1],
                     "matvecs": getattr(solver, "matvecs", None)}
    e64 = out["gpu_fp64"]["energies"][-1]
    out["dE_split_vs_fp64"] = abs(out["gpu_bf16x3_refined"]["energies"][-1] - e64)
    if with_cpu:
        out["dE_gpu_vs_cpu_oracle"] = abs(out["cpu_oracle_fp64"]["energies"][-1] - e64)
    return out


def sweep_hubbard(torch, n: int, D: int, warm: int, timed: int):
    """Hubbard chain t=1, U=4, half filling, (N, 2Sz), JW MPO w=6, bond D:
    random right-canonical block MPS (seed 2024), `warm` split-precision
    sweeps, then `timed` sweeps from that same MPS with FP64 Davidson (the
    reference sweep's solver) and with split-precision Jacobi-Davidson."""
    from tk_gb300 import PREC_BF16X3, PREC_FP64, models, sweep

    m = models.hubbard()
    t0 = time.perf_counter()
    sites, bonds = sweep.random_site_tensors(m, n, D, (n, 0), np.random.default_rng(2024), width=0.75)
    out = {"config": f"hubbard L={n} t=1 U=4 N={n} 2Sz=0 D={D} davidson tol=1e-10 seed=2024",
           "init_seconds": time.perf_counter() - t0}
    warm_dmrg = sweep.DeviceDMRG(m, sites, bonds, precision=PREC_BF16X3, solver="davidson", tol=1e-10)
    rec = warm_dmrg.run(D, warm)
    torch.cuda.synchronize()
    out["warmup"] = {"sweeps": warm, "energies": rec.energies, "seconds": rec.seconds}
    snap = [sweep.SiteTensor(t.kind, t.legs, t.keys, t.offs, t.data.clone()) for t in warm_dmrg.sites]
    snap_bonds = list(warm_dmrg.bonds)
    del warm_dmrg
    for name, prec in (("fp64", PREC_FP64), ("bf16x3", PREC_BF16X3)):
        sites2 = [sweep.SiteTensor(t.kind, t.legs, t.keys, t.offs, t.data.clone()) for t in snap]
        dm = sweep.DeviceDMRG(m, sites2, list(snap_bonds), precision=prec, solver="davidson", tol=1e-10)
        torch.cuda.synchronize()
        rec = dm.run(D, timed)
        out[name] = {"seconds_per_sweep": sum(rec.seconds) / timed, "energies": rec.energies,
                     "max_trunc": max(rec.trunc), "max_bond": rec.max_bond[-1], "matvecs": rec.matvecs,
                     "fp64_matvecs": rec.fp64_matvecs,
                     "phase_seconds": {k: round(v, 3) for k, v in rec.phase_seconds.items()}}
        del dm
    out["sweep_speedup"] = out["fp64"]["seconds_per_sweep"] / out["bf16x3"]["seconds_per_sweep"]
    out["dE"] = abs(out["fp64"]["energies"][-1] - out["bf16x3"]["energies"][-1])
    return out


def tdvp_anderson(torch, steps: int, n: int = 16, D: int = 1024, dt: float = 0.05):
    """Anderson impurity (U=3, half filling, seeded bath, chain geometry) with n sites:
    ground state by two split-precision Davidson sweeps at bond D, phi = c+_{0 up}|gs>,
    then `steps` real-time two-site TDVP steps of dt (complex FP64 environments,
    Krylov 16); G(t) = <phi(0)|phi(t)> from the impurity site, time per step."""
    from tk_gb300 import PREC_BF16X3, models, sweep

    m = models.anderson_chain(n, U=3.0, seed=5)
    sites, bonds = sweep.random_site_tensors(m, n, D, (n, 0), np.random.default_rng(2024), width=0.75)
    dm = sweep.DeviceDMRG(m, sites, bonds, precision=PREC_BF16X3, solver="davidson", tol=1e-10, krylov=16)
    t0 = time.perf_counter()
    rec = dm.run(D, 2)
    out = {"config": f"anderson chain n={n} U=3 D={D} dt={dt} krylov=16 seed=5", "ground_energies": rec.energies,
           "ground_seconds": time.perf_counter() - t0}
    e0 = rec.energies[-1]
    dm.apply_site_operator(0, models.hubbard_local()["cdu"], (1, 1))
    phi0 = [t.clone() for t in dm.sites]
    norm = math.sqrt(sweep.mps_overlap(phi0, phi0).real)
    rec2 = sweep.SweepRecord()
    g, secs = [], []
    for k in range(steps):
        ts = time.perf_counter()
        dm.tdvp_step(dt, D, rec2, real_time=True)
        secs.append(time.perf_counter() - ts)
        # G>(t) = <gs| c exp(-i (H - E0) t) c+ |gs>; the evolved state is kept normalised
        t = dt * (k + 1)
        g.append(complex(np.exp(1j * e0 * t)) * norm * sweep.mps_overlap(phi0, dm.sites))
    out["seconds_per_step"] = sum(secs) / max(1, len(secs))
    out["g_greater"] = [[round(dt * (k + 1), 6), v.real, v.imag] for k, v in enumerate(g)]
    out["g_greater_0"] = norm * norm
    out["matvecs"] = rec2.matvecs
    out["max_bond"] = max(b.total_dim for b in dm.bonds)
    return out


def secondary_rows(torch, dev):
    """Timings of the rows around the matvec, each beside a CPU restatement:
    one left environment growth (contract_left_environment, FP64 grouped GEMM
    on the device) at the Hubbard D=2048 bond and at D=512 (where the dense
    numpy contraction of the oracle finishes in seconds); the dense GEMM of
    LinAlgBackend::gemm (tk_gemm_f64, 4096^3) against cuBLAS DGEMM in the same
    run; the rank-2 block GEMM of SparseLinAlgBackend::block_gemm
    (tk_block_gemm_f64, host buffers in and out) on 15 U(1) sectors summing
    to 1024 against numpy per-block products."""
    import ctypes as C

    import oracle.environments as oe
    from tk_gb300 import _abi, models, sweep
    from tk_gb300.heff import _Marshal, context
    from tk_gb300.symmetry import U1, BlockSparseTensor, key_pack

    out = {}

    def ev_ms(fn, reps):
        fn()
        torch.cuda.synchronize(dev)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(reps):
            fn()
        e.record()
        e.synchronize()
        return s.elapsed_time(e) / reps

    rng = np.random.default_rng(5)
    for scale in (1.0, 0.25):
        p = models.workload("hubbard_d2048", scale=scale)
        D = p.env_l.ket_idx.total_dim
        bl = p.env_l.ket_idx
        # the right bond: the same (N, 2Sz) distribution (a site adds 0..2 particles and keeps
        # N - 2Sz even, so every left sector reaches several right ones)
        mid = models.gaussian_bond_u1u1(D, 30)
        A = sweep.SiteTensor.from_dense(p.kind, [p.w_i.indices[0], bl, mid],
                                        rng.standard_normal((p.w_i.indices[0].total_dim, D, D)), dev.index or 0)
        if len(A.keys) == 0:
            raise RuntimeError("environment-growth timing: the site tensor has no allowed block")
        Ld = sweep.DeviceEnv.from_dense(p.kind, p.env_l.data, bl, p.env_l.mpo_idx, bl, dev.index or 0)
        ms = ev_ms(lambda: sweep.grow_left(Ld, A, p.w_i, device=dev.index or 0), 5)
        row = {"D": D, "site_blocks": int(len(A.keys)), "gpu_ms": ms}
        if scale < 1:
            Adense, Wd = A.to_dense(), p.w_i.to_dense()
            t0 = time.perf_counter()
            ref = oe.grow_left(p.env_l.data, Adense, Wd)
            row["cpu_numpy_dense_ms"] = (time.perf_counter() - t0) * 1e3
            got = sweep.grow_left(Ld, A, p.w_i, device=dev.index or 0).to_dense()
            row["rel_err_vs_numpy"] = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
        out[f"env_grow_left_hubbard_D{D}"] = row

    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    c = torch.empty(n, n, dtype=torch.float64, device=dev)
    ma = _abi.tk_mat(a.data_ptr(), n, n, n, 1, 0)
    mb = _abi.tk_mat(b.data_ptr(), n, n, n, 1, 0)
    mc = _abi.tk_mat_mut(c.data_ptr(), n, n, n, 1)
    lib = _abi.load()
    ctx = context(dev.index or 0)
    t_ours = ev_ms(lambda: _abi.check(lib.tk_gemm_f64(ctx, 1.0, C.byref(ma), C.byref(mb), 0.0, C.byref(mc), None)), 3)
    t_cublas = ev_ms(lambda: torch.matmul(a, b, out=c), 3)
    flop = 2.0 * n ** 3
    out["gemm_f64_4096"] = {"tk_gemm_f64_tflops": flop / t_ours / 1e9, "cublas_dgemm_tflops": flop / t_cublas / 1e9,
                            "fraction_of_cublas": t_cublas / t_ours}

    bond = models.gaussian_bond_u1(1024, 15, 3.0)
    tens = []
    for _ in range(2):
        t = BlockSparseTensor([bond, bond], (0,), [0, 1])
        for q, d in bond.sectors:
            t.set_block([q, q], rng.standard_normal((d, d)))
        tens.append(t)
    m = _Marshal()
    ba, bb = m.bst(tens[0]), m.bst(tens[1])

    def block_gemm():
        res = _abi.tk_bst_out()
        _abi.check(lib.tk_block_gemm_f64(ctx, C.byref(ba), C.byref(bb), C.byref(res)))
        lib.tk_bst_free(C.byref(res))

    block_gemm()
    t0 = time.perf_counter()
    for _ in range(5):
        block_gemm()
    t_blk = (time.perf_counter() - t0) / 5
    t0 = time.perf_counter()
    for _ in range(5):
        for q, _d in bond.sectors:
            tens[0].blocks[key_pack(U1, [q, q])] @ tens[1].blocks[key_pack(U1, [q, q])]
    t_np = (time.perf_counter() - t0) / 5
    flop = sum(2.0 * d ** 3 for _, d in bond.sectors)
    out["block_gemm_u1_15_sectors_1024"] = {"gpu_ms_host_buffers": t_blk * 1e3, "cpu_numpy_ms": t_np * 1e3,
                                            "gflop": flop / 1e9}
    return out


def dist_env():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0"))


def max_over_ranks(x: float, device) -> float:
    """The largest of the ranks' x (the timing of a replicas run is its
    slowest rank); x itself without an initialised process group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


CPU_BUILD = ("oracle/_build/liborc_timed.so: gcc -O3 -fopenmp -std=gnu11 -ffp-contract=fast -funroll-loops "
             "(FMA contraction on)")


def oracle_for(prob, timed: bool = False):
    import oracle

    q = lambda ix: ([list(c) for c, _ in ix.sectors], [d for _, d in ix.sectors])
    return oracle.BlockSparseOracle(prob.kind, q(prob.w_i.indices[0]), q(prob.w_j.indices[0]), q(prob.env_l.ket_idx),
                                    q(prob.env_r.ket_idx), prob.flux, prob.w_i.to_dense(), prob.w_j.to_dense(),
                                    prob.env_l.data, prob.env_r.data, timed=timed)


def cpu_baseline(prob, workload: str, seconds: float, one_core_seconds: float) -> dict:
    """The oracle's block-sparse FP64 matvec (its FMA build) timed on the host
    cores: all threads (the reported value) and, when a single-thread matvec
    fits the budget, one thread beside it."""
    import oracle

    orc = oracle_for(prob, timed=True)
    xc = np.random.default_rng(1).standard_normal(orc.total)
    cores = oracle.num_threads(timed=True)
    v, runs, el = time_cpu(orc, xc, seconds)
    out = {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "build": CPU_BUILD,
           "sample": f"{runs} full matvecs of {workload} in {el:.1f} s, all host threads"}
    # a single thread is at most `cores` times slower; skip it when two matvecs would not fit
    if one_core_seconds > 0 and 2.0 * cores / v <= one_core_seconds:
        oracle.set_threads(1, timed=True)
        try:
            v1, runs1, el1 = time_cpu(orc, xc, one_core_seconds)
        finally:
            oracle.set_threads(cores, timed=True)
        out["one_core"] = {"value": v1, "unit": UNIT, "sample": f"{runs1} full matvecs in {el1:.1f} s, one thread"}
    return out


def cpu_baseline_isolated(workload: str, seconds: float, one_core_seconds: float) -> dict:
    """cpu_baseline in a fresh child process (no torch, no CUDA context, the
    same process setup as the --impl reference arm), so that both arms time
    the CPU under the same conditions."""
    cmd = [sys.executable, str(Path(__file__).resolve()), "--cpu-child", "--workload", workload, "--cpu-seconds",
           str(seconds), "--cpu-one-core-seconds", str(one_core_seconds)]
    env = dict(os.environ)
    for k in ("RANK", "LOCAL_RANK", "WORLD_SIZE"):
        env.pop(k, None)
    r = subprocess.run(cmd, capture_output=True, text=True, env=env, timeout=600)
    if r.returncode != 0:
        raise RuntimeError(f"CPU baseline child failed:\n{r.stderr[-2000:]}")
    out = json.loads(r.stdout.strip().splitlines()[-1])
    out["process"] = "child process without torch or CUDA"
    return out


def run_cpu_child(args):
    from tk_gb300 import models

    prob = models.workload(args.workload)
    print(json.dumps(cpu_baseline(prob, args.workload, args.cpu_seconds, args.cpu_one_core_seconds)), flush=True)


def time_cpu(orc, x, seconds: float):
    y = np.empty_like(x)
    orc.apply_into(x, y)
    runs, t0 = 0, time.perf_counter()
    while True:
        orc.apply_into(x, y)
        runs += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            return runs / el, runs, el


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons, 100 ms period."""

    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.proc = device, None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"tk_clocks_{os.getpid()}_{device}.csv"

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        t0 = time.time()
        while self.proc and time.time() - t0 < 5.0 and self.path.stat().st_size == 0:
            time.sleep(0.05)
        return self

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self, t_begin: float, t_end: float):
        """Samples whose host timestamp falls in [t_begin, t_end] (loaded pre-phase + timed steps)."""
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        import datetime

        sm, mx, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                ts = datetime.datetime.strptime(f[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
                if ts < t_begin - 0.05 or ts > t_end + 0.05:
                    continue
                sm.append(float(f[1]))
                mx = float(f[2])
                power.append(float(f[3]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        try:
            self.path.unlink()
        except OSError:
            pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None,
                "window": "loaded pre-phase + timed steps"}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text()), "measured"
        except ValueError:
            pass
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def dgemm_peak_tflops(torch, dev):
    """cuBLAS FP64 GEMM throughput on this GPU (the FP64 roofline denominator)."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2.0 * n ** 3 / best / 1e12


TRAFFIC_SOURCE = ("stored: profiles/ncu_traffic.json, dram__bytes_read.sum + dram__bytes_write.sum per launch from "
                  "one ncu capture of the same workload and build (commands in profiles/), not measured in this run")


def traffic_for(workload: str, precision: str, kernel: str):
    p = ROOT / "profiles" / "ncu_traffic.json"
    if not p.exists():
        return None
    try:
        return json.loads(p.read_text()).get(workload, {}).get(precision, {}).get(kernel)
    except ValueError:
        return None


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle
    from tk_gb300 import models

    prob = models.workload(args.workload)
    orc = oracle_for(prob, timed=True)
    x = np.random.default_rng(1).standard_normal(orc.total)
    y = np.empty_like(x)
    cores = oracle.num_threads(timed=True)
    for _ in range(args.warmup):
        orc.apply_into(x, y)
    # at least --steps matvecs and at least --ref-seconds (at most 60 s) of CPU work
    steps, t0 = 0, time.perf_counter()
    while True:
        orc.apply_into(x, y)
        steps += 1
        el = time.perf_counter() - t0
        if (steps >= args.steps and el >= args.ref_seconds) or el >= 60.0:
            break
    v = steps / el
    line = {
        "impl": "reference", "metric": WORKLOADS.get(args.workload, (METRIC,))[0], "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": args.warmup, "ms_per_step": el / steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded N(0,1) environments, Gaussian sector dims)",
        "config": {"workload": args.workload, "block_dim": orc.total, "dense_dim": orc.dense_dim, "threads": cores},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port", "build": CPU_BUILD,
                         "sample": f"{steps} full matvecs of {args.workload} in {el:.1f} s (after {args.warmup} "
                                   "warm-up), block-sparse FP64 restatement of build_heff_two_site, OpenMP over "
                                   "sector tasks"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gflops": orc.flops() * v / 1e9,
    }
    print(json.dumps(line), flush=True)


def lanczos_compare(plan, torch, dev, prec_split: bool):
    """Time to the lowest eigenpair: FP64 path vs split precision + FP64 refinement."""
    from tk_gb300 import PREC_BF16X3, PREC_FP64

    out = {}
    cfg = dict(krylov_dim=30, max_restarts=40, tol=1e-9)
    runs = [("fp64", PREC_FP64, 0)] + ([("bf16x3_refined", PREC_BF16X3, 30)] if prec_split else [])
    for name, prec, refine in runs:
        plan.set_precision(prec)
        plan.lanczos(krylov_dim=cfg["krylov_dim"], max_restarts=0, tol=cfg["tol"], refine=0)  # graph capture, warm
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        r = plan.lanczos(refine=refine, **cfg)
        torch.cuda.synchronize(dev)
        out[name] = {"E": r.eigenvalue, "residual": r.residual_norm, "converged": r.converged,
                     "matvecs": r.matvec_count, "fp64_matvecs": r.fp64_matvec_count, "restarts": r.restarts,
                     "seconds": time.perf_counter() - t0}
    if prec_split:
        out["dE"] = abs(out["fp64"]["E"] - out["bf16x3_refined"]["E"])
        out["speedup"] = out["fp64"]["seconds"] / out["bf16x3_refined"]["seconds"]
        plan.set_precision(PREC_BF16X3)
    return out


def run_ours(args):
    import torch
    import torch.distributed as dist

    ws, rank, local = dist_env()
    if ws > 1:
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device(f"cuda:{local}"))
    dev = torch.device(f"cuda:{local}")
    import __graft_entry__

    __graft_entry__.build()
    from tk_gb300 import PREC_BF16X3, PREC_FP64, models

    prob = models.workload(args.workload)
    plan = prob.plan(precision=PREC_FP64, device=local)
    from tk_gb300 import _abi

    fp64_sched = {"grouped": _abi.SCHED_GROUPED, "stacked": _abi.SCHED_STACKED}[args.fp64_schedule]
    plan.set_schedule(fp64_sched)
    prec_name = "fp64"
    tune = None
    if args.precision in ("auto", "bf16x3"):
        plan.set_precision(PREC_BF16X3)
        prec_name = "bf16x3"
        # the autotuner times the candidate schedules on this workload and keeps the fastest
        if args.autotune:
            tune = plan.autotune(reps=10, use_cache=False)
        elif args.tc_options:
            plan.set_tc_options(*[int(v) for v in args.tc_options.split(",")])
            tune = {"chosen": plan.tc_options(), "set_by": "--tc-options"}
    n = plan.block_dim
    flops_total, alg_bytes = plan.cost()
    launches_per_matvec = plan.launches()
    rng = np.random.default_rng(1 + rank)
    xh = rng.standard_normal(n)
    xh /= np.linalg.norm(xh)
    x = torch.from_numpy(xh).to(dev)
    y = torch.empty_like(x)
    flush = torch.empty(2 * L2_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    clk = ClockSampler(local).start()
    for _ in range(args.warmup):
        flush.zero_()
        plan.profile(x, y, reps=1, stream=stream)
    torch.cuda.synchronize(dev)
    # loaded pre-phase (untimed) so that the clock sampler sees the GPU under this load
    t_load = time.time()
    while time.time() - t_load < 0.4:
        flush.zero_()
        plan.profile(x, y, reps=1, stream=stream)
    torch.cuda.synchronize(dev)
    if ws > 1:
        dist.barrier()
    # timed steps: one matvec each (the same launches as tk_heff2_apply), CUDA
    # events on the launching stream around it, L2 flushed before each step
    # outside the events
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    torch.cuda.synchronize(dev)
    for e0, e1 in evs:
        flush.zero_()
        e0.record()
        plan.apply(x, y, stream=stream)
        e1.record()
    torch.cuda.synchronize(dev)
    step_ms = [e0.elapsed_time(e1) for e0, e1 in evs]
    # per-stage split (an event between the stages) for the roofline of the dominant kernel
    prof_steps = min(args.steps, 50)
    stage_ms = np.zeros(3)
    for _ in range(prof_steps):
        flush.zero_()
        ms, fl, by = plan.profile(x, y, reps=1, stream=stream)
        stage_ms += np.array(ms)
    torch.cuda.synchronize(dev)
    t_end = time.time()
    clk.stop()
    if ws > 1:
        dist.barrier()
    max_s = max_over_ranks(sum(step_ms) / 1e3, dev)
    value = args.steps * ws / max_s
    stage_ms /= prof_steps
    clocks = clk.summary(t_load, t_end)
    y_fp = None
    fp64 = None
    if prec_name != "fp64":
        yb = y.clone()
        plan.set_precision(PREC_FP64)
        y64 = torch.empty_like(x)
        plan.apply(x, y64)
        torch.cuda.synchronize(dev)
        y_fp = float(torch.linalg.norm(yb - y64) / torch.linalg.norm(y64))
        # the FP64 path (--fp64-schedule) on the same workload and input, timed the same way
        n64 = max(3, min(args.steps, 50))
        ev64 = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n64)]
        for e0, e1 in ev64:
            flush.zero_()
            e0.record()
            plan.apply(x, y64, stream=stream)
            e1.record()
        torch.cuda.synchronize(dev)
        t64 = max_over_ranks(sum(a.elapsed_time(b) for a, b in ev64) / 1e3, dev)
        fp64 = {"value": n64 * ws / t64, "unit": UNIT, "steps": n64, "ms_per_step": t64 / n64 * 1e3,
                "schedule": args.fp64_schedule,
                "launches_per_matvec": plan.launches(), "split_speedup": value / (n64 * ws / t64)}
        plan.set_precision(PREC_BF16X3)
    # end-to-end through the C ABI with pinned host buffers (H2D + matvec + D2H per step)
    from tk_gb300 import _abi

    hx = torch.from_numpy(xh).pin_memory()
    hy = torch.empty_like(hx).pin_memory()

    def e2e_run(mode):
        plan.set_host_io(mode)
        for _ in range(max(1, args.warmup)):
            plan.apply_host_flat_ptr(hx.data_ptr(), hy.data_ptr())
        if ws > 1:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            plan.apply_host_flat_ptr(hx.data_ptr(), hy.data_ptr())
        return args.steps * ws / max_over_ranks(time.perf_counter() - t0, dev)

    # the three transfer forms, then the library's default (its per-plan choice)
    e2e_modes = {name: e2e_run(m) for name, m in (("staged", _abi.HOST_IO_STAGED), ("direct", _abi.HOST_IO_DIRECT),
                                                  ("direct_out", _abi.HOST_IO_DIRECT_OUT))}
    e2e_value = e2e_run(_abi.HOST_IO_AUTO)
    lz = None
    if not args.no_lanczos and rank == 0:
        lz = lanczos_compare(plan, torch, dev, prec_name != "fp64")
    if rank != 0:
        if ws > 1:
            dist.barrier()
            dist.destroy_process_group()
        return
    # roofline of the dominant stage: tensor or HBM bound by arithmetic intensity
    peaks, peak_kind = measured_peaks()
    dom = int(np.argmax(stage_ms))
    sec = stage_ms[dom] / 1e3
    products = 3.0 if prec_name != "fp64" else 1.0
    if prec_name == "fp64":
        tpeak = dgemm_peak_tflops(torch, dev)
        tsrc = "cuBLAS DGEMM 4096^3 measured in this run (MEASURED_PEAKS.json has no FP64 entry)"
    else:
        tpeak = peaks["bf16_tflops"]
        tsrc = f"bf16_tflops ({peak_kind})"
    hpeak = peaks["hbm_gbs"]
    intensity = products * fl[dom] / max(by[dom], 1.0)  # pipe flops per compulsory byte
    ridge = tpeak * 1e12 / (hpeak * 1e9)
    t_ach = fl[dom] / sec / 1e12
    h_ach = by[dom] / sec / 1e9
    if dom == 1 or intensity < ridge:
        roof = {"bound": "hbm", "achieved": h_ach, "peak": hpeak, "unit": "GB/s", "frac": h_ach / hpeak,
                "peak_source": f"hbm_gbs ({peak_kind})"}
    else:
        roof = {"bound": "tensor", "achieved": t_ach, "peak": tpeak, "unit": "TFLOP/s", "frac": t_ach / tpeak,
                "peak_source": tsrc}
    roof.update({"kernel": STAGES[dom], "traffic": traffic_for(args.workload, prec_name, STAGES[dom]),
                 "traffic_source": TRAFFIC_SOURCE,
                 "alg_bytes": by[dom], "alg_flops": fl[dom], "pipe_flops_per_byte": intensity, "ridge": ridge,
                 "tensor_achieved_tflops": t_ach * products, "tensor_peak_tflops": tpeak,
                 "stage_ms": [float(v) for v in stage_ms], "stage_bytes": by, "stage_flops": fl})
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_isolated(args.workload, args.cpu_seconds, args.cpu_one_core_seconds)
    line = {
        "metric": WORKLOADS[args.workload][0], "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": max_s / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec_name == "fp64" else "bf16x3 (fp32 accumulate)",
        "data": WORKLOADS[args.workload][1],
        "config": {"workload": args.workload, "precision": prec_name, "block_dim": n, "dense_dim": plan.dense_dim,
                   "n_blocks": plan.n_blocks, "alg_gflop_per_matvec": flops_total / 1e9,
                   "alg_mbytes_per_matvec": alg_bytes / 1e6, "l2": "flushed between timed steps",
                   "parallelism": f"replicas x{ws}"},
        "gflops": flops_total * value / ws / 1e9,
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                "api": "tk_heff2_apply_host_flat (pinned FlatBlockStorage host buffers)",
                "host_io": ("library default (TK_HOST_IO_AUTO): psi copied in (in two halves overlapped with "
                            "stage 1 where the plan allows), the stage-3 kernel writes y to the pinned host buffer"
                            if prec_name != "fp64" else "staged: H2D copy, matvec, D2H copy"),
                "by_host_io": e2e_modes},
        "gpu_launches": launches_per_matvec * args.steps,
        "clocks": clocks,
    }
    if y_fp is not None:
        line["split_vs_fp64_rel_err"] = y_fp
    if fp64 is not None:
        line["fp64_value"] = fp64["value"]
        line["fp64"] = fp64
    if tune is not None:
        line["autotune"] = tune
    if lz is not None:
        line["lanczos"] = lz
    if args.compare_schedules > 0:
        line["schedules"] = compare_schedules(plan, x, y, torch, dev, args.compare_schedules, flush)
    if args.rows:
        line["rows"] = secondary_rows(torch, dev)
    if args.dmrg:
        line["dmrg_cfg1"] = dmrg_cfg1(torch, args.dmrg_cpu)
    if args.sweeps > 0:
        sw = sweep_hubbard(torch, args.sweep_sites, args.sweep_bond, args.sweep_warmup, args.sweeps)
        line["sweeps_hubbard"] = sw
        # the metric's second half: seconds per sweep at D=2048, split vs FP64, at |dE| <= 1e-10
        line["sweep"] = {"fp64_seconds": sw["fp64"]["seconds_per_sweep"],
                         "split_seconds": sw["bf16x3"]["seconds_per_sweep"], "speedup": sw["sweep_speedup"],
                         "dE": sw["dE"], "dE_ok": bool(sw["dE"] <= 1e-10)}
    if args.tdvp_steps > 0:
        line["tdvp_anderson"] = tdvp_anderson(torch, args.tdvp_steps)
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.cpu_child:
        run_cpu_child(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
