#!/usr/bin/env python
"""Two-site DMRG H_eff matvec throughput on GB300.

One step = one matvec y = H_eff x of the named two-site workload (synthetic,
seeded; inputs resident in HBM for `value`).  `--impl reference` times the
CPU restatement of the reference's matvec (the Rust reference cannot be
built here) on the host cores instead.  With N ranks every rank runs an
independent replica of the workload (the matvec does not shard across GPUs:
replicas only); value = matvecs of all ranks / max-over-ranks time.

Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import json
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
UNIT = "matvec/s"
L2_BYTES = 129 * 1024 * 1024


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hubbard_d2048")
    ap.add_argument("--precision", default="auto", choices=["auto", "fp64", "bf16x3"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def oracle_for(prob):
    import oracle

    q = lambda ix: ([list(c) for c, _ in ix.sectors], [d for _, d in ix.sectors])
    return oracle.BlockSparseOracle(prob.kind, q(prob.w_i.indices[0]), q(prob.w_j.indices[0]), q(prob.env_l.ket_idx),
                                    q(prob.env_r.ket_idx), prob.flux, prob.w_i.to_dense(), prob.w_j.to_dense(),
                                    prob.env_l.data, prob.env_r.data)


def time_cpu(orc, x, seconds: float, min_runs: int = 1):
    """Runs whole matvecs until `seconds` elapse; returns (matvecs/s, runs, elapsed)."""
    y = np.empty_like(x)
    orc.apply_into(x, y)  # warm
    runs, t0 = 0, time.perf_counter()
    while True:
        orc.apply_into(x, y)
        runs += 1
        el = time.perf_counter() - t0
        if el >= seconds and runs >= min_runs:
            return runs / el, runs, el


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"tk_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
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
                "samples": len(sm)}


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


def traffic_for(workload: str, precision: str, kernel: str):
    p = ROOT / "profiles" / "ncu_traffic.json"
    if not p.exists():
        return None
    try:
        d = json.loads(p.read_text())
        return d.get(workload, {}).get(precision, {}).get(kernel)
    except ValueError:
        return None


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import oracle
    from tk_gb300 import models

    prob = models.workload(args.workload)
    orc = oracle_for(prob)
    x = np.random.default_rng(1).standard_normal(orc.total)
    y = np.empty_like(x)
    cores = oracle.num_threads()
    for _ in range(args.warmup):
        orc.apply_into(x, y)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.apply_into(x, y)
    el = time.perf_counter() - t0
    v = args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded N(0,1) environments, Gaussian sector dims)",
        "config": {"workload": args.workload, "block_dim": orc.total, "dense_dim": orc.dense_dim,
                   "threads": cores},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full matvecs of {args.workload} (after {args.warmup} warm-up)"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gflops": orc.flops() * v / 1e9,
    }
    print(json.dumps(line), flush=True)


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
    prec_name = "fp64"
    if args.precision in ("auto", "bf16x3"):
        try:
            plan.set_precision(PREC_BF16X3)
            prec_name = "bf16x3"
        except Exception as e:  # noqa: BLE001
            if args.precision == "bf16x3":
                raise
            print(f"# split precision unavailable: {e}", file=sys.stderr)
    n = plan.block_dim
    flops_total, alg_bytes = plan.cost()
    rng = np.random.default_rng(1 + rank)
    xh = rng.standard_normal(n)
    xh /= np.linalg.norm(xh)
    x = torch.from_numpy(xh).to(dev)
    y = torch.empty_like(x)
    flush = torch.empty(2 * L2_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    # warm-up
    for _ in range(args.warmup):
        flush.zero_()
        plan.profile(x, y, reps=1, stream=stream)
    torch.cuda.synchronize(dev)
    if ws > 1:
        dist.barrier()
    stage_ms = np.zeros(3)
    step_ms = []
    with ClockSampler(local) as clk:
        torch.cuda.synchronize(dev)
        for _ in range(args.steps):
            flush.zero_()  # L2 flushed between timed steps (outside the events)
            ms, fl = plan.profile(x, y, reps=1, stream=stream)
            stage_ms += np.array(ms)
            step_ms.append(sum(ms))
        torch.cuda.synchronize(dev)
    if ws > 1:
        dist.barrier()
    total_s = sum(step_ms) / 1e3
    t = torch.tensor([total_s], dtype=torch.float64, device=dev)
    if ws > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    max_s = float(t.item())
    value = args.steps * ws / max_s
    stage_ms /= args.steps
    clocks = clk.summary()
    # parity spot check of the timed matvec against the FP64 path (result read back, not timed)
    y_fp = None
    if prec_name != "fp64":
        yb = y.clone()
        plan.set_precision(PREC_FP64)
        y64 = torch.empty_like(x)
        plan.apply(x, y64)
        torch.cuda.synchronize(dev)
        y_fp = float(torch.linalg.norm(yb - y64) / torch.linalg.norm(y64))
        plan.set_precision(PREC_BF16X3)
    # end-to-end through the C ABI with pinned host buffers (H2D + matvec + D2H per step)
    hx = torch.from_numpy(xh).pin_memory()
    hy = torch.empty_like(hx).pin_memory()
    for _ in range(max(1, args.warmup)):
        plan.apply_host_flat_ptr(hx.data_ptr(), hy.data_ptr())
    if ws > 1:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        plan.apply_host_flat_ptr(hx.data_ptr(), hy.data_ptr())
    e2e_s = time.perf_counter() - t0
    te = torch.tensor([e2e_s], dtype=torch.float64, device=dev)
    if ws > 1:
        dist.all_reduce(te, op=dist.ReduceOp.MAX)
    e2e_value = args.steps * ws / float(te.item())
    if rank != 0:
        if ws > 1:
            dist.barrier()
            dist.destroy_process_group()
        return
    # roofline of the dominant kernel (largest mean stage time)
    peaks, peak_kind = measured_peaks()
    names = ["stage1_L_psi_gemm", "stage2_wij_combine", "stage3_R_gemm"]
    dom = int(np.argmax(stage_ms))
    if dom == 1:
        bound, unit = "hbm", "GB/s"
        comb_bytes = 8.0 * 2 * n * 4  # rough: the combine reads T1 and writes T2 (each ~ w x |psi|)
        achieved = comb_bytes / (stage_ms[1] / 1e3) / 1e9
        peak = peaks["hbm_gbs"]
        peak_src = f"hbm_gbs ({peak_kind})"
    elif prec_name == "fp64":
        bound, unit = "tensor", "TFLOP/s"
        achieved = fl[dom] / (stage_ms[dom] / 1e3) / 1e12
        peak = dgemm_peak_tflops(torch, dev)
        peak_src = "cuBLAS DGEMM 4096^3 measured in this run (no FP64 entry in MEASURED_PEAKS.json)"
    else:
        bound, unit = "tensor", "TFLOP/s"
        achieved = fl[dom] / (stage_ms[dom] / 1e3) / 1e12
        peak = peaks["bf16_tflops"]
        peak_src = f"bf16_tflops ({peak_kind}); achieved counts FP64-equivalent flops, the pipe runs 3 bf16 products each"
    roof = {"bound": bound, "kernel": names[dom], "achieved": achieved, "peak": peak, "unit": unit,
            "frac": achieved / peak if peak else None, "peak_source": peak_src,
            "traffic": traffic_for(args.workload, prec_name, names[dom]),
            "stage_ms": [float(v) for v in stage_ms]}
    cpu = None
    if ws == 1 and not args.no_cpu_baseline:
        import oracle

        orc = oracle_for(prob)
        xc = np.random.default_rng(1).standard_normal(orc.total)
        v, runs, el = time_cpu(orc, xc, args.cpu_seconds)
        cpu = {"value": v, "unit": UNIT, "cores": oracle.num_threads(), "kind": "port",
               "sample": f"{runs} full matvecs of {args.workload} in {el:.1f} s, all host threads"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": max_s / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64" if prec_name == "fp64" else "bf16x3(fp32 acc)",
        "data": "synthetic (seeded N(0,1) environments, Gaussian (N,2Sz) sector dims)",
        "config": {"workload": args.workload, "precision": prec_name, "block_dim": n, "dense_dim": plan.dense_dim,
                   "n_blocks": plan.n_blocks, "alg_gflop_per_matvec": flops_total / 1e9,
                   "alg_mbytes_per_matvec": alg_bytes / 1e6, "l2": "flushed between timed steps",
                   "parallelism": f"replicas x{ws}"},
        "gflops": flops_total * value / ws / 1e9,
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                "api": "tk_heff2_apply_host_flat (pinned FlatBlockStorage host buffers)"},
        "gpu_launches": 3 * args.steps,
        "clocks": clocks,
    }
    if y_fp is not None:
        line["split_vs_fp64_rel_err"] = y_fp
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
