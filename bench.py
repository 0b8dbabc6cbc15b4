#!/usr/bin/env python3
"""Benchmark of the batched MsFEC basis build (fine-DoF x RHS per second).

Default workload: batched uneven-depth Q1 basis build, coarse 16^3 cells of
the unit cube, local depth L ~ U{2,3,4,5} per cell (seed 3), 8 coarse-basis
RHS per cell, oscillatory coefficient (eps = 1/64) times a per-cell
log-normal factor, load sin(pi x) sin(pi y) sin(pi z); mixed precision
(FP32 PCG + FP64 iterative refinement) with the plain FP64 path timed beside
it. One step = one full build (local solves + Galerkin K_H, F_H) of every
cell of this rank's share.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 runs under torchrun: coarse cells are partitioned contiguously by work
(no data-path collective; only the timing max is reduced), scaling "weak" is
NOT claimed since the global workload is fixed -> "strong".
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "mpi-msfec_gb300")
for _p in (PKG, REPO):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "fine-DoF·RHS/s of batched basis solves, mixed vs FP64 @1e-10 rel; bwd/fwd time"
UNIT = "fine-DoF·RHS/s"


def peaks():
    p = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def partition(cells, world, rank):
    """Contiguous cell ranges with balanced fine-DoF x RHS work."""
    import workloads
    w = workloads.fine_counts(cells)[1].astype(np.float64)
    cum = np.concatenate([[0.0], np.cumsum(w)])
    bounds = [int(np.searchsorted(cum, cum[-1] * r / world, side="left")) for r in range(world + 1)]
    bounds[0], bounds[-1] = 0, len(cells)
    lo, hi = bounds[rank], bounds[rank + 1]
    return lo, hi


def make_workload(name):
    import workloads
    if name == "q1_uneven":
        cells, a, r, load = workloads.q1_uneven(m=16, seed=3)
        cfg = {"workload": "q1_uneven_coarse16^3_L2-5_8rhs", "coarse_cells": 4096, "depths": [2, 3, 4, 5],
               "eps": 1.0 / 64, "seed": 3}
    elif name == "q1_small":
        cells, a, r, load = workloads.q1_lognormal(m=4, depth=3, seed=1, reaction=True)
        cfg = {"workload": "q1_lognormal_coarse4^3_L3_8rhs_reaction1", "coarse_cells": 64, "depths": [3],
               "seed": 1}
    elif name == "q1_adjoint_fwd":
        cells, a, r, load = workloads.q1_lognormal(m=8, depth=4, seed=4, reaction=False)
        cfg = {"workload": "q1_lognormal_coarse8^3_L4_8rhs", "coarse_cells": 512, "depths": [4], "seed": 4}
    else:
        raise SystemExit(f"unknown workload {name}")
    return cells, a, r, load, cfg


def coef_slice(cells, lo, hi):
    import workloads
    nf = workloads.fine_counts(cells)[0]
    off = np.concatenate([[0], np.cumsum(nf)])
    return int(off[lo]), int(off[hi])


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for ln in open(self.path).read().splitlines():
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = np.array([float(r[1]) for r in rows if r[1].replace(".", "").isdigit()] or [0.0])
        smax = max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        under = sm[sm > 0.5 * np.max(sm)] if sm.size else sm
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(under)) if under.size else None, "sm_max_mhz": smax,
                "reasons": reasons, "samples": len(rows)}


def cpu_sample_cells(cells, target_s, nthreads):
    """Stratified sample (every depth represented) sized for ~target_s of CPU work."""
    depths = sorted(set(int(d) for d in cells["depth"]))
    # rough per-cell CG+SSOR cost model in seconds on one core (measured: L4 ~ 0.1 s)
    per_cell = {1: 1e-4, 2: 5e-4, 3: 8e-3, 4: 0.1, 5: 1.6}
    per_depth = target_s * nthreads / max(1, len(depths))
    idx = []
    for d in depths:
        cand = np.where(cells["depth"] == d)[0]
        k = int(max(1, min(len(cand), per_depth / per_cell.get(d, 1.0))))
        idx.extend(cand[:k].tolist())
    return np.array(sorted(idx))


def time_oracle(cells, a, r, load, sel, nthreads):
    from oracle import oracle
    import workloads
    nf = workloads.fine_counts(cells)[0]
    off = np.concatenate([[0], np.cumsum(nf)])
    asub = np.concatenate([a[off[c]:off[c + 1]] for c in sel])
    rsub = None if r is None else np.concatenate([r[off[c]:off[c + 1]] for c in sel])
    sub = cells[sel]
    t0 = time.perf_counter()
    res = oracle.q1_build(sub["origin"], sub["size"], sub["depth"], asub, rsub, load_kind=load.kind,
                          load_params=list(load.params), solver=oracle.SOLVER_CG_SSOR, tol=1e-12,
                          max_iter=1000, want_phi=False, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return workloads.work_dof_rhs(sub) / dt, dt, len(sel), res["status"]


def run_reference(args):
    world, rank, _ = dist_env()
    if rank != 0:
        return
    cells, a, r, load, cfg = make_workload(args.workload)
    nthreads = os.cpu_count() or 1
    sel = cpu_sample_cells(cells, args.cpu_seconds / 2.0, nthreads)
    vals = []
    for _ in range(args.warmup):
        time_oracle(cells, a, r, load, sel[: max(1, len(sel) // 8)], nthreads)
    t_all = []
    for _ in range(args.steps):
        v, dt, ncell, st = time_oracle(cells, a, r, load, sel, nthreads)
        vals.append(v)
        t_all.append(dt)
    value = float(np.median(vals))
    sample = f"{len(sel)} of {len(cells)} cells, every depth represented; CG+SSOR(1.6) 1e-12 per RHS"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.median(t_all) * 1e3), "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import msfec
    import workloads

    world, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    cells_all, a_all, r_all, load, cfg = make_workload(args.workload)
    lo, hi = partition(cells_all, world, rank)
    flo, fhi = coef_slice(cells_all, lo, hi)
    cells = cells_all[lo:hi]
    a = np.ascontiguousarray(a_all[flo:fhi])
    r = None if r_all is None else np.ascontiguousarray(r_all[flo:fhi])
    work_local = workloads.work_dof_rhs(cells)
    work_total = workloads.work_dof_rhs(cells_all)
    nc = len(cells)

    stream = torch.cuda.Stream()
    d_a = torch.from_numpy(a).cuda()
    d_r = None if r is None else torch.from_numpy(r).cuda()
    d_KH = torch.zeros((nc, 8, 8), dtype=torch.float64, device="cuda")
    d_FH = torch.zeros((nc, 8), dtype=torch.float64, device="cuda")
    d_rep = torch.zeros(nc * msfec.REPORT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def reduce_max(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def timed_device(precision, steps, warmup):
        h = msfec.Handle(precision=precision, device=local)
        h.set_stream(stream.cuda_stream)
        h.set_timing(True)
        rp = 0 if d_r is None else d_r.data_ptr()
        for _ in range(warmup):
            h.q1_build_device(cells, d_a.data_ptr(), rp, load, d_KH.data_ptr(), d_FH.data_ptr(), d_rep.data_ptr())
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        solve_ms, gal_ms, launches = [], [], 0
        e0.record(stream)
        for _ in range(steps):
            h.q1_build_device(cells, d_a.data_ptr(), rp, load, d_KH.data_ptr(), d_FH.data_ptr(), d_rep.data_ptr())
            t = h.timings()
            solve_ms.append(t["solve_ms"])
            gal_ms.append(t["galerkin_ms"])
            launches += t["kernel_launches"]
        e1.record(stream)
        barrier()
        ms = e0.elapsed_time(e1) / steps
        rep = np.frombuffer(d_rep.cpu().numpy().tobytes(), dtype=msfec.REPORT_DTYPE)
        h.close()
        return ms, float(np.mean(solve_ms)), float(np.mean(gal_ms)), launches, rep

    # ---- mixed precision (headline) with clocks sampled during the timed region
    sampler = ClockSampler(local)
    sampler.start()
    ms_mixed, solve_ms, gal_ms, launches, rep = timed_device(msfec.PRECISION_MIXED, args.steps, args.warmup)
    clocks = sampler.stop()
    ms_mixed = reduce_max(ms_mixed)
    value = work_total / (ms_mixed * 1e-3)

    # ---- plain FP64 path on the same workload (fewer steps: it is the slow baseline)
    fp64 = None
    if not args.skip_fp64:
        k64 = max(1, min(args.steps, 3))
        ms64, solve64, gal64, _, rep64 = timed_device(msfec.PRECISION_FP64, k64, 1)
        ms64 = reduce_max(ms64)
        fp64 = {"value": work_total / (ms64 * 1e-3), "ms_per_step": ms64, "solve_ms": solve64,
                "steps": k64, "converged": bool(rep64["converged"].all()),
                "mixed_over_fp64": (work_total / (ms_mixed * 1e-3)) / (work_total / (ms64 * 1e-3))}

    # ---- end to end through the host-buffer C ABI (pinned host inputs, H2D + D2H inside)
    h = msfec.Handle(precision=msfec.PRECISION_MIXED, device=local)
    h.set_stream(stream.cuda_stream)
    a_pin = torch.from_numpy(a).pin_memory().numpy()
    r_pin = None if r is None else torch.from_numpy(r).pin_memory().numpy()
    h.q1_build(cells, a_pin, r_pin, load)
    barrier()
    t0 = time.perf_counter()
    ke = max(1, min(args.steps, 3))
    for _ in range(ke):
        KH, FH, rep_e, st = h.q1_build(cells, a_pin, r_pin, load)
    barrier()
    e2e_s = reduce_max((time.perf_counter() - t0) / ke)
    h.close()
    h2d = a.nbytes + (0 if r is None else r.nbytes) + nc * msfec.CELL_DTYPE.itemsize
    d2h = KH.nbytes + FH.nbytes + nc * msfec.REPORT_DTYPE.itemsize

    if rank != 0:
        if dist is not None:
            dist.destroy_process_group()
        return

    # ---- roofline of the dominant kernel (persistent local solver)
    peak, peak_kind = peaks()
    nfine = int(np.sum(workloads.fine_counts(cells)[0]))
    nnodes = int(np.sum(workloads.fine_counts(cells)[1]))
    alg_solve = nfine * 8 * (1 if r is None else 2) + nnodes * 8 * 8 * 2  # a(,r) in; phi, y out
    alg_gal = nnodes * 8 * 8 * 2 + nc * 72 * 8
    roof = {"bound": "hbm", "kernel": "q1_solve_kernel (persistent PCG, on-chip state)",
            "achieved": alg_solve / (solve_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
            "frac": alg_solve / (solve_ms * 1e-3) / 1e9 / peak, "traffic": None,
            "algorithmic_bytes": alg_solve, "launch_ms": solve_ms, "peak_source": peak_kind,
            "galerkin": {"kernel": "q1_galerkin_kernel (DMMA)", "launch_ms": gal_ms,
                         "achieved": alg_gal / (gal_ms * 1e-3) / 1e9, "frac": alg_gal / (gal_ms * 1e-3) / 1e9 / peak,
                         "algorithmic_bytes": alg_gal}}

    # ---- CPU baseline: oracle CG+SSOR (faithful-iterative) on a bounded sample
    cpu = None
    if not args.skip_cpu:
        nthreads = os.cpu_count() or 1
        sel = cpu_sample_cells(cells_all, args.cpu_seconds, nthreads)
        v, dt, ncell, st = time_oracle(cells_all, a_all, r_all, load, sel, nthreads)
        cpu = {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
               "sample": f"{ncell} of {len(cells_all)} cells (every depth), CG+SSOR(1.6) 1e-12, {dt:.1f} s"}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": dict(cfg, precision="mixed", l2="inputs and basis (>5 GB) exceed L2",
                           parallelism=f"cells partitioned over {world} GPU(s)"),
            "roofline": roof, "cpu_baseline": cpu,
            "e2e": {"value": work_total / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches), "clocks": clocks, "fp64_path": fp64,
            "converged": bool(rep["converged"].all()),
            "max_iterations": int(rep["iterations"].max()), "work_dof_rhs": work_total}
    print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="q1_uneven", choices=["q1_uneven", "q1_small", "q1_adjoint_fwd"])
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
