#!/usr/bin/env python
"""Sampled-ALS throughput on one GB300 (sweeps/s).

Workload (default): the 4-mode Zipf tensor 5e6 x 5e6 x 2e4 x 1e3 with 1e8
nonzeros (alpha 1.2, log-normal float32 values, seed 0), CP-ARLS-LEV, R=25,
J=2^17 samples per least-squares solve.  A sweep updates every mode once.
Randomly initialised factors give this very sparse tensor empty sampled
fibres (zero factors, then NaN), so one exact-ALS sweep runs first, untimed —
the reference's "-p exact" preprocessing (decompose.py:82-96).

  value      sweeps/s, tensor resident on the GPU, K timed sweeps after W
             warm-up sweeps (CUDA events, synchronised on both sides).
  e2e        same metric through the public API with host buffers: every
             sweep copies its uniform draws from pinned host memory (on a copy
             stream, overlapping the previous sweep) and reads sigma back.
  roofline   sampled MTTKRP (fibre lookup, hit gather/sort, weighted scatter
             fused with the R x R solve) against the measured HBM copy
             bandwidth; algorithmic bytes per step (see algorithmic_bytes)
             summed over a sweep, divided by the region's CUDA-event time.
  cpu_baseline  the oracle port of the reference on this machine's cores.

--impl reference times the CPU port alone and prints its own line.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "sampled-ALS sweeps/s at equal fit (±1e-3): mixed vs FP64 form, 1 GB300"
WORKLOADS = {
    "zipf4": dict(desc="4-mode Zipf(1.2) tensor 5e6 x 5e6 x 2e4 x 1e3, 1e8 nonzeros, log-normal values, "
                       "CP-ARLS-LEV, R=25, J=2^17",
                  dims=(5_000_000, 5_000_000, 20_000, 1_000), nnz=100_000_000, alpha=1.2, R=25, J=1 << 17,
                  sampler="cp_arls_lev"),
    "zipf4_small": dict(desc="4-mode Zipf(1.2) tensor 5e5 x 5e5 x 2e4 x 1e3, 1e7 nonzeros (reduced)",
                        dims=(500_000, 500_000, 20_000, 1_000), nnz=10_000_000, alpha=1.2, R=25, J=1 << 17,
                        sampler="cp_arls_lev"),
}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 50 ms, started before the
    warm-up; the samples whose timestamps fall inside the timed region
    (begin() .. end(), host clock) are reported, or the one nearest to it
    when the region is shorter than the sampling interval."""

    FIELDS = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    REASONS = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []
        self.t_begin = self.t_end = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def begin(self):
        import datetime
        self.t_begin = datetime.datetime.now()

    def end(self):
        import datetime
        self.t_end = datetime.datetime.now()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    @classmethod
    def summarise(cls, lines, t_begin, t_end):
        """(sm MHz median, max MHz, reasons, samples in the region) of nvidia-smi CSV lines."""
        import datetime
        rows = []
        for line in lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 10:
                continue
            try:
                ts = datetime.datetime.strptime(p[0], "%Y/%m/%d %H:%M:%S.%f")
                rows.append((ts, float(p[2]), float(p[3]), p[6:10]))
            except ValueError:
                continue
        inside = [r for r in rows if t_begin is not None and t_end is not None and t_begin <= r[0] <= t_end]
        if not inside and rows and t_begin is not None and t_end is not None:
            mid = t_begin + (t_end - t_begin) / 2
            inside = [min(rows, key=lambda r: abs((r[0] - mid).total_seconds()))]
        reasons = set()
        for r in inside:
            for nm, v in zip(cls.REASONS, r[3]):
                if v.lower() == "active":
                    reasons.add(nm)
        sm = [r[1] for r in inside]
        return (statistics.median(sm) if sm else None, inside[-1][2] if inside else None, sorted(reasons),
                len(inside))

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons, n = self.summarise(self.lines, self.t_begin, self.t_end)
        return {"sm_mhz": sm, "sm_max_mhz": smax, "reasons": reasons, "samples": n,
                "sampled": "every 50 ms; the samples inside the timed region, else the nearest one"}


# DRAM bytes (read + write) of the sampled-MTTKRP region per sweep, summed over its
# kernels from one ncu capture of this bench on the same workload and form (the
# capture and its command: profiles/sweep_launches_zipf4_1e8_{tf32,fp64}.md).  The
# bench cannot run ncu itself; other workloads and forms report null.
REGION_TRAFFIC = {("zipf4", "tf32"): 2.0958e9, ("zipf4", "fp64"): 3.2366e9}


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def make_workload(w, seed=0):
    import torch

    from rdist_tensor_gb300 import synthetic

    t = time.perf_counter()
    dims, idx, vals = synthetic.zipf_tensor_device(w["dims"], w["nnz"], alpha=w["alpha"], values="lognormal",
                                                   seed=seed, device="cuda")
    torch.cuda.synchronize()
    log(f"generated {idx.shape[0]} nonzeros in {time.perf_counter() - t:.1f}s")
    return dims, idx, vals


def build_optimizer(w, dims, idx, vals, J, precision="fp64"):
    import torch

    from rdist_tensor_gb300.api import (AccumulatorStationary, CP_ARLS_LEV, Grid, LowRankTensor, STS_CP,
                                        SparseTensor, TensorGrid)

    N = len(dims)
    grid = Grid(np.ones(N, dtype=np.int32))
    tg = TensorGrid(dims, grid)
    st = SparseTensor(tg, idx, vals, "none")
    lr = LowRankTensor(w["R"], tg)
    lr.initialize_factors_gaussian_random(seed=1)
    sampler = CP_ARLS_LEV(lr) if w["sampler"] == "cp_arls_lev" else STS_CP(lr)
    opt = AccumulatorStationary(st, lr, sampler, max_samples=J, precision=precision)
    t = time.perf_counter()
    opt.initialize_ground_truth_for_als()
    torch.cuda.synchronize()
    log(f"initialised (sorted copies, hash tables, sampler) in {time.perf_counter() - t:.1f}s")
    t = time.perf_counter()
    for n in range(N):
        opt.exact_step(n)
    torch.cuda.synchronize()
    log(f"exact-ALS preprocessing sweep in {time.perf_counter() - t:.2f}s, fit {opt.compute_exact_fit():.6f}")
    return opt, lr, st


def algorithmic_bytes(N, R, Ju, H, touched):
    """Sampled MTTKRP bytes of one step: sample keys, weights and design rows
    read once, each hit's mode-n index and value, touched output rows written
    once (zeroing of the previous rows and the write of the new ones)."""
    return Ju * (N - 1) * 4 + Ju * 8 + Ju * R * 8 + H * (4 + 8) + 2 * touched * R * 8


def cpu_port_sweeps(dims, idx_np, vals_np, R, J, sweeps, warmup, sampler="cp_arls_lev"):
    """The oracle port of the reference (OpenMP C loops + numpy/LAPACK) on the
    host cores: set-up and one exact sweep untimed, then sampled sweeps."""
    from oracle import oracle as O
    from rdist_tensor_gb300 import synthetic

    factors = synthetic.gaussian_factors(dims, R, seed=1)
    t = time.perf_counter()
    ora = O.OracleALS(dims, idx_np, vals_np, factors, sampler)
    log(f"cpu port: set-up {time.perf_counter() - t:.1f}s")
    t = time.perf_counter()
    O.exact_als_sweep(ora, 1)
    log(f"cpu port: exact sweep {time.perf_counter() - t:.1f}s")
    rng = np.random.default_rng(3)
    N = len(dims)
    for _ in range(warmup):
        for n in range(N):
            ora.step(n, J, rng.random((N, J)))
    t = time.perf_counter()
    for _ in range(sweeps):
        for n in range(N):
            ora.step(n, J, rng.random((N, J)))
    el = time.perf_counter() - t
    return sweeps / el, el, O.lib().or_num_threads(), ora.fit()


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, w):
    ws, rank, local = dist_init()
    if rank != 0:
        return 0
    import torch

    dims, idx, vals = make_workload(w)
    idx_np = idx.cpu().numpy().astype(np.uint32)
    vals_np = vals.cpu().numpy().astype(np.float64)
    del idx, vals
    torch.cuda.empty_cache()
    sweeps = max(1, min(args.steps, args.ref_sweeps))
    warm = min(args.warmup, 1)
    value, el, cores, fit = cpu_port_sweeps(dims, idx_np, vals_np, w["R"], w["J"], sweeps, warm)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": args.gpus,
            "steps": sweeps, "warmup": warm, "ms_per_step": 1000.0 * el / sweeps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, see config)",
            "config": {"workload": w["desc"], "nnz": int(len(vals_np)), "preprocessing": "one exact-ALS sweep",
                       "fit_after": fit},
            "cpu_baseline": {"value": value, "unit": "sweeps/s", "cores": cores, "kind": "port",
                             "sample": f"{sweeps} sampled sweep(s) of the full workload after one warm-up; the "
                                       "reference's C++ cannot be rebuilt on this machine, so the oracle "
                                       "restatement (pinned to it by golden vectors) runs"},
            "e2e": {"value": value, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, w):
    import torch

    from rdist_tensor_gb300 import _lib

    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    lib = _lib.load()
    dims, idx, vals = make_workload(w, seed=args.seed + rank)
    N, R, J = len(dims), w["R"], w["J"]
    nnz = int(idx.shape[0])

    def timed(opt, clocks=None):
        # execute_sweeps: the first sweep runs step by step, later ones replay
        # one captured sweep (a CUDA graph); the capture happens in the warm-up.
        if clocks:
            clocks.start()
        opt.execute_sweeps(args.warmup, J)
        torch.cuda.synchronize()
        l0 = lib.exafac_kernel_launches()
        barrier(ws)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if clocks:
            clocks.begin()
        e0.record()
        opt.execute_sweeps(args.steps, J)
        e1.record()
        torch.cuda.synchronize()
        if clocks:
            clocks.end()
        barrier(ws)
        el = max_over_ranks(e0.elapsed_time(e1) * 1e-3, ws)
        return el, lib.exafac_kernel_launches() - l0, opt.compute_exact_fit()

    # ---- the FP64 form (the reference's arithmetic) -----------------------
    ref_form = None
    if args.precision != "fp64" and not args.no_fp64_form:
        opt64, _, _ = build_optimizer(w, dims, idx, vals, J, "fp64")
        el64, _, fit64 = timed(opt64)
        opt64.deinitialize()
        del opt64
        torch.cuda.empty_cache()
        ref_form = {"precision": "fp64", "sweeps_per_s": ws * args.steps / el64, "fit_after": fit64}

    # ---- timed region: K sweeps of the measured form, tensor resident -----
    opt, lr, st = build_optimizer(w, dims, idx, vals, J, args.precision)
    clocks = ClockSampler(local)
    elapsed, launches, fit = timed(opt, clocks)
    clk = clocks.stop()
    value = ws * args.steps / elapsed

    # ---- roofline of the sampled MTTKRP (region timers, one sweep) -------
    _lib.call("exafac_als_enable_timing", opt._h, 1)
    tot_bytes, units = 0.0, []
    for n in range(N):
        opt.execute_ALS_step(n, J)
        info = opt.step_info()
        tot_bytes += algorithmic_bytes(N, R, info.unique_samples, info.hits, info.touched_rows)
        units.append((info.unique_samples, info.hits, info.touched_rows))
    regions = (ctypes.c_double * 7)()
    _lib.call("exafac_als_region_times", opt._h, regions)
    _lib.call("exafac_als_enable_timing", opt._h, 0)
    spmm_s = regions[3]
    peak, peak_kind = measured_peaks()
    achieved = tot_bytes / spmm_s / 1e9 if spmm_s > 0 else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None,
                "traffic": REGION_TRAFFIC.get((args.workload, args.precision)),
                "kernel": "sampled MTTKRP region (lookup, hit sort, scatter + solve), per sweep",
                "algorithmic_bytes": tot_bytes, "duration_s": spmm_s, "peak_source": peak_kind,
                "regions_s": {k: v for k, v in zip(["leverage_sampling", "row_gather", "design_matrix_prep",
                                                    "spmm", "dense_reduce", "postprocessing", "sampler_update"],
                                                   list(regions))},
                "units_per_step": [{"unique_samples": a, "hits": b, "touched_rows": c} for a, b, c in units]}

    # ---- e2e through the public API with host buffers ---------------------
    # Every sweep's uniforms come from pinned host memory and its sigma goes
    # back to pinned host memory, inside the timed region.  The copy of sweep
    # s+1's uniforms runs on a copy stream into a staging buffer while sweep s
    # computes; a device copy moves it into the buffer the captured sweep
    # reads.  The host reads sweep s-1's sigma (and checks it) once sweep s is
    # queued, so at most two sweeps are in flight.
    nbuf = min(args.steps, 8)  # distinct pinned input blocks, used in turn (16.8 MB each)
    host_uni = torch.empty((nbuf, N, N, J), dtype=torch.float64, pin_memory=True)
    host_uni.copy_(torch.rand((nbuf, N, N, J), dtype=torch.float64))
    dev_uni = torch.empty((N, N, J), dtype=torch.float64, device="cuda")
    stage = [torch.empty_like(dev_uni) for _ in range(2)]
    sig_host = torch.empty((args.steps, R), dtype=torch.float64, pin_memory=True)
    main_st = torch.cuda.current_stream()
    copy_st = torch.cuda.Stream()
    ev_staged = [torch.cuda.Event() for _ in range(2)]
    ev_free = [torch.cuda.Event() for _ in range(2)]
    ev_done = [torch.cuda.Event() for _ in range(args.steps)]

    def stage_in(s):
        b = s % 2
        with torch.cuda.stream(copy_st):
            copy_st.wait_event(ev_free[b])  # the device copy out of this buffer is done
            stage[b].copy_(host_uni[s % nbuf], non_blocking=True)
            ev_staged[b].record(copy_st)

    def check_sigma(s):
        ev_done[s].synchronize()
        if not bool(torch.isfinite(sig_host[s]).all()):
            raise RuntimeError(f"sweep {s}: sigma is not finite")

    # one untimed sweep with these buffers: it captures the sweep graph for them
    dev_uni.copy_(host_uni[0], non_blocking=True)
    opt.execute_sweeps(1, J, dev_uni)
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    stage_in(0)
    for s in range(args.steps):
        b = s % 2
        if s + 1 < args.steps:
            stage_in(s + 1)
        main_st.wait_event(ev_staged[b])
        dev_uni.copy_(stage[b], non_blocking=True)
        ev_free[b].record(main_st)
        opt.execute_sweeps(1, J, dev_uni)
        sig_host[s].copy_(lr.sigma, non_blocking=True)
        ev_done[s].record(main_st)
        if s >= 1:
            check_sigma(s - 1)
    check_sigma(args.steps - 1)
    torch.cuda.synchronize()
    e2e_el = max_over_ranks(time.perf_counter() - t0, ws)
    opt.step_info()  # raises if a kernel reported an out-of-range index
    e2e = {"value": ws * args.steps / e2e_el, "unit": "sweeps/s", "h2d_bytes_per_step": N * N * J * 8,
           "d2h_bytes_per_step": R * 8}

    # ---- CPU baseline (rank 0, one GPU only) ------------------------------
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        idx_np = st.indices.cpu().numpy().astype(np.uint32)
        vals_np = st.values.cpu().numpy()
        cval, cel, cores, cfit = cpu_port_sweeps(dims, idx_np, vals_np, R, J, 1, 0)
        cpu = {"value": cval, "unit": "sweeps/s", "cores": cores, "kind": "port",
               "sample": "one sampled sweep of the full workload (after untimed set-up and one exact sweep); "
                         "oracle restatement, OpenMP over all host threads"}
    opt.deinitialize()
    if rank != 0:
        return 0
    dtype = "f64" if args.precision == "fp64" else f"{args.precision} design Gram, fp32 row products, fp64 solve/CDF"
    cfg = {"workload": w["desc"], "nnz": nnz, "R": R, "J": J, "sampler": w["sampler"], "precision": args.precision,
           "preprocessing": "one exact-ALS sweep, untimed", "parallelism": f"{ws} independent replica(s)",
           "l2": "inputs larger than L2 (per-mode sorted copies and hash tables, tens of GB)", "fit_after": fit}
    if ref_form is not None:
        cfg["fp64_form"] = ref_form
        cfg["speedup_vs_fp64_form"] = value / ref_form["sweeps_per_s"]
        cfg["fit_gap_vs_fp64_form"] = abs(fit - ref_form["fit_after"])
        cfg["equal_fit_1e-3"] = bool(abs(fit - ref_form["fit_after"]) <= 1e-3)
    line = {"metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic (seeded Zipf coordinates, log-normal values; no public dataset)",
            "config": cfg,
            "roofline": roofline, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk}
    if cpu is not None:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="zipf4", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="tf32", choices=["fp64", "tf32", "bf16"],
                    help="form timed for `value`; a mixed form is also compared with the FP64 form")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-sweeps", type=int, default=3)
    ap.add_argument("--no-fp64-form", action="store_true",
                    help="skip timing the FP64 form beside a mixed form (for kernel profiling runs)")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, w)
    return run_gpu(args, w)


if __name__ == "__main__":
    sys.exit(main())
