#!/usr/bin/env python
"""Sampled-ALS throughput on one GB300 (sweeps/s), mixed vs FP64 form.

Workloads (--workload; the seeded synthetic stand-ins for the shapes the
sampled-ALS solvers are quoted on; no public dataset is named):

  zipf5         (default) 5-mode Zipf(1.1) tensor 1e6 x 1e6 x 1e5 x 1e3 x 100,
                2e8 nonzeros, N(0,1) float32 values, STS-CP, R=128, J=2^19,
                BF16 design products vs the FP64 form, 10 sweeps.
  planted3_r64  3-mode 2000^3 planted rank-10 tensor, 2e6 nonzeros, STS-CP,
                R=64, J=2^18, TF32 (and BF16) vs the FP64 form.
  planted3      the same tensor, STS-CP, R=25, J=65536, FP64 form.
  zipf4         4-mode Zipf(1.2) tensor 5e6 x 5e6 x 2e4 x 1e3, 1e8 nonzeros,
                log-normal values, CP-ARLS-LEV, R=25, J=2^17, TF32 vs FP64.
  gcp4          3-mode Poisson count tensor 1e6 x 1e6 x 1e4, 5e7 nonzeros,
                gradient-based GCP (Poisson loss, sampled entries, Adam),
                R=32, 200 steps: its own metric, GCP steps/s (no reference
                counterpart; --impl reference prints an unavailable line).

A sweep updates every mode once.  Randomly initialised factors give the Zipf
tensors empty sampled fibres (zero factors, then NaN, in the reference too),
so one exact-ALS sweep runs first, untimed: the reference's "-p exact"
preprocessing (decompose.py:82-96).

  value      sweeps/s of the measured form, tensor resident on the GPU, K
             timed sweeps after W warm-up sweeps (CUDA events, synchronised on
             both sides), replayed from one captured CUDA graph.
  e2e        the same metric through the public API with host buffers: every
             sweep copies its uniform draws from pinned host memory (on a copy
             stream, overlapping the previous sweep) and reads sigma back.
  roofline   the dominant kernel against the measured HBM copy bandwidth:
             for the mixed STS-CP forms at R >= 32 the resident-node tcgen05
             level kernel (level_kernel_roofline; the double-buffered one of
             the deeper levels in roofline_deep_levels, the sampled MTTKRP
             region in roofline_sampled_mttkrp); otherwise the sampled
             MTTKRP (fibre lookup, hit grouping, weighted reduction fused
             with the R x R solve): algorithmic bytes per step (see
             algorithmic_bytes) summed over a sweep, divided by the region's
             CUDA-event time.
  cpu_baseline  the oracle port of the reference on this machine's cores
             (a bounded sample, scaled to the workload: see its "sample").

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
GCP_METRIC = "GCP Adam steps/s (Poisson loss on sampled entries), 1 GB300"
WORKLOADS = {
    "zipf5": dict(desc="5-mode Zipf(1.1) tensor 1e6 x 1e6 x 1e5 x 1e3 x 100, 2e8 nonzeros, N(0,1) values, STS-CP, "
                       "R=128, J=2^19",
                  gen="zipf", dims=(1_000_000, 1_000_000, 100_000, 1_000, 100), nnz=200_000_000, alpha=1.1,
                  values="normal", R=128, J=1 << 19, sampler="sts_cp", precision="bf16", exact_pre=True, steps=10,
                  cpu_nnz=20_000_000, cpu_J=1 << 15),
    "planted3_r64": dict(desc="3-mode 2000^3 planted rank-10 tensor (|N(0,1)| factors, noise variance 0.01), "
                              "2e6 nonzeros, STS-CP, R=64, J=2^18",
                         gen="planted", dims=(2000, 2000, 2000), nnz=2_000_000, R=64, J=1 << 18, sampler="sts_cp",
                         precision="tf32", other_forms=("bf16",), exact_pre=False, steps=20, cpu_J=1 << 15),
    "planted3": dict(desc="3-mode 2000^3 planted rank-10 tensor (|N(0,1)| factors, noise variance 0.01), "
                          "2e6 nonzeros, STS-CP, R=25, J=65536",
                     gen="planted", dims=(2000, 2000, 2000), nnz=2_000_000, R=25, J=65536, sampler="sts_cp",
                     precision="fp64", exact_pre=False, steps=20, cpu_J=65536),
    "zipf4": dict(desc="4-mode Zipf(1.2) tensor 5e6 x 5e6 x 2e4 x 1e3, 1e8 nonzeros, log-normal values, "
                       "CP-ARLS-LEV, R=25, J=2^17",
                  gen="zipf", dims=(5_000_000, 5_000_000, 20_000, 1_000), nnz=100_000_000, alpha=1.2,
                  values="lognormal", R=25, J=1 << 17, sampler="cp_arls_lev", precision="tf32", exact_pre=True,
                  steps=100, cpu_J=1 << 17),
    "gcp4": dict(desc="3-mode Poisson count tensor 1e6 x 1e6 x 1e4, 5e7 nonzeros (Zipf(1.1) support, rates from a "
                      "planted rank-16 CP model with Gamma(0.5,1) factors), GCP Poisson loss, R=32, J=2^17 sampled "
                      "entries per step (2^16 nonzeros + 2^16 zeros), Adam lr=1e-2, FP32",
                 kind="gcp", dims=(1_000_000, 1_000_000, 10_000), nnz=50_000_000, planted_rank=16, R=32, J=1 << 17,
                 lr=1e-2, steps=200, cpu_steps=3),
    "zipf4_small": dict(desc="4-mode Zipf(1.2) tensor 5e5 x 5e5 x 2e4 x 1e3, 1e7 nonzeros (reduced)",
                        gen="zipf", dims=(500_000, 500_000, 20_000, 1_000), nnz=10_000_000, alpha=1.2,
                        values="lognormal", R=25, J=1 << 17, sampler="cp_arls_lev", precision="tf32", exact_pre=True,
                        steps=100, cpu_J=1 << 17),
}
DEFAULT_WORKLOAD = "zipf5"


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


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def level_kernel_roofline(R, J, nodes=64, use_tc=2, launches=5, seed=0):
    """Roofline of a tcgen05 level kernel of the mixed forms' breadth-first
    STS-CP descents, timed live: exafac_quad_forms_f32 (the level kernel's
    quadratic forms, without the branch epilogue) over J FP32 vectors of
    rank R, slots sorted by node over `nodes` distinct packed nodes.
    use_tc = 2: the resident-node kernel (bfs_level_tcr_kernel, the root and
    the shallow levels: 64 nodes of 8192 slots is level 6 at J = 2^19);
    use_tc = 1: the double-buffered kernel of the deeper levels
    (bfs_level_tc_kernel; 1024 nodes of 512 slots).  One launch reads every
    vector once (J R 4 bytes, gathered rows) and each node's packed Gram
    once; its tensor-core work is two TF32 MMAs per K step (2 J R^2
    multiply-adds).  CUDA events on the launching stream, the average of
    `launches` launches after two warm-up launches; inputs (J R 4 bytes,
    268 MB at J = 2^19, R = 128) larger than L2."""
    import torch

    from rdist_tensor_gb300 import _lib

    Pf = (R * (R + 1) // 2 + 3) & ~3
    g = torch.Generator(device="cuda").manual_seed(seed)
    X = torch.randn((J, R), generator=g, device="cuda", dtype=torch.float32)
    G = torch.randn((nodes, Pf), generator=g, device="cuda", dtype=torch.float32)
    node = torch.sort(torch.randint(0, nodes, (J,), generator=g, device="cuda")).values.contiguous()
    q = torch.empty(J, dtype=torch.float32, device="cuda")
    st = torch.cuda.current_stream()
    args = (R, J, ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(node.data_ptr()), ctypes.c_void_p(G.data_ptr()),
            ctypes.c_void_p(q.data_ptr()), use_tc, ctypes.c_void_p(st.cuda_stream))
    for _ in range(2):
        _lib.call("exafac_quad_forms_f32", *args)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(launches):
        _lib.call("exafac_quad_forms_f32", *args)
    e1.record(st)
    torch.cuda.synchronize()
    dur = e0.elapsed_time(e1) * 1e-3 / launches
    used = int(torch.unique(node).numel())
    algo = J * R * 4 + used * Pf * 4
    peak, peak_kind = measured_peaks()
    achieved = algo / dur / 1e9
    name = ("bfs_level_tcr_kernel (tcgen05 quadratic forms of a descent level, node resident)" if use_tc == 2 else
            "bfs_level_tc_kernel (tcgen05 quadratic forms of a descent level, double-buffered slots)")
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": name, "algorithmic_bytes": algo, "duration_s": dur, "launches": launches,
            "peak_source": peak_kind, "tensor_tflops": 2.0 * J * R * R / dur / 1e12, "J": J, "R": R,
            "nodes": used}


def gcp_adjoint_roofline(model, J_nz, J_z, launches=20):
    """Roofline of the GCP step's dominant kernel of this library, the
    sampled adjoint (cp_adjoint_kernel, the sampled MTTKRP of the loss
    derivatives into every factor), timed live: `launches` launches, each on
    its own fresh stratified sample (so the rows it touches are not the last
    launch's), CUDA events on the launching stream after two warm-ups.
    Algorithmic bytes per launch, J entries: per entry its N coordinates and
    its loss derivative (4 N + 4), the N factor rows it reads (N R 4) and the
    N gradient rows it adds into (N R 4, each counted once)."""
    import torch

    from rdist_tensor_gb300 import _lib, gcp

    N, R, J = model.N, model.R, J_nz + J_z
    samples = [model.step_sample(J_nz, J_z)[0] for _ in range(launches)]
    gm = torch.rand(J, dtype=torch.float32, device="cuda")
    grads = [torch.zeros_like(U) for U in model.factors]
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream()
    dims = gcp._dims_arg(model.dims)

    def launch(idx):
        _lib.call("exafac_cp_sampled_adjoint", N, R, dims, J, ctypes.c_void_p(idx.data_ptr()),
                  ctypes.c_void_p(gm.data_ptr()), gcp._ptrs([U.detach() for U in model.factors]), gcp._ptrs(grads),
                  0, ctypes.c_void_p(status.data_ptr()), ctypes.c_void_p(st.cuda_stream))

    for k in range(2):
        launch(samples[k])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for idx in samples:
        launch(idx)
    e1.record(st)
    torch.cuda.synchronize()
    if int(status.item()) != 0:
        raise RuntimeError("adjoint flagged an out-of-range entry")
    dur = e0.elapsed_time(e1) * 1e-3 / launches
    algo = J * (4 * N + 4) + 2 * J * N * R * 4
    peak, peak_kind = measured_peaks()
    achieved = algo / dur / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": None, "kernel": "cp_adjoint_kernel (sampled MTTKRP of the loss derivatives, every mode)",
            "algorithmic_bytes": algo, "duration_s": dur, "launches": launches, "peak_source": peak_kind, "J": J,
            "R": R}


def gcp_cpu_sample(dims, idx_np, vals_np, R, J_nz, J_z, lr, steps, seed=0):
    """The same GCP step restated with torch on the host cores (no
    counterpart exists in the reference): stratified sample, model values
    from gathered factor rows, weighted Poisson loss, autograd gradient
    (index-add backward), Adam and the projection onto nonnegative factors,
    on factors of the workload's full size.  Returns (steps/s, threads)."""
    import torch

    g = torch.Generator().manual_seed(seed)
    idx = torch.as_tensor(idx_np.astype(np.int64))
    vals = torch.as_tensor(vals_np.astype(np.float32))
    U = [torch.rand((int(d), R), generator=g) * 0.5 for d in dims]
    for u in U:
        u.requires_grad_()
    opt = torch.optim.Adam(U, lr=lr)
    nnz, total = idx.shape[0], float(np.prod([float(d) for d in dims]))
    wnz, wz = nnz / J_nz, (total - nnz) / J_z

    def step():
        pick = torch.randint(0, nnz, (J_nz,), generator=g)
        rows = torch.cat([idx[pick], torch.stack([torch.randint(0, int(d), (J_z,), generator=g) for d in dims], 1)])
        x = torch.cat([vals[pick], torch.zeros(J_z)])
        w = torch.cat([torch.full((J_nz,), wnz), torch.full((J_z,), wz)])
        m = U[0][rows[:, 0]]
        for k in range(1, len(U)):
            m = m * U[k][rows[:, k]]
        m = m.sum(dim=1)
        opt.zero_grad(set_to_none=True)
        f = (w * (m - x * torch.log(m + 1e-10))).sum()
        f.backward()
        opt.step()
        with torch.no_grad():
            for u in U:
                u.clamp_(min=0.0)

    step()
    t = time.perf_counter()
    for _ in range(steps):
        step()
    return steps / (time.perf_counter() - t), torch.get_num_threads()


def run_gcp(args, w):
    """The GCP line: gradient-based Poisson GCP through the autograd sampled
    adjoint, K Adam steps timed with CUDA events after W warm-up steps, the
    tensor resident on the GPU."""
    import torch

    from rdist_tensor_gb300 import _lib, gcp, synthetic

    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    lib = _lib.load()
    t = time.perf_counter()
    dims, idx, vals, _ = synthetic.poisson_counts_device(w["dims"], w["nnz"], rank=w["planted_rank"],
                                                         seed=args.seed + rank)
    torch.cuda.synchronize()
    log(f"generated {idx.shape[0]} nonzeros in {time.perf_counter() - t:.1f}s")
    R, J, lr = w["R"], w["J"], w["lr"]
    J_nz = J // 2
    J_z = J - J_nz
    steps = args.steps if args.steps is not None else w["steps"]
    warmup = args.warmup
    model = gcp.GCP(idx, vals, dims, rank=R, loss="poisson", seed=1)
    if args.nvtx_sweep:  # W steps, then 5 inside the NVTX range 'sweep' (for a launch list)
        for _ in range(warmup):
            model.step(J_nz, J_z, lr)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        torch.cuda.nvtx.range_push("sweep")
        for _ in range(5):
            model.step(J_nz, J_z, lr)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        print(json.dumps({"nvtx_steps": 5, "elapsed_s": time.perf_counter() - t0, "workload": w["desc"]}),
              flush=True)
        return 0
    f_start = model.full_objective()
    clocks = ClockSampler(local)
    clocks.start()
    for _ in range(warmup):
        model.step(J_nz, J_z, lr)
    torch.cuda.synchronize()
    l0 = lib.exafac_kernel_launches()
    barrier(ws)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks.begin()
    e0.record()
    for _ in range(steps):
        f = model.step(J_nz, J_z, lr)
    e1.record()
    torch.cuda.synchronize()
    clocks.end()
    barrier(ws)
    elapsed = max_over_ranks(e0.elapsed_time(e1) * 1e-3, ws)
    launches = lib.exafac_kernel_launches() - l0
    clk = clocks.stop()
    value = ws * steps / elapsed
    f_end = model.full_objective()
    log(f"gcp: {value:.1f} steps/s, objective {f_start:.6e} -> {f_end:.6e}")

    # optimizer share: the fused Adam + projection alone, on the last step's
    # gradients
    opt = model.optimizer(lr)
    k_opt = 20
    torch.cuda.synchronize()
    o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    o0.record()
    for _ in range(k_opt):
        opt.step()
    o1.record()
    torch.cuda.synchronize()
    opt_ms = o0.elapsed_time(o1) / k_opt

    roofline = gcp_adjoint_roofline(model, J_nz, J_z)

    # e2e: the public API step with every step's objective read back to
    # pinned host memory inside the timed region
    e2e_steps = min(steps, 50)
    host_f = torch.empty(e2e_steps, dtype=torch.float32, pin_memory=True)
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    for k in range(e2e_steps):
        host_f[k].copy_(model.step(J_nz, J_z, lr), non_blocking=True)
    torch.cuda.synchronize()
    e2e_el = max_over_ranks(time.perf_counter() - t0, ws)
    if not bool(torch.isfinite(host_f).all()):
        raise RuntimeError("a sampled objective is not finite")
    e2e = {"value": ws * e2e_steps / e2e_el, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 4,
           "steps": e2e_steps,
           "note": "GCP.step through the public API; the step's sample is drawn on the device from (seed, "
                   "counter), so it has no host input; its sampled objective is read back every step"}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        idx_np, vals_np = idx.cpu().numpy(), vals.cpu().numpy()
        cval, cores = gcp_cpu_sample(dims, idx_np, vals_np, R, J_nz, J_z, lr, w["cpu_steps"])
        cpu = {"value": cval, "unit": "steps/s", "cores": cores, "kind": "port",
               "sample": f"{w['cpu_steps']} full-size steps (after one untimed) of the same GCP step restated "
                         "with torch on the host cores; the reference has no GCP"}
    if rank != 0:
        return 0
    cfg = {"workload": w["desc"], "nnz": int(idx.shape[0]), "R": R, "J": J, "J_nonzeros": J_nz, "J_zeros": J_z,
           "lr": lr, "loss": "poisson", "init": "Uniform(0, 0.5) factors",
           "parallelism": f"{ws} independent replica(s)",
           "l2": "inputs larger than L2 (factors, Adam moments and gradients: 1.03 GB)",
           "objective_start": f_start, "objective_end": f_end,
           "objective": "exact Poisson objective over all 1e16 entries (model mass - sum_nz x log m)",
           "steps_run": warmup + steps, "optimizer_ms_per_step": opt_ms,
           "optimizer_bytes_per_step": 7 * 4 * sum(int(d) for d in dims) * R,
           "optimizer_gbs": 7 * 4 * sum(int(d) for d in dims) * R / (opt_ms * 1e-3) / 1e9,
           "step_kernels_of_this_library": "gcp_sample_kernel, cp_model_kernel, cp_adjoint_kernel, "
                                           "adam_step_kernel (Adam fused with the projection); the loss terms and "
                                           "their derivative are torch elementwise ops under autograd"}
    line = {"metric": GCP_METRIC, "value": value, "unit": "steps/s", "n_gpus": ws, "steps": steps,
            "warmup": warmup, "ms_per_step": 1000.0 * elapsed / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded; no public dataset is named for this shape)", "config": cfg,
            "roofline": roofline, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk}
    if cpu is not None:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    return 0


def make_workload(w, seed=0):
    """Seeded synthetic tensor of the workload on the GPU: (dims, int32
    coordinates, values) as device tensors."""
    import torch

    from rdist_tensor_gb300 import synthetic

    t = time.perf_counter()
    if w["gen"] == "planted":
        dims, idx, vals = synthetic.planted_uniform(dims=w["dims"], nnz=w["nnz"], seed=seed)
        idx = torch.as_tensor(idx.astype(np.int32)).cuda()
        vals = torch.as_tensor(vals).cuda()
    else:
        dims, idx, vals = synthetic.zipf_tensor_device(w["dims"], w["nnz"], alpha=w["alpha"], values=w["values"],
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
    log(f"{precision}: initialised (sorted copies, hash tables, sampler) in {time.perf_counter() - t:.1f}s")
    if w["exact_pre"]:
        t = time.perf_counter()
        for n in range(N):
            opt.exact_step(n)
        torch.cuda.synchronize()
        log(f"{precision}: exact-ALS preprocessing sweep in {time.perf_counter() - t:.2f}s, "
            f"fit {opt.compute_exact_fit():.6f}")
    return opt, lr, st


def design_bytes(precision):
    """Bytes of one design-row element the sampled MTTKRP reads: FP64 rows in
    the FP64 form, FP32 rows in the mixed forms."""
    return 8 if precision == "fp64" else 4


def algorithmic_bytes(N, R, Ju, H, touched, s_d=8):
    """Sampled MTTKRP bytes of one step: sample keys, weights and design rows
    (s_d bytes per element) read once, each hit's mode-n index and value,
    touched output rows written once (zeroing of the previous rows and the
    write of the new ones)."""
    return Ju * (N - 1) * 4 + Ju * 8 + Ju * R * s_d + H * (4 + 8) + 2 * touched * R * 8


def uniforms_per_step(N, J, sampler):
    return N * (2 if sampler == "sts_cp" else 1) * J


def cpu_port_sample(w, dims, ora, sweeps, warmup):
    """The oracle port of the reference (OpenMP C loops + numpy/LAPACK) on the
    host cores: `sweeps` sampled sweeps at the workload's CPU sample size
    (J = cpu_J samples per step; the first cpu_nnz nonzeros when the workload
    names a subsample), after set-up and `warmup` untimed sweeps.  Returns
    (sweeps/s scaled to the workload's J, elapsed s, threads, fit, sample
    text).  The sampling (tree descents or CDF draws) and the design rows cost
    J per step; the scaling by cpu_J / J holds for them, and is stated."""
    from oracle import oracle as O

    J = w.get("cpu_J", w["J"])
    rng = np.random.default_rng(3)
    N = len(dims)
    shape = (N, J) if w["sampler"] == "cp_arls_lev" else (N, 2, J)
    for _ in range(warmup):
        for n in range(N):
            ora.step(n, J, rng.random(shape))
    t = time.perf_counter()
    for _ in range(sweeps):
        for n in range(N):
            ora.step(n, J, rng.random(shape))
    el = time.perf_counter() - t
    scale = J / w["J"]
    sample = (f"{sweeps} sampled sweep(s) at J={J} per step" +
              (f" on the first {ora.idx.shape[0]} nonzeros" if w.get("cpu_nnz") else " on the full tensor") +
              (f", scaled by {J}/{w['J']} to the workload's J (sampling cost is linear in J)" if scale != 1 else "") +
              f"; starting factors {'after one exact-ALS sweep on the GPU' if w['exact_pre'] else 'N(0,1)'}; "
              "oracle restatement (pinned to the reference by golden vectors), OpenMP over all host threads")
    return sweeps / el * scale, el, O.lib().or_num_threads(), ora.fit(), sample


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


def host_copy(dims, idx, vals):
    return idx.cpu().numpy().astype(np.uint32), vals.cpu().numpy().astype(np.float64)


def oracle_start(w, dims, idx_np, vals_np):
    """The oracle port on the CPU sample's nonzeros (the first cpu_nnz when
    the workload names a subsample), from N(0,1) factors with normalised
    columns, after (Zipf workloads) one exact-ALS sweep as the GPU arm's
    preprocessing.  Set-up and that sweep are untimed."""
    from oracle import oracle as O
    from rdist_tensor_gb300 import synthetic

    nnz = w.get("cpu_nnz")
    if nnz is not None and nnz < len(vals_np):
        idx_np, vals_np = idx_np[:nnz], vals_np[:nnz]
    factors = synthetic.gaussian_factors(dims, w["R"], seed=1)
    t = time.perf_counter()
    ora = O.OracleALS(dims, idx_np, vals_np, factors, w["sampler"])
    log(f"cpu port: set-up {time.perf_counter() - t:.1f}s")
    if w["exact_pre"]:
        t = time.perf_counter()
        O.exact_als_sweep(ora, 1)
        log(f"cpu port: exact-ALS sweep {time.perf_counter() - t:.1f}s")
    return ora


def run_reference(args, w):
    ws, rank, local = dist_init()
    if rank != 0:
        return 0
    import torch

    dims, idx, vals = make_workload(w)
    idx_np, vals_np = host_copy(dims, idx, vals)
    del idx, vals
    torch.cuda.empty_cache()
    sweeps = max(1, min(args.steps, args.ref_sweeps))
    warm = min(args.warmup, 1)
    ora = oracle_start(w, dims, idx_np, vals_np)
    value, el, cores, fit, sample = cpu_port_sample(w, dims, ora, sweeps, warm)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": args.gpus,
            "steps": sweeps, "warmup": warm, "ms_per_step": 1000.0 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded, see config)",
            "config": {"workload": w["desc"], "nnz": int(len(vals_np)), "R": w["R"], "J": w["J"],
                       "sampler": w["sampler"], "fit_after_sample": fit},
            "cpu_baseline": {"value": value, "unit": "sweeps/s", "cores": cores, "kind": "port",
                             "sample": sample + "; the reference's C++ cannot be rebuilt on this machine (its "
                                                "sources are not here), so the oracle restatement runs"},
            "e2e": {"value": value, "unit": "sweeps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args, w):
    import torch

    from rdist_tensor_gb300 import _lib

    ws, rank, local = dist_init()
    torch.cuda.set_device(local)
    lib = _lib.load()
    if args.kernel_only:  # the level kernels alone (for a kernel profile): resident-node, then double-buffered
        print(json.dumps({"roofline": level_kernel_roofline(w["R"], w["J"]),
                          "roofline_deep_levels": level_kernel_roofline(w["R"], w["J"], nodes=1024, use_tc=1)}),
              flush=True)
        return 0
    dims, idx, vals = make_workload(w, seed=args.seed + rank)
    N, R, J = len(dims), w["R"], w["J"]
    nnz = int(idx.shape[0])
    precision = args.precision or w["precision"]
    steps = args.steps if args.steps is not None else w["steps"]
    warmup = args.warmup

    def timed(opt, sweeps, clocks=None):
        # execute_sweeps: the first sweep runs step by step, later ones replay
        # one captured sweep (a CUDA graph); the capture happens in the warm-up.
        if clocks:
            clocks.start()
        opt.execute_sweeps(warmup, J)
        torch.cuda.synchronize()
        l0 = lib.exafac_kernel_launches()
        barrier(ws)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if clocks:
            clocks.begin()
        e0.record()
        opt.execute_sweeps(sweeps, J)
        e1.record()
        torch.cuda.synchronize()
        if clocks:
            clocks.end()
        barrier(ws)
        el = max_over_ranks(e0.elapsed_time(e1) * 1e-3, ws)
        opt.step_info()  # raises if a kernel reported a device-side error
        return el, lib.exafac_kernel_launches() - l0, opt.compute_exact_fit()

    def e2e_run(opt, lr, sweeps):
        """The same metric through the public API with host buffers: every
        sweep's uniforms come from pinned host memory and its sigma goes back
        to pinned host memory, inside the timed region.  The copy of sweep
        s+1's uniforms runs on a copy stream into a staging buffer while sweep
        s computes; a device copy moves it into the buffer the captured sweep
        reads.  The host reads sweep s-1's sigma (and checks it) once sweep s
        is queued, so at most two sweeps are in flight."""
        per = uniforms_per_step(N, J, w["sampler"])
        nbuf = min(sweeps, 4)  # distinct pinned input blocks, used in turn
        host_uni = torch.empty((nbuf, N * per), dtype=torch.float64, pin_memory=True)
        host_uni.copy_(torch.rand((nbuf, N * per), dtype=torch.float64))
        dev_uni = torch.empty(N * per, dtype=torch.float64, device="cuda")
        stage = [torch.empty_like(dev_uni) for _ in range(2)]
        sig_host = torch.empty((sweeps, R), dtype=torch.float64, pin_memory=True)
        main_st = torch.cuda.current_stream()
        copy_st = torch.cuda.Stream()
        ev_staged = [torch.cuda.Event() for _ in range(2)]
        ev_free = [torch.cuda.Event() for _ in range(2)]
        ev_done = [torch.cuda.Event() for _ in range(sweeps)]

        def stage_in(k):
            b = k % 2
            with torch.cuda.stream(copy_st):
                copy_st.wait_event(ev_free[b])  # the device copy out of this buffer is done
                stage[b].copy_(host_uni[k % nbuf], non_blocking=True)
                ev_staged[b].record(copy_st)

        def check_sigma(k):
            ev_done[k].synchronize()
            if not bool(torch.isfinite(sig_host[k]).all()):
                raise RuntimeError(f"sweep {k}: sigma is not finite")

        # one untimed sweep with these buffers: it captures the sweep graph for them
        dev_uni.copy_(host_uni[0], non_blocking=True)
        opt.execute_sweeps(1, J, dev_uni)
        torch.cuda.synchronize()
        barrier(ws)
        t0 = time.perf_counter()
        stage_in(0)
        for k in range(sweeps):
            b = k % 2
            if k + 1 < sweeps:
                stage_in(k + 1)
            main_st.wait_event(ev_staged[b])
            dev_uni.copy_(stage[b], non_blocking=True)
            ev_free[b].record(main_st)
            opt.execute_sweeps(1, J, dev_uni)
            sig_host[k].copy_(lr.sigma, non_blocking=True)
            ev_done[k].record(main_st)
            if k >= 1:
                check_sigma(k - 1)
        check_sigma(sweeps - 1)
        torch.cuda.synchronize()
        el = max_over_ranks(time.perf_counter() - t0, ws)
        opt.step_info()  # raises if a kernel reported a device-side error
        return {"value": ws * sweeps / el, "unit": "sweeps/s", "h2d_bytes_per_step": N * per * 8,
                "d2h_bytes_per_step": R * 8, "sweeps": sweeps}

    if args.nvtx_sweep:  # one sweep step by step inside an NVTX range (for a launch list)
        opt, lr, _ = build_optimizer(w, dims, idx, vals, J, precision)
        for _ in range(warmup):
            for n in range(N):
                opt.execute_ALS_step(n, J)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        torch.cuda.nvtx.range_push("sweep")
        for n in range(N):
            opt.execute_ALS_step(n, J)
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        opt.step_info()
        print(json.dumps({"nvtx_sweep_s": el, "precision": precision, "workload": w["desc"],
                          "fit": opt.compute_exact_fit()}), flush=True)
        opt.deinitialize()
        return 0

    # ---- the FP64 form (the reference's arithmetic), and other mixed forms --
    forms = {}
    compare = [] if (precision == "fp64" or args.no_fp64_form) else ["fp64"]
    compare += [f for f in w.get("other_forms", ()) if f != precision and not args.no_fp64_form]
    for prec in compare:
        opt, lr, _ = build_optimizer(w, dims, idx, vals, J, prec)
        el, _, fit = timed(opt, steps)
        rec = {"precision": prec, "sweeps_per_s": ws * steps / el, "fit_after": fit,
               "sweeps": warmup + steps + (1 if w["exact_pre"] else 0)}
        if prec == "fp64":
            rec["e2e"] = e2e_run(opt, lr, min(steps, 3))
        forms[prec] = rec
        log(f"{prec} form: {rec['sweeps_per_s']:.3f} sweeps/s, fit {fit:.6f}")
        opt.deinitialize()
        del opt, lr
        torch.cuda.empty_cache()

    # ---- timed region: K sweeps of the measured form, tensor resident -----
    opt, lr, st = build_optimizer(w, dims, idx, vals, J, precision)
    clocks = ClockSampler(local)
    elapsed, launches, fit = timed(opt, steps, clocks)
    clk = clocks.stop()
    value = ws * steps / elapsed
    log(f"{precision} form: {value:.3f} sweeps/s, fit {fit:.6f}")

    # ---- roofline of the sampled MTTKRP (region timers, one sweep) -------
    _lib.call("exafac_als_enable_timing", opt._h, 1)
    tot_bytes, units = 0.0, []
    for n in range(N):
        opt.execute_ALS_step(n, J)
        info = opt.step_info()
        tot_bytes += algorithmic_bytes(N, R, info.unique_samples, info.hits, info.touched_rows,
                                       design_bytes(precision))
        units.append((info.unique_samples, info.hits, info.touched_rows))
    regions = (ctypes.c_double * 7)()
    _lib.call("exafac_als_region_times", opt._h, regions)
    _lib.call("exafac_als_enable_timing", opt._h, 0)
    opt.timing = False
    spmm_s = regions[3]
    peak, peak_kind = measured_peaks()
    achieved = tot_bytes / spmm_s / 1e9 if spmm_s > 0 else None
    region_names = ["leverage_sampling", "row_gather", "design_matrix_prep", "spmm", "dense_reduce",
                    "postprocessing", "sampler_update"]
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": (achieved / peak) if achieved else None, "traffic": None,
                "traffic_note": "ncu DRAM bytes of this region: see the profiles of this workload",
                "kernel": "sampled MTTKRP region (lookup, hit grouping, segmented reduction + solve), per sweep",
                "algorithmic_bytes": tot_bytes, "duration_s": spmm_s, "peak_source": peak_kind,
                "design_element_bytes": design_bytes(precision),
                "regions_s": dict(zip(region_names, list(regions))),
                "units_per_step": [{"unique_samples": a, "hits": b, "touched_rows": c} for a, b, c in units]}

    # ---- roofline of the dominant kernel (the mixed STS-CP descents') -----
    mttkrp = deep = None
    if w["sampler"] == "sts_cp" and precision != "fp64" and R >= 32:
        mttkrp = roofline
        roofline = level_kernel_roofline(R, J)
        deep = level_kernel_roofline(R, J, nodes=1024, use_tc=1)

    # ---- the drop-in round loop (execute_ALS_rounds, region timers on) ----
    rounds = 2
    opt.execute_ALS_rounds(rounds, J, rounds)
    stats = json.loads(opt.get_statistics_json())
    drop_in = {"sweeps_per_s": rounds / stats["als_total_time"], "rounds": rounds,
               "note": "ALS_Optimizer.execute_ALS_rounds with its region timers, step by step (no graph replay)"}

    # ---- e2e through the public API with host buffers ---------------------
    e2e = e2e_run(opt, lr, steps)

    # ---- CPU baseline (rank 0, one GPU only) ------------------------------
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        idx_np, vals_np = host_copy(dims, st.indices, st.values)
        opt.deinitialize()
        ora = oracle_start(w, dims, idx_np, vals_np)
        cval, cel, cores, cfit, sample = cpu_port_sample(w, dims, ora, 1, 0)
        cpu = {"value": cval, "unit": "sweeps/s", "cores": cores, "kind": "port", "sample": sample}
    opt.deinitialize()
    if rank != 0:
        return 0
    dtype = {"fp64": "f64", "tf32": "tf32 design Gram; fp32 rows, MTTKRP, solve and tree descents; "
                                    "fp64 Gram chain, pinv, tree sums, CDF",
             "bf16": "bf16 design Gram; fp32 rows, MTTKRP, solve and tree descents; "
                     "fp64 Gram chain, pinv, tree sums, CDF"}[precision]
    cfg = {"workload": w["desc"], "nnz": nnz, "R": R, "J": J, "sampler": w["sampler"], "precision": precision,
           "preprocessing": "one exact-ALS sweep, untimed" if w["exact_pre"] else "none (N(0,1) factors)",
           "parallelism": f"{ws} independent replica(s)",
           "l2": "inputs larger than L2 (per-mode sorted copies and hash tables)", "fit_after": fit,
           "sweeps_run": warmup + steps + (1 if w["exact_pre"] else 0), "drop_in_rounds": drop_in}
    if "fp64" in forms:
        ref = forms["fp64"]
        cfg["fp64_form"] = ref
        cfg["speedup_vs_fp64_form"] = value / ref["sweeps_per_s"]
        cfg["fit_gap_vs_fp64_form"] = abs(fit - ref["fit_after"])
        cfg["equal_fit_1e-3"] = bool(abs(fit - ref["fit_after"]) <= 1e-3)
    for prec, rec in forms.items():
        if prec != "fp64":
            cfg[f"{prec}_form"] = rec
    line = {"metric": METRIC, "value": value, "unit": "sweeps/s", "n_gpus": ws, "steps": steps,
            "warmup": warmup, "ms_per_step": 1000.0 * elapsed / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype,
            "data": "synthetic (seeded; no public dataset is named for these shapes)",
            "config": cfg, "roofline": roofline, "e2e": e2e, "gpu_launches": int(launches), "clocks": clk}
    if mttkrp is not None:
        line["roofline_sampled_mttkrp"] = mttkrp
        line["roofline_deep_levels"] = deep
    if cpu is not None:
        line["cpu_baseline"] = cpu
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed sweeps (default: the workload's count)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default=None, choices=["fp64", "tf32", "bf16"],
                    help="form timed for `value` (default: the workload's); a mixed form is also compared with "
                         "the FP64 form")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-sweeps", type=int, default=1)
    ap.add_argument("--no-fp64-form", action="store_true",
                    help="skip timing the FP64 form beside a mixed form (for kernel profiling runs)")
    ap.add_argument("--nvtx-sweep", action="store_true",
                    help="after the warm-up sweeps, run one sweep step by step inside the NVTX range 'sweep', "
                         "print its time and exit (for an ncu launch list)")
    ap.add_argument("--kernel-only", action="store_true",
                    help="time the dominant kernel alone on the workload's J and R and exit (for a kernel profile)")
    args = ap.parse_args()
    w = WORKLOADS[args.workload]
    if w.get("kind") == "gcp":
        if args.impl == "reference":
            if int(os.environ.get("RANK", "0")) == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference has no GCP; its "
                                                                      "CPU restatement is this line's cpu_baseline"}))
            return 0
        return run_gcp(args, w)
    if args.impl == "reference":
        if args.steps is None:
            args.steps = w["steps"]
        return run_reference(args, w)
    return run_gpu(args, w)


if __name__ == "__main__":
    sys.exit(main())
