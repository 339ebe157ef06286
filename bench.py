#!/usr/bin/env python
"""Benchmark of the FDTD step loop (one JSON line on stdout, rank 0).

Workload: the heterogeneous-dielectric grid, 320×192×128 cells, 12-cell CPML
(CUDA-path CPML semantics), Si strip + random 2×2×0.22 µm design region,
y-polarised Gaussian current plane, two 21-frequency flux planes with
Kahan-compensated FP32 DFT accumulation; FP32 bulk arithmetic.  A "step" is
one full FDTD time step (H half-step + E half-step + DFT on decimation steps)
over the whole grid; the metric is cell-updates per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU: replicas only (one independent simulation per GPU, no collective
on the data path); value = all ranks' cell-updates / max-over-ranks time.
The reference arm times the CPU restatement of the reference's CPU step loop
(the reference is Julia and cannot run here) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

METRIC = "Gcell-updates/s & %HBM roofline; serve p50/p99 latency at 1e-4 flux error"
UNIT = "Gcell-updates/s"
WORKLOAD = ("waveguide 320x192x128 FP32, 12-cell CPML (CUDA-path semantics), Si strip eps 12.25 in "
            "eps 2.085 + random 2x2x0.22um design (seed 1234, 3-cell box filter), Ey Gaussian current "
            "plane (waist 0.4um), Gaussian pulse fcen=1/1.55 fwidth=0.25fcen, 2 flux planes x 21 freqs, "
            "Kahan FP32 DFT")


def dist_env():
    return int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), int(
        os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, period_ms: int = 100):
        self.cmd = ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.FIELDS}",
                    "--format=csv,noheader,nounits", f"-lms", str(period_ms)]
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(self.cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=5)

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    p = ROOT / "profiles" / "dram_traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    v = d.get(kernel)
    return None if v is None else float(v)


WORKLOADS = {
    "waveguide": WORKLOAD,
    "dispersive": ("dispersive 256^3 FP32, 12-cell CPML (CUDA-path semantics), eps 2.25 slab with chi3=1e-3, "
                   "4 Lorentz (eps_inf 2, sigma 1, f0 1, gamma 0.05) + 4 Drude (eps_inf 1, wp 5, gamma 0.1) "
                   "spheres (seed 42), Ez Gaussian plane source, 6-face box flux x 11 freqs, Kahan FP32 DFT"),
}
_workload_name = "waveguide"


def build_workload(dtype="f32", semantics="cpml"):
    __graft_entry__.package()
    from khronos_gb300 import configs

    w = configs.BUILDERS[_workload_name](dtype=dtype)
    w.sim.semantics = semantics
    return w, w.sim.spec()


def cpu_baseline(spec, budget_s=12.0):
    """The CPU restatement on the host cores, on a bounded number of full-grid steps."""
    orc = __graft_entry__._oracle()
    o = orc.OracleSim(spec)
    t0 = time.perf_counter()
    o.step(2)
    per = max((time.perf_counter() - t0) / 2, 1e-6)
    n = int(max(3, min(200, budget_s / per)))
    t0 = time.perf_counter()
    o.step(n)
    dt = time.perf_counter() - t0
    o.close()
    cells = spec.cells
    return {"value": cells * n / dt / 1e9, "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
            "sample": f"{n} full-grid steps of the same workload after 2 warm-up steps "
                      f"({cells} cells, FP32, C++ restatement of the reference CPU step loop, OpenMP)"}


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    w, spec = build_workload("f32", "reference_cpu")
    orc = __graft_entry__._oracle()
    o = orc.OracleSim(spec)
    o.step(max(args.warmup, 1))
    # each timed step is one full-grid step; bound the run to about a minute
    t0 = time.perf_counter()
    o.step(1)
    per = max(time.perf_counter() - t0, 1e-6)
    k = int(max(1, min(args.steps, 60.0 / per)))
    t0 = time.perf_counter()
    o.step(k)
    dt = time.perf_counter() - t0
    value = spec.cells * k / dt / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": k, "warmup": args.warmup, "ms_per_step": dt / k * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOADS[_workload_name].replace("CUDA-path semantics",
                                                                  "reference CPU-path semantics"),
                   "grid": list(spec.n), "note": "reference is Julia (absent); timed: its CPU step loop "
                                                 "restated in C++ (oracle/), all host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
                         "sample": f"{k} full-grid steps (requested {args.steps}) after {args.warmup} warm-up"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, world, rank, local_rank):
    import torch

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
        dist = dist_mod
    __graft_entry__.package()
    from khronos_gb300.device import GpuSim

    w, spec = build_workload("f32", "cpml")
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    # ---- device-resident run: inputs already in HBM --------------------------
    gpu = GpuSim(spec)
    gpu.step(args.warmup, sh)
    torch.cuda.synchronize()
    h_bytes, e_bytes, dft_bytes = gpu.model_bytes_split()
    launches0 = gpu.launches
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        start.record(stream)
        h_ms, e_ms, dft_ms = gpu.step_timed(args.steps, sh)
        end.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = start.elapsed_time(end)
    launches = gpu.launches - launches0
    from khronos_gb300.replicas import aggregate_rate, max_over_ranks

    ms_max = max_over_ranks(ms, dist, device="cuda")
    cells = spec.cells
    value = aggregate_rate(cells * args.steps, ms_max / 1e3, world) / 1e9
    gpu.close()

    # ---- end to end through the C ABI with host buffers ------------------------
    e2e = None
    if not args.no_e2e:
        e2e = end_to_end(args, spec, w, sh, world, dist, cells)
    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    peak, peak_kind = measured_peaks()
    simt = os.environ.get("KHRONOS_GB300_KERNEL") == "simt"
    e_kernel = "half_step_kernel<float,E>" if simt else "half_step_tma_kernel<float,E>"
    e_launch_ms = e_ms / args.steps
    achieved = e_bytes / (e_launch_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOADS[_workload_name], "grid": list(spec.n), "cells": cells,
                   "l2": "inputs larger than L2 (fields+materials+CPML state ~0.9 GB per replica vs 129 MB L2); no flush",
                   "parallelism": f"replicas{world}" if world > 1 else "single"},
        "roofline": {"bound": "hbm", "kernel": e_kernel, "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "algorithmic_bytes_per_launch": e_bytes,
                     "traffic": ncu_traffic(e_kernel) if _workload_name == "waveguide" else None,
                     "h_kernel": {"achieved": h_bytes / (h_ms / args.steps / 1e3) / 1e9,
                                  "algorithmic_bytes_per_launch": h_bytes, "ms_per_launch": h_ms / args.steps},
                     "e_ms_per_launch": e_launch_ms, "dft_ms_per_step": dft_ms / args.steps,
                     "step_model_bytes": h_bytes + e_bytes + dft_bytes,
                     "step_achieved": (h_bytes + e_bytes + dft_bytes) / (ms_max / args.steps / 1e3) / 1e9},
        "clocks": clk.summary(),
        "gpu_launches": launches,
    }
    if e2e is not None:
        line["e2e"] = e2e
    if not args.no_flux_check:
        line["flux_error"] = flux_accuracy(w, sh)
    if world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(spec)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def flux_accuracy(w, sh):
    """Flux spectra of the full FP32 run against the full FP64 run of the same
    inputs (the FP32 spec promoted; the FP64 kernels match the FP64 oracle to
    1e-10 in the parity tests); relative L2 over the frequencies, worst plane."""
    from khronos_gb300.device import GpuSim
    from khronos_gb300.monitors import flux_error

    fluxes = {}
    _, spec32 = build_workload("f32", "cpml")
    for dt, spec in (("f32", spec32), ("f64", spec32.promoted())):
        g = GpuSim(spec)
        g.step(w.steps, sh)
        fluxes[dt] = [g.flux(list(range(4 * i, 4 * i + 4)), fm.normal_axis, fm.dA)
                      for i, fm in enumerate(w.flux_monitors)]
        g.close()
    errs = [flux_error(a, b) for a, b in zip(fluxes["f32"], fluxes["f64"])]
    return {"rel_l2": max(e["rel_l2"] for e in errs), "max_rel": max(e["max_rel"] for e in errs),
            "per_plane": errs, "steps": w.steps, "frequencies": len(w.flux_monitors[0].frequencies),
            "vs": "FP64 run of the same inputs (FP32 spec promoted) and step count"}


def end_to_end(args, spec, w, sh, world, dist, cells):
    """Same metric through the C ABI from host buffers: create + upload, K steps,
    DFT arrays and fluxes read back to the host, all inside the timed region."""
    import torch
    from khronos_gb300.device import GpuSim

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g2 = GpuSim(spec)  # host arrays -> device (materials, σ, sources, monitors)
    g2.step(args.steps, sh)
    dft_host = [g2.dft(m) for m in range(len(spec.monitors))]
    fluxes = [g2.flux(list(range(4 * i, 4 * i + 4)), fm.normal_axis, fm.dA)
              for i, fm in enumerate(w.flux_monitors)]
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    g2.close()
    h2d = sum(a.nbytes for _, _, a in spec.materials) // 2  # values cross as the run's FP32
    h2d += sum(s.amp.size * 16 for s in spec.sources) + sum(x.size * 8 for x in spec.sigma_b + spec.sigma_d
                                                            if x is not None)
    d2h = sum(d.size * 16 for d in dft_host) + sum(f.size * 8 for f in fluxes)
    from khronos_gb300.replicas import aggregate_rate, max_over_ranks

    e2e_max = max_over_ranks(e2e_s, dist, device="cuda")
    return {"value": aggregate_rate(cells * args.steps, e2e_max, world) / 1e9, "unit": UNIT,
            "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
            "scope": "GpuSim(spec) from host arrays + K steps + DFT arrays and flux read back to host"}


def _pct(v, q):
    import numpy as np

    return float(np.percentile(np.asarray(v, dtype=np.float64), q)) if len(v) else None


def serving_leg(n_requests, seed=2024, budget_gb=150.0, max_resident=16, quantum=64, load=1.5, world=1, rank=0):
    """The serving stream twice: one plain simulation at a time (the
    reference's run_batch), then through the request server with Poisson
    arrivals at `load` × the sequential throughput.  Latency = result read
    back on the host − scheduled arrival."""
    import threading

    import numpy as np
    import torch

    from khronos_gb300 import configs
    from khronos_gb300.device import GpuSim
    from khronos_gb300.serve import Server

    stream = configs.serving_stream(n_requests, seed)
    if world > 1:  # replicas: this rank serves its share of the independent requests
        from khronos_gb300.replicas import shard

        mine = set(shard([r.work for r in stream], world, rank))
        stream = [r for i, r in enumerate(stream) if i in mine]
    work = [r.work for r in stream]

    def flux_of(g, w):
        fm = w.flux_monitors[0]
        return g.flux([0, 1, 2, 3], fm.normal_axis, fm.dA)

    # 1) sequential, back to back: per-request service time
    torch.cuda.synchronize()
    service, seq_flux = [], []
    for r in stream:
        t0 = time.perf_counter()
        w = r.make()
        g = GpuSim(w.sim.spec())
        g.step(r.steps)
        seq_flux.append(flux_of(g, w))
        g.close()
        service.append(time.perf_counter() - t0)
    seq_rate = sum(work) / sum(service) / 1e9
    gap = float(np.mean(service)) / load
    arrivals = [r.arrival_unit * gap for r in stream]
    # sequential latencies under the same arrivals (a FIFO single server)
    finish, seq_lat = 0.0, []
    for a, sv in zip(arrivals, service):
        finish = max(finish, a) + sv
        seq_lat.append(finish - a)
    seq_span = finish - arrivals[0]

    # 2) the request server, requests submitted at their arrival times
    srv = Server(int(budget_gb * 1e9), max_resident=max_resident, quantum_steps=quantum)
    srv_flux = [None] * len(stream)
    done_at = [0.0] * len(stream)
    t_start = time.perf_counter()
    index = {}
    lock = threading.Lock()
    errors = []

    def submitter():
        try:
            for r, a in zip(stream, arrivals):
                delay = t_start + a - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                w = r.make()
                req = srv.submit(w.sim.spec(), r.steps)
                with lock:
                    index[req.ticket] = (r.index, w)
        except Exception as e:  # surfaced below
            errors.append(e)

    th = threading.Thread(target=submitter)
    th.start()
    peak_resident = 0
    for _ in range(len(stream)):
        req = srv.next_done(timeout=600.0)
        if req is None:
            raise RuntimeError("serving leg: no request finished within 600 s")
        req.wait()
        with lock:
            i, w = index[req.ticket]
        srv_flux[i] = flux_of(req.sim, w)
        done_at[i] = time.perf_counter() - t_start
        req.release()
        peak_resident = max(peak_resident, srv.stats()["resident"])
    th.join()
    srv.close()
    if errors:
        raise errors[0]
    # 3) sustained capacity: the whole stream submitted at once
    model_bytes = 0.0
    srv = Server(int(budget_gb * 1e9), max_resident=max_resident, quantum_steps=quantum)
    t0 = time.perf_counter()
    pending = []
    for r in stream:
        spec = r.make().sim.spec()
        pending.append(srv.submit(spec, r.steps))
    for _ in stream:
        req = srv.next_done(timeout=600.0)
        if req is None:
            raise RuntimeError("serving leg: no request finished within 600 s")
        req.wait()
        model_bytes += req.sim.model_bytes_per_step() * req.steps
        req.release()
    sat_span = time.perf_counter() - t0
    srv.close()
    peak_gbs, _ = measured_peaks()
    srv_lat = [d - a for d, a in zip(done_at, arrivals)]
    srv_span = max(done_at) - arrivals[0]
    diff = max(float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))
               for a, b in zip(srv_flux, seq_flux))
    lat = lambda v: {"p50": _pct(v, 50), "p95": _pct(v, 95), "p99": _pct(v, 99), "max": max(v)}
    return {
        "requests": len(stream), "seed": seed, "budget_gb": budget_gb, "max_resident": max_resident,
        "quantum_steps": quantum, "offered_load_vs_sequential": load, "mean_interarrival_s": gap,
        "cell_updates": int(sum(work)),
        "server": {"gcell_per_s": sum(work) / srv_span / 1e9, "latency_s": lat(srv_lat), "makespan_s": srv_span},
        "sequential": {"gcell_per_s": sum(work) / seq_span / 1e9, "busy_gcell_per_s": seq_rate,
                       "latency_s": lat(seq_lat), "makespan_s": seq_span,
                       "mean_service_s": float(np.mean(service))},
        "saturated": {"gcell_per_s": sum(work) / sat_span / 1e9, "makespan_s": sat_span,
                      "model_bytes": model_bytes, "achieved_gbs": model_bytes / sat_span / 1e9,
                      "hbm_frac": model_bytes / sat_span / 1e9 / peak_gbs},
        "speedup_aggregate": (sum(work) / srv_span) / (sum(work) / seq_span),
        "capacity_vs_sequential": (sum(work) / sat_span) / (sum(work) / sum(service)),
        "flux_max_rel_diff_served_vs_solo": diff,
    }


def run_serving(args, world=1, rank=0, local_rank=0):
    """The serving stream on one GPU, or sharded over `world` replicas (one
    server per GPU, requests split by shard(); the only collectives are the
    host-side (gloo) reductions of the legs' rates and makespans)."""
    import torch

    torch.cuda.set_device(local_rank)
    __graft_entry__.package()
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("gloo")
        dist = dist_mod
    res = serving_leg(args.serve_requests, world=world, rank=rank)
    if dist is not None:
        from khronos_gb300.replicas import max_over_ranks

        total = {}
        for leg in ("server", "sequential", "saturated"):
            span = max_over_ranks(res[leg]["makespan_s"], dist)
            t = torch.tensor([float(res["cell_updates"])], dtype=torch.float64)
            dist.all_reduce(t)
            total[leg] = float(t.item()) / span / 1e9
        res["replicas"] = {"world": world, "aggregate_gcell_per_s": total}
        dist.destroy_process_group()
        if rank != 0:
            return 0
    line = {"metric": "serve p50/p95/p99 latency and aggregate Gcell-updates/s", "unit": "s",
            "dtype": "f32", "data": "synthetic", "n_gpus": world, "config": {"workload": "serving stream", **{
                k: res[k] for k in ("requests", "seed", "budget_gb", "max_resident", "quantum_steps")}},
            "serving": res}
    print(json.dumps(line), flush=True)
    return 0


def adjoint_leg(steps=6000, fd_voxels=0, scale=1.0, fp64=True):
    """Waveguide-bend inverse design (400×400×128, 120×120×22 design voxels,
    5 frequencies): FP32 objective + adjoint gradient wall time through the
    public API; optionally the FP64 gradient of the same inputs (error of the
    FP32 gradient) and central finite differences (δρ = 1e-3, FP64) on
    `fd_voxels` seeded design voxels."""
    import numpy as np
    import torch

    from khronos_gb300 import configs
    from khronos_gb300.adjoint import bend_problem, reference_fields

    out = {"steps": steps, "scale": scale}
    w = configs.bend(dtype="f32", steps=steps, scale=scale)
    cells = int(np.prod(w.sim.n))
    out["grid"] = list(w.sim.n)
    out["design_dims"] = list(w.design_dims)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e_ref = reference_fields(w)
    t_ref = time.perf_counter() - t0
    opt = bend_problem(w, e_ref)
    opt(w.rho0, need_gradient=False)  # creates both simulations (set-up, uploads)
    t0 = time.perf_counter()
    opt.update_design(w.rho0)
    f0 = opt.forward_run()
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    g32 = opt.adjoint_run().copy()
    t_adj = time.perf_counter() - t0
    if opt.gradient_per_freq is None:  # windowed mode: one adjoint run for all frequencies
        n_adj = 1
    else:
        n_adj = int(np.count_nonzero(np.any(opt.gradient_per_freq != 0, axis=(1, 2, 3))))
    launches = opt._fwd.launches + opt._adj.launches
    opt.close()
    out.update({
        "mode": opt.mode, "history_gb": opt.history_bytes() / 1e9,
        "f0_fp32": f0, "straight_ref_s": t_ref, "forward_s": t_fwd, "adjoint_s": t_adj,
        "adjoint_runs": n_adj, "gradient_s": t_fwd + t_adj,
        "gcell_per_s": cells * steps * (1 + n_adj) / (t_fwd + t_adj) / 1e9,
        "gpu_launches_fwd_adj": launches,
    })
    if fp64:
        # the FP64 run of the same inputs (FP32 specs promoted)
        o64 = bend_problem(w, reference_fields(w, promote=True), promote=True)
        t0 = time.perf_counter()
        f64, g64 = o64(w.rho0)
        g64 = g64.copy()
        out["fp64_gradient_s"] = time.perf_counter() - t0
        out["f0_fp64"] = f64
        out["f0_rel_err_fp32"] = abs(f0 - f64) / abs(f64)
        out["gradient_rel_l2_fp32_vs_fp64"] = float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64))
        if fd_voxels:
            rng = np.random.default_rng(99)
            idx = [tuple(int(rng.integers(0, d)) for d in w.design_dims) for _ in range(fd_voxels)]
            t0 = time.perf_counter()
            fd = o64.calculate_fd_gradient(w.rho0, idx, db=1e-3)
            rel = [abs(g64[i] - f) / abs(f) for i, f in zip(idx, fd)]
            rel32 = [abs(g32[i] - f) / abs(f) for i, f in zip(idx, fd)]
            out["fd"] = {"voxels": [list(i) for i in idx], "fd": fd.tolist(),
                         "adjoint_fp64": [float(g64[i]) for i in idx],
                         "adjoint_fp32": [float(g32[i]) for i in idx],
                         "rel_err_fp64_max": max(rel), "rel_err_fp32_max": max(rel32),
                         "seconds": time.perf_counter() - t0, "db": 1e-3}
        o64.close()
    return out


def run_adjoint(args):
    import torch

    torch.cuda.set_device(0)
    __graft_entry__.package()
    res = adjoint_leg(args.adjoint_steps, args.adjoint_fd, args.adjoint_scale, not args.adjoint_no_fp64)
    line = {"metric": "adjoint gradient of the waveguide-bend objective (wall time, s)", "unit": "s",
            "value": res["gradient_s"], "higher_is_better": False, "dtype": "f32", "data": "synthetic",
            "n_gpus": 1, "config": {"workload": "waveguide bend inverse design 400x400x128 (scaled by "
                                                f"{args.adjoint_scale}), 5 frequencies"}, "adjoint": res}
    print(json.dumps(line), flush=True)
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--no-flux-check", action="store_true", help="skip the FP32-vs-FP64 flux leg")
    ap.add_argument("--serve-only", action="store_true", help="run only the serving-stream leg")
    ap.add_argument("--serve-requests", type=int, default=512)
    ap.add_argument("--adjoint-only", action="store_true", help="run only the waveguide-bend adjoint leg")
    ap.add_argument("--adjoint-steps", type=int, default=6000)
    ap.add_argument("--adjoint-scale", type=float, default=1.0)
    ap.add_argument("--adjoint-fd", type=int, default=0, help="finite-difference voxels (FP64)")
    ap.add_argument("--adjoint-no-fp64", action="store_true")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="waveguide",
                    help="waveguide: the 320x192x128 heterogeneous grid (default); dispersive: 256^3 ADE + chi3")
    args = ap.parse_args(argv)
    global _workload_name
    _workload_name = args.workload
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local_rank = dist_env()
    if args.impl == "reference":
        return run_reference(args, world, rank)
    if args.serve_only:
        return run_serving(args, world, rank, local_rank)
    if args.adjoint_only:
        return run_adjoint(args)
    return run_ours(args, world, rank, local_rank)


if __name__ == "__main__":
    sys.exit(main())
