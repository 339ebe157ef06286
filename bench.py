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
The reference arm times the CPU restatement of the reference's step loop (the
reference is Julia and cannot run here) on the same workload and CPML stage
logic, on all host threads.

The default line also carries: `e2e` (the same run through the public API
from pinned host arrays, set-up and flux read-back included), `flux_error`
(full FP32 run against the FP64 run of the same inputs), `serve` (64-request
serving stream against one-at-a-time runs under the same arrivals) and
`cpu_baseline`.
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


class _Nvml:
    """Minimal NVML reader (ctypes on the driver's libnvidia-ml): SM clock,
    its maximum and the active clock-event (throttle) reasons.  Read-only."""

    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown",
               0x4: "sw_power_cap"}

    def __init__(self, uuid, index: int):
        import ctypes as C

        self.C = C
        self.lib = C.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = C.c_void_p()
        st = -1
        if uuid:
            st = self.lib.nvmlDeviceGetHandleByUUID(uuid.encode(), C.byref(self.h))
        if st != 0:
            st = self.lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(index), C.byref(self.h))
        if st != 0:
            raise OSError("no NVML handle for the device")
        self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        v = C.c_uint()
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, C.byref(v))  # NVML_CLOCK_SM
        self.max_sm = float(v.value)

    def sample(self):
        C = self.C
        v, r = C.c_uint(), C.c_ulonglong()
        self.lib.nvmlDeviceGetClockInfo(self.h, 1, C.byref(v))
        self.reasons_fn(self.h, C.byref(r))
        return float(v.value), int(r.value)


class ClockSampler:
    """SM clock and throttle reasons sampled every millisecond (NVML) from
    __enter__ to __exit__; mark() brackets the timed region, and summary()
    reports the samples taken inside it.  Falls back to nvidia-smi polling
    when NVML cannot be opened."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, period_ms: float = 1.0):
        self.index = gpu_index
        self.period = period_ms / 1e3
        self.samples = []  # (time, sm_mhz, max_mhz, reasons set)
        self.window = None
        self._stop = threading.Event()
        self.proc = None
        self.thread = None
        self.source = "nvml"

    def __enter__(self):
        uuid = None
        try:
            import torch

            u = getattr(torch.cuda.get_device_properties(self.index), "uuid", None)
            if u is not None:
                uuid = "GPU-" + str(u)
        except Exception:
            pass
        try:
            self.nvml = _Nvml(uuid, self.index)
            self.thread = threading.Thread(target=self._poll_nvml, daemon=True)
        except OSError:
            self.nvml = None
            self.source = "nvidia-smi"
            try:
                self.proc = subprocess.Popen(
                    ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                     "--format=csv,noheader,nounits", "-lms", "20"],
                    stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            except OSError:
                self.proc = None
                return self
            self.thread = threading.Thread(target=self._read_smi, daemon=True)
        self.thread.start()
        return self

    def _poll_nvml(self):
        names = _Nvml.REASONS
        while not self._stop.is_set():
            try:
                sm, r = self.nvml.sample()
            except Exception:
                break
            self.samples.append((time.perf_counter(), sm, self.nvml.max_sm,
                                 {n for bit, n in names.items() if r & bit}))
            time.sleep(self.period)

    def _read_smi(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm, smax = float(parts[0]), float(parts[1])
            except ValueError:
                continue
            self.samples.append((time.perf_counter(), sm, smax,
                                 {nm for nm, v in zip(names, parts[4:8]) if v.lower().startswith("active")}))

    def mark(self, t0: float, t1: float):
        self.window = (t0, t1)

    def __exit__(self, *exc):
        self._stop.set()
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=5)

    def summary(self):
        inside = self.samples
        scope = "sampler lifetime"
        if self.window is not None:
            w = [s for s in self.samples if self.window[0] <= s[0] <= self.window[1]]
            if w:
                inside, scope = w, "timed region"
        if not inside:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0, "source": self.source}
        reasons = set().union(*(s[3] for s in inside))
        return {"sm_mhz": statistics.median(s[1] for s in inside), "sm_max_mhz": max(s[2] for s in inside),
                "reasons": sorted(reasons), "samples": len(inside), "scope": scope, "source": self.source,
                "period_ms": self.period * 1e3}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic(kernel: str, workload: str = "waveguide"):
    """DRAM bytes per launch of `kernel` on `workload` from the committed ncu
    summary, if any (keys "<workload>:<kernel>", the waveguide's without prefix)."""
    p = ROOT / "profiles" / "dram_traffic.json"
    if not p.exists():
        return None
    d = json.loads(p.read_text())
    v = d.get(kernel if workload == "waveguide" else f"{workload}:{kernel}")
    return None if v is None else float(v)


WORKLOADS = {
    "waveguide": WORKLOAD,
    "dispersive": ("dispersive 256^3 FP32, 12-cell CPML (CUDA-path semantics), eps 2.25 slab with chi3=1e-3, "
                   "4 Lorentz (eps_inf 2, sigma 1, f0 1, gamma 0.05) + 4 Drude (eps_inf 1, wp 5, gamma 0.1) "
                   "spheres (seed 42), Ez Gaussian plane source, 6-face box flux x 11 freqs, Kahan FP32 DFT"),
    "periodic": ("photonic-crystal slab 256x256x128 FP32, periodic x and y (halo wrap after every half-step), "
                 "12-cell CPML in z (CUDA-path semantics), Si slab 0.22 um with a 0.4 um square lattice of "
                 "0.12 um air holes, Ex plane-wave current plane, two 21-frequency flux planes, Kahan FP32 DFT"),
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
    o = orc.OracleSim(spec, timed=True)
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
                      f"({cells} cells, FP32, C++ restatement of the reference step loop, OpenMP, "
                      f"-O3 with FMA contraction)"}


def run_reference(args, world, rank):
    """The reference arm: the C++ restatement of the reference's step loop
    (the reference is Julia and cannot run here) on the host cores, on the
    same workload and CPML stage logic as the GPU arm; the reference CPU
    path's own stage dispatch is timed beside it on a short sample."""
    if rank != 0:
        return 0
    orc = __graft_entry__._oracle()

    def timed(semantics, steps, warmup, budget_s):
        w, spec = build_workload("f32", semantics)
        o = orc.OracleSim(spec, timed=True)
        o.step(max(warmup, 1))
        t0 = time.perf_counter()
        o.step(1)
        per = max(time.perf_counter() - t0, 1e-6)
        k = int(max(1, min(steps, budget_s / per)))
        t0 = time.perf_counter()
        o.step(k)
        dt = time.perf_counter() - t0
        o.close()
        return spec, k, dt

    spec, k, dt = timed("cpml", args.steps, args.warmup, 60.0)
    value = spec.cells * k / dt / 1e9
    _, k2, dt2 = timed("reference_cpu", min(args.steps, 10), 1, 10.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": k, "warmup": args.warmup, "ms_per_step": dt / k * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(spec, 1),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": orc.num_threads(), "kind": "port",
                         "sample": f"{k} full-grid steps (requested {args.steps}) after {args.warmup} warm-up; "
                                   "C++ restatement of the reference step loop (Julia is absent), OpenMP over "
                                   "all host threads, -O3 with FMA contraction"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_cpu_path_stages": {
            "value": spec.cells * k2 / dt2 / 1e9, "unit": UNIT, "steps": k2,
            "note": "same grid with the reference CPU path's own CPML stage dispatch (generic_curl!, "
                    "Helpers.jl:39-270), which this arm's CUDA-path stage logic replaces"},
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(spec, world):
    return {"workload": WORKLOADS[_workload_name], "grid": list(spec.n), "cells": spec.cells,
            "l2": "inputs larger than L2 (fields+materials+CPML state ~0.9 GB per replica vs 129 MB L2); no flush",
            "parallelism": f"replicas{world}" if world > 1 else "single"}


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
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        gpu.step(args.warmup, sh)
        torch.cuda.synchronize()
        h_bytes, e_bytes, dft_bytes = gpu.model_bytes_split()
        launches0 = gpu.launches
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        start.record(stream)
        gpu.step(args.steps, sh)
        end.record(stream)
        torch.cuda.synchronize()
        clk.mark(t0, time.perf_counter())
    if dist:
        dist.barrier()
    ms = start.elapsed_time(end)
    launches = gpu.launches - launches0
    # Per-kernel split for the roofline: a separate pass after the timed
    # region, with CUDA events around the launches of every 8th step (events
    # inside the timed region would cost it ~4 %).
    rsteps = max(args.steps, 64)
    h_ms, e_ms, dft_ms = gpu.step_timed(rsteps, sh)
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
    e_launch_ms = e_ms / rsteps
    achieved = e_bytes / (e_launch_ms / 1e3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(spec, world),
        "roofline": {"bound": "hbm", "kernel": e_kernel, "achieved": achieved, "peak": peak,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / peak,
                     "algorithmic_bytes_per_launch": e_bytes,
                     "traffic": ncu_traffic(e_kernel, _workload_name),
                     "h_kernel": {"achieved": h_bytes / (h_ms / rsteps / 1e3) / 1e9,
                                  "algorithmic_bytes_per_launch": h_bytes, "ms_per_launch": h_ms / rsteps,
                                  "frac": h_bytes / (h_ms / rsteps / 1e3) / 1e9 / peak},
                     "e_ms_per_launch": e_launch_ms, "dft_ms_per_step": dft_ms / rsteps,
                     "timing": f"CUDA events around the launches of every 8th step of a {rsteps}-step pass "
                               "after the timed region",
                     "step_model_bytes": h_bytes + e_bytes + dft_bytes,
                     "step_achieved": (h_bytes + e_bytes + dft_bytes) / (ms_max / args.steps / 1e3) / 1e9},
        "clocks": clk.summary(),
        "gpu_launches": launches,
    }
    if e2e is not None:
        line["e2e"] = e2e
    if not args.no_flux_check:
        line["flux_error"] = flux_accuracy(w, sh)
    if world == 1 and not args.no_serve and _workload_name == "waveguide":
        line["serve"] = serving_leg(args.serve_requests_default, compact=True)
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
    """Same metric through the public API from host buffers: the simulation
    created from material arrays in pinned host memory in the run's precision
    (FP32), prepared (uploads, device classification), K steps, and the flux
    spectra of both planes (the run's result) read back to the host, all inside
    the timed region."""
    import dataclasses

    import torch
    from khronos_gb300.device import GpuSim

    # inputs staged in pinned host memory before the timed region, as a caller
    # that keeps its GeometryData arrays in page-locked memory would hold them
    pinned, mats = [], []
    for kind, comp, arr in spec.materials:
        buf = torch.empty(int(arr.size), dtype=torch.float32, pin_memory=True)
        h = buf.numpy().reshape(arr.shape, order="F")
        h[...] = arr
        pinned.append(buf)
        mats.append((kind, comp, h))
    spec_h = dataclasses.replace(spec, materials=mats)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g2 = GpuSim(spec_h)  # create, attach the pinned arrays, prepare
    t1 = time.perf_counter()
    g2.step(args.steps, sh)
    g2.synchronize()
    t2 = time.perf_counter()
    fluxes = [g2.flux(list(range(4 * i, 4 * i + 4)), fm.normal_axis, fm.dA)
              for i, fm in enumerate(w.flux_monitors)]
    t3 = time.perf_counter()
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    g2.close()
    h2d = sum(a.nbytes for _, _, a in mats)
    h2d += sum(s.amp.size * 16 for s in spec.sources) + sum(x.size * 8 for x in spec.sigma_b + spec.sigma_d
                                                            if x is not None)
    d2h = sum(f.size * 8 for f in fluxes)
    from khronos_gb300.replicas import aggregate_rate, max_over_ranks

    e2e_max = max_over_ranks(e2e_s, dist, device="cuda")
    return {"value": aggregate_rate(cells * args.steps, e2e_max, world) / 1e9, "unit": UNIT,
            "h2d_bytes_per_step": h2d / args.steps, "d2h_bytes_per_step": d2h / args.steps,
            "breakdown_ms": {"create_prepare": (t1 - t0) * 1e3, "steps": (t2 - t1) * 1e3,
                             "flux_readback": (t3 - t2) * 1e3},
            "scope": "GpuSim(spec) from FP32 material arrays in pinned host memory (create, attach, prepare: "
                     "uploads + device classification) + K steps + both planes' flux spectra read back to host"}


def _pct(v, q):
    import numpy as np

    return float(np.percentile(np.asarray(v, dtype=np.float64), q)) if len(v) else None


def serving_leg(n_requests, seed=2024, budget_gb=150.0, max_resident=16, quantum=64, load=1.5, world=1, rank=0,
                compact=False):
    """The serving stream under Poisson arrivals, twice: one plain simulation
    at a time in arrival order (the reference's run_batch, src/Batch.jl:103-145,
    fed by the same arrivals), then through the request server.  Latency =
    flux read back on the host − scheduled arrival.  The offered load is
    `load` × the sequential throughput measured on the first few requests.
    Without `compact`, the saturated capacity (whole stream submitted at
    once) is measured too."""
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
    # each request's host-side Simulation → spec, built before the clocks start
    made = [r.make() for r in stream]
    specs = [m.sim.spec() for m in made]

    def flux_of(g, w):
        fm = w.flux_monitors[0]
        return g.flux([0, 1, 2, 3], fm.normal_axis, fm.dA)

    def run_plain(i):
        g = GpuSim(specs[i])
        g.step(stream[i].steps)
        f = flux_of(g, made[i])
        g.close()
        return f

    # 0) calibration: sequential throughput on the first requests
    torch.cuda.synchronize()
    ncal = min(8, len(stream))
    t0 = time.perf_counter()
    for i in range(ncal):
        run_plain(i)
    cal_rate = sum(work[:ncal]) / (time.perf_counter() - t0)
    gap = float(np.mean(work)) / (load * cal_rate)
    arrivals = [r.arrival_unit * gap for r in stream]

    # 1) sequential: one plain simulation at a time, each started no earlier
    #    than its arrival
    seq_flux, seq_done = [], []
    t_start = time.perf_counter()
    for i, a in enumerate(arrivals):
        delay = t_start + a - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        seq_flux.append(run_plain(i))
        seq_done.append(time.perf_counter() - t_start)
    seq_lat = [d - a for d, a in zip(seq_done, arrivals)]
    seq_span = max(seq_done) - arrivals[0]

    # 2) the request server, requests submitted at their arrival times
    srv = Server(int(budget_gb * 1e9), max_resident=max_resident, quantum_steps=quantum)
    srv_flux = [None] * len(stream)
    done_at = [0.0] * len(stream)
    index = {}
    lock = threading.Lock()
    errors = []
    t_start = time.perf_counter()

    def submitter():
        try:
            for i, a in enumerate(arrivals):
                delay = t_start + a - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                req = srv.submit(specs[i], stream[i].steps)
                with lock:
                    index[req.ticket] = i
        except Exception as e:  # surfaced below
            errors.append(e)

    th = threading.Thread(target=submitter)
    th.start()
    for _ in range(len(stream)):
        req = srv.next_done(timeout=600.0)
        if req is None:
            raise RuntimeError("serving leg: no request finished within 600 s")
        req.wait()
        with lock:
            i = index[req.ticket]
        srv_flux[i] = flux_of(req.sim, made[i])
        done_at[i] = time.perf_counter() - t_start
        req.release()
    th.join()
    srv.close()
    if errors:
        raise errors[0]
    srv_lat = [d - a for d, a in zip(done_at, arrivals)]
    srv_span = max(done_at) - arrivals[0]
    diff = max(float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))
               for a, b in zip(srv_flux, seq_flux))
    lat = lambda v: {"p50": _pct(v, 50), "p95": _pct(v, 95), "p99": _pct(v, 99), "max": max(v)}
    total = float(sum(work))
    out = {
        "requests": len(stream), "seed": seed, "budget_gb": budget_gb, "max_resident": max_resident,
        "quantum_steps": quantum, "offered_load_vs_sequential": load, "mean_interarrival_s": gap,
        "cell_updates": int(total), "calibration_gcell_per_s": cal_rate / 1e9,
        "server": {"gcell_per_s": total / srv_span / 1e9, "latency_s": lat(srv_lat), "makespan_s": srv_span},
        "sequential": {"gcell_per_s": total / seq_span / 1e9, "latency_s": lat(seq_lat), "makespan_s": seq_span,
                       "how": "one GpuSim at a time in arrival order, started at max(arrival, previous done)"},
        "speedup_aggregate": seq_span / srv_span,
        "flux_max_rel_diff_served_vs_solo": diff,
    }
    if not compact:
        model_bytes = 0.0
        srv = Server(int(budget_gb * 1e9), max_resident=max_resident, quantum_steps=quantum)
        t0 = time.perf_counter()
        for i in range(len(stream)):
            srv.submit(specs[i], stream[i].steps)
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
        out["saturated"] = {"gcell_per_s": total / sat_span / 1e9, "makespan_s": sat_span,
                            "model_bytes": model_bytes, "achieved_gbs": model_bytes / sat_span / 1e9,
                            "hbm_frac": model_bytes / sat_span / 1e9 / peak_gbs}
        out["capacity_vs_sequential"] = (total / sat_span) / (total / seq_span)
    return out


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
            if leg not in res:
                continue
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


def adjoint_leg(steps=6000, fd_voxels=0, scale=1.0, fp64=True, mode="time", compare_modes=False):
    """Waveguide-bend inverse design (400×400×128, 120×120×22 design voxels,
    5 frequencies): FP32 objective + adjoint gradient wall time through the
    public API in `mode` ("time": windowed, exact for the finite run; "dft":
    forward DFT fields kept, one adjoint run per frequency); optionally the
    other mode's FP32 gradient of the same inputs (`compare_modes`), the FP64
    gradient (error of the FP32 gradient) and central finite differences
    (δρ = 1e-3, FP64, forward runs only) on `fd_voxels` seeded design voxels."""
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
    opt = bend_problem(w, e_ref, mode=mode)
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
    others = {}
    if compare_modes:
        other = "dft" if opt.mode == "time" else "time"
        o2 = bend_problem(w, e_ref, mode=other)
        t0 = time.perf_counter()
        _, g_other = o2(w.rho0)
        others[other] = g_other.copy()
        o2.close()
        out["other_mode"] = {"mode": other, "seconds": time.perf_counter() - t0,
                             "gradient_rel_l2_vs_this_mode": float(np.linalg.norm(g32 - others[other]) /
                                                                   np.linalg.norm(others[other]))}
    rng = np.random.default_rng(99)
    idx = [tuple(int(rng.integers(0, d)) for d in w.design_dims) for _ in range(16)][:fd_voxels]
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
        # FP64 forward runs only: a DFT-mode problem keeps no time history
        ofd = bend_problem(w, reference_fields(w, promote=True), promote=True, mode="dft")
        t0 = time.perf_counter()
        fd = ofd.calculate_fd_gradient(w.rho0, idx, db=1e-3)
        rel = lambda g: max(abs(g[i] - f) / abs(f) for i, f in zip(idx, fd))
        out["fd"] = {"voxels": [list(i) for i in idx], "fd": fd.tolist(),
                     "adjoint_fp32": [float(g32[i]) for i in idx], "rel_err_fp32_max": rel(g32),
                     "seconds": time.perf_counter() - t0, "db": 1e-3, "mode": opt.mode}
        if fp64:
            out["fd"]["adjoint_fp64"] = [float(g64[i]) for i in idx]
            out["fd"]["rel_err_fp64_max"] = rel(g64)
        for m, g in others.items():
            out["fd"][f"adjoint_fp32_{m}"] = [float(g[i]) for i in idx]
            out["fd"][f"rel_err_fp32_{m}_max"] = rel(g)
        ofd.close()
    if fp64:
        o64.close()
    return out


def run_adjoint(args):
    import torch

    torch.cuda.set_device(0)
    __graft_entry__.package()
    res = adjoint_leg(args.adjoint_steps, args.adjoint_fd, args.adjoint_scale, not args.adjoint_no_fp64,
                      args.adjoint_mode, args.adjoint_compare_modes)
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
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg of the default line")
    ap.add_argument("--serve-requests-default", type=int, default=64,
                    help="requests of the serving leg in the default line")
    ap.add_argument("--adjoint-only", action="store_true", help="run only the waveguide-bend adjoint leg")
    ap.add_argument("--adjoint-steps", type=int, default=6000)
    ap.add_argument("--adjoint-scale", type=float, default=1.0)
    ap.add_argument("--adjoint-fd", type=int, default=0, help="finite-difference voxels (FP64)")
    ap.add_argument("--adjoint-no-fp64", action="store_true")
    ap.add_argument("--adjoint-mode", choices=["time", "dft"], default="time")
    ap.add_argument("--adjoint-compare-modes", action="store_true",
                    help="also the other mode's FP32 gradient of the same inputs")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="waveguide",
                    help="waveguide: the 320x192x128 heterogeneous grid (default); dispersive: 256^3 ADE + chi3; "
                         "periodic: 256x256x128 photonic-crystal slab, periodic x/y")
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
