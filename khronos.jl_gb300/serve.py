"""Serving: many independent simulations on one GPU.

``Server`` wraps the library's request server (``kh_server_*``): requests are
admitted in arrival order whenever the device-memory budget and a resident
slot allow, prepared while other requests step, and stepped in quanta on
per-slot streams so their kernels overlap.  ``run_batch`` and
``run_batch_concurrent`` keep the reference's batch drivers
(src/Batch.jl:103-145 and :170-263): the first runs one plain simulation at a
time, the second submits the whole batch to a ``Server`` (continuous batching
instead of fixed waves).  ``plan_batch`` mirrors src/Batch.jl:21-66 with the
library's own per-simulation memory estimate.
"""
from __future__ import annotations

import ctypes as C
import time
from dataclasses import dataclass, field
from typing import Callable, Dict, List, Optional, Sequence

from . import _abi
from .device import GpuSim
from .spec import SimSpec


@dataclass
class RequestInfo:
    state: int
    status: int
    steps: int
    bytes: int
    t_submit: float
    t_admit: float
    t_start: float
    t_done: float

    @property
    def latency(self) -> float:
        return self.t_done - self.t_submit


class Request:
    """One submitted simulation; its results are read through ``sim`` once
    ``wait()`` returned, then ``release()`` frees its device memory."""

    def __init__(self, server: "Server", sim: GpuSim, ticket: int, steps: int):
        self.server = server
        self.sim = sim
        self.ticket = ticket
        self.steps = steps

    def wait(self, timeout: Optional[float] = None) -> bool:
        st = self.server.lib.kh_server_wait(self.server.handle, self.ticket, -1.0 if timeout is None else timeout)
        if st == _abi.KH_ERR_TIMEOUT:
            return False
        self.server._check(st)
        return True

    def info(self) -> RequestInfo:
        ri = _abi.RequestInfo()
        self.server._check(self.server.lib.kh_server_info(self.server.handle, self.ticket, C.byref(ri)))
        return RequestInfo(ri.state, ri.status, ri.steps, ri.bytes, ri.t_submit, ri.t_admit, ri.t_start, ri.t_done)

    def release(self):
        if self.sim is not None:
            self.server._check(self.server.lib.kh_server_release(self.server.handle, self.ticket))
            self.sim.handle = C.c_void_p()
            self.sim = None


class Server:
    """Request server on the current CUDA device."""

    def __init__(self, budget_bytes: int, max_resident: int = 16, quantum_steps: int = 64, lib=None):
        self.lib = lib or _abi.load()
        d = _abi.ServerDesc(int(budget_bytes), int(max_resident), int(quantum_steps))
        self.handle = C.c_void_p()
        st = self.lib.kh_server_create(C.byref(d), C.byref(self.handle))
        if st != _abi.KH_OK:
            raise _abi.KhError(st, "kh_server_create failed")
        self._requests: Dict[int, Request] = {}

    def _check(self, st: int):
        if st != _abi.KH_OK:
            raise _abi.KhError(st, self.lib.kh_server_last_error(self.handle).decode())

    def submit(self, spec: SimSpec, steps: int) -> Request:
        sim = GpuSim(spec, lib=self.lib, prepare=False)
        ticket = C.c_int64()
        st = self.lib.kh_server_submit(self.handle, sim.handle, int(steps), C.byref(ticket))
        if st != _abi.KH_OK:
            sim.close()
            self._check(st)
        sim.detach()
        req = Request(self, sim, ticket.value, int(steps))
        self._requests[req.ticket] = req
        return req

    def next_done(self, timeout: Optional[float] = None) -> Optional[Request]:
        """The next finished request (each reported once), None on timeout."""
        t = C.c_int64()
        st = self.lib.kh_server_wait_any(self.handle, -1.0 if timeout is None else timeout, C.byref(t))
        if st == _abi.KH_ERR_TIMEOUT:
            return None
        self._check(st)
        return self._requests.pop(t.value)

    def stats(self) -> dict:
        q, r, b = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.lib.kh_server_stats(self.handle, C.byref(q), C.byref(r), C.byref(b)))
        return {"queued": q.value, "resident": r.value, "budget_used": b.value}

    def close(self):
        if self.handle:
            self.lib.kh_server_destroy(self.handle)
            self.handle = C.c_void_p()
            for r in self._requests.values():
                if r.sim is not None:
                    r.sim.handle = C.c_void_p()
                    r.sim = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def estimate_bytes(spec: SimSpec, lib=None) -> int:
    """Device bytes a simulation of `spec` allocates (estimate_memory,
    src/Memory.jl:120-251), from the library's own allocation rule."""
    g = GpuSim(spec, lib=lib, prepare=False)
    try:
        est = C.c_int64()
        g._check(g.lib.kh_sim_memory_bytes(g.handle, C.byref(est), None))
        return int(est.value)
    finally:
        g.close()


def plan_batch(spec: SimSpec, n_sims: int, budget_bytes: int, lib=None) -> dict:
    """How many simulations like `spec` fit the budget at once
    (plan_batch, src/Batch.jl:21-66)."""
    per = estimate_bytes(spec, lib)
    max_batch = max(1, min(n_sims, budget_bytes // max(per, 1)))
    return {"max_batch": int(max_batch), "n_waves": -(-n_sims // max_batch), "per_sim_bytes": per,
            "total_bytes": per * max_batch}


def collect_dft(sim: GpuSim) -> List:
    return [sim.dft(i) for i in range(len(sim.spec.monitors))]


def run_batch(specs: Sequence[SimSpec], steps: Sequence[int], collect: Callable[[GpuSim], object] = collect_dft,
              lib=None) -> List[object]:
    """One plain simulation at a time (run_batch, src/Batch.jl:103-145)."""
    out = []
    for spec, n in zip(specs, steps):
        g = GpuSim(spec, lib=lib)
        g.step(int(n))
        out.append(collect(g))
        g.close()
    return out


def run_batch_concurrent(specs: Sequence[SimSpec], steps: Sequence[int],
                         collect: Callable[[GpuSim], object] = collect_dft, budget_bytes: Optional[int] = None,
                         max_concurrent: int = 0, quantum_steps: int = 64, lib=None) -> List[object]:
    """The batch through a Server (run_batch_concurrent, src/Batch.jl:170-263):
    requests are admitted as budget and slots free up instead of in waves."""
    if budget_bytes is None:
        import torch

        free, _ = torch.cuda.mem_get_info()
        budget_bytes = int(0.85 * free)
    out: List[object] = [None] * len(specs)
    with Server(budget_bytes, max_resident=max_concurrent or 16, quantum_steps=quantum_steps, lib=lib) as srv:
        index = {}
        for i, (spec, n) in enumerate(zip(specs, steps)):
            index[srv.submit(spec, int(n)).ticket] = i
        for _ in range(len(specs)):
            req = srv.next_done()
            req.wait()
            out[index[req.ticket]] = collect(req.sim)
            req.release()
    return out
