"""DFT and flux monitors (host side).

* DFTMonitor / init_monitors        src/Monitors/Monitors.jl:202-272
* auto_decimate!                    src/Monitors/Monitors.jl:33-78
* FluxMonitor / get_flux            src/Monitors/FluxMonitor.jl:18-172

The accumulation itself runs on the GPU (kh_sim_step); the flux reduction runs
in FP64 on the GPU (kh_sim_flux).  ``flux_from_dft`` is the host restatement
of get_flux used to cross-check it.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np

from .grid import EX, EY, EZ, HX, HY, HZ, Grid, GridVolume
from .sources import ContinuousWaveSource, CustomSource, GaussianPulseSource


@dataclass
class DFTMonitor:
    """DFTMonitor(component, center, size, frequencies, decimation=1)."""

    component: int
    center: Sequence[float]
    size: Sequence[float]
    frequencies: Sequence[float]
    decimation: int = 1
    # filled by Simulation.prepare
    gv: Optional[GridVolume] = None
    monitor_id: int = -1
    sim: object = None

    def data(self) -> np.ndarray:
        """Complex DFT array of shape (Nx, Ny, Nz, Nf) (column-major like Julia)."""
        return self.sim._read_dft(self)


@dataclass
class FluxMonitor:
    """FluxMonitor(center, size, frequencies, decimation=1): 4 tangential DFTs."""

    center: Sequence[float]
    size: Sequence[float]
    frequencies: Sequence[float]
    decimation: int = 1
    normal_axis: int = -1
    e_monitors: List[DFTMonitor] = field(default_factory=list)
    h_monitors: List[DFTMonitor] = field(default_factory=list)
    dA: float = 0.0
    sim: object = None

    def expand(self, grid: Grid):
        """init_flux_monitor (FluxMonitor.jl:18-70)."""
        zeros = [a for a in range(3) if self.size[a] == 0.0]
        if not zeros:
            raise ValueError("FluxMonitor size must have exactly one zero dimension")
        self.normal_axis = zeros[0]
        comps = {0: ((EY, EZ), (HY, HZ)), 1: ((EX, EZ), (HX, HZ)), 2: ((EX, EY), (HX, HY))}
        ec, hc = comps[self.normal_axis]
        mk = lambda c: DFTMonitor(component=c, center=list(self.center), size=list(self.size),
                                  frequencies=list(self.frequencies), decimation=self.decimation)
        self.e_monitors = [mk(c) for c in ec]
        self.h_monitors = [mk(c) for c in hc]
        d = [float(v) for v in grid.delta]
        self.dA = {0: d[1] * d[2], 1: d[0] * d[2], 2: d[0] * d[1]}[self.normal_axis]
        return self.e_monitors + self.h_monitors

    def flux(self) -> np.ndarray:
        return self.sim._flux(self)


def auto_decimation(sources, dt) -> int:
    """D = max(1, floor(1/(2·f_max·Δt))) from the stored source bandwidths
    (auto_decimate!, Monitors.jl:33-78).  Returns 1 when no benefit."""
    T = type(dt)
    f_max = 0.0
    for s in sources:
        tp = s.time_profile
        if isinstance(tp, GaussianPulseSource):
            st = tp.stored(T)
            f_max = max(f_max, float(st["fcen"]) + float(st["fwidth"]) / 2)
        elif isinstance(tp, ContinuousWaveSource):
            f_max = max(f_max, float(T(tp.fcen)))
        elif isinstance(tp, CustomSource):
            f_max = max(f_max, float(T(tp.fcen)) + float(T(tp.fwidth)) / 2)
        else:
            f_max = max(f_max, 1.0 / (2.0 * float(dt)))
    if f_max <= 0:
        return 1
    return max(1, int(math.floor(1.0 / (2.0 * f_max * float(dt)))))


def flux_from_dft(normal_axis: int, e1, e2, h1, h2, dA: float) -> np.ndarray:
    """get_flux on host arrays shaped (Nx, Ny, Nz, Nf) (FluxMonitor.jl:92-156)."""

    def avg(f, d):
        if f.shape[d] >= 2:
            a = np.take(f, [0], axis=d)
            b = np.take(f, [1], axis=d)
            return (a + b) / 2
        return f

    e1, e2, h1, h2 = (avg(x, normal_axis) for x in (e1, e2, h1, h2))
    tang = [a for a in range(3) if a != normal_axis]
    n1 = min(x.shape[tang[0]] for x in (e1, e2, h1, h2))
    n2 = min(x.shape[tang[1]] for x in (e1, e2, h1, h2))
    sl = [slice(None)] * 4
    sl[normal_axis] = slice(0, 1)
    sl[tang[0]] = slice(0, n1)
    sl[tang[1]] = slice(0, n2)
    sl = tuple(sl)
    s = (e1[sl] * np.conj(h2[sl]) - e2[sl] * np.conj(h1[sl])).real * dA
    return s.reshape(-1, s.shape[-1]).sum(axis=0)


def flux_error(test, ref) -> dict:
    """Error of a flux spectrum against a reference spectrum (same frequencies):
    relative L2 over the frequencies, and the largest per-frequency error
    relative to the largest reference magnitude."""
    test = np.asarray(test, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    if test.shape != ref.shape:
        raise ValueError("flux spectra differ in shape")
    scale = float(np.max(np.abs(ref))) if ref.size else 0.0
    if scale == 0.0:
        d = float(np.max(np.abs(test))) if test.size else 0.0
        return {"rel_l2": d, "max_rel": d}
    return {"rel_l2": float(np.linalg.norm(test - ref) / np.linalg.norm(ref)),
            "max_rel": float(np.max(np.abs(test - ref)) / scale)}
