"""Sources: time profiles and spatial amplitude arrays.

Restates the reference's host-side source set-up:

* GaussianPulseSource / ContinuousWaveSource / CustomSource
                                   src/Sources/TimeSources.jl:53-192
* UniformSource                    src/Sources/SpatialSources.jl:92-131
* amplitude arrays                 src/Sources/Sources.jl:44-131, 235-248

The per-step time factor f(t) is evaluated by the CUDA library on the host in
the run's precision (kh_sim_step); the Python functions here exist for
set-up (cutoffs, decimation) and for tests.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, Optional, Sequence

import numpy as np

from .grid import Grid, interpolation_weight


def gaussian_bandwidth(width: float) -> float:
    """_gaussian_bandwidth (TimeSources.jl:118-121)."""
    tol = 1e-7
    return math.sqrt(-2.0 * math.log(tol)) / (width * math.pi)


@dataclass
class GaussianPulseSource:
    """GaussianPulseSource(; fcen, fwidth, start_time, cutoff_scale) (TimeSources.jl:91-109).

    Stored values are rounded to the run's number type when the simulation is
    prepared (``GaussianPulseData{backend_number}``).
    """

    fcen: float
    fwidth: float
    start_time: float = 0.0
    cutoff_scale: float = 5.0

    def __post_init__(self):
        width = 1.0 / self.fwidth
        cutoff = width * self.cutoff_scale + self.start_time
        fwidth_stored = gaussian_bandwidth(width)
        while math.exp(-cutoff * cutoff / (2 * width * width)) < 1e-100:
            cutoff *= 0.9
        peak_time_raw = cutoff / 2
        period = 1.0 / self.fcen
        # Julia round(): nearest, ties to even — Python's round() does the same.
        peak_time = round(peak_time_raw / period) * period
        self.width = width
        self.cutoff = cutoff
        self.fwidth_stored = fwidth_stored
        self.peak_time = peak_time

    kind = 0

    def stored(self, T):
        return dict(fcen=T(self.fcen), fwidth=T(self.fwidth_stored), width=T(self.width),
                    peak_time=T(self.peak_time), cutoff=T(self.cutoff))

    def cutoff_time(self, T):
        return float(T(self.cutoff))

    def eval(self, t: float, T=np.float64) -> complex:
        """eval_time_source(::GaussianPulseData, t) in precision T (TimeSources.jl:123-132)."""
        s = self.stored(T)
        tt = T(T(t) - s["peak_time"])
        if tt > s["cutoff"]:
            return complex(0.0, 0.0)
        two_pi = T(T(2) * T(math.pi))
        g = np.exp(T(T(T(-tt) * tt) / T(T(T(2) * s["width"]) * s["width"])))
        b = T(T(T(-two_pi) * s["fcen"]) * tt)
        return complex(float(T(g * np.cos(b))), float(T(g * np.sin(b))))


@dataclass
class ContinuousWaveSource:
    """ContinuousWaveSource(; fcen) (TimeSources.jl:53-72): never cuts off."""

    fcen: float
    kind = 1

    def cutoff_time(self, T):
        return math.inf

    def eval(self, t: float, T=np.float64) -> complex:
        two_pi = T(T(2) * T(math.pi))
        b = T(T(T(-two_pi) * T(self.fcen)) * T(t))
        return complex(float(np.cos(b)), float(np.sin(b)))


@dataclass
class CustomSource:
    """CustomSource(; src_func, fcen, fwidth, end_time) (TimeSources.jl:157-190).

    The library cannot call back into Python per step, so the profile is
    tabulated on the host at every half-step time the run will use:
    entries (f(nΔt), f(nΔt + Δt/2)) for n < table_steps.
    """

    src_func: Callable[[float], complex]
    fcen: float
    fwidth: float
    end_time: float
    table_steps: int = 0
    kind = 2

    def cutoff_time(self, T):
        return float(T(self.end_time))


@dataclass
class Source:
    """Base for spatial sources: a component, a box and an amplitude."""

    time_profile: object
    component: int
    center: Sequence[float] = (0.0, 0.0, 0.0)
    size: Sequence[float] = (0.0, 0.0, 0.0)
    amplitude: complex = 1.0

    def components(self):
        return [self.component]

    def profile(self, point, component) -> complex:
        return 1.0

    def amplitude_array(self, grid: Grid, component: int):
        """(GridVolume, complex amplitude array indexed [ix, iy, iz]) for one component.

        _fill_amplitude_data! generic path (Sources.jl:101-131): the value at
        each index is interpolation weight × amplitude × spatial profile.
        """
        gv = grid.grid_volume(self.center, self.size, component)
        origin = grid.component_origin(component)
        d = [float(v) for v in grid.delta]
        lo = [self.center[a] - self.size[a] / 2 for a in range(3)]
        hi = [self.center[a] + self.size[a] / 2 for a in range(3)]
        vs = [float(s) for s in self.size]
        cc3 = grid.cell_center[2]
        dims = (gv.dims[0], gv.dims[1], max(1, gv.dims[2]))
        amp = np.zeros(dims, dtype=np.complex128)  # amp[ix, iy, iz]
        for iz in range(1, dims[2] + 1):
            pz = origin[2] + (iz + gv.start_idx[2] - 2) * d[2]
            if math.isinf(pz) or math.isnan(pz):
                pz = cc3
            for iy in range(1, dims[1] + 1):
                py = origin[1] + (iy + gv.start_idx[1] - 2) * d[1]
                for ix in range(1, dims[0] + 1):
                    px = origin[0] + (ix + gv.start_idx[0] - 2) * d[0]
                    p = (px, py, pz)
                    w = interpolation_weight(p, lo, hi, vs, d, 3)
                    if w == 0.0:
                        continue
                    amp[ix - 1, iy - 1, iz - 1] = w * self.amplitude * self.profile(p, component)
        return gv, amp


@dataclass
class UniformSource(Source):
    """UniformSource (SpatialSources.jl:92-131): constant profile."""


@dataclass
class ProfileSource(Source):
    """A current source with a user spatial profile ``profile_func(x, y, z)``.

    Goes through the reference's generic amplitude path
    (``get_source_profile(source, point, component)``, Sources.jl:242-248), the
    same path its GaussianBeam/Equivalent sources take.
    """

    profile_func: Optional[Callable[[float, float, float], complex]] = None

    def profile(self, point, component) -> complex:
        return self.profile_func(*point) if self.profile_func else 1.0
