"""Sources: time profiles and spatial amplitude arrays.

Restates the reference's host-side source set-up:

* GaussianPulseSource / ContinuousWaveSource / CustomSource
                                   src/Sources/TimeSources.jl:53-192
* UniformSource                    src/Sources/SpatialSources.jl:92-131
* PlaneWaveSource                  src/Sources/SpatialSources.jl:428-575,
                                   src/Sources/Sources.jl:144-231
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


def _cross(a, b):
    return [a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]]


@dataclass
class PlaneWaveSource(Source):
    """PlaneWaveSource (SpatialSources.jl:428-575): a plane of electric and
    magnetic current that launches a plane wave along ``k_vector`` (or the
    direction given by ``angle_theta``/``angle_phi``) with polarisation angle
    ``polarization_angle`` about it.

    The injection plane is the zero-size axis of ``size``.  The polarisation
    basis follows the reference: for k along the plane normal the s/p pair is
    degenerate and the reference fixes the basis vector by k's axis
    (x → ŷ, y → ẑ, z → x̂); otherwise it is n̂ × k̂ (zero, hence no source,
    for k anti-parallel to the normal, as in the reference).  Currents
    Ĵ = n̂ × (k̂ × Ê)/Z₀ and M̂ = −n̂ × Ê with Z₀ = √(μ/ε), each carrying the
    phase exp(−i k k̂·r) at its own Yee position; only transverse components
    with a nonzero factor are injected.  ``component`` is ignored.
    """

    component: int = -1
    polarization_angle: float = 0.0
    k_vector: Optional[Sequence[float]] = None
    angle_theta: Optional[float] = None
    angle_phi: Optional[float] = None
    eps: float = 1.0
    mu: float = 1.0

    def __post_init__(self):
        if self.k_vector is None:
            if self.angle_theta is None or self.angle_phi is None:
                raise ValueError("give either k_vector or angle_phi and angle_theta")
            th, ph = self.angle_theta, self.angle_phi
            kv = [math.sin(ph) * math.cos(th), math.sin(ph) * math.sin(th), math.cos(ph)]
        else:
            kv = [float(v) for v in self.k_vector]
        nrm = math.sqrt(sum(v * v for v in kv))
        self.khat = [v / nrm for v in kv]
        self.k = 2 * math.pi * float(self.time_profile.fcen) * math.sqrt(self.eps * self.mu)
        zero = [a for a in range(3) if float(self.size[a]) == 0.0]
        if len(zero) != 1:
            raise ValueError(f"the injection volume is not a plane (size={tuple(self.size)})")
        self.normal_axis = zero[0]
        n = [0.0, 0.0, 0.0]
        n[self.normal_axis] = 1.0
        self.normal = n
        if sum(a * b for a, b in zip(n, self.khat)) == 1.0:
            first = next(a for a in range(3) if self.khat[a] != 0.0)
            ppn = [[0.0, 1.0, 0.0], [0.0, 0.0, 1.0], [1.0, 0.0, 0.0]][first]
        else:
            ppn = _cross(n, self.khat)
        c, s_ = math.cos(self.polarization_angle), math.sin(self.polarization_angle)
        kxp = _cross(self.khat, ppn)
        self.polarization = [ppn[a] * c + kxp[a] * s_ for a in range(3)]

    def scaling(self, component: int) -> float:
        """get_planewave_polarization_scaling (SpatialSources.jl:518-545)."""
        if component < 3:
            inv_z0 = 1.0 / math.sqrt(self.mu / self.eps)
            j = _cross(self.normal, _cross(self.khat, [inv_z0 * p for p in self.polarization]))
            return j[component]
        return -_cross(self.normal, self.polarization)[component - 3]

    def components(self):
        """get_source_components (SpatialSources.jl:547-565): the plane's
        transverse E and H components with a nonzero factor."""
        t = [a for a in range(3) if a != self.normal_axis]
        cand = [t[0], t[1], 3 + t[0], 3 + t[1]]
        return [c for c in cand if self.scaling(c) != 0.0]

    def profile(self, point, component) -> complex:
        """get_source_profile (SpatialSources.jl:567-575)."""
        ph = sum(p * k for p, k in zip(point, self.khat)) * self.k
        return self.scaling(component) * complex(math.cos(ph), -math.sin(ph))

    def amplitude_array(self, grid: Grid, component: int):
        """The reference's separable plane-wave fill (_fill_amplitude_data!
        specialised for PlaneWaveSourceData, Sources.jl:144-231): per axis a
        factor w_a(p_a)·exp(−i k k̂_a p_a), w_a the 1-D interpolation weight
        (1 on an axis of infinite extent), multiplied together and by
        pol_factor · amplitude.  Reproduced as the reference has it: when the
        component's grid volume is one cell thick in z, the z factor (weight
        and phase) is left out."""
        gv = grid.grid_volume(self.center, self.size, component)
        origin = grid.component_origin(component)
        d = [float(v) for v in grid.delta]
        size = [float(v) for v in self.size]
        lo = [self.center[a] - size[a] / 2 for a in range(3)]
        hi = [self.center[a] + size[a] / 2 for a in range(3)]
        cc3 = grid.cell_center[2]
        dims = (gv.dims[0], gv.dims[1], max(1, gv.dims[2]))
        fac = []
        for a in range(3):
            col = np.zeros(dims[a], dtype=np.complex128)
            for i in range(1, dims[a] + 1):
                p = origin[a] + (i + gv.start_idx[a] - 2) * d[a]
                if a == 2 and (math.isinf(p) or math.isnan(p)):
                    p = cc3
                w = 1.0 if math.isinf(size[a]) else interpolation_weight(
                    (p, 0.0, 0.0), (lo[a], 0.0, 0.0), (hi[a], 0.0, 0.0), (size[a], 0.0, 0.0),
                    (d[a], 0.0, 0.0), 1)
                th = (-self.k * self.khat[a]) * p
                col[i - 1] = w * complex(math.cos(th), math.sin(th))
            fac.append(col)
        scale = complex(self.scaling(component) * self.amplitude)
        cz = fac[2] if dims[2] > 1 else np.ones(1, dtype=np.complex128)
        amp = (fac[0][:, None, None] * fac[1][None, :, None]) * cz[None, None, :] * scale
        return gv, amp
