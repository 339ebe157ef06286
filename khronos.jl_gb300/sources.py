"""Sources: time profiles and spatial amplitude arrays.

Restates the reference's host-side source set-up:

* GaussianPulseSource / ContinuousWaveSource / CustomSource
                                   src/Sources/TimeSources.jl:53-192
* UniformSource                    src/Sources/SpatialSources.jl:92-131
* PlaneWaveSource                  src/Sources/SpatialSources.jl:428-575,
                                   src/Sources/Sources.jl:144-231
* EquivalentSource / TFSFSource    src/Sources/SpatialSources.jl:155-247, 297-410
                                   (interpolation: src/utils.jl:584-727)
* GaussianBeamSource               src/Sources/SpatialSources.jl:650-860
* amplitude arrays                 src/Sources/Sources.jl:44-131, 235-248

The per-step time factor f(t) is evaluated by the CUDA library on the host in
the run's precision (kh_sim_step); the Python functions here exist for
set-up (cutoffs, decimation) and for tests.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

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


# ---------------------------------------------------------------------------
# Interpolation of sampled field data (utils.jl:584-727), as the reference
# writes it: within an interval the weight (p − x_left)/Δ multiplies the LEFT
# sample and (x_right − p)/Δ the right one, i.e. the two weights are swapped
# with respect to linear interpolation; at a sample point (and outside the
# sampled range) the nearest sample is returned.

def _neighbors(x: np.ndarray, point: float):
    """get_neighbors (utils.jl:584-602): the two indices around ``point``."""
    ci = int(np.argmin(np.abs(x - point)))
    if x[ci] == point or ci == 0 or ci == len(x) - 1:
        return ci, ci
    if x[ci] > point:
        return ci - 1, ci
    return ci, ci + 1


def _linear(x, y, point):
    lo, hi = _neighbors(x, point)
    if lo == hi:
        return y[lo]
    d = x[hi] - x[lo]
    return ((point - x[lo]) / d) * y[lo] + ((x[hi] - point) / d) * y[hi]


def _bilinear(x1, x2, y, point):
    lo, hi = _neighbors(x2, point[1])
    top = _linear(x1, y[:, hi], point[0])
    if lo == hi:
        return top
    bottom = _linear(x1, y[:, lo], point[0])
    d = x2[hi] - x2[lo]
    return ((point[1] - x2[lo]) / d) * bottom + ((x2[hi] - point[1]) / d) * top


def trilinear_interpolator(x1, x2, x3, y, point):
    """trilinear_interpolator (utils.jl:659-687)."""
    lo, hi = _neighbors(x3, point[2])
    top = _bilinear(x1, x2, y[:, :, hi], point[:2])
    if lo == hi:
        return top
    bottom = _bilinear(x1, x2, y[:, :, lo], point[:2])
    d = x3[hi] - x3[lo]
    return ((point[2] - x3[lo]) / d) * bottom + ((x3[hi] - point[2]) / d) * top


def interpolator_from_array(data, center, size):
    """gen_interpolator_from_array (utils.jl:697-727): samples spread evenly
    over the volume (an axis with one sample sits at the centre)."""
    data = np.asarray(data)
    if data.ndim != 3:
        raise ValueError(f"The supplied data array must be 3D (supplied {data.ndim} dimensions).")
    axes = []
    for a in range(3):
        if data.shape[a] == 1:
            axes.append(np.array([float(center[a])]))
        else:
            axes.append(np.linspace(center[a] - size[a] / 2, center[a] + size[a] / 2, data.shape[a]))
    return lambda p: trilinear_interpolator(axes[0], axes[1], axes[2], data, p)


def _plane_axis(size):
    zero = [a for a in range(3) if float(size[a]) == 0.0]
    if len(zero) != 1:
        raise ValueError(f"The specified volume is not a plane (size={tuple(size)})")
    return zero[0]


def _transverse(axis):
    """get_plane_transverse_fields (utils.jl:339-353)."""
    t = [a for a in range(3) if a != axis]
    return [t[0], t[1], 3 + t[0], 3 + t[1]]


@dataclass
class EquivalentSource(Source):
    """EquivalentSource (SpatialSources.jl:155-247): the currents that launch
    a given field from a plane, Ĵ = n̂ × Ĥ and M̂ = −n̂ × Ê, from 3-D arrays
    of all six field components (``fields`` keyed EX..HZ) sampled evenly over
    the plane and interpolated to each Yee position with the reference's
    interpolator.  Only the plane's transverse components are injected.
    ``component`` is ignored."""

    component: int = -1
    fields: Optional[dict] = None

    def __post_init__(self):
        if self.fields is None or any(c not in self.fields for c in range(6)):
            raise ValueError("An equivalent source requires all 6 field components.")
        f = {c: np.asarray(self.fields[c], dtype=np.complex128) for c in range(6)}
        if any(v.ndim != 3 for v in f.values()):
            raise ValueError("The supplied field profiles must be 3D.")
        self.normal_axis = _plane_axis(self.size)
        n = [0.0, 0.0, 0.0]
        n[self.normal_axis] = 1.0
        ex, ey, ez, hx, hy, hz = (f[c] for c in range(6))
        currents = {
            0: n[1] * hz - n[2] * hy, 1: n[2] * hx - n[0] * hz, 2: n[0] * hy - n[1] * hx,
            3: n[2] * ey - n[1] * ez, 4: n[0] * ez - n[2] * ex, 5: n[1] * ex - n[0] * ey,
        }
        keep = _transverse(self.normal_axis)
        self._interp = {c: interpolator_from_array(currents[c], self.center, self.size) for c in keep}

    def components(self):
        return list(self._interp)

    def profile(self, point, component) -> complex:
        return complex(self._interp[component](np.asarray(point, dtype=float)))


def TFSFSource(*, time_profile, size, center=(0.0, 0.0, 0.0), injection_axis: int = 2, direction: int = -1,
               polarization_angle: float = 0.0, amplitude: complex = 1.0, eps: float = 1.0, mu: float = 1.0,
               n_grid: int = 50) -> List[EquivalentSource]:
    """TFSFSource (SpatialSources.jl:297-410): a total-field/scattered-field
    box as six EquivalentSource faces carrying the analytic incident plane
    wave along ±``injection_axis`` (0..2 here, 1..3 in the reference), each
    face sampled on about ``n_grid`` points per largest box side; the upper
    face of each axis injects with amplitude −1, the lower one with +1."""
    if injection_axis not in (0, 1, 2) or direction not in (-1, 1):
        raise ValueError("injection_axis must be 0, 1 or 2 and direction ±1")
    k_hat = [0.0, 0.0, 0.0]
    k_hat[injection_axis] = float(direction)
    k_mag = 2 * math.pi * float(time_profile.fcen) * math.sqrt(eps * mu)
    z0 = math.sqrt(mu / eps)
    tr = [a for a in range(3) if a != injection_axis]
    e_pol = [0.0, 0.0, 0.0]
    e_pol[tr[0]] = math.cos(polarization_angle)
    e_pol[tr[1]] = math.sin(polarization_angle)
    h_pol = [v / z0 for v in _cross(k_hat, e_pol)]
    half = [float(s) / 2 for s in size]
    smax = max(float(s) for s in size)
    out = []
    for axis in range(3):
        for side in (-1, 1):
            fc = [float(c) for c in center]
            fc[axis] += side * half[axis]
            fs = [float(s) for s in size]
            fs[axis] = 0.0
            o = [a for a in range(3) if a != axis]
            n1 = max(2, int(round(fs[o[0]] * n_grid / smax)))
            n2 = max(2, int(round(fs[o[1]] * n_grid / smax)))
            r1 = np.linspace(fc[o[0]] - fs[o[0]] / 2, fc[o[0]] + fs[o[0]] / 2, n1)
            r2 = np.linspace(fc[o[1]] - fs[o[1]] / 2, fc[o[1]] + fs[o[1]] / 2, n2)
            shape = [1, 1, 1]
            shape[o[0]], shape[o[1]] = n1, n2
            arrs = {c: np.zeros(shape, dtype=np.complex128) for c in range(6)}
            for i2, c2 in enumerate(r2):
                for i1, c1 in enumerate(r1):
                    pos = [0.0, 0.0, 0.0]
                    pos[axis] = fc[axis]
                    pos[o[0]], pos[o[1]] = c1, c2
                    th = -k_mag * sum(a * b for a, b in zip(k_hat, pos))
                    ph = complex(math.cos(th), math.sin(th))
                    idx = [0, 0, 0]
                    idx[o[0]], idx[o[1]] = i1, i2
                    for c in range(3):
                        arrs[c][tuple(idx)] = amplitude * e_pol[c] * ph
                        arrs[3 + c][tuple(idx)] = amplitude * h_pol[c] * ph
            out.append(EquivalentSource(time_profile=time_profile, fields=arrs, center=tuple(fc),
                                        size=tuple(fs), amplitude=-1.0 if side == 1 else 1.0))
    return out


@dataclass
class GaussianBeamSource(Source):
    """GaussianBeamSource (SpatialSources.jl:650-860): the complex-source-point
    beam with waist ``beam_waist`` at ``beam_center`` travelling along
    ``k_vector``, polarised along ``polarization``, injected from a plane
    through Ĵ = n̂ × Ĥ and M̂ = −n̂ × Ê; every transverse component is
    injected.  Only real polarisation vectors (the reference's complex branch
    does not run).  ``component`` is ignored."""

    component: int = -1
    beam_center: Sequence[float] = (0.0, 0.0, 0.0)
    beam_waist: float = 1.0
    k_vector: Sequence[float] = (0.0, 0.0, 1.0)
    polarization: Sequence[float] = (1.0, 0.0, 0.0)
    eps: float = 1.0
    mu: float = 1.0

    def __post_init__(self):
        self.normal_axis = _plane_axis(self.size)
        if any(isinstance(v, complex) and v.imag != 0 for v in self.polarization):
            raise NotImplementedError("complex beam polarisation")
        self._cache = {}

    def components(self):
        return _transverse(self.normal_axis)

    def fields_at(self, point):
        """get_gaussianbeam_field_profiles (SpatialSources.jl:715-831): E, H."""
        key = tuple(float(v) for v in point)
        hit = self._cache.get(key)
        if hit is not None:
            return hit
        import cmath

        k = complex(2 * math.pi * float(self.time_profile.fcen) * math.sqrt(self.eps * self.mu))
        zr = math.sqrt(self.mu / self.eps)
        pol = np.asarray(self.polarization, dtype=float)
        z0 = k * self.beam_waist ** 2 / 2.0
        kz0 = k * z0
        xrel = np.asarray(key) - np.asarray(self.beam_center, dtype=float)
        zhat = np.asarray(self.k_vector, dtype=float) / np.linalg.norm(self.k_vector)
        rho = float(np.linalg.norm(np.cross(zhat, xrel)))
        z = float(xrel @ zhat)
        zc = z - 1j * z0
        rsq = rho * rho + zc * zc
        R = cmath.sqrt(rsq)
        kR = k * R
        kRsq = kR * kR
        kR3 = kRsq * kR
        rescaled = False
        if abs(kR) > 1e-15:
            if abs(kR.imag) > 30.0:
                rescaled = True
                exp_i = cmath.exp(1j * kR.real)
                exp_p = cmath.exp(kR.imag - kz0)
                exp_m = cmath.exp(-kR.imag - kz0)
                cos_kr = 0.5 * (exp_i * exp_m + exp_i.conjugate() * exp_p)
                sin_kr = -1j * 0.5 * (exp_i * exp_m - exp_i.conjugate() * exp_p)
            else:
                cos_kr = cmath.cos(kR)
                sin_kr = cmath.sin(kR)
            f = -3 * (cos_kr / kRsq - sin_kr / kR3)
            g = 1.5 * (sin_kr / kR + cos_kr / kRsq - sin_kr / kR3)
            fmg = (f - g) / rsq
        else:
            kR4 = kRsq * kRsq
            f = kR4 / 280.0 - kRsq / 10.0 + 1.0
            g = kR4 * 3.0 / 280.0 - kRsq / 5.0 + 1.0
            fmg = (kR4 / 5040.0 - kRsq / 140.0 + 0.1) * (k * k)
        i2fk = 0.5j * f * k
        E = np.zeros(3, dtype=np.complex128)
        H = np.zeros(3, dtype=np.complex128)
        rnorm = float(np.linalg.norm(pol))
        if rnorm > 1e-6:
            xh = pol / rnorm
            yh = np.cross(zhat, xh)
            basis = np.stack([xh, yh, zhat], axis=1)
            x = float(xh @ xrel)
            y = float(yh @ xrel)
            e_n = np.array([g + fmg * x * x + i2fk * zc, fmg * x * y, fmg * x * zc - i2fk * x])
            h_n = np.array([fmg * x * y, g + fmg * y * y + i2fk * zc, fmg * y * zc - i2fk * y])
            E = E + rnorm * (basis @ e_n)
            H = H + rnorm * (basis @ h_n)
        if rescaled:
            e0 = 3.0 / (2 * kz0 ** 3) * (kz0 * (kz0 - 1) + 0.5 * (1.0 - cmath.exp(-2.0 * kz0)))
        else:
            e0 = 3.0 / (2 * kz0 ** 3) * (cmath.exp(kz0) * kz0 * (kz0 - 1) + cmath.sinh(kz0))
        E = E / e0
        H = H / (e0 * zr)
        self._cache[key] = (E, H)
        return E, H

    def profile(self, point, component) -> complex:
        """get_source_profile (SpatialSources.jl:833-846)."""
        E, H = self.fields_at(point)
        n = [0.0, 0.0, 0.0]
        n[self.normal_axis] = 1.0
        if component < 3:
            return complex(np.cross(n, H)[component])
        return complex(-np.cross(n, E)[component - 3])
