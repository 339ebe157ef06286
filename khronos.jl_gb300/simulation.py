"""Simulation: host mirror of Khronos's user API over the CUDA step loop.

Mirrors the reference's ``Simulation(...)`` / ``prepare_simulation!`` /
``run(sim; until, until_after_sources)`` (a time or a stop function such as
``stop_when_dft_decayed``) / ``get_flux`` calls (src/DataStructures.jl:714-801,
src/Simulation.jl:92-539, src/Monitors/FluxMonitor.jl:92-156).  Geometry is given as per-voxel material
arrays on the Center range (rasterisation of shapes is set-up, not part of the
step loop); everything else follows the reference's arithmetic.
"""
from __future__ import annotations

import logging
import math
import time
import warnings
from typing import Callable, List, Optional, Sequence, Union

import numpy as np

from . import grid as G

log = logging.getLogger("khronos_gb300")
from .monitors import DFTMonitor, FluxMonitor, auto_decimation, flux_from_dft
from .sources import ContinuousWaveSource, CustomSource, GaussianPulseSource
from .spec import (KH_F32, KH_F64, MAT_CHI3, MAT_EPS_INV, MAT_MU_INV, MAT_SIGMA_B, MAT_SIGMA_D,
                   SEM_CPML, SEM_REFERENCE_CPU,
                   TIME_CW, TIME_GAUSSIAN, TIME_TABLE, LorentzianSusceptibility, MonitorSpec, PoleSpec,
                   SimSpec, SourceSpec, ade_coefficients)


class Simulation:
    """A 3D Khronos simulation whose step loop runs on the GPU.

    ``semantics`` selects the CPML stage logic: "cpml" (default) follows the
    reference's CUDA PML kernels and is stable; "reference_cpu" restates the
    reference's CPU-backend dispatch exactly, including the dropped σ_prev
    stage that makes that path grow without bound once PML is present.

    ``boundary_conditions`` ([[lo, hi]] per axis of ``boundaries.PECBoundary``,
    ``PMCBoundary``, ...) zeroes the PML conductivity on those sides while the
    PML regions keep following ``boundaries``, as the reference's prepare
    does; an axis with Periodic (or Bloch with k = 0) on both sides wraps its
    fields' halo after every half-step.

    Materials (all optional; arrays are (Nx, Ny, Nz), cell-indexed):
      geometry: list of geometry.Object (Ball / Cuboid / Cylinder with an
      isotropic ε) rasterised on the device at each component's Yee position,
      with background_eps elsewhere and subpixel_smoothing "none", "volume" or
      "anisotropic" (instead of eps_inv arrays),
      eps_inv: scalar or 3 arrays (ε⁻¹ per Yee component), mu_inv likewise,
      sigma_d / sigma_b: 3 conductivity arrays, chi3: one Center array,
      poles: list of (LorentzianSusceptibility, σ array) — ε⁻¹ must already
      carry the χ1 semi-implicit correction (``apply_chi1_correction``).
    """

    def __init__(self, *, cell_size, resolution, sources=(), cell_center=(0.0, 0.0, 0.0),
                 boundaries=None, monitors=(), dtype="f32", courant=0.5, eps_inv=1.0, mu_inv=1.0,
                 sigma_d=None, sigma_b=None, chi3=None, poles=(), semantics="cpml", geometry=None,
                 background_eps=1.0, subpixel_smoothing="none", boundary_conditions=None):
        self.grid = G.Grid.build(cell_size, cell_center, resolution, dtype, courant)
        self.dtype = dtype
        self.sources = list(sources)
        self.boundaries = boundaries
        from .boundaries import effective_pml, periodic_mask

        self.boundary_conditions = boundary_conditions
        self._sigma_boundaries = effective_pml(boundaries, boundary_conditions)
        self._periodic = periodic_mask(boundary_conditions)
        self.monitors = list(monitors)
        self.eps_inv = eps_inv
        self.mu_inv = mu_inv
        self.sigma_d = sigma_d
        self.sigma_b = sigma_b
        self.chi3 = chi3
        self.poles = list(poles)
        if semantics not in ("cpml", "reference_cpu"):
            raise ValueError("semantics must be 'cpml' or 'reference_cpu'")
        self.semantics = semantics
        if geometry is not None and not np.isscalar(eps_inv):
            raise ValueError("give either geometry objects or per-voxel eps_inv arrays, not both")
        self.geometry = list(geometry) if geometry is not None else None
        self.background_eps = background_eps
        self.subpixel_smoothing = subpixel_smoothing
        self._dev = None
        self._dft_monitors: List[DFTMonitor] = []
        self._norm_cache = None

    # -- convenience --------------------------------------------------------
    @property
    def n(self):
        return self.grid.n

    @property
    def dt(self):
        return self.grid.dt

    def round_time(self, timestep: Optional[int] = None) -> float:
        """round_time(sim) = Float64(timestep·Δt) in the run's precision (Simulation.jl:22)."""
        ts = self.timestep if timestep is None else timestep
        T = self.grid.T
        return float(T(T(ts) * self.grid.dt))

    def last_source_time(self) -> float:
        """max cutoff over sources; ∞ if any CW source (TimeSources.jl:40-47, Kernels.jl:27-35)."""
        T = self.grid.T
        if not self.sources:
            return math.inf
        return max(s.time_profile.cutoff_time(T) for s in self.sources)

    # -- prepare ------------------------------------------------------------
    def spec(self) -> SimSpec:
        """Host-side set-up of prepare_simulation! as a backend-independent SimSpec."""
        g = self.grid
        T = g.T
        sp = SimSpec(n=g.n, dtype=KH_F32 if T is np.float32 else KH_F64,
                     delta=tuple(float(d) for d in g.delta), dt=float(g.dt),
                     semantics=SEM_CPML if self.semantics == "cpml" else SEM_REFERENCE_CPU,
                     periodic=self._periodic)
        if self.boundaries is not None:
            lo, hi = G.pml_widths(g, self.boundaries)
            sp.pml_lo, sp.pml_hi = lo, hi
            for a in range(3):
                L, R = self._sigma_boundaries[a]
                s = G.cell_sigma(g, a, L, R).astype(np.float64)
                sp.sigma_b[a] = s
                sp.sigma_d[a] = s.copy()
        # materials
        geo_poles = []
        if self.geometry is not None:
            from .geometry import pole_arrays

            geo_poles = pole_arrays(self.geometry, g, self.boundaries)
        if self.geometry is not None and geo_poles:
            # dispersive objects: ε∞ on the host too, so that the χ1
            # correction (Geometry.jl:1236-1250) can act on it
            from .geometry import rasterize_values

            if self.subpixel_smoothing != "none":
                raise NotImplementedError("subpixel smoothing together with dispersive objects")
            if self.poles:
                raise ValueError("give poles either on geometry objects or as arrays, not both")
            eps = [1.0 / rasterize_values(self.geometry, g, G.EX + c, [o.material.eps for o in self.geometry],
                                          self.background_eps) for c in range(3)]
            eps = apply_chi1_correction(eps, geo_poles, g.dt, T=np.float64)
            for c in range(3):
                sp.materials.append((MAT_EPS_INV, c, _xfast(eps[c])))
        elif self.geometry is not None:  # rasterised on the device (kh_sim_set_geometry)
            from .geometry import geometry_spec

            sp.geometry = geometry_spec(self.geometry, g, self.background_eps, self.subpixel_smoothing)
        elif np.isscalar(self.eps_inv):
            sp.eps_inv = float(T(self.eps_inv))
        else:
            for c in range(3):
                sp.materials.append((MAT_EPS_INV, c, _xfast(self.eps_inv[c])))
        if np.isscalar(self.mu_inv):
            sp.mu_inv = float(T(self.mu_inv))
        else:
            for c in range(3):
                sp.materials.append((MAT_MU_INV, c, _xfast(self.mu_inv[c])))
        for kind, arrs in ((MAT_SIGMA_D, self.sigma_d), (MAT_SIGMA_B, self.sigma_b)):
            if arrs is not None:
                for c in range(3):
                    if arrs[c] is not None:
                        sp.materials.append((kind, c, _xfast(arrs[c])))
        if self.chi3 is not None:
            sp.materials.append((MAT_CHI3, 0, _xfast(self.chi3)))
        if self.geometry is not None:  # μ, σD, σB, χ3 of the objects (host rasterisation)
            from .geometry import material_arrays

            geo_mats = material_arrays(self.geometry, g)
            given = {(kind, c) for kind, c, _ in sp.materials}
            clash = [(kind, c) for kind, c, _ in geo_mats if (kind, c) in given or
                     (kind == MAT_MU_INV and not np.isscalar(self.mu_inv))]
            if clash:
                raise ValueError("a material property is given both by geometry objects and by an array")
            sp.materials.extend(geo_mats)
        for sus, sigma in list(self.poles) + geo_poles:
            sp.poles.append(PoleSpec(coeffs=ade_coefficients(sus, float(g.dt)),
                                     sigma=_xfast(sigma)))
        # sources (assemble_sources, Sources.jl:44-92)
        for src in self.sources:
            tp = src.time_profile
            for comp in src.components():
                gv, amp = src.amplitude_array(g, comp)
                s = SourceSpec(component=comp, start=gv.start0, dims=tuple(amp.shape), amp=amp,
                               time_kind=TIME_GAUSSIAN)
                if isinstance(tp, GaussianPulseSource):
                    st = tp.stored(T)
                    s.fcen, s.width, s.peak_time, s.cutoff = (float(st["fcen"]), float(st["width"]),
                                                              float(st["peak_time"]), float(st["cutoff"]))
                elif isinstance(tp, ContinuousWaveSource):
                    s.time_kind = TIME_CW
                    s.fcen = float(T(tp.fcen))
                elif isinstance(tp, CustomSource):
                    s.time_kind = TIME_TABLE
                    s.fcen = float(T(tp.fcen))
                    s.cutoff = float(T(tp.end_time))
                    tab = np.zeros((tp.table_steps, 2), dtype=np.complex128)
                    dt = g.dt
                    for n in range(tp.table_steps):
                        t0 = float(T(T(n) * dt))
                        t1 = t0 + float(dt / T(2))
                        tab[n, 0] = complex(tp.src_func(float(T(t0))))
                        tab[n, 1] = complex(tp.src_func(float(T(t1))))
                    s.table = tab
                else:
                    raise TypeError(f"unsupported time profile {type(tp).__name__}")
                sp.sources.append(s)
        # monitors: auto-decimation then init (Simulation.jl:165-172)
        D = auto_decimation(self.sources, g.dt) if self.sources else 1
        self._dft_monitors = []
        for m in self.monitors:
            if m.decimation == 1 and D > 1:
                m.decimation = D
            if isinstance(m, FluxMonitor):
                self._dft_monitors.extend(m.expand(g))
            else:
                self._dft_monitors.append(m)
        for m in self._dft_monitors:
            gv = g.grid_volume(m.center, m.size, m.component)
            m.gv = gv
            sp.monitors.append(MonitorSpec(component=m.component, start=gv.start0, dims=gv.dims,
                                           freqs=np.array([float(T(f)) for f in m.frequencies]),
                                           decimation=int(m.decimation)))
        return sp

    def prepare(self):
        """prepare_simulation!: build the spec and the device state."""
        if self._dev is not None:
            return self
        from .device import GpuSim

        sp = self.spec()
        self._spec = sp
        self._dev = GpuSim(sp)
        for idx, m in enumerate(self._dft_monitors):
            m.monitor_id = idx
            m.sim = self
        for m in self.monitors:
            m.sim = self
        return self

    # -- running --------------------------------------------------------------
    @property
    def timestep(self) -> int:
        return self._dev.timestep if self._dev is not None else 0

    def step(self, nsteps: int = 1, stream: Optional[int] = None):
        self.prepare()
        self._dev.step(nsteps, stream)

    def steps_until(self, until: float) -> int:
        """Steps `run(sim; until)` takes: while !(round_time > until) step!."""
        ts = self.timestep
        n = 0
        while not (self.round_time(ts + n) > until):
            n += 1
        return n

    def run(self, until: Union[float, Callable, None] = None,
            until_after_sources: Union[float, Callable, None] = None):
        """run(sim; until | until_after_sources) (Simulation.jl:295-382).

        Each is a time or a function ``f(sim) -> bool`` called before every
        step, the run ending at the first True (``stop_when_dft_decayed``).
        With ``until_after_sources`` the run first steps while
        ``round_time <= last_source_time``.  A function may also offer
        ``steps_before_decision(sim)``: how many steps from now it would
        answer False without changing any state; those steps are then taken
        in one batch instead of one call per step."""
        if (until is None) == (until_after_sources is None):
            raise ValueError("Must specify exactly one of until / until_after_sources")
        self.prepare()
        log.info("Starting simulation...")
        t_start = time.perf_counter()
        step_start = self.timestep
        try:
            self._run_steps(until, until_after_sources)
        finally:
            self._dev.synchronize()
            total = self.timestep - step_start
            elapsed = time.perf_counter() - t_start
            if total > 0 and elapsed > 0:
                n = self.grid.n
                rate = n[0] * n[1] * max(1, n[2]) * total / elapsed / 1e6
                log.info("Simulation complete: %d steps in %.3fs (%.1f MVoxels/s)", total, elapsed, rate)

    def _run_steps(self, until, until_after_sources):
        if until_after_sources is not None:
            last = self.last_source_time()
            n = 0
            ts = self.timestep
            while self.round_time(ts + n) <= last:
                n += 1
            self.step(n)
            log.info("All sources have terminated...")
            until = until_after_sources
        if not callable(until):
            self.step(self.steps_until(until))
            return
        skip = getattr(until, "steps_before_decision", None)
        while True:
            k = skip(self) if skip is not None else 0
            if k > 0:
                self.step(k)
                continue
            if until(self):
                return
            self.step(1)

    def dft_fields_norms(self) -> np.ndarray:
        """dft_fields_norm of every DFT monitor, flux sub-monitors included
        (Simulation.jl:530-539): sqrt(Σ|F|²) over its accumulated array,
        reduced in FP64 on the device.  Re-read only when a monitor has
        updated since the last read (an update happens in the step taken at
        timestep s when s is a multiple of its decimation)."""
        self.prepare()
        ts = self.timestep
        c = self._norm_cache
        if c is not None:
            t0, norms = c
            if t0 == ts or (t0 < ts and not any(s % m.decimation == 0 for s in range(t0, ts)
                                                for m in self._dft_monitors)):
                self._norm_cache = (ts, norms)
                return norms
        norms = self._dev.dft_norms()
        self._norm_cache = (ts, norms)
        return norms

    def run_benchmark(self, until: int) -> float:
        """run_benchmark(sim, until) (Simulation.jl:492-527): `until` steps,
        timed from step 10 on with the device synchronised; returns the step
        rate in MCells/s (cells × (until − 10) / seconds / 1e6)."""
        import time

        if until <= 10:
            raise ValueError("run_benchmark times steps 10..until: until must exceed 10")
        self.prepare()
        self.step(10)
        self._dev.synchronize()
        t0 = time.perf_counter()
        self.step(until - 10)
        self._dev.synchronize()
        dt = time.perf_counter() - t0
        n = self.grid.n
        return n[0] * n[1] * max(1, n[2]) * (until - 10) / dt / 1e6

    def reset_fields(self):
        """reset_fields! (Simulation.jl:571-637): fields, auxiliary state, DFT
        accumulators and the step counter back to zero; materials, sources
        and monitors stay."""
        self.prepare()
        self._dev.reset()
        self._norm_cache = None

    # -- results ----------------------------------------------------------------
    def get_field(self, comp: int) -> np.ndarray:
        self.prepare()
        return self._dev.field(comp)

    def _read_dft(self, m: DFTMonitor) -> np.ndarray:
        return self._dev.dft(m.monitor_id)

    def _flux(self, fm: FluxMonitor) -> np.ndarray:
        ids = [m.monitor_id for m in fm.e_monitors + fm.h_monitors]
        return self._dev.flux(ids, fm.normal_axis, fm.dA)

    def get_flux(self, fm: FluxMonitor, on_device: bool = True) -> np.ndarray:
        if on_device:
            return self._flux(fm)
        e1, e2 = (self._read_dft(m) for m in fm.e_monitors)
        h1, h2 = (self._read_dft(m) for m in fm.h_monitors)
        return flux_from_dft(fm.normal_axis, e1, e2, h1, h2, fm.dA)

    def close(self):
        if self._dev is not None:
            self._dev.close()
            self._dev = None


def _xfast(a) -> np.ndarray:
    """A cell-indexed [i, j, k] array in FP64 with x fastest in memory (the
    ABI's layout, Julia's column-major order), so that handing it to the
    library needs no transposing copy."""
    return np.asfortranarray(a, dtype=np.float64)


class stop_when_dft_decayed:
    """stop_when_dft_decayed(; tolerance, minimum_runtime, maximum_runtime)
    (Simulation.jl:411-485): a stop function for ``run`` that is True once
    every DFT monitor that has seen signal has a step-to-step change of its
    norm at most ``tolerance`` times the largest change it has seen.

    The reference's logic, call for call: nothing before ``minimum_runtime``;
    True (with a warning) past ``maximum_runtime``; a monitor's first nonzero
    norm only records it; a monitor with no change yet keeps the run going;
    no active monitor keeps it going.  The norm of a decimated monitor does
    not change between its updates, so on those steps its change is 0: once
    each monitor has changed once after the first record, the next step
    without an update reports convergence.  Reproduced as is.
    """

    def __init__(self, tolerance: float = 1e-6, minimum_runtime: float = 0.0,
                 maximum_runtime: float = math.inf):
        if minimum_runtime > maximum_runtime:
            raise ValueError(f"Minimum runtime ({minimum_runtime}) cannot be greater than maximum "
                             f"runtime ({maximum_runtime}).")
        self.tolerance = tolerance
        self.minimum_runtime = minimum_runtime
        self.maximum_runtime = maximum_runtime
        self.state = {}  # monitor index -> (previous norm, largest change)

    def __call__(self, sim) -> bool:
        t = sim.round_time()
        if t < self.minimum_runtime:
            return False
        if t > self.maximum_runtime:
            warnings.warn("Maximum runtime reached.")
            return True
        all_converged = True
        n_active = 0
        for i, cur in enumerate(sim.dft_fields_norms()):
            cur = float(cur)
            if cur == 0.0:
                continue
            if i not in self.state:
                self.state[i] = (cur, 0.0)
                all_converged = False
                continue
            prev, maxchange = self.state[i]
            change = abs(cur - prev)
            maxchange = max(maxchange, change)
            self.state[i] = (cur, maxchange)
            if maxchange == 0.0:
                all_converged = False
                continue
            n_active += 1
            if change / maxchange > self.tolerance:
                all_converged = False
        if n_active == 0:
            return False
        return all_converged

    def steps_before_decision(self, sim) -> int:
        """Steps from now whose calls would return False untouched (before
        the minimum runtime)."""
        ts = sim.timestep
        n = 0
        while sim.round_time(ts + n) < self.minimum_runtime:
            n += 1
        return n


def apply_chi1_correction(eps_inv, poles, dt, T=np.float64):
    """ε⁻¹ → ε⁻¹ / (1 + ε⁻¹·χ1), χ1 = Σ_p γ₁⁻¹·C_p·σ_p/2 (Geometry.jl:1236-1250, 1335-1341).

    Applied cell by cell (the reference indexes the three component arrays by
    the linear index of a Center-sized array; with component-sized arrays that
    is an offset, and the aligned cell-by-cell form is the intended one).
    """
    chi1 = None
    for sus, sigma in poles:
        c = ade_coefficients(sus, float(dt))
        k = c["gamma1_inv"] * (c["drude_coeff"] if c["is_drude"] else c["sigma_omega0_dt_sq"]) / 2
        term = np.asarray(sigma, dtype=T) * T(k)
        chi1 = term if chi1 is None else chi1 + term
    if chi1 is None:
        return eps_inv
    out = []
    for e in eps_inv:
        e = np.array(e, dtype=T, copy=True)
        mask = chi1 != 0
        e[mask] = e[mask] / (T(1) + e[mask] * chi1[mask])
        out.append(e)
    return out
