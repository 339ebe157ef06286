"""Adjoint gradients of DFT-field objectives over the CUDA step loop.

Host mirror of the reference's adjoint stack (src/Adjoint/*.jl):

* ``DesignRegion``            DesignRegion.jl (per-voxel density ρ, linear ε(ρ))
* ``FourierFields``           FourierFieldsObjective (ObjectiveQuantities.jl:252-345)
* ``FieldOverlap``            its DFT contracted with fixed weights (mode-overlap objectives)
* ``OptimizationProblem``     OptimizationProblem.jl:21-320 — ``opt(rho)`` returns
                              ``(f0, gradient)``; INIT → FWD → ADJ state machine
* ``calculate_gradient``      calculate_gradient! (GradientKernel.jl:35-109)
* ``calculate_fd_gradient``   calculate_fd_gradient (GradientKernel.jl:117-152)
* ``simulate``                the ChainRules rrule of ChainRulesIntegration.jl:38-60,
                              as a torch.autograd.Function whose backward runs the adjoint

Method.  An objective J(Y) depends on DFT values Y_f = Σ_o w_f(o)·Ê_f(o) of E
components on monitor cells o, so its first variation is a real linear
functional of the time-domain field there: dJ = Σ_n Σ_o s_o(n)·dE_o(n) with
s_o(n) = Re Σ_f conj(G_f)·w_f(o)·φ_f(n) (G = ∂J/∂Re Y + i ∂J/∂Im Y, φ_f(n) the
per-step DFT factor Δt·e^{iωt_n}).  Perturbing ε⁻¹ at a design voxel v acts on
the forward run like a transient current source δ·ε_v²·E_v(m) at v each step
(the reference's sources are transient: E = ε⁻¹(D + S), S cleared each step,
Helpers.jl:329-332).  The Yee update is reciprocal: with A the one-step matrix
on (D, B), Aᵀ = Q·A·Q⁻¹ for Q = diag(ε⁻¹, −μ⁻¹), so the response at v to a
transient source at o equals the response at o to one at v.  Hence the
adjoint field is a FORWARD run of the same kernels, with sources on the
objective cells:

* "time" mode (exact for the finite run): inject s_o(N−1−j), the weights
  time-reversed, and correlate ∂J/∂ε_c(v) = −Σ_m E_c(v, m)·A_c(v, N−1−m), with
  E recorded on the design voxels during the forward run; one adjoint run for
  all frequencies.
* "dft" mode (forward DFT fields kept, no time history): one adjoint run per
  frequency f injecting the complex pattern a(o) = Σ_m conj(G_{m,f})·w_{m,f}(o)
  with a pulse g whose DFT at f is Ŝ_f; then
  ∂Y_f/∂ε_c(v) = −Ê_c^fwd(v, f)·Ê_c^adj(v, f)/Ŝ_f.  A real run carries a complex
  pattern exactly at f through the table source Re(a·(g(n) + i·q(n))) with
  q(n) = (cos(ωΔt)·g(n) − g(n−1))/sin(ωΔt), whose DFT is −i times that of g at
  ω.  Exact for the DTFT, i.e. once the fields have decayed within the run.

Both need the design voxels and the objective cells outside the CPML (the
discrete CPML is not reciprocal), and every DFT involved runs at every step
(decimation 1): a decimated sum would alias.

The reference's multi-frequency adjoint source is an average-amplitude
placeholder (ObjectiveQuantities.jl:333-343, AdjointSourceScale.jl:111-122);
this module computes the exact gradient of the discrete system instead.
"""
from __future__ import annotations

import copy
import math
from dataclasses import dataclass, field
from typing import Callable, List, Optional, Sequence

import numpy as np

from .spec import MAT_CHI3, MAT_EPS_INV, KH_F32, HistorySpec, MonitorSpec, SimSpec, SourceSpec, TIME_TABLE


@dataclass
class DesignRegion:
    """Per-voxel density ρ ∈ [0, 1] on a cell box; ε = ε_min + ρ·(ε_max − ε_min)
    on all three diagonal components of each voxel (the linear interpolation
    of GradientKernel.jl:30-31; one design parameter per Yee cell, so the
    restriction step is the identity)."""

    start: tuple
    dims: tuple
    eps_min: float
    eps_max: float

    @property
    def n(self) -> int:
        return int(np.prod(self.dims))

    def eps_inv(self, rho: np.ndarray) -> np.ndarray:
        rho = np.clip(np.asarray(rho, dtype=np.float64).reshape(self.dims, order="F"), 0.0, 1.0)
        return 1.0 / (self.eps_min + rho * (self.eps_max - self.eps_min))


@dataclass
class FieldOverlap:
    """Y_f = Σ_c Σ_cells weights[c][cell, f] · Ê_c(cell, f) over E-component DFT
    monitors, one cell box per component: the FourierFieldsObjective DFT
    (ObjectiveQuantities.jl:252-288) contracted with fixed weights, e.g.
    conj(E_ref) for a mode-overlap objective |∫E·E_ref*|².  The contraction
    runs in FP64 on the device (kh_sim_dft_overlap)."""

    components: Sequence[int]          # subset of EX, EY, EZ
    starts: Sequence[tuple]
    dims: Sequence[tuple]
    weights: Sequence[np.ndarray]      # complex (dims + (nf,)) per component

    def value_from_dfts(self, dfts: Sequence[np.ndarray]) -> np.ndarray:
        return sum(np.einsum("xyzf,xyzf->f", d, w) for d, w in zip(dfts, self.weights))

    def pattern(self, G: np.ndarray, part: int, k: int) -> np.ndarray:
        """Adjoint-source amplitudes on part `part`'s cells at frequency k:
        conj(G_k)·w (dJ = Re Σ_k conj(G_k)·dY_k)."""
        return np.conj(G[k]) * self.weights[part][..., k]


@dataclass
class FourierFields:
    """FourierFieldsObjective (ObjectiveQuantities.jl:252-288): the DFT of one
    E component over a cell box; the objective function receives the complex
    array itself, shape (Nx, Ny, Nz, Nf)."""

    component: int
    start: tuple
    dim: tuple

    @property
    def components(self):
        return [self.component]

    @property
    def starts(self):
        return [tuple(self.start)]

    @property
    def dims(self):
        return [tuple(self.dim)]

    def value_from_dfts(self, dfts: Sequence[np.ndarray]) -> np.ndarray:
        return np.array(dfts[0], dtype=np.complex128)

    def pattern(self, G: np.ndarray, part: int, k: int) -> np.ndarray:
        return np.conj(G[..., k])


def adjoint_time_table(freq: float, dt: float, steps: int, T, bandwidth: float = 0.5):
    """Time table of an adjoint source at ``freq`` for ``steps`` steps.

    Column 1 (the E half-step value of step n, time t_n = nΔt + Δt/2 as the
    run forms it) holds g(n) + i·q(n): g a Gaussian pulse centred on freq with
    fwidth = bandwidth·freq over ±4.5 widths, q its exact quadrature at ω =
    2π·freq.  Column 0 (H half-step) is zero: the sources are E components.
    Returns (table, cutoff_time, Ŝ), Ŝ = Σ_n Δt·e^{iωt_n}·g(n) with the phase
    factors the device DFT uses.
    """
    T = np.dtype(T).type
    f = float(T(freq))
    w = 2 * math.pi * f
    dtT = T(dt)
    t = e_sample_times(dt, steps, T)
    width = 1.0 / (bandwidth * f)
    t0 = 4.5 * width
    g = np.exp(-((t - t0) ** 2) / (2 * width * width)) * np.cos(w * (t - t0))
    g[t > 2 * t0] = 0.0
    g = g.astype(T).astype(np.float64)
    c, s = math.cos(w * float(dtT)), math.sin(w * float(dtT))
    g_prev = np.concatenate([[0.0], g[:-1]])
    q = ((c * g - g_prev) / s).astype(T).astype(np.float64)
    tab = np.zeros((steps, 2), dtype=np.complex128)
    tab[:, 1] = g + 1j * q
    S_hat = complex(np.sum(dft_phases(freq, dt, steps, T) * g))
    return tab, 2 * t0, S_hat


def e_sample_times(dt: float, steps: int, T) -> np.ndarray:
    """Time of the E half of step n as the run forms it: round_time(n) + Δt/2
    (Simulation.jl:22, Kernels.jl:70,85), n < steps."""
    T = np.dtype(T).type
    dtT = T(dt)
    return np.array([T(T(k) * dtT) for k in range(steps)], dtype=np.float64) + float(dtT / T(2))


def dft_phases(freq: float, dt: float, steps: int, T) -> np.ndarray:
    """Per-step DFT factors of an E monitor at ``freq`` exactly as the device
    applies them: Δt·e^{iθ}, θ = f·2π·t in FP64, each part rounded to T."""
    T = np.dtype(T).type
    th = float(T(freq)) * (2 * math.pi * e_sample_times(dt, steps, T))
    dtT = float(T(dt))
    return (np.cos(th) * dtT).astype(T).astype(np.float64) + 1j * (np.sin(th) * dtT).astype(T).astype(np.float64)


def wirtinger(objective: Callable, Ys: List[np.ndarray]):
    """(J, [G_m]) with G = ∂J/∂Re Y + i ∂J/∂Im Y for each argument, by torch
    autograd when J accepts torch tensors (the reference's _compute_jacobian,
    OptimizationProblem.jl:331-374, uses ForwardDiff), else central differences."""
    try:
        import torch
    except ImportError:
        torch = None
    if torch is not None:
        # grad mode may be off (e.g. inside an autograd.Function's forward)
        with torch.enable_grad():
            ts = [torch.tensor(np.asarray(Y, dtype=np.complex128), requires_grad=True) for Y in Ys]
            try:
                J = objective(*ts)
            except (TypeError, RuntimeError, ValueError):
                J = None  # not written for torch tensors: differentiate numerically
            if isinstance(J, torch.Tensor) and J.requires_grad:
                J.backward()
                return float(J.detach().real), [t.grad.detach().numpy().astype(np.complex128) for t in ts]
    J0 = float(np.real(objective(*Ys)))
    Gs = []
    for m, Y in enumerate(Ys):
        G = np.zeros_like(np.asarray(Y, dtype=np.complex128))
        for idx in np.ndindex(G.shape):
            h = 1e-6 * max(abs(Y[idx]), 1e-300)
            parts = []
            for d in (h, 1j * h):
                Yp = [np.array(y, dtype=np.complex128, copy=True) for y in Ys]
                Ym = [np.array(y, dtype=np.complex128, copy=True) for y in Ys]
                Yp[m][idx] += d
                Ym[m][idx] -= d
                parts.append((float(np.real(objective(*Yp))) - float(np.real(objective(*Ym)))) / (2 * h))
            G[idx] = parts[0] + 1j * parts[1]
        Gs.append(G)
    return J0, Gs


class OptimizationProblem:
    """opt(rho; need_gradient=True) → (f0, gradient), OptimizationProblem.jl:59-80.

    ``spec`` is the forward simulation (sources, materials with per-voxel ε⁻¹
    arrays covering the design box).  Each call updates the design
    (update_design_all!), runs ``steps`` forward steps, evaluates the
    objective function of the objective arguments' Y values, and, when a
    gradient is wanted, runs the adjoint and reduces forward × adjoint fields
    on the device.  The run length is the fixed ``steps`` (the reference runs
    until its DFTs decay, Simulation.jl:411-485).

    ``mode``:
      "time" (default) — exact gradient of the finite run.  The forward run
        records E on the design voxels every step (history monitors); ONE
        adjoint run injects, on the objective cells, the time-reversed real
        weights s_o(N−1−j) = Re Σ_f conj(G_f)·w_f(o)·φ_f(N−1−j) (φ the
        per-step DFT factors); ∂J/∂ε_c(v) = −Σ_m E_c(v, m)·A_c(v, N−1−m)
        (kh_history_correlate).  Memory: 2 × steps × design voxels × 3
        values of the run's precision.
      "dft" — forward DFT fields only, one adjoint run per frequency
        (kh_adjoint_accumulate); exact once the fields have decayed within
        ``steps``, no time history.
    """

    def __init__(self, spec: SimSpec, objective_function: Callable, objective_arguments: Sequence,
                 design_region: DesignRegion, frequencies: Sequence[float], steps: int,
                 adjoint_bandwidth: float = 0.5, mode: str = "time", lib=None):
        if mode not in ("time", "dft"):
            raise ValueError("mode must be 'time' or 'dft'")
        self.base = spec
        self.objective_function = objective_function
        self.objective_arguments = list(objective_arguments)
        self.design_region = design_region
        self.frequencies = [float(f) for f in frequencies]
        self.steps = int(steps)
        self.adjoint_bandwidth = adjoint_bandwidth
        self.mode = mode
        self.lib = lib
        self.current_state = "INIT"
        self.f0 = None
        self.results_list = None
        self.gradient = None
        self.gradient_per_freq = None
        self.f_bank: list = []
        self._fwd = None
        self._adj = None
        self._check_design_materials()
        self._build_specs()

    # -- set-up ---------------------------------------------------------------
    def _check_design_materials(self):
        eps = [a for (k, c, a) in self.base.materials if k == MAT_EPS_INV]
        if len(eps) != 3:
            raise ValueError("the forward spec needs per-voxel ε⁻¹ arrays for all three components")
        # the adjoint runs the same kernels as the forward run, which is exact
        # for a linear system (dielectrics, conductors, Lorentz/Drude poles);
        # a χ3 medium makes the step nonlinear
        if any(k == MAT_CHI3 and np.any(np.asarray(a) != 0) for (k, c, a) in self.base.materials):
            raise ValueError("adjoint gradients need a linear system: the spec carries χ3")

    def _np_T(self):
        return np.float32 if self.base.dtype == KH_F32 else np.float64

    def history_bytes(self) -> int:
        """Device bytes of the two design-voxel histories of the time mode."""
        return 2 * 3 * self.design_region.n * self.steps * np.dtype(self._np_T()).itemsize

    def _build_specs(self):
        T = self._np_T()
        freqs = np.array([float(T(f)) for f in self.frequencies])
        dr = self.design_region
        fwd = copy.copy(self.base)
        fwd.monitors = list(self.base.monitors)
        fwd.sources = list(self.base.sources)
        fwd.histories = list(self.base.histories)
        self._obj_ids = []
        for oq in self.objective_arguments:
            ids = []
            for c, st, dm in zip(oq.components, oq.starts, oq.dims):
                fwd.monitors.append(MonitorSpec(c, tuple(st), tuple(dm), freqs, 1))
                ids.append(len(fwd.monitors) - 1)
            self._obj_ids.append(ids)
        adj = copy.copy(self.base)
        adj.sources, adj.monitors, adj.histories = [], [], []
        self._fwd_design, self._adj_design = [], []
        for c in range(3):
            if self.mode == "dft":
                fwd.monitors.append(MonitorSpec(c, tuple(dr.start), tuple(dr.dims), freqs, 1))
                self._fwd_design.append(len(fwd.monitors) - 1)
                adj.monitors.append(MonitorSpec(c, tuple(dr.start), tuple(dr.dims), freqs, 1))
                self._adj_design.append(len(adj.monitors) - 1)
            else:
                fwd.histories.append(HistorySpec(c, tuple(dr.start), tuple(dr.dims), self.steps))
                self._fwd_design.append(len(fwd.histories) - 1)
                adj.histories.append(HistorySpec(c, tuple(dr.start), tuple(dr.dims), self.steps))
                self._adj_design.append(len(adj.histories) - 1)
        # adjoint sources on the objective cells: one per objective component
        # ("dft": one frequency per run) or per component and frequency ("time")
        self._adj_src = []
        kset = [None] if self.mode == "dft" else list(range(len(self.frequencies)))
        for m, oq in enumerate(self.objective_arguments):
            for ci, (c, st, dm) in enumerate(zip(oq.components, oq.starts, oq.dims)):
                for k in kset:
                    adj.sources.append(SourceSpec(component=c, start=tuple(st), dims=tuple(dm),
                                                  amp=np.ones(tuple(dm), dtype=np.complex128),
                                                  time_kind=TIME_TABLE, cutoff=0.0,
                                                  table=np.zeros((1, 2), dtype=np.complex128)))
                    self._adj_src.append((m, ci, k, len(adj.sources) - 1))
        self.fwd_spec = fwd
        self.adj_spec = adj

    def _sims(self):
        from .device import GpuSim

        if self._fwd is None:
            self._fwd = GpuSim(self.fwd_spec, lib=self.lib)
        if self._adj is None:
            self._adj = GpuSim(self.adj_spec, lib=self.lib)
        return self._fwd, self._adj

    def close(self):
        for s in (self._fwd, self._adj):
            if s is not None:
                s.close()
        self._fwd = self._adj = None

    # -- the state machine ------------------------------------------------------
    def update_design(self, rho: np.ndarray):
        """update_design_all! (OptimizationProblem.jl:87-93): new ε⁻¹ on the
        design box of both simulations, fields reset."""
        fwd, adj = self._sims()
        einv = self.design_region.eps_inv(rho)
        for s in (fwd, adj):
            for c in range(3):
                s.update_material_box(MAT_EPS_INV, c, self.design_region.start, einv)
            s.reset()
        self.rho = np.asarray(rho, dtype=np.float64).reshape(self.design_region.dims, order="F").copy()
        self.current_state = "INIT"

    def forward_run(self):
        """forward_run! (OptimizationProblem.jl:104-164) with a fixed step count."""
        fwd, _ = self._sims()
        fwd.reset()
        fwd.step(self.steps)
        Ys = []
        for oq, ids in zip(self.objective_arguments, self._obj_ids):
            if isinstance(oq, FieldOverlap):  # contracted on the device
                Y = np.zeros(len(self.frequencies), dtype=np.complex128)
                for w, mid in zip(oq.weights, ids):
                    Y += fwd.dft_overlap(mid, w)
            else:
                Y = oq.value_from_dfts([fwd.dft(mid) for mid in ids])
            Ys.append(Y)
        self.results_list = Ys
        self.f0, self._G = wirtinger(self.objective_function, Ys)
        self.f_bank.append(self.f0)
        self.current_state = "FWD"
        return self.f0

    def adjoint_run(self):
        """adjoint_run! + calculate_gradient! (OptimizationProblem.jl:177-320,
        GradientKernel.jl:35-109); gradient = ∂J/∂ρ over the design box."""
        if self.mode == "time":
            self.gradient = self._adjoint_time()
        else:
            self.gradient = self._adjoint_dft()
        self.current_state = "ADJ"
        return self.gradient

    def _adjoint_time(self):
        fwd, adj = self._sims()
        T = self._np_T()
        dr = self.design_region
        N = self.steps
        end = float(T(T(N) * T(self.base.dt))) + float(self.base.dt)  # active for all N steps
        phases = [dft_phases(f, float(self.base.dt), N, T) for f in self.frequencies]
        for (m, ci, k, si) in self._adj_src:
            tab = np.zeros((N, 2), dtype=np.complex128)
            tab[:, 1] = phases[k][::-1]
            amp = self.objective_arguments[m].pattern(self._G[m], ci, k)
            adj.update_source(si, amp=amp, table=tab, cutoff=end)
        adj.reset()
        adj.step(N)
        g = np.zeros(tuple(dr.dims))
        fwd.history_correlate(self._fwd_design, adj, self._adj_design, N, -(dr.eps_max - dr.eps_min), g)
        self.gradient_per_freq = None
        return g

    def _adjoint_dft(self):
        fwd, adj = self._sims()
        T = self._np_T()
        dr = self.design_region
        nf = len(self.frequencies)
        self.gradient_per_freq = np.zeros((nf,) + tuple(dr.dims))
        for k, f in enumerate(self.frequencies):
            if all(not np.any(np.asarray(G)[..., k] != 0) for G in self._G):
                continue
            tab, cutoff, S_hat = adjoint_time_table(f, float(self.base.dt), self.steps, T, self.adjoint_bandwidth)
            for (m, ci, _, si) in self._adj_src:
                amp = self.objective_arguments[m].pattern(self._G[m], ci, k)
                adj.update_source(si, amp=amp, table=tab, cutoff=cutoff)
            adj.reset()
            adj.step(self.steps)
            g = np.zeros(tuple(dr.dims))
            # dJ/dε_c(v) = Re(−F·A/Ŝ); dε/dρ = ε_max − ε_min on all three components
            coef = -(dr.eps_max - dr.eps_min) / S_hat
            fwd.adjoint_accumulate(self._fwd_design, k, adj, self._adj_design, k, coef, g)
            self.gradient_per_freq[k] = g
        return self.gradient_per_freq.sum(axis=0)

    def __call__(self, rho: np.ndarray, need_gradient: bool = True):
        self.update_design(rho)
        if self.current_state == "INIT":
            self.forward_run()
        if need_gradient and self.current_state == "FWD":
            self.adjoint_run()
        return self.f0, (self.gradient if need_gradient else None)

    def calculate_fd_gradient(self, rho: np.ndarray, indices: Sequence[tuple], db: float = 1e-3):
        """Central finite differences of the objective at the given design
        voxels (calculate_fd_gradient, GradientKernel.jl:117-152; ρ clamped to
        [0, 1] and the actual step used)."""
        rho = np.asarray(rho, dtype=np.float64).reshape(self.design_region.dims, order="F")
        out = []
        for idx in indices:
            lo = rho.copy()
            hi = rho.copy()
            lo[idx] = max(rho[idx] - db, 0.0)
            hi[idx] = min(rho[idx] + db, 1.0)
            fl, _ = self(lo, need_gradient=False)
            fh, _ = self(hi, need_gradient=False)
            out.append((fh - fl) / (hi[idx] - lo[idx]))
        return np.array(out)


def power_overlap(*Ys):
    """J = Σ_m Σ_f |Y_{m,f}|² (numpy or torch complex arrays)."""
    return sum((Y.real ** 2 + Y.imag ** 2).sum() for Y in Ys)


def plane_monitors(spec: SimSpec, plane, frequencies, T) -> List[int]:
    """Append decimation-1 DFT monitors for [(component, start, dims)] to spec."""
    freqs = np.array([float(T(f)) for f in frequencies])
    ids = []
    for comp, st, dm in plane:
        spec.monitors.append(MonitorSpec(comp, tuple(st), tuple(dm), freqs, 1))
        ids.append(len(spec.monitors) - 1)
    return ids


def reference_fields(w, lib=None, promote: bool = False) -> List[np.ndarray]:
    """E_ref on the objective plane: the straight-strip run of a BendWorkload
    (same grid, same step count), one DFT array per component.  ``promote``
    runs the same inputs in FP64 (SimSpec.promoted)."""
    from .device import GpuSim

    sp = w.straight.spec()
    sp.monitors = []
    ids = plane_monitors(sp, w.plane, w.frequencies, w.straight.grid.T)
    if promote:
        sp = sp.promoted()
    g = GpuSim(sp, lib=lib)
    try:
        g.step(w.steps)
        return [g.dft(i) for i in ids]
    finally:
        g.close()


def bend_problem(w, e_ref: Optional[List[np.ndarray]] = None, lib=None, mode: str = "time",
                 promote: bool = False) -> OptimizationProblem:
    """The waveguide-bend objective J = Σ_f |Σ_plane E·E_ref*|² as an
    OptimizationProblem over the workload's design box.  ``promote`` builds
    the FP64 problem of the same inputs (cell indices, boxes, source
    footprints and values of the workload's precision, FP64 arithmetic), the
    reference an FP32 gradient's error is measured against."""
    if e_ref is None:
        e_ref = reference_fields(w, lib=lib, promote=promote)
    spec = w.sim.spec()
    spec.monitors = []
    if promote:
        spec = spec.promoted()
    oq = FieldOverlap(components=[c for c, _, _ in w.plane], starts=[s for _, s, _ in w.plane],
                      dims=[d for _, _, d in w.plane], weights=[np.conj(e) for e in e_ref])
    dr = DesignRegion(tuple(w.design_start), tuple(w.design_dims), w.eps_min, w.eps_max)
    freqs = [float(w.sim.grid.T(f)) for f in w.frequencies]  # as the workload's precision stores them
    return OptimizationProblem(spec, power_overlap, [oq], dr, freqs, w.steps, mode=mode, lib=lib)


def simulate(opt: OptimizationProblem, rho):
    """simulate(opt, designs) with its rrule (ChainRulesIntegration.jl:20-60):
    a torch.autograd.Function whose forward is the forward run and whose
    backward runs the adjoint simulations and returns grad_output·∂J/∂ρ."""
    import torch

    class _Simulate(torch.autograd.Function):
        @staticmethod
        def forward(ctx, r):
            f0, _ = opt(r.detach().cpu().double().numpy(), need_gradient=False)
            return torch.tensor(f0, dtype=torch.float64)

        @staticmethod
        def backward(ctx, grad_out):
            g = opt.adjoint_run()
            return grad_out * torch.from_numpy(np.ascontiguousarray(g)).to(torch.float64)

    return _Simulate.apply(rho)
