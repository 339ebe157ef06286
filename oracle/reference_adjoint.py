"""ORACLE — test infrastructure, not product code.

The reference's own adjoint gradient for a single-frequency
FourierFieldsObjective, restated step by step on the oracle step loop so its
accuracy can be reported next to central finite differences (the reference
is Julia and cannot run here):

* forward run with Dx/Dy/Dz DFT monitors on the design region
  (install_design_region_monitors!, src/Adjoint/DesignRegion.jl:293-312);
  at design voxels D = ε·E (E = ε⁻¹(D + S − P) with no source or pole there);
* dJ = (∂J/∂Re Y + i ∂J/∂Im Y)/2 (_compute_jacobian,
  src/Adjoint/OptimizationProblem.jl:331-374);
* adjoint source: one SourceData per objective on its monitor cells with
  amplitude dJ·scale and the forward source's time profile
  (place_adjoint_source, src/Adjoint/ObjectiveQuantities.jl:290-332), scale =
  2·dV/(π·√(2π)·fwd_dtft) with dV = 1 and fwd_dtft = Σ_{n < floor(T/Δt)}
  Δt/√(2π)·e^{i2πf nΔt}·f_src(nΔt) (adj_src_scale,
  src/Adjoint/AdjointSourceScale.jl:67-125, single frequency,
  include_resolution = false);
* ∂J/∂ρ_v = Σ_c Re[dε⁻¹/dρ · D_adj,c(v) · D_fwd,c(v)], dε⁻¹/dρ = −Δε/ε²
  (calculate_gradient!, src/Adjoint/GradientKernel.jl:35-109; one design
  parameter per Yee cell, so the interpolation weight is 1 and no z sum).

The run length is the problem's fixed step count on both runs.

Measured on the 24×20×16 test case (J = Σ|Ez|² on a plane, one frequency,
3500 steps, fields decayed): as written the procedure's gradient has the
wrong sign and a voxel-dependent ratio to central differences (correlation
−0.58); with the amplitude conjugated it equals cos(ωΔt/2)/(2π) times the
finite-difference gradient at every voxel (the 1/(2π) from scale·DFT(f)/2,
the cosine from the E sources running at (n + ½)Δt while the scale's DTFT
samples nΔt).
"""
from __future__ import annotations

import copy
import math

import numpy as np

from .adjoint import _with_design
from .oracle import OracleSim


def _gaussian(src, t: float) -> complex:
    """eval_time_source(::GaussianPulseData, t) in FP64 (TimeSources.jl:123-132)."""
    tt = t - src.peak_time
    if tt > src.cutoff:
        return 0j
    g = math.exp(-tt * tt / (2 * src.width * src.width))
    b = -2 * math.pi * src.fcen * tt
    return complex(g * math.cos(b), g * math.sin(b))


def reference_gradient(opt, rho, conjugate_amplitude: bool = False):
    """∂J/∂ρ by the reference's procedure.  ``conjugate_amplitude`` uses
    conj(dJ)·scale as the adjoint amplitude (the time reversal the exact
    derivation calls for) instead of the reference's dJ·scale."""
    from khronos_gb300.adjoint import FourierFields, wirtinger
    from khronos_gb300.spec import MonitorSpec, TIME_GAUSSIAN

    if len(opt.frequencies) != 1 or not all(isinstance(o, FourierFields) for o in opt.objective_arguments):
        raise ValueError("the reference's exact-scale adjoint covers one frequency and FourierFields objectives")
    T = opt._np_T()
    f = opt.frequencies[0]
    dr = opt.design_region
    freqs = np.array([float(T(f))])
    src0 = opt.base.sources[0]
    if src0.time_kind != TIME_GAUSSIAN:
        raise ValueError("the forward source must be a Gaussian pulse")

    def with_design_monitors(spec):
        sp = _with_design(spec, opt, rho)
        sp.monitors = list(sp.monitors)
        sp.histories = []
        ids = []
        for c in range(3):
            sp.monitors.append(MonitorSpec(c, tuple(dr.start), tuple(dr.dims), freqs, 1))
            ids.append(len(sp.monitors) - 1)
        return sp, ids

    # forward run
    sp, dids = with_design_monitors(opt.fwd_spec)
    o = OracleSim(sp)
    o.step(opt.steps)
    Ys = [oq.value_from_dfts([o.dft(i) for i in ids]) for oq, ids in zip(opt.objective_arguments, opt._obj_ids)]
    eps = 1.0 / dr.eps_inv(rho)
    d_fwd = [eps * o.dft(i)[..., 0] for i in dids]
    o.close()
    J, G = wirtinger(opt.objective_function, Ys)
    dJ = [g / 2 for g in G]
    if conjugate_amplitude:
        dJ = [np.conj(d) for d in dJ]

    # adj_src_scale: DTFT of the forward source over the run's time
    dt = float(opt.base.dt)
    T_sim = float(T(T(opt.steps) * T(dt)))
    n = int(math.floor(T_sim / dt))
    t_vals = np.arange(n) * dt
    y = np.array([_gaussian(src0, t) for t in t_vals])
    fwd_dtft = np.sum(dt / math.sqrt(2 * math.pi) * np.exp(1j * 2 * math.pi * f * t_vals) * y)
    scale = 2.0 / (math.pi * math.sqrt(2 * math.pi) * fwd_dtft)

    # adjoint run: the objectives' cells as sources with the forward time profile
    spa, aids = with_design_monitors(opt.fwd_spec)
    spa.sources = []
    for oq, d in zip(opt.objective_arguments, dJ):
        s = copy.copy(src0)
        s.component, s.start, s.dims = oq.component, tuple(oq.start), tuple(oq.dim)
        s.amp = d[..., 0] * scale
        spa.sources.append(s)
    oa = OracleSim(spa)
    oa.step(opt.steps)
    d_adj = [eps * oa.dft(i)[..., 0] for i in aids]
    oa.close()
    d_eps_inv = -(dr.eps_max - dr.eps_min) / eps ** 2
    return sum(np.real(d_eps_inv * a * b) for a, b in zip(d_adj, d_fwd))
