"""ORACLE — test infrastructure, not product code.

CPU restatement of an OptimizationProblem's objective and adjoint gradient
on the oracle step loop (oracle/khronos_oracle.cpp), used by tests/ as the
checker of the CUDA adjoint path (khronos_gb300.adjoint):

* ``objective``       forward run + FieldOverlap values + J (numpy overlap)
* ``gradient``        the same adjoint runs on the oracle ("time" mode: E on
                      the design box recorded every step and correlated with
                      the time-reversed adjoint run; "dft" mode: one adjoint
                      run per frequency) and the same per-voxel reduction in
                      numpy FP64.  The oracle has no history monitors: it steps
                      one step at a time and reads the fields.
* ``fd_gradient``     central finite differences of ``objective``

The reference's own gradient (src/Adjoint/GradientKernel.jl:35-109) cannot run
here (Julia); central differences of the reference's forward step loop,
restated in the oracle, are the pin.
"""
from __future__ import annotations

import copy

import numpy as np

from .oracle import OracleSim


def _with_design(spec, opt, rho):
    """Copy of spec with the design box's ε⁻¹ set from rho (update_design!)."""
    from khronos_gb300.spec import MAT_EPS_INV

    dr = opt.design_region
    einv = dr.eps_inv(rho)
    sp = copy.copy(spec)
    mats = []
    for kind, comp, arr in spec.materials:
        if kind == MAT_EPS_INV:
            arr = np.array(arr, dtype=np.float64, copy=True)
            sl = tuple(slice(dr.start[a], dr.start[a] + dr.dims[a]) for a in range(3))
            arr[sl] = einv
        mats.append((kind, comp, arr))
    sp.materials = mats
    return sp


def objective(opt, rho, want_fields=False):
    from khronos_gb300.adjoint import wirtinger

    sp = _with_design(opt.fwd_spec, opt, rho)
    o = OracleSim(sp)
    o.step(opt.steps)
    Ys = []
    for oq, ids in zip(opt.objective_arguments, opt._obj_ids):
        Ys.append(oq.value_from_dfts([o.dft(mid) for mid in ids]))
    J, G = wirtinger(opt.objective_function, Ys)
    if not want_fields:
        o.close()
        return J
    fwd = [o.dft(i) for i in opt._fwd_design]  # "dft" mode: design-box DFT monitors
    o.close()
    return J, G, fwd


def gradient(opt, rho):
    """∂J/∂ρ over the design box (and, in "dft" mode, the per-frequency parts)."""
    if opt.mode == "time":
        return _gradient_time(opt, rho), None
    return _gradient_dft(opt, rho)


def _record(o, opt, steps):
    """Step the oracle `steps` times, recording E_x..E_z on the design box."""
    dr = opt.design_region
    sl = tuple(slice(dr.start[a], dr.start[a] + dr.dims[a]) for a in range(3))
    hist = np.zeros((steps, 3) + tuple(dr.dims))
    for n in range(steps):
        o.step(1)
        for c in range(3):
            hist[n, c] = o.field(c)[sl]
    return hist


def _gradient_time(opt, rho):
    from khronos_gb300.adjoint import dft_phases, wirtinger

    T = opt._np_T()
    dr = opt.design_region
    N = opt.steps
    o = OracleSim(_with_design(opt.fwd_spec, opt, rho))
    hist_f = _record(o, opt, N)
    Ys = []
    for oq, ids in zip(opt.objective_arguments, opt._obj_ids):
        Ys.append(oq.value_from_dfts([o.dft(mid) for mid in ids]))
    o.close()
    _, G = wirtinger(opt.objective_function, Ys)
    sp = _with_design(opt.adj_spec, opt, rho)
    sp.sources = [copy.copy(s) for s in opt.adj_spec.sources]
    for (m, ci, k, si) in opt._adj_src:
        s = sp.sources[si]
        tab = np.zeros((N, 2), dtype=np.complex128)
        tab[:, 1] = dft_phases(opt.frequencies[k], float(opt.base.dt), N, T)[::-1]
        s.amp = opt.objective_arguments[m].pattern(G[m], ci, k)
        s.table = tab
        s.cutoff = 1e300
    oa = OracleSim(sp)
    hist_a = _record(oa, opt, N)
    oa.close()
    return -(dr.eps_max - dr.eps_min) * np.einsum("ncxyz,ncxyz->xyz", hist_f, hist_a[::-1])


def _gradient_dft(opt, rho):
    from khronos_gb300.adjoint import adjoint_time_table

    T = opt._np_T()
    dr = opt.design_region
    J, G, fwd = objective(opt, rho, want_fields=True)
    per = np.zeros((len(opt.frequencies),) + tuple(dr.dims))
    for k, f in enumerate(opt.frequencies):
        if all(not np.any(np.asarray(g)[..., k] != 0) for g in G):
            continue
        tab, cutoff, S_hat = adjoint_time_table(f, float(opt.base.dt), opt.steps, T, opt.adjoint_bandwidth)
        sp = _with_design(opt.adj_spec, opt, rho)
        sp.sources = [copy.copy(s) for s in opt.adj_spec.sources]
        for (m, ci, _, si) in opt._adj_src:
            s = sp.sources[si]
            s.amp = opt.objective_arguments[m].pattern(G[m], ci, k)
            s.table = tab
            s.cutoff = cutoff
        o = OracleSim(sp)
        o.step(opt.steps)
        acc = np.zeros(tuple(dr.dims), dtype=np.complex128)
        for c in range(3):
            acc += fwd[c][..., k] * o.dft(opt._adj_design[c])[..., k]
        o.close()
        per[k] = np.real(-(dr.eps_max - dr.eps_min) / S_hat * acc)
    return per.sum(axis=0), per


def fd_gradient(opt, rho, indices, db=1e-3):
    rho = np.asarray(rho, dtype=np.float64)
    out = []
    for idx in indices:
        lo, hi = rho.copy(), rho.copy()
        lo[idx] = max(rho[idx] - db, 0.0)
        hi[idx] = min(rho[idx] + db, 1.0)
        out.append((objective(opt, hi) - objective(opt, lo)) / (hi[idx] - lo[idx]))
    return np.array(out)
