"""A small inverse-design case shared by the adjoint tests.

36×30×24 cells (2.4 × 2.0 × 1.6 µm at 15 cells/µm) with a 6-cell CPML,
background ε = 2, a 6×6×5-voxel design box with ρ ~ U(0, 1) and ε ∈ [2, 6],
(``small=True``: 24×20×16 cells at 10 cells/µm, 4-cell CPML, 4×4×3 voxels)
an Ez Gaussian-pulse point source, and an x-normal objective plane of Ex, Ey,
Ez with seeded random complex weights; J = Σ_f |Y_f|².  Everything sits
outside the CPML, as the adjoint method requires.
"""
import numpy as np

FCEN = 1 / 1.55
LAYOUTS = {
    # resolution: (design start, design dims, plane start, plane dims)
    15: ((15, 12, 9), (6, 6, 5), (26, 8, 6), (1, 14, 12)),
    10: ((10, 8, 6), (4, 4, 3), (17, 5, 4), (1, 10, 8)),
}


def make_problem(dtype="f64", steps=3000, nfreq=3, lib=None, seed=3, small=False, mode="time"):
    from khronos_gb300 import grid as G
    from khronos_gb300.adjoint import DesignRegion, FieldOverlap, OptimizationProblem, power_overlap
    from khronos_gb300.simulation import Simulation
    from khronos_gb300.sources import GaussianPulseSource, UniformSource

    res = 10 if small else 15
    DESIGN_START, DESIGN_DIMS, PLANE_START, PLANE_DIMS = LAYOUTS[res]
    rng = np.random.default_rng(seed)
    rho0 = rng.uniform(0, 1, size=DESIGN_DIMS)
    freqs = list(np.linspace(0.9 * FCEN, 1.1 * FCEN, nfreq)) if nfreq > 1 else [FCEN]
    weights = [rng.normal(size=PLANE_DIMS + (nfreq,)) + 1j * rng.normal(size=PLANE_DIMS + (nfreq,))
               for _ in range(3)]
    size = (2.4, 2.0, 1.6)
    g = G.Grid.build(size, (0, 0, 0), res, dtype)
    eps = np.full(g.n, 2.0)
    sl = tuple(slice(DESIGN_START[a], DESIGN_START[a] + DESIGN_DIMS[a]) for a in range(3))
    eps[sl] = 2.0 + rho0 * 4.0
    einv = 1.0 / eps
    src = UniformSource(time_profile=GaussianPulseSource(fcen=FCEN, fwidth=0.3 * FCEN),
                        component=G.EZ, center=(-0.6, 0.05, 0.0), size=(0, 0, 0))
    sim = Simulation(cell_size=size, resolution=res, sources=[src], boundaries=[[0.4, 0.4]] * 3,
                     dtype=dtype, eps_inv=[einv, einv, einv])
    spec = sim.spec()
    oq = FieldOverlap(components=[G.EX, G.EY, G.EZ], starts=[PLANE_START] * 3, dims=[PLANE_DIMS] * 3,
                      weights=weights)
    dr = DesignRegion(DESIGN_START, DESIGN_DIMS, 2.0, 6.0)
    opt = OptimizationProblem(spec, power_overlap, [oq], dr, freqs, steps, mode=mode, lib=lib)
    return opt, rho0
