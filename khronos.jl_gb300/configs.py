"""Synthetic workloads with the shapes of the benchmark configurations.

All inputs are synthetic and seeded (no dataset exists for these runs):

* ``dipole``     — 64³ vacuum, 10-cell CPML, Ez point dipole, x-normal flux
                   plane at 3 frequencies, 1000 steps (FP32 and FP64).
* ``waveguide``  — 320×192×128, 12-cell CPML, Si strip (ε 12.25) in ε 2.085
                   cladding through a 2×2×0.22 µm random design region
                   (ρ ~ U(0,1), seed 1234, 3-cell box filter), Ey current plane
                   with a 0.4 µm Gaussian profile, two 21-frequency flux planes,
                   4000 steps.
* ``dispersive`` — 256³, 12-cell CPML, ε 2.25 slab with χ3 = 1e-3, 4 Lorentz +
                   4 Drude spheres (seed 42), Ez plane source, 6-face box flux at
                   11 frequencies, 3000 steps.
* ``serving_stream`` — request stream (seed 2024): grids from {64³, 96³, 128³,
                   160×160×96, 256×128×64} with a 10-cell CPML, 1–20 spheres,
                   Ez dipole, 5-frequency flux plane, U(500, 4000) steps,
                   Poisson arrivals.

``scale`` shrinks the cell counts (same physical layout, coarser or smaller
grid) so the CPU oracle can run the same layout in seconds.

Shapes are rasterised by sampling each Yee component at its own position
(first object wins), which is how the reference samples material points
(src/Geometry.jl:241-248, 353-366), without subpixel smoothing.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List

import numpy as np

from . import grid as G
from .monitors import FluxMonitor
from .simulation import Simulation, apply_chi1_correction
from .sources import GaussianPulseSource, ProfileSource, UniformSource
from .spec import DrudeSusceptibility, LorentzianSusceptibility

FCEN = 1 / 1.55


@dataclass
class Workload:
    name: str
    sim: Simulation
    steps: int
    flux_monitors: List[FluxMonitor] = field(default_factory=list)
    description: str = ""


def yee_coords(g: G.Grid, comp: int):
    """Physical coordinates of component ``comp`` at cells 0..n-1 per axis."""
    o = g.component_origin(comp)
    return [o[a] + np.arange(g.n[a]) * float(g.delta[a]) for a in range(3)]


def _box_mask(xs, ys, zs, center, size):
    mx = np.abs(xs - center[0]) <= size[0] / 2
    my = np.abs(ys - center[1]) <= size[1] / 2
    mz = np.abs(zs - center[2]) <= size[2] / 2
    return mx[:, None, None] & my[None, :, None] & mz[None, None, :]


def _sphere_mask(xs, ys, zs, c, r):
    d2 = (xs[:, None, None] - c[0]) ** 2 + (ys[None, :, None] - c[1]) ** 2 + (zs[None, None, :] - c[2]) ** 2
    return d2 <= r * r


def _freqs(n, lo, hi):
    return list(np.linspace(lo, hi, n)) if n > 1 else [0.5 * (lo + hi)]


def dipole(dtype="f32", steps=1000, resolution=20, size=3.2, pml=0.5) -> Workload:
    src = UniformSource(time_profile=GaussianPulseSource(fcen=FCEN, fwidth=0.2 * FCEN),
                        component=G.EZ, center=(0.0, 0.0, 0.0), size=(0.0, 0.0, 0.0))
    inner = size - 2 * pml
    fm = FluxMonitor(center=(0.8 * size / 3.2, 0.0, 0.0), size=(0.0, 0.9 * inner, 0.9 * inner),
                     frequencies=[0.9 * FCEN, FCEN, 1.1 * FCEN])
    sim = Simulation(cell_size=(size, size, size), resolution=resolution, sources=[src],
                     boundaries=[[pml, pml]] * 3, monitors=[fm], dtype=dtype)
    return Workload("dipole", sim, steps, [fm],
                    f"{sim.n[0]}x{sim.n[1]}x{sim.n[2]} vacuum, PML {pml} um, Ez point dipole")


def waveguide(dtype="f32", steps=4000, scale=1.0, seed=1234) -> Workload:
    res = 25 * scale
    size = (12.8, 7.68, 5.12)
    pml = 12 / 25
    sim_probe = G.Grid.build(size, (0, 0, 0), res, dtype)
    g = sim_probe
    # ε per component: cladding, Si strip along x, random design region
    eps = []
    rng = np.random.default_rng(seed)
    design_c, design_s = (0.0, 0.0, 0.0), (2.0, 2.0, 0.22)
    # design density on the cell grid, 3-cell box filter with clamped edges
    xs_c, ys_c, zs_c = yee_coords(g, G.CENTER)
    rho = rng.uniform(0.0, 1.0, size=g.n)
    pad = np.pad(rho, 1, mode="edge")
    filt = np.zeros_like(rho)
    for dx in range(3):
        for dy in range(3):
            for dz in range(3):
                filt += pad[dx:dx + g.n[0], dy:dy + g.n[1], dz:dz + g.n[2]]
    filt /= 27.0
    for comp in (G.EX, G.EY, G.EZ):
        xs, ys, zs = yee_coords(g, comp)
        e = np.full(g.n, 2.085)
        strip = _box_mask(xs, ys, zs, (0.0, 0.0, 0.0), (1e9, 0.5, 0.22))
        e[strip] = 12.25
        dm = _box_mask(xs, ys, zs, design_c, design_s)
        e[dm] = 2.085 + filt[dm] * (12.25 - 2.085)
        eps.append(1.0 / e)
    inner_y = size[1] - 2 * pml
    inner_z = size[2] - 2 * pml
    src = ProfileSource(time_profile=GaussianPulseSource(fcen=FCEN, fwidth=0.25 * FCEN),
                        component=G.EY, center=(-5.0, 0.0, 0.0), size=(0.0, 0.9 * inner_y, 0.9 * inner_z),
                        profile_func=lambda x, y, z: math.exp(-((y ** 2 + z ** 2) / 0.4 ** 2)))
    fw = 0.25 * FCEN
    freqs = _freqs(21, FCEN - 0.5 * fw, FCEN + 0.5 * fw)
    fms = [FluxMonitor(center=(xp, 0.0, 0.0), size=(0.0, 0.9 * inner_y, 0.9 * inner_z), frequencies=freqs)
           for xp in (-4.0, 4.0)]
    sim = Simulation(cell_size=size, resolution=res, sources=[src], boundaries=[[pml, pml]] * 3,
                     monitors=fms, dtype=dtype, eps_inv=eps)
    return Workload("waveguide", sim, steps, fms,
                    f"{sim.n[0]}x{sim.n[1]}x{sim.n[2]} Si strip + random design, PML 12 cells")


def dispersive(dtype="f32", steps=3000, scale=1.0, seed=42) -> Workload:
    res = 20 * scale
    L = 12.8
    pml = 12 / 20
    g = G.Grid.build((L, L, L), (0, 0, 0), res, dtype)
    rng = np.random.default_rng(seed)
    lo_int = -L / 2 + pml + 0.2
    spheres = []
    for s in range(8):
        r = rng.uniform(0.2, 0.6)
        c = tuple(rng.uniform(lo_int + r, -lo_int - r) for _ in range(3))
        spheres.append((c, r, "lorentz" if s < 4 else "drude"))
    lor = LorentzianSusceptibility(1.0, 0.05, 1.0)
    dru = DrudeSusceptibility(0.1, (2 * math.pi * 5.0) ** 2 / (2 * math.pi * 0.1))
    eps_c, chi3 = [], None
    sig_l = np.zeros(g.n)
    sig_d = np.zeros(g.n)
    xs, ys, zs = yee_coords(g, G.EX)  # pole σ on Ex positions, shared by x/y/z (Geometry.jl:1146-1177)
    for (c, r, kind) in spheres:
        m = _sphere_mask(xs, ys, zs, c, r)
        if kind == "lorentz":
            sig_l[m & (sig_d == 0)] = lor.sigma
        else:
            sig_d[m & (sig_l == 0)] = dru.sigma
    for comp in (G.EX, G.EY, G.EZ):
        cx, cy, cz = yee_coords(g, comp)
        e = np.ones(g.n)
        slab = (np.abs(cz) <= 1.0)[None, None, :] & np.ones(g.n, dtype=bool)
        e[slab] = 2.25
        for (c, r, kind) in reversed(spheres):  # first object wins
            e[_sphere_mask(cx, cy, cz, c, r)] = 2.0 if kind == "lorentz" else 1.0
        eps_c.append(1.0 / e)
    xc, yc, zc = yee_coords(g, G.CENTER)
    chi3 = np.zeros(g.n)
    chi3[:, :, np.abs(zc) <= 1.0] = 1e-3
    for (c, r, kind) in spheres:
        chi3[_sphere_mask(xc, yc, zc, c, r)] = 0.0
    poles = [(lor, sig_l), (dru, sig_d)]
    eps_c = apply_chi1_correction(eps_c, poles, g.dt, T=np.float64)
    inner = L - 2 * pml
    src = UniformSource(time_profile=GaussianPulseSource(fcen=FCEN, fwidth=0.2 * FCEN), component=G.EZ,
                        center=(-5.0 * L / 12.8, 0.0, 0.0), size=(0.0, inner, inner))
    freqs = _freqs(11, 0.8 * FCEN, 1.2 * FCEN)
    h = 4.5 * L / 12.8
    fms = []
    for a in range(3):
        for sgn in (-1, 1):
            c = [0.0, 0.0, 0.0]
            c[a] = sgn * h
            sz = [2 * h, 2 * h, 2 * h]
            sz[a] = 0.0
            fms.append(FluxMonitor(center=tuple(c), size=tuple(sz), frequencies=freqs))
    sim = Simulation(cell_size=(L, L, L), resolution=res, sources=[src], boundaries=[[pml, pml]] * 3,
                     monitors=fms, dtype=dtype, eps_inv=eps_c, chi3=chi3, poles=poles)
    return Workload("dispersive", sim, steps, fms,
                    f"{sim.n[0]}^3, chi3 slab, 4 Lorentz + 4 Drude spheres, PML 12 cells")


def photonic_slab(dtype="f32", steps=3000, scale=1.0) -> Workload:
    """Periodic along x and y (no PML there), 12-cell CPML along z: a silicon
    slab (ε 12.25, 0.22 µm thick) with a square lattice of air holes (period
    0.4 µm, radius 0.12 µm) in a 6.4 × 6.4 µm supercell, an Ex current plane
    1 µm below it spanning the cell (a normal-incidence plane wave), flux
    planes below and above at 21 frequencies.  256×256×128 at 40 cells/µm;
    the periodic set-up of the reference's slab examples at benchmark size,
    with the wrap of both periodic axes after every half-step."""
    from .boundaries import Periodic

    res = 40 * scale
    size = (6.4, 6.4, 3.2)
    pml = 12 / 40
    g = G.Grid.build(size, (0, 0, 0), res, dtype)
    a, r = 0.4, 0.12
    eps = []
    for comp in (G.EX, G.EY, G.EZ):
        xs, ys, zs = yee_coords(g, comp)
        dx = np.mod(xs + a / 2, a) - a / 2
        dy = np.mod(ys + a / 2, a) - a / 2
        hole = (dx[:, None] ** 2 + dy[None, :] ** 2 < r * r)[:, :, None]
        slab = (np.abs(zs) <= 0.11)[None, None, :]
        e = np.where(slab & ~hole, 12.25, 1.0)
        eps.append(1.0 / e)
    src = UniformSource(time_profile=GaussianPulseSource(fcen=FCEN, fwidth=0.25 * FCEN), component=G.EX,
                        center=(0.0, 0.0, -1.0), size=(math.inf, math.inf, 0.0))
    fw = 0.25 * FCEN
    freqs = _freqs(21, FCEN - 0.5 * fw, FCEN + 0.5 * fw)
    # flux planes just inside the periodic span (a full-span plane would read
    # the staggered layer on the wrap faces)
    fms = [FluxMonitor(center=(0.0, 0.0, zp), size=(0.98 * size[0], 0.98 * size[1], 0.0), frequencies=freqs)
           for zp in (-1.2, 1.0)]
    sim = Simulation(cell_size=size, resolution=res, sources=[src], boundaries=[[0.0, 0.0], [0.0, 0.0], [pml, pml]],
                     boundary_conditions=[[Periodic(), Periodic()], [Periodic(), Periodic()], [None, None]],
                     monitors=fms, dtype=dtype, eps_inv=eps)
    return Workload("periodic", sim, steps, fms,
                    f"{sim.n[0]}x{sim.n[1]}x{sim.n[2]} photonic-crystal slab, periodic x/y, PML 12 cells in z")


@dataclass
class BendWorkload:
    """Inverse-design workload: forward and straight-reference simulations,
    the design box and the output plane (see ``bend``)."""

    sim: Simulation                 # the bend with the initial design
    straight: Simulation            # straight strip along +y (E_ref run)
    design_start: tuple
    design_dims: tuple
    rho0: np.ndarray                # initial density over the design box
    eps_min: float
    eps_max: float
    plane: list                     # [(component, start, dims)] of Ex, Ey, Ez on the output plane
    frequencies: list
    steps: int
    description: str = ""


def bend(dtype="f32", steps=6000, scale=1.0, seed=7) -> BendWorkload:
    """3-D waveguide-bend inverse design: 400×400×128 cells at 25 cells/µm
    (16 × 16 × 5.12 µm) with a 12-cell CPML, ε = 2.085 cladding.  Input strip
    along +x and output strip along +y (ε 12.25, 0.5 × 0.22 µm) meet a centred
    120×120×22-voxel design box (4.8 × 4.8 × 0.88 µm) with ρ ~ U(0, 1) (seed 7)
    and ε = 2.085 + ρ·(12.25 − 2.085) on all three components of each voxel.
    Source: Ey current plane at x = −6 µm with a Gaussian transverse profile
    (waist 0.4 µm), Gaussian pulse fcen = 1/1.55, fwidth = 0.25·fcen.
    Objective plane: y = +6 µm, 2 × 1.2 µm across the output strip, Ex/Ey/Ez at
    5 frequencies fcen·(0.9 … 1.1).  The straight run (strip along +y, Ex
    plane source at y = −6 µm) gives E_ref on the same plane.  ``scale``
    shrinks the resolution (same physical layout)."""
    res = 25 * scale
    L, H = 16.0, 5.12
    pml = 12 / 25
    e_clad, e_core = 2.085, 12.25
    g = G.Grid.build((L, L, H), (0, 0, 0), res, dtype)
    di = max(2, int(round(120 * scale)))
    dk = max(2, int(round(22 * scale)))
    dstart = tuple((g.n[a] - d) // 2 for a, d in enumerate((di, di, dk)))
    ddims = (di, di, dk)
    rng = np.random.default_rng(seed)
    rho0 = rng.uniform(0.0, 1.0, size=ddims)

    def eps_arrays(kind: str):
        out = []
        for comp in (G.EX, G.EY, G.EZ):
            xs, ys, zs = yee_coords(g, comp)
            e = np.full(g.n, e_clad)
            if kind == "bend":
                inp = _box_mask(xs, ys, zs, (-L / 4, 0.0, 0.0), (L / 2, 0.5, 0.22))
                outp = _box_mask(xs, ys, zs, (0.0, L / 4, 0.0), (0.5, L / 2, 0.22))
                e[inp | outp] = e_core
                sl = tuple(slice(dstart[a], dstart[a] + ddims[a]) for a in range(3))
                e[sl] = e_clad + rho0 * (e_core - e_clad)
            else:
                e[_box_mask(xs, ys, zs, (0.0, 0.0, 0.0), (0.5, 1e9, 0.22))] = e_core
            out.append(1.0 / e)
        return out

    fw = 0.25 * FCEN
    prof = lambda x, y, z: math.exp(-((y ** 2 + z ** 2) / 0.4 ** 2))
    src = ProfileSource(time_profile=GaussianPulseSource(fcen=FCEN, fwidth=fw), component=G.EY,
                        center=(-6.0, 0.0, 0.0), size=(0.0, 2.0, 1.2), profile_func=prof)
    prof_s = lambda x, y, z: math.exp(-((x ** 2 + z ** 2) / 0.4 ** 2))
    src_s = ProfileSource(time_profile=GaussianPulseSource(fcen=FCEN, fwidth=fw), component=G.EX,
                          center=(0.0, -6.0, 0.0), size=(2.0, 0.0, 1.2), profile_func=prof_s)
    kw = dict(cell_size=(L, L, H), resolution=res, boundaries=[[pml, pml]] * 3, dtype=dtype)
    sim = Simulation(sources=[src], eps_inv=eps_arrays("bend"), **kw)
    straight = Simulation(sources=[src_s], eps_inv=eps_arrays("straight"), **kw)
    plane = []
    for comp in (G.EX, G.EY, G.EZ):
        gv = g.grid_volume((0.0, 6.0, 0.0), (2.0, 0.0, 1.2), comp)
        plane.append((comp, gv.start0, gv.dims))
    freqs = list(np.linspace(0.9 * FCEN, 1.1 * FCEN, 5))
    return BendWorkload(sim, straight, dstart, ddims, rho0, e_clad, e_core, plane, freqs, steps,
                        f"{g.n[0]}x{g.n[1]}x{g.n[2]} bend, design {di}x{di}x{dk}, PML 12 cells")


SERVING_GRIDS = [(64, 64, 64), (96, 96, 96), (128, 128, 128), (160, 160, 96), (256, 128, 64)]


@dataclass
class ServingRequest:
    index: int
    grid: tuple
    steps: int
    arrival_unit: float   # arrival time in units of the mean inter-arrival time
    work: int             # cell-updates
    make: object = None   # () -> Workload (built on demand)


def serving_request(index: int, grid, steps: int, seed: int, dtype="f32") -> Workload:
    """One request of the serving stream: `grid` cells at 20 cells/µm with a
    10-cell CPML, 1–20 dielectric spheres (ε ~ U(2, 12), radius 3–15 cells,
    centres inside the CPML-free region; the first sphere wins where they
    overlap) rasterised on the device at each component's Yee position, an Ez
    Gaussian-pulse dipole at a random interior point and one x-normal
    5-frequency flux plane."""
    from .geometry import Ball, Material, Object

    res = 20
    pml = 10 / res
    size = tuple(n / res for n in grid)
    rng = np.random.default_rng(seed)
    nsph = int(rng.integers(1, 21))
    lo = [int(res * pml)] * 3
    hi = [grid[a] - lo[a] for a in range(3)]
    objs = []
    for _ in range(nsph):
        r = float(rng.uniform(3, 15))
        c = [float(rng.uniform(lo[a], hi[a])) for a in range(3)]
        e = float(rng.uniform(2, 12))
        centre = tuple(c[a] / res - size[a] / 2 for a in range(3))  # cell units -> µm (cell_center 0)
        objs.append(Object(Ball(centre, r / res), Material(e)))
    margin = 2
    pos = [float(rng.uniform(lo[a] + margin, hi[a] - margin)) / res - size[a] / 2 for a in range(3)]
    src = UniformSource(time_profile=GaussianPulseSource(fcen=FCEN, fwidth=0.2 * FCEN), component=G.EZ,
                        center=tuple(pos), size=(0.0, 0.0, 0.0))
    inner = [size[a] - 2 * pml for a in range(3)]
    fm = FluxMonitor(center=(0.3 * inner[0], 0.0, 0.0), size=(0.0, 0.9 * inner[1], 0.9 * inner[2]),
                     frequencies=_freqs(5, 0.8 * FCEN, 1.2 * FCEN))
    sim = Simulation(cell_size=size, resolution=res, sources=[src], boundaries=[[pml, pml]] * 3,
                     monitors=[fm], dtype=dtype, geometry=objs, background_eps=1.0)
    assert tuple(sim.n) == tuple(grid), (sim.n, grid)
    return Workload(f"serve{index}", sim, steps, [fm],
                    f"{grid[0]}x{grid[1]}x{grid[2]}, {nsph} spheres, Ez dipole, {steps} steps")


def serving_stream(n_requests: int = 512, seed: int = 2024, dtype="f32") -> List[ServingRequest]:
    """The request stream: grids uniformly from SERVING_GRIDS, steps
    ~ U(500, 4000), Poisson arrivals (exponential gaps of unit mean; scale by
    the chosen mean inter-arrival time)."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for i in range(n_requests):
        grid = SERVING_GRIDS[int(rng.integers(0, len(SERVING_GRIDS)))]
        steps = int(rng.integers(500, 4001))
        t += float(rng.exponential(1.0))
        sub_seed = int(rng.integers(0, 2 ** 31 - 1))
        cells = grid[0] * grid[1] * grid[2]
        out.append(ServingRequest(i, grid, steps, t, cells * steps,
                                  make=(lambda i=i, g=grid, n=steps, s=sub_seed: serving_request(i, g, n, s, dtype))))
    return out


BUILDERS = {"dipole": dipole, "waveguide": waveguide, "dispersive": dispersive, "periodic": photonic_slab}
