"""Geometry objects whose ε⁻¹ the device rasterises (kh_sim_set_geometry).

Mirrors the reference's ``Object(shape, Material(ε = …))`` with the
GeometryPrimitives shapes it paints (``Ball``, ``Cuboid``, ``Cylinder``;
src/Geometry.jl:156-250) and its ``subpixel_smoothing`` modes
(``NoSmoothing``, ``VolumeAveraging``, ``AnisotropicSmoothing``,
src/Geometry.jl:795-990).  Only isotropic non-dispersive permittivity is
rasterised on the device; other material data keep using per-voxel arrays.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Sequence

SHAPE_BALL, SHAPE_CUBOID, SHAPE_CYLINDER = range(3)
SMOOTHING = {"none": 0, "volume": 1, "anisotropic": 2}


@dataclass
class Ball:
    center: Sequence[float]
    radius: float

    def raw(self):
        return SHAPE_BALL, 0, tuple(map(float, self.center)), (float(self.radius), 0.0, 0.0)


@dataclass
class Cuboid:
    """Axis-aligned box."""

    center: Sequence[float]
    size: Sequence[float]

    def raw(self):
        return SHAPE_CUBOID, 0, tuple(map(float, self.center)), tuple(map(float, self.size))


@dataclass
class Cylinder:
    """Axis-aligned cylinder (axis 0, 1, 2 = x, y, z)."""

    center: Sequence[float]
    radius: float
    height: float
    axis: int = 2

    def raw(self):
        return SHAPE_CYLINDER, int(self.axis), tuple(map(float, self.center)), (float(self.radius),
                                                                               float(self.height), 0.0)


@dataclass
class Material:
    """Material(ε, μ, σD, σB, χ3, susceptibilities) of an object (isotropic
    scalars; ε is ε∞ when poles are given).  ε is rasterised on the device
    with optional subpixel smoothing; μ, σD, σB and χ3 on the host
    (``material_arrays``), unsmoothed, as the reference rasterises them
    (Geometry.jl:223-250, 610-636); poles through ``pole_arrays``."""

    eps: float = 1.0
    mu: float = 1.0
    sigma_d: float = 0.0
    sigma_b: float = 0.0
    chi3: float = 0.0
    susceptibilities: tuple = ()  # LorentzianSusceptibility / DrudeSusceptibility poles


@dataclass
class Object:
    shape: object
    material: Material


@dataclass
class GeometrySpec:
    """What kh_sim_set_geometry receives: raw objects (shape, axis, center,
    size, ε), the background ε, the centre of cell (0,0,0) and the mode."""

    objects: List[tuple]
    background: float
    origin: tuple
    smoothing: int


def geometry_spec(objects: Sequence[Object], grid, background: float = 1.0, smoothing: str = "none") -> GeometrySpec:
    from .grid import CENTER

    if smoothing not in SMOOTHING:
        raise ValueError(f"smoothing must be one of {sorted(SMOOTHING)}")
    raw = []
    for o in objects:
        shape, axis, c, s = o.shape.raw()
        raw.append((shape, axis, c, s, float(o.material.eps)))
    return GeometrySpec(raw, float(background), tuple(grid.component_origin(CENTER)), SMOOTHING[smoothing])


def _component_axes(grid, comp: int):
    """Sample coordinates of a component along x, y, z: the centre of cell
    (0,0,0) moved by the component's Yee shift, plus i·Δ (the device's
    arithmetic for ε)."""
    import numpy as np

    from .grid import CENTER

    base = grid.component_origin(CENTER)
    sh = grid.yee_shift(comp)
    d = [float(v) for v in grid.delta]
    return [(base[a] + sh[a]) + np.arange(grid.n[a], dtype=np.float64) * d[a] for a in range(3)]


def _inside_mask(raw, axes):
    """Inclusive inside test of one raw object over the sample lattice
    (the device predicate, same operation order, no fused multiply-add)."""
    import numpy as np

    shape, axis, c, s = raw[:4]
    X = [axes[a].reshape([-1 if b == a else 1 for b in range(3)]) - c[a] for a in range(3)]
    if shape == SHAPE_BALL:
        return np.sqrt(X[0] * X[0] + X[1] * X[1] + X[2] * X[2]) <= s[0]
    if shape == SHAPE_CUBOID:
        m = np.ones(tuple(len(x) for x in axes), dtype=bool)
        for a in range(3):
            m &= np.abs(X[a]) <= 0.5 * s[a]
        return m
    a1, a2 = (axis + 1) % 3, (axis + 2) % 3
    return (np.sqrt(X[a1] * X[a1] + X[a2] * X[a2]) <= s[0]) & (np.abs(X[axis]) <= 0.5 * s[1])


def rasterize_values(objects: Sequence[Object], grid, comp: int, values: Sequence[float], background: float):
    """One value per object painted at component ``comp``'s Yee positions:
    the first object that contains a point sets it (objects painted in
    reverse order, Geometry.jl:223-250), ``background`` elsewhere.  Returns
    an [i, j, k] array, x fastest in memory."""
    import numpy as np

    axes = _component_axes(grid, comp)
    out = np.full(tuple(grid.n), float(background), dtype=np.float64, order="F")
    for o, v in reversed(list(zip(objects, values))):
        out[_inside_mask(o.shape.raw(), axes)] = float(v)
    return out


def material_arrays(objects: Sequence[Object], grid):
    """Per-voxel μ⁻¹, σD, σB and χ3 arrays of the objects, each only when some
    object departs from free space (the reference allocates them on the same
    condition, needs_perm / needs_conductivities, Geometry.jl:314-351):
    list of (kind, component, array) in the SimSpec materials format.
    μ⁻¹ and σB sample the H components' positions, σD the E components', χ3
    the cell centres.  Dispersive susceptibilities of objects are not
    rasterised (give poles as arrays)."""
    from .grid import CENTER, EX, HX
    from .spec import MAT_CHI3, MAT_MU_INV, MAT_SIGMA_B, MAT_SIGMA_D

    out = []
    mats = [o.material for o in objects]
    if any(m.mu != 1.0 for m in mats):
        for c in range(3):
            out.append((MAT_MU_INV, c, rasterize_values(objects, grid, HX + c, [1.0 / m.mu for m in mats], 1.0)))
    if any(m.sigma_d != 0.0 for m in mats):
        for c in range(3):
            out.append((MAT_SIGMA_D, c, rasterize_values(objects, grid, EX + c, [m.sigma_d for m in mats], 0.0)))
    if any(m.sigma_b != 0.0 for m in mats):
        for c in range(3):
            out.append((MAT_SIGMA_B, c, rasterize_values(objects, grid, HX + c, [m.sigma_b for m in mats], 0.0)))
    if any(m.chi3 != 0.0 for m in mats):
        out.append((MAT_CHI3, 0, rasterize_values(objects, grid, CENTER, [m.chi3 for m in mats], 0.0)))
    return out


def pole_arrays(objects: Sequence[Object], grid, boundaries):
    """init_polarization! (Geometry.jl:1059-1250): one σ array per distinct
    pole (keyed by (ω0, γ), in the order first met), sampled at the Ex
    positions and shared by the three components.  Each pole's array is
    painted by the objects that carry that pole, in reverse order (so an
    earlier object without the pole does not clear it, as in the
    reference), then zeroed at points inside a PML slab by physical
    coordinate.  Returns [(susceptibility, σ array)]."""
    import numpy as np

    from .grid import EX

    poles, seen = [], set()
    for o in objects:
        for sus in o.material.susceptibilities:
            key = (float(sus.omega_0), float(sus.gamma))
            if key not in seen:
                seen.add(key)
                poles.append(sus)
    if not poles:
        return []
    axes = _component_axes(grid, EX)
    out = []
    for pole in poles:
        key = (float(pole.omega_0), float(pole.gamma))
        sig = np.zeros(tuple(grid.n), dtype=np.float64, order="F")
        for o in reversed(list(objects)):
            val = next((float(x.sigma) for x in o.material.susceptibilities
                        if (float(x.omega_0), float(x.gamma)) == key), None)
            if val is not None:
                sig[_inside_mask(o.shape.raw(), axes)] = val
        if boundaries is not None:
            pml = np.zeros(tuple(grid.n), dtype=bool)
            for a in range(3):
                lo = grid.cell_center[a] - float(grid.cell_size[a]) / 2
                hi = grid.cell_center[a] + float(grid.cell_size[a]) / 2
                left, right = float(boundaries[a][0]), float(boundaries[a][1])
                m = np.zeros(grid.n[a], dtype=bool)
                if left > 0:
                    m |= axes[a] < lo + left
                if right > 0:
                    m |= axes[a] > hi - right
                pml |= m.reshape([-1 if b == a else 1 for b in range(3)])
            sig[pml] = 0.0
        out.append((pole, sig))
    return out
