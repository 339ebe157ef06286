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
    eps: float = 1.0


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
