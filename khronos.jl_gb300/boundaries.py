"""Boundary conditions of a simulation side (DataStructures.jl:157-162).

The reference's prepare step (init_boundaries, Boundaries.jl:99-164) zeroes
the PML conductivity on every side whose condition is ``Periodic``,
``Bloch``, ``PECBoundary`` or ``PMCBoundary``; the PML *regions* (which cells
keep CPML state, Chunking.jl:108-138) still follow the ``boundaries``
thicknesses.  A PEC or PMC side is otherwise the zero ghost wall every side
without PML has.  Periodic and Bloch sides also wrap the halo
(_add_periodic_connections!, Chunking.jl:1725-1800): that wrap is not part
of this step loop, and such sides are refused.
"""
from __future__ import annotations

from dataclasses import dataclass


class BoundaryCondition:
    pass


class PECBoundary(BoundaryCondition):
    pass


class PMCBoundary(BoundaryCondition):
    pass


class Periodic(BoundaryCondition):
    pass


@dataclass
class Bloch(BoundaryCondition):
    k: float = 0.0


def effective_pml(boundaries, boundary_conditions):
    """PML thicknesses the σ profiles are computed with: zero on the sides
    whose condition is Periodic, Bloch, PEC or PMC (Boundaries.jl:101-110).
    Raises NotImplementedError for Periodic / Bloch sides (no halo wrap)."""
    if boundaries is None:
        return None
    eff = [list(map(float, b)) for b in boundaries]
    if boundary_conditions is None:
        return eff
    for axis, bcs in enumerate(boundary_conditions):
        for side, bc in enumerate(bcs):
            if isinstance(bc, (Periodic, Bloch)):
                raise NotImplementedError(
                    "periodic and Bloch boundaries wrap the halo every half-step; this step loop "
                    "has zero ghost walls only")
            if isinstance(bc, (PECBoundary, PMCBoundary)):
                eff[axis][side] = 0.0
    return eff
