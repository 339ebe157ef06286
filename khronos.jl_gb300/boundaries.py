"""Boundary conditions of a simulation side (DataStructures.jl:157-162).

The reference's prepare step (init_boundaries, Boundaries.jl:99-164) zeroes
the PML conductivity on every side whose condition is ``Periodic``,
``Bloch``, ``PECBoundary`` or ``PMCBoundary``; the PML *regions* (which cells
keep CPML state, Chunking.jl:108-138) still follow the ``boundaries``
thicknesses.  A PEC or PMC side is otherwise the zero ghost wall every side
without PML has.  An axis whose two sides are both Periodic or Bloch also
wraps its halo after every half-step (_add_periodic_connections!,
Chunking.jl:1725-1800): ``periodic_mask`` gives those axes to the step loop.
A Bloch phase k·L ≠ 0 needs complex fields (Chunking.jl:1058) and is refused.

With more than one chunk the reference connects only the first and the last
chunk by position along the axis (Chunking.jl:1770-1798), which for the
PML-grid plan of a periodic axis (all chunks at the same coordinate) joins
two slabs of different regions and leaves the others unwrapped.  This single
domain wraps every cell of the face, as the reference's single-chunk plan does.
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
    whose condition is Periodic, Bloch, PEC or PMC (Boundaries.jl:101-110)."""
    if boundaries is None:
        return None
    eff = [list(map(float, b)) for b in boundaries]
    if boundary_conditions is None:
        return eff
    for axis, bcs in enumerate(boundary_conditions):
        for side, bc in enumerate(bcs):
            if isinstance(bc, (Periodic, Bloch, PECBoundary, PMCBoundary)):
                eff[axis][side] = 0.0
    return eff


def periodic_mask(boundary_conditions) -> int:
    """Bit a set when both sides of axis a are Periodic or Bloch, the axes
    _add_periodic_connections! wraps (Chunking.jl:1729-1733).  Raises
    NotImplementedError for a Bloch k ≠ 0 on such an axis: its phase
    exp(±i·k·L) needs complex fields."""
    if boundary_conditions is None:
        return 0
    mask = 0
    for axis, bcs in enumerate(boundary_conditions):
        if len(bcs) < 2 or not all(isinstance(bc, (Periodic, Bloch)) for bc in bcs):
            continue
        k = next((bc.k for bc in bcs if isinstance(bc, Bloch)), 0.0)
        if k != 0:
            raise NotImplementedError(
                "a Bloch phase exp(i·k·L) needs complex fields; this step loop keeps real fields "
                "(Periodic, or Bloch with k = 0, is supported)")
        mask |= 1 << axis
    return mask
