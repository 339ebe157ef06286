"""Host-side grid arithmetic of a Khronos simulation.

These functions restate the set-up arithmetic that the reference performs on
the host before any kernel runs, with the same operation order and the same
Julia type promotion (the run's number type ``T`` is ``numpy.float32`` or
``numpy.float64``; Julia promotes ``T op Float64`` to ``Float64`` and
``Int op T`` to ``T``):

* grid size, spacing and time step   src/DataStructures.jl:714-742
* Yee shifts and component origins   src/utils.jl:133-170
* GridVolume and grid indices        src/utils.jl:98-211
* source/monitor interpolation       src/utils.jl:480-541
* PML conductivity profile           src/Boundaries.jl:23-72, 99-164
* PML region widths (chunk plan)     src/Chunking.jl:108-138, 622-738, 907-966

Cells here are 0-based; the reference's 1-based Center index is ``i + 1``.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# Component ids, in the reference's order.
EX, EY, EZ, HX, HY, HZ = range(6)
COMPONENT_NAMES = ("Ex", "Ey", "Ez", "Hx", "Hy", "Hz")
CENTER = 6  # Center() pseudo-component (no Yee shift)

# Extra staggered layer per axis of each component's array
# (get_component_voxel_count, src/utils.jl:26-38).
COMPONENT_EXTRA = {
    EX: (0, 1, 1), EY: (1, 0, 1), EZ: (1, 1, 0),
    HX: (1, 0, 0), HY: (0, 1, 0), HZ: (0, 0, 1),
    CENTER: (0, 0, 0),
}


def is_electric(c: int) -> bool:
    return c in (EX, EY, EZ)


def is_magnetic(c: int) -> bool:
    return c in (HX, HY, HZ)


@dataclass
class Grid:
    """Grid numbers exactly as ``SimulationData`` stores them.

    ``cell_size`` entries are rounded to ``T`` (``N.(cell_size)``), ``N`` is
    ``floor(cell_size * resolution)``, ``Δ = cell_size / N`` and
    ``Δt = Courant * min(Δ)``, all in ``T`` (DataStructures.jl:719-740).
    """

    T: type
    cell_size: tuple
    cell_center: tuple
    n: tuple
    delta: tuple
    dt: float

    @classmethod
    def build(cls, cell_size, cell_center, resolution, dtype="f64", courant=0.5):
        T = np.float32 if dtype in ("f32", np.float32) else np.float64
        cs = tuple(T(c) for c in cell_size)
        # floor(Int, cell_size[i] * resolution): T * Int -> T
        n = tuple(int(math.floor(float(c * T(resolution)))) for c in cs)
        if any(v <= 0 for v in n):
            raise ValueError("every axis needs at least one cell (3D only)")
        delta = tuple(T(c / T(v)) for c, v in zip(cs, n))
        dt = T(min(delta) * T(courant))
        center = tuple(float(c) for c in cell_center)
        return cls(T=T, cell_size=cs, cell_center=center, n=n, delta=delta, dt=dt)

    # -- Yee geometry (utils.jl:139-170) ---------------------------------
    def yee_shift(self, comp: int):
        dx, dy, dz = (float(d) for d in self.delta)
        return {
            CENTER: (0.0, 0.0, 0.0),
            EX: (0.0, -float(self.delta[1] / self.T(2)), -float(self.delta[2] / self.T(2))),
            EY: (-float(self.delta[0] / self.T(2)), 0.0, -float(self.delta[2] / self.T(2))),
            EZ: (-float(self.delta[0] / self.T(2)), -float(self.delta[1] / self.T(2)), 0.0),
            HX: (-float(self.delta[0] / self.T(2)), 0.0, 0.0),
            HY: (0.0, -float(self.delta[1] / self.T(2)), 0.0),
            HZ: (0.0, 0.0, -float(self.delta[2] / self.T(2))),
        }[comp]

    def component_origin(self, comp: int):
        base = tuple(
            self.cell_center[a] - float(self.cell_size[a] / self.T(2)) + float(self.delta[a] / self.T(2))
            for a in range(3)
        )
        sh = self.yee_shift(comp)
        return tuple(base[a] + sh[a] for a in range(3))

    def component_dims(self, comp: int):
        ex = COMPONENT_EXTRA[comp]
        return tuple(self.n[a] + ex[a] for a in range(3))

    # -- grid indices (utils.jl:176-211) ---------------------------------
    def grid_idx(self, point, comp: int):
        """Fractional 1-based grid index of ``point`` (get_grid_idx)."""
        d = [float(v) for v in self.delta]
        sim_min = [self.cell_center[a] - float(self.cell_size[a]) / 2 for a in range(3)]
        sim_max = [self.cell_center[a] + float(self.cell_size[a]) / 2 for a in range(3)]
        ctc = [float(self.delta[a] / self.T(2)) for a in range(3)]
        sh = self.yee_shift(comp)
        out = []
        for a in range(3):
            lo = sim_min[a] + ctc[a] + sh[a]
            hi = sim_max[a] - ctc[a] - sh[a]
            p = min(point[a], hi)
            p = max(p, lo)
            v = (p - lo) / d[a] + 1
            out.append(0.0 if math.isnan(v) else v)
        return out

    def grid_volume(self, center, size, comp: int) -> "GridVolume":
        """GridVolume(sim, Volume(center, size), component) (utils.jl:103-113)."""
        lo = [center[a] - size[a] / 2 for a in range(3)]
        hi = [center[a] + size[a] / 2 for a in range(3)]
        s = [int(math.floor(v)) for v in self.grid_idx(lo, comp)]
        e = [int(math.ceil(v)) for v in self.grid_idx(hi, comp)]
        dims = [e[a] - s[a] + 1 for a in range(3)]
        return GridVolume(comp, tuple(s), tuple(e), tuple(dims))


@dataclass(frozen=True)
class GridVolume:
    """1-based inclusive index box of one component (DataStructures.jl:87-94)."""

    component: int
    start_idx: tuple
    end_idx: tuple
    dims: tuple

    @property
    def start0(self):
        """0-based cell of element (1,1,1)."""
        return tuple(v - 1 for v in self.start_idx)


def interpolation_weight(point, min_corner, max_corner, vol_size, delta, ndims=3) -> float:
    """_compute_interpolation_weight_fast (utils.jl:486-541)."""
    weight = 1.0
    for dim in range(ndims):
        p = point[dim]
        lo = min_corner[dim]
        hi = max_corner[dim]
        d = delta[dim]
        sz = vol_size[dim]
        if (p <= (lo - d)) or (p >= (hi + d)):
            return 0.0
        elif sz == 0.0:
            weight *= 1 - min(abs(p - (lo + hi) * 0.5) / d, 1.0)
        elif sz < d:
            if (p >= lo) and (p <= hi):
                weight *= 1 - 0.5 * (1.0 - (p - lo) / d) ** 2 - 0.5 * (1.0 - (hi - p) / d) ** 2
            elif (p <= lo) and (abs(p - lo) < d):
                if hi < (p + d):
                    weight *= 0.5 * (1.0 - (lo - p) / d) ** 2 - 0.5 * (1.0 - (hi - p) / d) ** 2
                else:
                    weight *= 0.5 * (1.0 - (lo - p) / d) ** 2
            elif (p >= hi) and (abs(p - hi) < d):
                if lo > (p - d):
                    weight *= 0.5 * (1.0 - (p - hi) / d) ** 2 - 0.5 * (1.0 - (p - lo) / d) ** 2
                else:
                    weight *= 0.5 * (1.0 - (p - hi) / d) ** 2
        else:
            if (p < lo) and (abs(p - lo) < d):
                weight *= 0.5 * (1.0 - (lo - p) / d) ** 2
            elif (p >= lo) and (abs(p - lo) < d):
                weight *= 1 - 0.5 * (1.0 - (p - lo) / d) ** 2
            elif (p <= hi) and (abs(p - hi) < d):
                weight *= 1 - 0.5 * (1.0 - (hi - p) / d) ** 2
            elif (p > hi) and (abs(p - hi) < d):
                weight *= 0.5 * (1.0 - (p - hi) / d) ** 2
    return weight


# -- PML (Boundaries.jl:23-72) --------------------------------------------
def sigma_helper(idx: int, N: int, dx, dt, length_left, length_right, T):
    """σ at half-cell sample ``idx`` (1-based), already scaled by Δt/2."""
    f64 = np.float64
    dx, dt = T(dx), T(dt)

    def u0(L):
        den = T(T(T(4) * L) * T(1)) / T(3)  # 4 * pml_length * 1 / 3 in T
        return f64(-math.log(1e-15)) / f64(den) * (0.5 * f64(dt))

    def u(x):  # x^2 * 0.5 * (sign(x) + 1)
        return f64(T(x * x)) * 0.5 * f64(T(np.sign(x)) + T(1))

    total_length = T(T(T(N) * dx) / T(2))
    real_idx = T(T(T(idx) * dx) / T(2))
    Ll, Lr = T(length_left), T(length_right)
    if real_idx < Ll:
        return T(u0(Ll) * u(T(T(Ll - real_idx) / Ll)))
    elif T(total_length - real_idx) < Lr:
        return T(u0(Lr) * u(T(T(Lr - T(total_length - real_idx)) / Lr)))
    return T(0)


def compute_sigma(N: int, dx, dt, length_left, length_right, T) -> np.ndarray:
    """compute_sigma: length-N array of half-cell samples (Boundaries.jl:64-72)."""
    sig = np.zeros(N, dtype=T)
    if length_left != 0.0 or length_right != 0.0:
        for idx in range(1, N + 1):
            sig[idx - 1] = sigma_helper(idx, N, dx, dt, length_left, length_right, T)
    return sig


def cell_sigma(grid: Grid, axis: int, length_left, length_right) -> np.ndarray:
    """σ at the cell centres the kernels read: σ[2i-1] (Helpers.jl:276-277)."""
    n = grid.n[axis]
    full = compute_sigma(2 * n + 1, grid.delta[axis], grid.dt, length_left, length_right, grid.T)
    return full[0 : 2 * n : 2].copy()


def pml_widths(grid: Grid, boundaries):
    """Per-axis PML region widths in cells: ceil(L/Δ) (Chunking.jl:121-122, 642-643).

    Returns (lo, hi) tuples.  Reproduces plan_chunks (Chunking.jl:907-966): with
    PML present but no PML-free region left, the reference falls back to one
    chunk whose PML flags cover whole axes; that is encoded as lo = n.
    """
    lo, hi = [0, 0, 0], [0, 0, 0]
    if boundaries is None:
        return tuple(lo), tuple(hi)
    T = grid.T
    for a in range(3):
        Ll, Lr = T(boundaries[a][0]), T(boundaries[a][1])
        if Ll > 0:
            lo[a] = int(math.ceil(float(T(Ll / grid.delta[a]))))
        if Lr > 0:
            hi[a] = int(math.ceil(float(T(Lr / grid.delta[a]))))
    n_regions = 1
    interior_exists = True
    for a in range(3):
        cnt = (1 if lo[a] >= 1 else 0) + (1 if hi[a] >= 1 else 0)
        inner = grid.n[a] - lo[a] - hi[a] >= 1
        cnt += 1 if inner else 0
        if cnt == 0:
            cnt = 1
        n_regions *= cnt
        interior_exists &= inner
    if n_regions > 1 and not interior_exists:
        # single-chunk fallback: flags from overlap with the whole domain
        for a in range(3):
            if lo[a] > 0 or hi[a] > 0:
                lo[a], hi[a] = grid.n[a], 0
    return tuple(lo), tuple(hi)
