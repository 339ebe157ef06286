"""SimSpec: the host-side description one C-ABI simulation is created from.

``Simulation.spec()`` produces it from user-level objects, restating what
``prepare_simulation!`` (src/Simulation.jl:92-283) computes on the host:
PML σ samples and region widths, source amplitude arrays, monitor boxes with
auto-decimation, ADE coefficients.  Arrays are numpy, cell-indexed a[i, j, k]
(x fastest when flattened with order='F'), values in float64 already rounded to
the run's precision where the reference stores them in that precision.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence, Tuple

import numpy as np

KH_F32, KH_F64 = 0, 1
MAT_EPS_INV, MAT_MU_INV, MAT_SIGMA_D, MAT_SIGMA_B, MAT_CHI3 = range(5)
TIME_GAUSSIAN, TIME_CW, TIME_TABLE = range(3)
SEM_REFERENCE_CPU, SEM_CPML = 0, 1


@dataclass
class LorentzianSusceptibility:
    """χ(ω) = σ·ω0² / (ω0² − ω² − iωγ) (Susceptibility.jl:17-33), frequencies in Meep units."""

    omega_0: float
    gamma: float
    sigma: float


def DrudeSusceptibility(gamma: float, sigma: float) -> LorentzianSusceptibility:
    """Drude pole = Lorentzian with ω0 = 0 (Susceptibility.jl:44-45)."""
    return LorentzianSusceptibility(0.0, float(gamma), float(sigma))


def ade_coefficients(s: LorentzianSusceptibility, dt: float) -> dict:
    """compute_ade_coefficients (Susceptibility.jl:74-85), in Float64."""
    gamma_pi_dt = s.gamma * math.pi * dt
    gamma1 = 1.0 - gamma_pi_dt
    gamma1_inv = 1.0 / (1.0 + gamma_pi_dt)
    omega0_dt_sq = (2 * math.pi * s.omega_0 * dt) ** 2
    return dict(
        gamma1_inv=gamma1_inv,
        gamma1=gamma1,
        omega0_dt_sq=omega0_dt_sq,
        sigma_omega0_dt_sq=omega0_dt_sq,
        drude_coeff=s.gamma * 2 * math.pi * dt * dt,
        is_drude=1 if s.omega_0 == 0.0 else 0,
    )


def eval_susceptibility(s: LorentzianSusceptibility, freq: float) -> complex:
    """eval_susceptibility (Susceptibility.jl:92-101)."""
    w = 2 * math.pi * freq
    w0 = 2 * math.pi * s.omega_0
    g = 2 * math.pi * s.gamma
    if s.omega_0 == 0:
        return -s.sigma * g / (w ** 2 + 1j * w * g)
    return s.sigma * w0 ** 2 / (w0 ** 2 - w ** 2 - 1j * w * g)


@dataclass
class SourceSpec:
    component: int
    start: Tuple[int, int, int]      # 0-based cell of element (0,0,0)
    dims: Tuple[int, int, int]
    amp: np.ndarray                  # complex128, shape dims (x, y, z)
    time_kind: int
    fcen: float = 0.0
    width: float = 0.0
    peak_time: float = 0.0
    cutoff: float = 0.0
    table: Optional[np.ndarray] = None  # complex128, shape (steps, 2)

    def __post_init__(self):
        # x fastest in memory, as the library reads it: handing it over is a view
        self.amp = np.asfortranarray(np.asarray(self.amp, dtype=np.complex128))


@dataclass
class MonitorSpec:
    component: int
    start: Tuple[int, int, int]
    dims: Tuple[int, int, int]
    freqs: np.ndarray               # float64 (rounded to the run's precision)
    decimation: int


@dataclass
class HistorySpec:
    """A history monitor: ``component`` over a cell box at every step < capacity."""

    component: int
    start: Tuple[int, int, int]
    dims: Tuple[int, int, int]
    capacity: int


@dataclass
class PoleSpec:
    coeffs: dict
    sigma: np.ndarray               # (nx, ny, nz) oscillator strength per voxel


@dataclass
class SimSpec:
    n: Tuple[int, int, int]
    dtype: int
    delta: Tuple[float, float, float]
    dt: float
    pml_lo: Tuple[int, int, int] = (0, 0, 0)
    pml_hi: Tuple[int, int, int] = (0, 0, 0)
    sigma_b: List[Optional[np.ndarray]] = field(default_factory=lambda: [None, None, None])
    sigma_d: List[Optional[np.ndarray]] = field(default_factory=lambda: [None, None, None])
    eps_inv: float = 1.0
    mu_inv: float = 1.0
    semantics: int = 1   # SEM_CPML (stable, the reference's CUDA-path CPML); 0 = CPU path
    periodic: int = 0    # bit a: axis a wraps its halo (Periodic / Bloch with k = 0)
    materials: List[Tuple[int, int, np.ndarray]] = field(default_factory=list)  # (kind, comp, array)
    poles: List[PoleSpec] = field(default_factory=list)
    sources: List[SourceSpec] = field(default_factory=list)
    monitors: List[MonitorSpec] = field(default_factory=list)
    histories: List[HistorySpec] = field(default_factory=list)
    geometry: Optional[object] = None  # geometry.GeometrySpec: ε⁻¹ rasterised on the device

    @property
    def np_dtype(self):
        return np.float32 if self.dtype == KH_F32 else np.float64

    @property
    def cells(self) -> int:
        return int(self.n[0]) * int(self.n[1]) * int(self.n[2])

    def promoted(self) -> "SimSpec":
        """The same run (identical cell indices, monitor boxes, source
        footprints and input values) computed in FP64: the full-FP64 run an
        FP32 run's error is measured against.  Only the arithmetic type
        changes; inputs already rounded to FP32 stay as they are."""
        import dataclasses

        return dataclasses.replace(self, dtype=KH_F64)


def flat_f(a: np.ndarray) -> np.ndarray:
    """x-fastest contiguous float64 view (or copy) of a cell-indexed array: no
    copy when it is already FP64 with x fastest."""
    return np.asarray(a, dtype=np.float64).ravel(order="F")


def flat_complex(a: np.ndarray) -> np.ndarray:
    """Interleaved (re, im) float64, x fastest."""
    # a contiguous complex128 array is already (re, im) pairs in memory
    z = np.ascontiguousarray(np.asarray(a, dtype=np.complex128).ravel(order="F"))
    return z.view(np.float64)
