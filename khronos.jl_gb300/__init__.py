"""khronos_gb300 — GB300-native FDTD step loop of Khronos.jl.

The step loop (curl + CPML + constitutive update + sources + χ3 + ADE poles,
DFT monitors, FP64 flux) runs as hand-written sm_103a CUDA kernels in
``libkhronos_gb300.so`` behind the C ABI of ``include/khronos_gb300.h``.
This package is the host side: the set-up arithmetic of the reference's
``prepare_simulation!`` and a ctypes binding of the ABI.
"""
from .boundaries import Bloch, PECBoundary, PMCBoundary, Periodic
from .grid import CENTER, EX, EY, EZ, HX, HY, HZ, Grid, GridVolume, interpolation_weight
from .monitors import DFTMonitor, FluxMonitor, flux_from_dft
from .simulation import Simulation, apply_chi1_correction, stop_when_dft_decayed
from .sources import (ContinuousWaveSource, CustomSource, EquivalentSource, GaussianBeamSource,
                      GaussianPulseSource, PlaneWaveSource, ProfileSource, TFSFSource, UniformSource)
from .spec import (DrudeSusceptibility, LorentzianSusceptibility, SimSpec, ade_coefficients,
                   eval_susceptibility)

__all__ = [
    "Bloch", "PECBoundary", "PMCBoundary", "Periodic",
    "CENTER", "EX", "EY", "EZ", "HX", "HY", "HZ", "Grid", "GridVolume", "interpolation_weight",
    "DFTMonitor", "FluxMonitor", "flux_from_dft", "Simulation", "apply_chi1_correction",
    "stop_when_dft_decayed",
    "ContinuousWaveSource", "CustomSource", "GaussianPulseSource", "PlaneWaveSource", "ProfileSource", "EquivalentSource", "TFSFSource",
    "GaussianBeamSource",
    "UniformSource",
    "DrudeSusceptibility", "LorentzianSusceptibility", "SimSpec", "ade_coefficients",
    "eval_susceptibility",
]
