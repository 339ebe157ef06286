"""Design-parameter filters and projections for inverse design.

Restates the reference's Adjoint/Filters.jl (raw ρ → filter → project → ε(ρ̄))
in torch, so that a filtered, projected design stays differentiable in front
of ``adjoint.simulate``:

* convolve_design_weights / conic_filter / cylindrical_filter / gaussian_filter
                                       Filters.jl:24-215
* tanh_projection                      Filters.jl:231-240
* exponential_/heaviside_ erosion and dilation, gray_indicator
                                       Filters.jl:249-305
* get_eta_from_conic, get_conic_radius_from_eta_e   Filters.jl:316-342

Designs are 2-D (Nx, Ny) grids flattened x fastest, as in the reference;
functions accept numpy arrays or torch tensors and return a torch tensor
(float64) of the same flattened shape.
"""
from __future__ import annotations

import math

import numpy as np
import torch


def _t(x) -> torch.Tensor:
    return x if isinstance(x, torch.Tensor) else torch.as_tensor(np.asarray(x, dtype=np.float64))


def _mesh_grid(Lx: float, Ly: float, resolution: float):
    """_mesh_grid (Filters.jl:127-135): design grid size and the kernel's
    nonnegative-quadrant coordinates 0, 1/res, … ≤ L/2."""
    nx = int(round(Lx * resolution)) + 1
    ny = int(round(Ly * resolution)) + 1

    def half(L):
        if resolution <= 0:
            return np.array([0.0])
        n = int(math.floor((L / 2) * resolution + 1e-9)) + 1
        return np.arange(n, dtype=np.float64) * (1.0 / resolution)

    return nx, ny, half(Lx), half(Ly)


def _quarter_to_full(hq: np.ndarray, shape) -> np.ndarray:
    """_quarter_to_full_kernel (Filters.jl:73-101): the C4v-symmetric kernel
    from its nonnegative quadrant, wrapped into a zero array of ``shape``."""
    kx, ky = hq.shape
    full = np.zeros(shape, dtype=np.float64)
    full[:kx, :ky] = hq
    full[shape[0] - np.arange(1, kx), :ky] = hq[1:, :]
    full[:kx, shape[1] - np.arange(1, ky)] = hq[:, 1:]
    full[np.ix_(shape[0] - np.arange(1, kx), shape[1] - np.arange(1, ky))] = hq[1:, 1:]
    return full


def convolve_design_weights(x2d: torch.Tensor, hq: np.ndarray) -> torch.Tensor:
    """convolve_design_weights (Filters.jl:106-121): edge-pad the design by its
    own size on every side, circular FFT convolution with the normalised full
    kernel, keep the centre."""
    sx, sy = x2d.shape
    h = _quarter_to_full(hq, (3 * sx, 3 * sy))
    h = torch.as_tensor(h / h.sum(), dtype=x2d.dtype)
    xp = torch.nn.functional.pad(x2d[None, None], (sy, sy, sx, sx), mode="replicate")[0, 0]
    res = torch.fft.ifftn(torch.fft.fftn(xp) * torch.fft.fftn(h)).real
    return res[sx:2 * sx, sy:2 * sy]


def _filter(x, kernel, Lx, Ly, resolution):
    x = _t(x)
    nx, ny, xv, yv = _mesh_grid(Lx, Ly, resolution)
    X, Y = np.meshgrid(xv, yv, indexing="ij")
    hq = kernel(X, Y)
    x2d = x.reshape(ny, nx).T  # flattened x fastest
    return convolve_design_weights(x2d, hq).T.reshape(-1)


def conic_filter(x, radius: float, Lx: float, Ly: float, resolution: float) -> torch.Tensor:
    """Linear conic ("hat") filter of radius ``radius`` (Filters.jl:146-168)."""
    def k(X, Y):
        r2 = X * X + Y * Y
        return np.where(r2 < radius * radius, 1.0 - np.sqrt(r2) / radius, 0.0)

    return _filter(x, k, Lx, Ly, resolution)


def cylindrical_filter(x, radius: float, Lx: float, Ly: float, resolution: float) -> torch.Tensor:
    """Top-hat filter of radius ``radius`` (Filters.jl:173-193)."""
    return _filter(x, lambda X, Y: np.where(X * X + Y * Y < radius * radius, 1.0, 0.0), Lx, Ly, resolution)


def gaussian_filter(x, sigma: float, Lx: float, Ly: float, resolution: float) -> torch.Tensor:
    """Gaussian filter exp(−r²/σ²) (Filters.jl:198-215)."""
    return _filter(x, lambda X, Y: np.exp(-(X * X + Y * Y) / (sigma * sigma)), Lx, Ly, resolution)


def tanh_projection(x, beta: float, eta: float) -> torch.Tensor:
    """Smoothed Heaviside threshold at ``eta`` of sharpness ``beta``; a step
    for β = ∞ (Filters.jl:231-240)."""
    x = _t(x)
    if math.isinf(beta):
        return (x > eta).to(x.dtype)
    return (math.tanh(beta * eta) + torch.tanh(beta * (x - eta))) / (math.tanh(beta * eta) +
                                                                   math.tanh(beta * (1 - eta)))


def exponential_erosion(x, radius, beta, Lx, Ly, resolution) -> torch.Tensor:
    """Filters.jl:249-256."""
    xh = torch.exp(beta * (1 - _t(x)))
    return 1 - torch.log(cylindrical_filter(xh, radius, Lx, Ly, resolution)) / beta


def exponential_dilation(x, radius, beta, Lx, Ly, resolution) -> torch.Tensor:
    """Filters.jl:262-269."""
    xh = torch.exp(beta * _t(x))
    return torch.log(cylindrical_filter(xh, radius, Lx, Ly, resolution)) / beta


def heaviside_erosion(x, radius, beta, Lx, Ly, resolution) -> torch.Tensor:
    """Filters.jl:275-282."""
    xh = cylindrical_filter(x, radius, Lx, Ly, resolution)
    return torch.exp(-beta * (1 - xh)) + math.exp(-beta) * (1 - xh)


def heaviside_dilation(x, radius, beta, Lx, Ly, resolution) -> torch.Tensor:
    """Filters.jl:288-295."""
    xh = cylindrical_filter(x, radius, Lx, Ly, resolution)
    return 1 - torch.exp(-beta * xh) + math.exp(-beta) * xh


def gray_indicator(x) -> float:
    """Grayness in percent: mean(4x(1−x))·100 (Filters.jl:302-304)."""
    x = _t(x)
    return float(torch.mean(4 * x * (1 - x)) * 100)


def get_eta_from_conic(b: float, R: float) -> float:
    """Eroded threshold for minimum length ``b`` with a conic filter of radius
    ``R`` (Filters.jl:316-329)."""
    nl = b / R
    if nl < 0:
        return 0.0
    if nl < 1:
        return 0.25 * nl * nl + 0.5
    if nl < 2:
        return -0.25 * nl * nl + nl
    return 1.0


def get_conic_radius_from_eta_e(b: float, eta_e: float) -> float:
    """Conic filter radius from the minimum length and the erosion threshold
    (Filters.jl:334-342)."""
    if 0.5 <= eta_e < 0.75:
        return b / (2 * math.sqrt(eta_e - 0.5))
    if 0.75 <= eta_e <= 1.0:
        return b / (2 - 2 * math.sqrt(1 - eta_e))
    raise ValueError(f"eta_e must be between 0.5 and 1.0, got {eta_e}")
