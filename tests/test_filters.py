"""Design filters and projections (Adjoint/Filters.jl), host side."""
import math

import numpy as np
import pytest
import torch


def _direct(x2d, hq):
    """Brute-force restatement: edge-padded design, full C4v kernel,
    normalised, centred linear convolution."""
    sx, sy = x2d.shape
    kx, ky = hq.shape
    full = {}
    for i in range(-(kx - 1), kx):
        for j in range(-(ky - 1), ky):
            full[(i, j)] = hq[abs(i), abs(j)]
    tot = sum(full.values())
    out = np.zeros_like(x2d)
    for a in range(sx):
        for b in range(sy):
            s = 0.0
            for (i, j), w in full.items():
                if w == 0:
                    continue
                # the padded design extends by one design width on each side
                ai = min(max(a - i, -sx), 2 * sx - 1)
                bj = min(max(b - j, -sy), 2 * sy - 1)
                s += w * x2d[min(max(ai, 0), sx - 1), min(max(bj, 0), sy - 1)]
            out[a, b] = s / tot
    return out


@pytest.mark.parametrize("name", ["conic_filter", "cylindrical_filter", "gaussian_filter"])
def test_filters_match_direct_convolution(kh, name):
    from khronos_gb300 import filters as F

    Lx, Ly, res, radius = 0.9, 0.6, 10, 0.25
    nx, ny, xv, yv = F._mesh_grid(Lx, Ly, res)
    rng = np.random.default_rng(1)
    x = rng.random(nx * ny)
    got = getattr(F, name)(x, radius, Lx, Ly, res).numpy()
    X, Y = np.meshgrid(xv, yv, indexing="ij")
    r2 = X * X + Y * Y
    hq = {"conic_filter": np.where(r2 < radius ** 2, 1 - np.sqrt(r2) / radius, 0.0),
          "cylindrical_filter": np.where(r2 < radius ** 2, 1.0, 0.0),
          "gaussian_filter": np.exp(-r2 / radius ** 2)}[name]
    want = _direct(x.reshape(ny, nx).T, hq).T.reshape(-1)
    assert np.allclose(got, want, rtol=1e-12, atol=1e-12)
    # a constant design stays constant (edge padding, normalised kernel)
    c = getattr(F, name)(np.full(nx * ny, 0.7), radius, Lx, Ly, res).numpy()
    assert np.allclose(c, 0.7, atol=1e-12)


def test_projection_and_indicators(kh):
    from khronos_gb300 import filters as F

    x = torch.linspace(0, 1, 11, dtype=torch.float64)
    p = F.tanh_projection(x, 8.0, 0.4)
    assert float(p[0]) == pytest.approx(0.0, abs=1e-15) and float(p[-1]) == pytest.approx(1.0)
    assert torch.all(p[1:] >= p[:-1])
    assert torch.equal(F.tanh_projection(x, math.inf, 0.45), (x > 0.45).double())
    assert F.gray_indicator(np.array([0.0, 1.0, 1.0])) == 0.0
    assert F.gray_indicator(np.full(4, 0.5)) == pytest.approx(100.0)
    for eta_e in (0.55, 0.6, 0.7, 0.8, 0.9, 0.95):
        R = F.get_conic_radius_from_eta_e(0.1, eta_e)
        assert F.get_eta_from_conic(0.1, R) == pytest.approx(eta_e, rel=1e-12)
    with pytest.raises(ValueError):
        F.get_conic_radius_from_eta_e(0.1, 0.3)


def test_morphology_and_gradient(kh):
    from khronos_gb300 import filters as F

    Lx, Ly, res = 0.8, 0.8, 10
    nx, ny, _, _ = F._mesh_grid(Lx, Ly, res)
    x = np.zeros((nx, ny))
    x[3:6, 3:6] = 1.0
    xf = x.T.reshape(-1)
    # (β kept moderate: exp(β) against FFT round-off, as in the reference)
    dil = F.exponential_dilation(xf, 0.15, 8.0, Lx, Ly, res).numpy()
    ero = F.exponential_erosion(xf, 0.15, 8.0, Lx, Ly, res).numpy()
    # soft max / min over the neighbourhood: dilation grows the block, erosion shrinks it
    assert dil.sum() > xf.sum() > ero.sum()
    assert dil.reshape(ny, nx)[4, 2] > 0.1 and ero.reshape(ny, nx)[4, 4] < 1.0
    hd = F.heaviside_dilation(xf, 0.15, 50.0, Lx, Ly, res).numpy()
    he = F.heaviside_erosion(xf, 0.15, 50.0, Lx, Ly, res).numpy()
    assert np.all((hd >= -1e-12) & (hd <= 1 + 1e-12)) and np.all((he >= -1e-12) & (he <= 1 + 1e-12))
    # the pipeline is differentiable end to end
    rho = torch.tensor(np.random.default_rng(2).random(nx * ny), dtype=torch.float64, requires_grad=True)

    def f(r):
        return torch.sum(F.tanh_projection(F.conic_filter(r, 0.2, Lx, Ly, res), 4.0, 0.5) ** 2)

    assert torch.autograd.gradcheck(f, (rho,), eps=1e-6, atol=1e-6)
