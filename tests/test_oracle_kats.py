"""Known-answer tests from the reference's own test suite, run against the
host-side restatement (grid volumes, interpolation weights, ADE coefficients,
susceptibilities, source footprints) and the Gaussian-pulse constants.

Each test cites the reference test it restates.
"""
import math

import numpy as np
import pytest


def _grid(kh, size=4.0, res=20, dtype="f64"):
    return kh.Grid.build((size, size, size), (0.0, 0.0, 0.0), res, dtype)


@pytest.mark.parametrize(
    "comp,size,dims,start,end",
    [
        # test/test_grid_volume.jl:22-52 (point)
        ("EX", (0, 0, 0), (2, 1, 1), (40, 41, 41), (41, 41, 41)),
        ("EY", (0, 0, 0), (1, 2, 1), (41, 40, 41), (41, 41, 41)),
        ("EZ", (0, 0, 0), (1, 1, 2), (41, 41, 40), (41, 41, 41)),
        # test/test_grid_volume.jl:57-87 (line along y)
        ("EX", (0, math.inf, 0), (2, 81, 1), (40, 1, 41), (41, 81, 41)),
        ("EY", (0, math.inf, 0), (1, 80, 1), (41, 1, 41), (41, 80, 41)),
        ("EZ", (0, math.inf, 0), (1, 81, 2), (41, 1, 40), (41, 81, 41)),
        # test/test_grid_volume.jl:93-123 (plane)
        ("EX", (0, math.inf, math.inf), (2, 81, 81), (40, 1, 1), (41, 81, 81)),
        ("EY", (0, math.inf, math.inf), (1, 80, 81), (41, 1, 1), (41, 80, 81)),
        ("EZ", (0, math.inf, math.inf), (1, 81, 80), (41, 1, 1), (41, 81, 80)),
    ],
)
def test_grid_volume_kat(kh, comp, size, dims, start, end):
    g = _grid(kh)
    gv = g.grid_volume((0.0, 0.0, 0.0), size, getattr(kh, comp))
    assert gv.dims == dims
    assert gv.start_idx == start
    assert gv.end_idx == end


def _restrict(kh, center, size):
    # test/test_interpolation.jl:14-37: 2D grid x = -0.5:0.1:0.5, y = -0.7:0.1:0.7
    dx = dy = 0.1
    xs = np.arange(-0.5, 0.5 + 1e-12, dx)
    ys = np.arange(-0.7, 0.7 + 1e-12, dy)
    lo = [center[a] - size[a] / 2 for a in range(3)]
    hi = [center[a] + size[a] / 2 for a in range(3)]
    w = np.zeros((len(xs), len(ys)))
    for j, y in enumerate(ys):
        for i, x in enumerate(xs):
            w[i, j] = kh.interpolation_weight((x, y, 0.0), lo, hi, size, (dx, dy, 0.0), 2)
    return w


def test_interpolation_point_and_line_kat(kh):
    # test/test_interpolation.jl:39-55
    assert abs(_restrict(kh, (0, 0, 0), (0, 0, 0)).sum() - 1.0) < 1e-15
    assert abs(_restrict(kh, (-0.12, -0.26, 0), (0, 0, 0)).sum() - 1.0) < 1e-15
    assert abs(_restrict(kh, (0.14, -0.21, 0), (0.5, 0, 0)).sum() * 0.1 - 0.5) < 1e-15
    assert abs(_restrict(kh, (0.14, -0.21, 0), (0, 0.5, 0)).sum() * 0.1 - 0.5) < 1e-15


def test_interpolation_volume_kat(kh):
    # test/test_interpolation.jl:57-74
    for sx, sy in ((0.4, 0.4), (0.4, 0.5)):
        for ix in np.arange(-1.6, 1.6 + 1e-9, 0.4):
            w = _restrict(kh, (ix * 0.1, ix * 0.1, 0), (sx, sy, 0))
            assert abs(w.sum() * 0.1 * 0.1 - sx * sy) < 1e-15


def test_interpolation_subpixel_kat(kh):
    # test/test_interpolation.jl:76-92
    for ix in np.arange(-1.6, 1.6 + 1e-9, 0.4):
        w = _restrict(kh, (0.14, ix * 0.1, 0), (5.0 * 0.1, 0.5 * 0.1, 0))
        assert abs(w.sum() - 2.5) < 1e-14
    for ix in np.arange(-0.8, 0.8 + 1e-9, 0.4):
        w = _restrict(kh, (ix * 0.1, 0.14, 0), (0.4 * 0.1, 6.0 * 0.1, 0))
        assert abs(w.sum() - 2.4) < 1e-14


def test_ade_coefficients_kat(kh):
    # test/test_dispersive.jl:23-39
    dt = 0.01
    c = kh.ade_coefficients(kh.LorentzianSusceptibility(1.0, 0.1, 2.0), dt)
    assert math.isclose(c["gamma1"], 1.0 - 0.1 * math.pi * dt)
    assert math.isclose(c["gamma1_inv"], 1.0 / (1.0 + 0.1 * math.pi * dt))
    assert math.isclose(c["omega0_dt_sq"], (2 * math.pi * 1.0 * dt) ** 2)
    assert math.isclose(c["sigma_omega0_dt_sq"], (2 * math.pi * 1.0 * dt) ** 2)
    assert c["is_drude"] == 0
    d = kh.ade_coefficients(kh.DrudeSusceptibility(0.5, 3.0), dt)
    assert d["is_drude"] == 1
    assert d["omega0_dt_sq"] == 0.0
    assert math.isclose(d["drude_coeff"], 0.5 * 2 * math.pi * dt ** 2)


def test_susceptibility_eval_kat(kh):
    # test/test_dispersive.jl:42-58
    s = kh.LorentzianSusceptibility(1.0, 0.1, 2.0)
    w, w0, g = 2 * math.pi * 0.5, 2 * math.pi, 2 * math.pi * 0.1
    assert np.isclose(kh.eval_susceptibility(s, 0.5), 2.0 * w0 ** 2 / (w0 ** 2 - w ** 2 - 1j * w * g))
    d = kh.DrudeSusceptibility(0.5, 3.0)
    gd = 2 * math.pi * 0.5
    assert np.isclose(kh.eval_susceptibility(d, 0.5), -3.0 * gd / (w ** 2 + 1j * w * gd))


@pytest.mark.parametrize("comp", ["EX", "EY", "EZ", "HX", "HY", "HZ"])
def test_point_source_footprint_kat(kh, comp):
    # test/test_sources.jl:42-59: a point in the middle of a voxel touches 8 nodes
    g = kh.Grid.build((10.0, 10.0, 10.0), (0, 0, 0), 10, "f64")
    src = kh.UniformSource(time_profile=kh.ContinuousWaveSource(fcen=1.0), component=getattr(kh, comp),
                           center=(0.023, 0.784, 0.631), size=(0.0, 0.0, 0.0))
    _, amp = src.amplitude_array(g, getattr(kh, comp))
    assert np.count_nonzero(amp) == 8


@pytest.mark.parametrize("comp", ["EX", "EY", "EZ", "HX", "HY", "HZ"])
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_line_source_footprint_kat(kh, comp, axis):
    # test/test_sources.jl:61-86: a line through the middle of voxels touches 4 nodes per cell
    g = kh.Grid.build((10.0, 10.0, 10.0), (0, 0, 0), 10, "f64")
    size = [0.0, 0.0, 0.0]
    size[axis] = math.inf
    c = getattr(kh, comp)
    src = kh.UniformSource(time_profile=kh.ContinuousWaveSource(fcen=1.0), component=c,
                           center=(0.023, 0.784, 0.631), size=tuple(size))
    _, amp = src.amplitude_array(g, c)
    assert np.count_nonzero(amp) == g.component_dims(c)[axis] * 4


def test_gaussian_pulse_constants(kh):
    # TimeSources.jl:91-121: width = 1/fwidth, cutoff = 5 width, stored fwidth widened,
    # peak snapped to a multiple of the period with ties to even.
    fcen = 1 / 1.55
    p = kh.GaussianPulseSource(fcen=fcen, fwidth=0.2 * fcen)
    assert p.width == pytest.approx(7.75)
    assert p.cutoff == pytest.approx(38.75)
    assert p.peak_time == pytest.approx(12 * 1.55)  # 12.5 periods rounds to 12
    assert p.fwidth_stored == pytest.approx(math.sqrt(-2 * math.log(1e-7)) / (7.75 * math.pi))
    q = kh.GaussianPulseSource(fcen=fcen, fwidth=0.25 * fcen)
    assert q.cutoff == pytest.approx(31.0) and q.peak_time == pytest.approx(15.5)
    # eval at the peak is 1 (no phase at an integer number of periods)
    assert abs(p.eval(p.peak_time) - 1.0) < 1e-12
    assert p.eval(p.peak_time + p.cutoff + 1.0) == 0
