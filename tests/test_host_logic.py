"""Host-side set-up logic: PML profile and regions, decimation, workload
specs, flux reduction formula, and the oracle's own physics sanity."""
import math

import numpy as np
import pytest

from conftest import field_errors, rel_l2


def test_pml_profile_asymmetry(kh):
    """σ sampled at (i-1/2)Δ on both sides (Boundaries.jl:23-38): a 10-cell PML
    has 10 nonzero cells on the left and 9 on the right, pre-scaled by Δt/2."""
    from khronos_gb300 import grid as G

    g = G.Grid.build((3.2, 3.2, 3.2), (0, 0, 0), 20, "f64")
    s = G.cell_sigma(g, 0, 0.5, 0.5)
    assert np.count_nonzero(s[:32]) == 10 and np.count_nonzero(s[32:]) == 9
    assert np.all(np.diff(s[:10]) < 0) and np.all(np.diff(s[55:]) > 0)
    u0 = -math.log(1e-15) / (4 * 0.5 / 3) * (0.5 * float(g.dt))
    assert s[0] == pytest.approx(u0 * ((0.5 - 0.025) / 0.5) ** 2, rel=1e-15)
    assert G.pml_widths(g, [[0.5, 0.5]] * 3) == ((10, 10, 10), (10, 10, 10))


def test_pml_widths_f32_and_fallback(kh):
    from khronos_gb300 import grid as G

    g = G.Grid.build((12.8, 7.68, 5.12), (0, 0, 0), 25, "f32")
    assert g.n == (320, 192, 128)
    assert G.pml_widths(g, [[0.48, 0.48]] * 3) == ((12, 12, 12), (12, 12, 12))
    small = G.Grid.build((1.0, 1.0, 1.0), (0, 0, 0), 10, "f64")
    assert G.pml_widths(small, [[0.6, 0.6], [0, 0], [0, 0]]) == ((10, 0, 0), (0, 0, 0))


def test_auto_decimation(kh):
    from khronos_gb300 import configs
    from khronos_gb300.monitors import auto_decimation

    w1 = configs.dipole(dtype="f64")
    assert auto_decimation(w1.sim.sources, w1.sim.dt) == 26
    w2 = configs.waveguide(dtype="f32", scale=1.0)
    assert auto_decimation(w2.sim.sources, w2.sim.dt) == 31
    assert w2.sim.n == (320, 192, 128)


def test_waveguide_spec_shapes(kh):
    from khronos_gb300 import configs

    w = configs.waveguide(dtype="f32", scale=0.25)
    sp = w.sim.spec()
    assert len(sp.monitors) == 8 and all(len(m.freqs) == 21 for m in sp.monitors)
    assert all(m.decimation > 1 for m in sp.monitors)
    for m in sp.monitors:
        for a in range(3):
            assert 0 <= m.start[a] and m.start[a] + m.dims[a] <= sp.n[a] + 1
    eps = [arr for kind, c, arr in sp.materials if kind == 0]
    assert len(eps) == 3 and all(a.shape == sp.n for a in eps)
    assert np.isclose(1 / np.min(eps[0]), 12.25) and np.isclose(1 / np.max(eps[0]), 2.085)


def test_flux_formula_matches_reference_loop(kh):
    from khronos_gb300.monitors import flux_from_dft

    rng = np.random.default_rng(3)
    shp = (2, 5, 4, 3)
    e1, e2, h1, h2 = (rng.normal(size=shp) + 1j * rng.normal(size=shp) for _ in range(4))
    dA = 0.01
    ref = np.zeros(3)
    for f in range(3):  # FluxMonitor.jl:104-153 written out
        E1 = (e1[0] + e1[1]) / 2
        E2 = (e2[0] + e2[1]) / 2
        H1 = (h1[0] + h1[1]) / 2
        H2 = (h2[0] + h2[1]) / 2
        s = 0.0
        for i2 in range(4):
            for i1 in range(5):
                s += (E1[i1, i2, f] * np.conj(H2[i1, i2, f]) - E2[i1, i2, f] * np.conj(H1[i1, i2, f])).real * dA
        ref[f] = s
    assert np.allclose(flux_from_dft(0, e1, e2, h1, h2, dA), ref, rtol=1e-13)


def _dipole(kh, semantics, dtype="f64", boundaries=((0.5, 0.5),) * 3):
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=1 / 1.55, fwidth=0.2 / 1.55),
                           component=kh.EZ)
    return kh.Simulation(cell_size=(3.2,) * 3, resolution=10, sources=[src], boundaries=list(boundaries),
                         dtype=dtype, semantics=semantics)


def _energy(o):
    return sum(float(np.sum(o.field(c) ** 2)) for c in range(6))


def test_oracle_cpml_absorbs(kh, oracle):
    """CUDA-path CPML semantics: once the pulse has left the source region the
    field energy decays."""
    o = oracle.OracleSim(_dipole(kh, "cpml").spec())
    o.step(700)
    e1 = _energy(o)
    o.step(300)
    e2 = _energy(o)
    assert np.isfinite(e2) and e2 < 0.5 * e1


def test_oracle_reference_cpu_path_grows(kh, oracle):
    """The reference CPU path drops the σ_prev stage in chunks without a U
    array (Helpers.jl:208-223): with PML the fields grow without bound."""
    o = oracle.OracleSim(_dipole(kh, "reference_cpu").spec())
    o.step(100)
    e1 = _energy(o)
    o.step(100)
    e2 = _energy(o)
    assert e2 > 1e6 * e1


def test_oracle_semantics_agree_without_pml(kh, oracle):
    a = oracle.OracleSim(_dipole(kh, "cpml", boundaries=((0, 0),) * 3).spec())
    b = oracle.OracleSim(_dipole(kh, "reference_cpu", boundaries=((0, 0),) * 3).spec())
    a.step(150)
    b.step(150)
    for c in range(6):
        assert np.array_equal(a.field(c), b.field(c))


def test_oracle_f32_tracks_f64(kh, oracle):
    a = oracle.OracleSim(_dipole(kh, "cpml", "f64").spec())
    b = oracle.OracleSim(_dipole(kh, "cpml", "f32").spec())
    a.step(300)
    b.step(300)
    errs = field_errors([b.field(c) for c in range(6)], [a.field(c) for c in range(6)])
    assert max(errs) < 1e-4


def test_flux_error_measure(kh):
    from khronos_gb300.monitors import flux_error

    ref = np.array([1.0, -2.0, 4.0])
    e = flux_error(ref * (1 + 1e-5), ref)
    assert abs(e["rel_l2"] - 1e-5) < 1e-12
    assert abs(e["max_rel"] - 1e-5) < 1e-12
    assert flux_error(np.zeros(2), np.zeros(2)) == {"rel_l2": 0.0, "max_rel": 0.0}
    with pytest.raises(ValueError):
        flux_error(np.zeros(2), np.zeros(3))


def test_promoted_spec_keeps_inputs(kh):
    from khronos_gb300 import configs
    from khronos_gb300.spec import KH_F32, KH_F64

    sp = configs.dipole(dtype="f32", resolution=10).sim.spec()
    pp = sp.promoted()
    assert sp.dtype == KH_F32 and pp.dtype == KH_F64
    assert pp.n == sp.n and pp.dt == sp.dt and pp.delta == sp.delta
    assert [m.start for m in pp.monitors] == [m.start for m in sp.monitors]
    assert all(np.array_equal(a.amp, b.amp) for a, b in zip(pp.sources, sp.sources))
