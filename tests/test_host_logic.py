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


def test_photonic_slab_spec(kh):
    """The periodic benchmark workload: x and y wrapped without PML, 12-cell
    CPML along z, flux planes inside the periodic span, a hole lattice in the
    slab (air at the lattice points, silicon between them)."""
    from khronos_gb300 import configs

    sp = configs.photonic_slab(dtype="f32").sim.spec()
    assert tuple(sp.n) == (256, 256, 128) and sp.periodic == 3
    assert tuple(sp.pml_lo) == (0, 0, 12) and tuple(sp.pml_hi) == (0, 0, 12)
    assert len(sp.monitors) == 8
    for m in sp.monitors:
        assert m.dims[0] < sp.n[0] and m.dims[1] < sp.n[1]
    eps_x = [arr for kind, c, arr in sp.materials if kind == 0 and c == 0][0]
    mid = sp.n[2] // 2
    slab = 1.0 / eps_x[:, :, mid]
    assert np.isclose(slab.max(), 12.25) and np.isclose(slab.min(), 1.0)
    assert 0.2 < np.mean(slab == 1.0) < 0.4  # π·0.12²/0.4² ≈ 0.28 of the area is hole
    assert np.all(1.0 / eps_x[:, :, 0] == 1.0)


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


def _absorber_sigma(n, delta, layers=20, order=3):
    """_apply_absorbers! (Geometry.jl:708-790) for one absorber on the high y
    side: σ = σ_max·(d/L)^p over the last `layers` entries of each component's
    own y extent (ny + 1 for Ex, Ez, Hy; ny for Ey, Hx, Hz), σ_max =
    −(p+1)·ln(1e-6)/(2L), on the cells 0..ny−1 this library's arrays hold."""
    L = layers * delta
    smax = -(order + 1) * np.log(1e-6) / (2.0 * L)

    def comp(ny_c):
        a = np.zeros(n)
        for layer in range(1, min(layers, ny_c) + 1):
            j = ny_c - layer  # 0-based index of this layer
            if j < n[1]:
                a[:, j, :] += smax * ((layers - layer + 1) / layers) ** order
        return a

    ny = n[1]
    sd = [comp(ny + 1), comp(ny), comp(ny + 1)]   # Ex, Ey, Ez
    sb = [comp(ny), comp(ny + 1), comp(ny)]       # Hx, Hy, Hz
    return sd, sb


def _absorber_case(kh, semantics):
    """The reference's absorber run (test/test_absorber.jl:84-121): a 4 µm cube
    at resolution 10 filled by an ε = 1 object, 1 µm PML on both x sides, the
    low y side and both z sides, a 20-layer absorber on the high y side, a CW
    Ez point source (fcen 1) at the centre."""
    src = kh.UniformSource(time_profile=kh.ContinuousWaveSource(fcen=1.0), component=kh.EZ)
    probe = kh.Simulation(cell_size=(4.0,) * 3, resolution=10, sources=[src], dtype="f64")
    n, delta = probe.grid.n, probe.grid.delta
    sd, sb = _absorber_sigma(n, delta[1])
    ones = [np.ones(n) for _ in range(3)]
    return kh.Simulation(cell_size=(4.0,) * 3, resolution=10, sources=[src], dtype="f64",
                         boundaries=[[1.0, 1.0], [1.0, 0.0], [1.0, 1.0]], eps_inv=ones,
                         sigma_d=sd, sigma_b=sb, semantics=semantics)


def test_reference_absorber_run_reaches_a_missing_dispatch(kh, oracle):
    """The reference's only multi-step test of a PML run on its CPU path,
    restated.  The absorber marks every region it overlaps as conductive
    (classify_region_physics, Chunking.jl:219-241), so the chunk with PML
    along x next to the high-y absorber allocates C_y (PML on prev(y) = x) but
    no U_y (no PML on next(y) = z); its σ arrays are zero-filled scalars
    (_slice_or_zero, Chunking.jl:1359-1366), and generic_curl! has no method
    for C without U with a scalar σ_next (Helpers.jl:39-270), so that run
    stops with a MethodError on the reference's CPU path.  The oracle, which
    restates the same dispatch, refuses the configuration at prepare."""
    sim = _absorber_case(kh, "reference_cpu")
    spec = sim.spec()
    assert tuple(spec.n) == (40, 40, 40)
    assert int(round(2.0 / spec.dt)) == 40  # run(until = 2.0)
    with pytest.raises(RuntimeError, match="status 6"):
        oracle.OracleSim(spec)


def test_cpu_path_growth_onset_on_the_dipole_grid(kh, oracle):
    """64³ dipole grid (10-cell CPML, Gaussian Ez dipole), FP64: the CPU-path
    fields leave the CUDA-path ones between steps 60 and 80 (energy ratio
    above 1.01), pass a ratio of 1e6 by step 140 and stay finite through step
    1000.  Mechanism: in a slab with PML along a only, the a-component's own
    W stage adds (1+σ)W_new − (1−σ)W_old, a gain that the σ_a damping of the
    other components' T and U stages cancels; the CPU path's method for a
    component without U (C, U and σD absent, Helpers.jl:208-223) drops its
    σ_prev = σ_a stage, so the gain is left uncancelled."""
    from khronos_gb300 import configs

    sims = {}
    for sem in ("cpml", "reference_cpu"):
        w = configs.dipole(dtype="f64", steps=1000)
        w.sim.semantics = sem
        sims[sem] = oracle.OracleSim(w.sim.spec())
    ratio = {}
    for step in range(10, 1001, 10):
        for o in sims.values():
            o.step(10)
        if step in (60, 80, 140, 1000):
            ratio[step] = _energy(sims["reference_cpu"]) / _energy(sims["cpml"])
    assert ratio[60] < 1.01 < ratio[80]
    assert ratio[140] > 1e6
    assert np.isfinite(ratio[1000]) and ratio[1000] > 1e100
