"""Physics checks that pin the step loop to known answers, independently of
the oracle: the reference's own validation example for normal-incidence
Fresnel reflectance (examples/fresnel_reflectance.jl), with its set-up
(air → n = 3.5 half-space, z-propagating plane wave, 1 µm PML on every face,
resolution 40, 50 wavelengths in 0.9–1.6 µm, two-run normalisation with the
incident field subtracted) and its pass bar (RMS error of R over the
frequencies that carry ≥ 1 % of the peak incident power < 0.05).  The
reference runs until its DFT monitors decay; here a fixed 60 time units
(the source switches off at t ≈ 10; the pulse has left the 10 µm cell long
before t = 60).

The reference's plane-wave fill drops the z factor (weight and propagation
phase) of a component whose source volume is one cell thick.  In FP64 the
example's source plane sits exactly on an Ex node, so the electric current
loses its phase against the magnetic one and most of the pulse leaves
backwards; the example then misses its own bar (RMS 0.105 measured).  In
FP32 the rounded grid index gives Ex a two-layer volume, the phase survives,
and the example as written passes.  The FP64 case therefore moves the plane
a quarter cell off the node and widens the PML-free transverse window to
2.5 µm.

Also the host-side PlaneWaveSource set-up: polarisation basis, current
factors and the reference's separable amplitude fill."""
import math

import numpy as np
import pytest


def _fresnel_sim(kh, res, with_slab, dtype, n_slab=3.5, dpml=1.0, nfreq=50, window=0.5, shift=0.0):
    from khronos_gb300.geometry import Cuboid, Material, Object

    lam = np.linspace(0.9, 1.6, nfreq)
    fcen = 0.5 * (1 / 0.9 + 1 / 1.6)
    fwidth = 1 / 0.9 - 1 / 1.6
    sxy, sz = 2 * dpml + window, 2 * dpml + 8.0
    src_z = -sz / 2 + dpml + 1.0 + shift / res
    src = kh.PlaneWaveSource(time_profile=kh.GaussianPulseSource(fcen=fcen, fwidth=fwidth),
                             center=(0.0, 0.0, src_z), size=(math.inf, math.inf, 0.0),
                             k_vector=(0.0, 0.0, 1.0), polarization_angle=0.0)
    geom = [Object(Cuboid((0.0, 0.0, sz / 4), (sxy, sxy, sz / 2)), Material(eps=n_slab ** 2))] if with_slab else []
    mon = kh.DFTMonitor(component=kh.EX, center=(0.0, 0.0, src_z + 1.0), size=(0.4, 0.4, 0.0),
                        frequencies=list(1.0 / lam))
    return kh.Simulation(cell_size=(sxy, sxy, sz), resolution=res, sources=[src], geometry=geom,
                         boundaries=[[dpml, dpml]] * 3, monitors=[mon], dtype=dtype)


def _reflectance(inc, tot):
    p_inc = np.sum(np.abs(inc) ** 2, axis=(0, 1, 2))
    p_ref = np.sum(np.abs(tot - inc) ** 2, axis=(0, 1, 2))
    good = p_inc > 0.01 * p_inc.max()
    return (p_ref / p_inc)[good]


def test_planewave_polarisation_and_components(kh):
    tp = kh.GaussianPulseSource(fcen=1.0, fwidth=0.3)
    # k along the plane normal: degenerate s/p, basis fixed by k's axis
    s = kh.PlaneWaveSource(time_profile=tp, size=(1.0, 1.0, 0.0), k_vector=(0.0, 0.0, 2.0))
    assert s.polarization == [1.0, 0.0, 0.0]
    assert s.components() == [kh.EX, kh.HY]
    assert s.scaling(kh.EX) == -1.0 and s.scaling(kh.HY) == -1.0
    assert s.k == 2 * math.pi
    s = kh.PlaneWaveSource(time_profile=tp, size=(0.0, 1.0, 1.0), k_vector=(1.0, 0.0, 0.0))
    assert s.polarization == [0.0, 1.0, 0.0] and s.components() == [kh.EY, kh.HZ]
    # oblique: basis n̂ × k̂, rotated about k̂ by the polarisation angle
    s = kh.PlaneWaveSource(time_profile=tp, size=(1.0, 1.0, 0.0), angle_theta=0.0,
                           angle_phi=math.pi / 6, polarization_angle=math.pi / 2, eps=2.25)
    k = s.khat
    assert np.allclose(k, [0.5, 0.0, math.cos(math.pi / 6)])
    assert abs(np.dot(s.polarization, k)) < 1e-15
    assert s.k == pytest.approx(2 * math.pi * 1.5)
    # Ĵ = n̂×(k̂×Ê)/Z₀, M̂ = −n̂×Ê
    e = np.array(s.polarization)
    j = np.cross([0, 0, 1], np.cross(k, e)) / math.sqrt(1 / 2.25)
    m = -np.cross([0, 0, 1], e)
    for c in range(3):
        assert s.scaling(c) == pytest.approx(j[c], abs=1e-15)
        assert s.scaling(3 + c) == pytest.approx(m[c], abs=1e-15)
    # k anti-parallel to the normal: n̂ × k̂ = 0, no component (as the reference)
    s = kh.PlaneWaveSource(time_profile=tp, size=(1.0, 1.0, 0.0), k_vector=(0.0, 0.0, -1.0))
    assert s.components() == []
    with pytest.raises(ValueError):
        kh.PlaneWaveSource(time_profile=tp, size=(1.0, 1.0, 1.0), k_vector=(0.0, 0.0, 1.0))


def test_planewave_separable_fill(kh):
    """Separable fill = weight × pol_factor × amplitude × exp(−i k k̂·r) per
    cell, except that a component one cell thick in z drops its z factor (the
    reference's fill does this for every single-layer volume); an infinite
    extent has weight 1 along that axis."""
    from khronos_gb300.grid import interpolation_weight

    sim = _fresnel_sim(kh, 10, False, "f64")
    src = sim.sources[0]
    g = sim.grid
    seen = set()
    for comp in src.components():
        gv, amp = src.amplitude_array(g, comp)
        origin = g.component_origin(comp)
        d = [float(v) for v in g.delta]
        lo_z, hi_z = src.center[2], src.center[2]
        one_layer = amp.shape[2] == 1
        seen.add(one_layer)
        for (ix, iy, iz), a in np.ndenumerate(amp):
            p = [origin[q] + ([ix, iy, iz][q] + 1 + gv.start_idx[q] - 2) * d[q] for q in range(3)]
            if one_layer:
                want = src.scaling(comp) * src.amplitude
            else:
                wz = interpolation_weight((p[2], 0, 0), (lo_z, 0, 0), (hi_z, 0, 0), (0.0, 0, 0), (d[2], 0, 0), 1)
                want = wz * src.scaling(comp) * src.amplitude * np.exp(-1j * src.k * p[2])
            assert a == pytest.approx(want, rel=1e-12, abs=1e-15)
    assert seen == {True, False}  # Ex on the plane (one layer), Hy straddling it (two)


def test_fresnel_source_volumes(kh):
    """The precision dependence described above, on the host: the example's
    Ex source volume is one layer in FP64 (z factor dropped) and two layers
    in FP32; the quarter-cell shift gives two layers in FP64."""
    def ex_layers(dtype, shift=0.0):
        sim = _fresnel_sim(kh, 40, False, dtype, shift=shift)
        return [s.dims[2] for s in sim.spec().sources if s.component == kh.EX][0]

    assert ex_layers("f64") == 1
    assert ex_layers("f32") == 2
    assert ex_layers("f64", shift=0.25) == 2


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_fresnel_reflectance(kh, gpu_lib, dtype):
    kw = dict(window=2.5, shift=0.25) if dtype == "f64" else {}
    out = {}
    for slab in (False, True):
        sim = _fresnel_sim(kh, 40, slab, dtype, **kw)
        sim.run(until=60.0)
        out[slab] = sim.monitors[0].data()
        sim.close()
    r = _reflectance(out[False], out[True])
    r_exact = ((3.5 - 1) / (3.5 + 1)) ** 2
    rms = math.sqrt(float(np.mean((r - r_exact) ** 2)))
    print(f"Fresnel {dtype}: R mean {r.mean():.4f} (exact {r_exact:.4f}), rms error {rms:.4f}, "
          f"max {np.max(np.abs(r - r_exact)):.4f}, {r.size} frequencies")
    assert r.size >= 20
    assert rms < 0.05


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_fresnel_case_matches_oracle(kh, oracle, gpu_lib, dtype):
    """The same set-up at resolution 10 (plane-wave source over the whole
    plane including the PML, rasterised dielectric half-space) against the
    oracle, step for step."""
    from test_gpu_parity import TOL, compare

    sim = _fresnel_sim(kh, 10, True, dtype)
    compare(sim.spec(), 400, oracle, gpu_lib, TOL[dtype])


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_oblique_planewave_matches_oracle(kh, oracle, gpu_lib, dtype):
    """An oblique, rotated plane wave (phase varying across the injection
    plane, four current components) over a dielectric block, device against
    the oracle."""
    from khronos_gb300.geometry import Cuboid, Material, Object
    from test_gpu_parity import TOL, compare

    src = kh.PlaneWaveSource(time_profile=kh.GaussianPulseSource(fcen=0.9, fwidth=0.3),
                             center=(0.0, 0.0, -0.6), size=(math.inf, math.inf, 0.0),
                             angle_theta=0.7, angle_phi=0.35, polarization_angle=0.6)
    assert len(src.components()) == 4
    geom = [Object(Cuboid((0.1, -0.1, 0.3), (0.8, 0.6, 0.4)), Material(eps=6.0))]
    mon = kh.DFTMonitor(component=kh.EY, center=(0, 0, 0.5), size=(1.2, 1.0, 0.0), frequencies=[0.8, 1.0])
    sim = kh.Simulation(cell_size=(2.2, 1.9, 2.1), resolution=10, sources=[src], geometry=geom,
                        boundaries=[[0.3, 0.3]] * 3, monitors=[mon], dtype=dtype)
    compare(sim.spec(), 120, oracle, gpu_lib, TOL[dtype])


# ---------------------------------------------------------------------------
# The reference's periodic validation example (examples/dielectric_slab.jl):
# an n = 2, 0.5 µm slab in a 0.1 µm periodic x/y cell with 1 µm of PML in z,
# resolution 40, a z-propagating PlaneWaveSource with a Gaussian pulse
# (fcen 1, fwidth = π), transmission flux_slab / flux_empty over 51
# frequencies in 0.67–1.67 against the Fresnel slab formula, bar 0.08.

def _slab_fresnel(f, n, d):
    r12 = (1 - n) / (1 + n)
    t12, r21, t21 = 2 / (1 + n), -r12, 2 * n / (1 + n)
    ph = n * 2 * np.pi * f * d
    return abs(t12 * t21 * np.exp(1j * ph) / (1 + r12 * r21 * np.exp(2j * ph))) ** 2


def _slab_transmission(kh, oracle, dtype, decimation):
    import math

    from khronos_gb300.geometry import Cuboid, Material, Object
    from khronos_gb300.monitors import flux_from_dft

    fmin, fmax = 1 / 1.5, 1 / 0.6
    freqs = list(np.linspace(fmin, fmax, 51))
    flux = []
    for slab in (False, True):
        src = kh.PlaneWaveSource(time_profile=kh.GaussianPulseSource(fcen=1.0, fwidth=math.pi * (fmax - fmin)),
                                 center=(0.0, 0.0, -1.0), size=(0.1, 0.1, 0.0), k_vector=(0.0, 0.0, 1.0))
        fm = kh.FluxMonitor(center=(0.0, 0.0, 1.0), size=(0.1, 0.1, 0.0), frequencies=freqs,
                            decimation=decimation)
        geo = [Object(Cuboid((0.0, 0.0, 0.0), (1.1, 1.1, 0.5)), Material(eps=4.0))] if slab else None
        bc = [[kh.Periodic(), kh.Periodic()], [kh.Periodic(), kh.Periodic()], [None, None]]
        sim = kh.Simulation(cell_size=(0.1, 0.1, 5.5), resolution=40, sources=[src], monitors=[fm],
                            boundaries=[[0, 0], [0, 0], [1.0, 1.0]], boundary_conditions=bc, dtype=dtype,
                            geometry=geo)
        spec = sim.spec()
        o = oracle.OracleSim(spec)
        o.step(int(math.ceil((src.time_profile.cutoff + 60.0) / spec.dt)))
        flux.append(flux_from_dft(fm.normal_axis, *[o.dft(i) for i in range(4)], fm.dA))
        auto = spec.monitors[0].decimation
        o.close()
    return np.asarray(freqs), flux[1] / flux[0], auto


@pytest.mark.parametrize("dtype,thickness", [("f64", 0.525), ("f32", 0.5)])
def test_periodic_slab_example_meets_its_bar(kh, oracle, dtype, thickness):
    """The example meets its 0.08 bar once its DFT is sampled densely
    (decimation 2).  As written, auto-decimation (Monitors.jl:33-78) samples at
    2·(fcen + fwidth_stored/2) = 8 per time unit, and the pulse, cut off at 18 %
    of its peak (cutoff 5/fwidth), leaves a transient near f = 6.75 that
    aliases into the band (to 8 − 6.75 = 1.25) differently in the two runs:
    max |ΔT| 0.17 (FP64) and 0.21 (FP32).  The slab's faces sit on z nodes and
    count as inside in FP64 (21 layers of Ex/Ey, 0.525 µm); the FP32 grid
    positions round to 20 layers (0.5 µm)."""
    f, T, _ = _slab_transmission(kh, oracle, dtype, decimation=2)
    err = float(np.max(np.abs(T - np.array([_slab_fresnel(x, 2.0, thickness) for x in f]))))
    assert err < 0.08, err


def test_periodic_slab_example_auto_decimation_aliases(kh, oracle):
    f, T, auto = _slab_transmission(kh, oracle, "f64", decimation=1)
    assert auto == 10
    err = float(np.max(np.abs(T - np.array([_slab_fresnel(x, 2.0, 0.525) for x in f]))))
    assert err > 0.08, err
