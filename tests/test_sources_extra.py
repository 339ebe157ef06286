"""Host-side source builders beyond uniform and plane-wave sources:
EquivalentSource (field arrays → J = n̂×H, M = −n̂×E through the reference's
interpolator), TFSFSource (six equivalent faces) and GaussianBeamSource
(complex-source-point beam), SpatialSources.jl:155-410, 650-860."""
import math

import numpy as np
import pytest


def test_interpolator_reference_semantics(kh):
    """gen_interpolator_from_array (utils.jl:584-727): exact at samples and
    outside the range; within an interval the two weights are swapped with
    respect to linear interpolation; a singleton axis sits at the centre.
    Also the reference's own check (test_interpolation.jl:96-107): no NaN at
    the centre of 24×12×1, 24×1×12, 1×24×12 and 24×12×12 samples."""
    from khronos_gb300.sources import interpolator_from_array

    rng = np.random.default_rng(3)
    data = rng.normal(size=(5, 4, 1))
    f = interpolator_from_array(data, (0.0, 0.0, 0.3), (2.0, 1.5, 0.0))
    xs, ys = np.linspace(-1, 1, 5), np.linspace(-0.75, 0.75, 4)
    for i, x in enumerate(xs):
        for j, y in enumerate(ys):
            assert f(np.array([x, y, 0.3])) == data[i, j, 0]
    # between x samples 1 and 2 at y sample 0: weight (p - x1)/Δ on sample 1
    p = xs[1] + 0.3 * (xs[2] - xs[1])
    want = 0.3 * data[1, 0, 0] + 0.7 * data[2, 0, 0]
    assert f(np.array([p, ys[0], 0.3])) == pytest.approx(want, rel=1e-14)
    assert f(np.array([5.0, ys[0], 7.0])) == data[4, 0, 0]
    for shape, size in (((24, 12, 1), (2.0, 1.0, 0.0)), ((24, 1, 12), (2.0, 0.0, 1.0)),
                        ((1, 24, 12), (1.0, 2.0, 1.0)), ((24, 12, 12), (2.0, 1.0, 1.0))):
        g = interpolator_from_array(rng.random(shape), (0.0, 0.0, 0.0), size)
        assert not np.isnan(g(np.zeros(3)))


def test_equivalent_source_currents(kh):
    tp = kh.GaussianPulseSource(fcen=1.0, fwidth=0.3)
    rng = np.random.default_rng(4)
    fields = {c: rng.normal(size=(3, 4, 1)) + 1j * rng.normal(size=(3, 4, 1)) for c in range(6)}
    s = kh.EquivalentSource(time_profile=tp, fields=fields, center=(0.1, 0.0, -0.2), size=(1.0, 1.5, 0.0))
    assert sorted(s.components()) == [kh.EX, kh.EY, kh.HX, kh.HY]
    p = np.array([0.1 - 0.5, 0.75, -0.2])  # the (0, 3) sample
    assert s.profile(p, kh.EX) == -fields[kh.HY][0, 3, 0]   # J = ẑ × H
    assert s.profile(p, kh.EY) == fields[kh.HX][0, 3, 0]
    assert s.profile(p, kh.HX) == fields[kh.EY][0, 3, 0]    # M = −ẑ × E
    assert s.profile(p, kh.HY) == -fields[kh.EX][0, 3, 0]
    with pytest.raises(ValueError):
        kh.EquivalentSource(time_profile=tp, fields={0: fields[0]}, size=(1.0, 1.0, 0.0))


def test_tfsf_faces(kh):
    tp = kh.GaussianPulseSource(fcen=1.0, fwidth=0.3)
    faces = kh.TFSFSource(time_profile=tp, size=(1.6, 1.2, 0.8), center=(0.1, 0.0, 0.0), injection_axis=2,
                          direction=1, polarization_angle=math.pi / 2)
    assert len(faces) == 6
    assert [f.amplitude for f in faces] == [1.0, -1.0] * 3
    assert faces[0].center == (0.1 - 0.8, 0.0, 0.0) and faces[0].size == (0.0, 1.2, 0.8)
    # n1, n2 = round(face extent · 50 / largest side)
    assert faces[0].fields[0].shape == (1, 38, 25)
    # y-polarised wave along +z: Ey = e^{-ikz}, Hx = −Ey / Z0
    f = faces[4]  # lower z face at z = −0.4
    ph = np.exp(-1j * 2 * math.pi * -0.4)
    assert np.allclose(f.fields[kh.EY], ph) and np.allclose(f.fields[kh.HX], -ph)
    assert np.all(f.fields[kh.EZ] == 0)


def test_gaussian_beam_waist_profile(kh):
    """At the waist the complex-source-point beam is a Gaussian of radius
    w0 up to non-paraxial corrections (w0 = 3 wavelengths: within 2 %), and
    E at the beam centre equals the polarisation vector."""
    tp = kh.GaussianPulseSource(fcen=1.0, fwidth=0.2)
    b = kh.GaussianBeamSource(time_profile=tp, center=(0, 0, -1), size=(8, 8, 0), beam_center=(0, 0, 0),
                              beam_waist=3.0, k_vector=(0, 0, 1), polarization=(0, 1, 0))
    E0, H0 = b.fields_at((0.0, 0.0, 0.0))
    assert np.allclose(E0, [0, 1, 0], atol=1e-12)
    assert abs(H0[0]) == pytest.approx(1.0, rel=1e-3)  # |H| = |E| / Z0, Z0 = 1
    for r in (1.0, 2.0, 3.0):
        for pt in ((r, 0, 0), (0, r, 0)):
            E, _ = b.fields_at(pt)
            assert abs(E[1]) / abs(E0[1]) == pytest.approx(math.exp(-r * r / 9.0), rel=2e-2)
    assert sorted(b.components()) == [kh.EX, kh.EY, kh.HX, kh.HY]
    # J = ẑ × H, M = −ẑ × E at a point of the plane
    E, H = b.fields_at((0.4, -0.3, -1.0))
    assert b.profile((0.4, -0.3, -1.0), kh.EX) == pytest.approx(-H[1])
    assert b.profile((0.4, -0.3, -1.0), kh.HY) == pytest.approx(-E[0])


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_tfsf_and_beam_sources_match_oracle(kh, oracle, gpu_lib, dtype):
    """Six TFSF faces (24 source arrays) and a Gaussian beam plane in one run,
    device against the oracle."""
    from test_gpu_parity import TOL, compare

    tp = kh.GaussianPulseSource(fcen=1.0, fwidth=0.3)
    srcs = kh.TFSFSource(time_profile=tp, size=(1.1, 0.9, 0.7), injection_axis=0, direction=-1,
                         polarization_angle=0.4)
    srcs.append(kh.GaussianBeamSource(time_profile=kh.GaussianPulseSource(fcen=0.8, fwidth=0.3),
                                      center=(0.0, 0.0, -0.75), size=(1.5, 1.3, 0.0), beam_center=(0.1, 0, 0),
                                      beam_waist=0.6, k_vector=(0, 0, 1), polarization=(1, 0.5, 0)))
    mon = kh.DFTMonitor(component=kh.EY, center=(0.2, 0, 0), size=(0, 1.0, 1.0), frequencies=[0.8, 1.0])
    sim = kh.Simulation(cell_size=(2.3, 2.1, 2.0), resolution=10, sources=srcs, monitors=[mon],
                        boundaries=[[0.3, 0.3]] * 3, dtype=dtype)
    compare(sim.spec(), 80, oracle, gpu_lib, TOL[dtype])
