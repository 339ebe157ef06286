"""Geometry set-up on the device (kh_sim_set_geometry).

CPU: the fill-fraction routine against closed forms and Monte Carlo, and the
reference's own subpixel-smoothing properties (test/test_subpixel.jl:38-147:
binary values without smoothing, intermediate values only at interfaces,
interior and exterior unchanged, values bounded, components differing under
anisotropic smoothing) on the oracle restatement.
GPU: the device arrays equal the restatement (FP64 to 1e-13 relative, FP32
to one rounding), the same properties through the C ABI, and a full run with
device geometry equals the CPU oracle run (FP64 1e-10).
"""
import math

import numpy as np
import pytest


def _sphere_scene(smoothing, dtype="f64"):
    """The reference's test scene: a Ball of ε = 12, radius 1, in a ε = 1
    Cuboid, 4 µm cube at 10 cells/µm (test_subpixel.jl:38-76)."""
    from khronos_gb300 import grid as G
    from khronos_gb300.geometry import Ball, Cuboid, Material, Object, geometry_spec

    g = G.Grid.build((4.0, 4.0, 4.0), (0, 0, 0), 10, dtype)
    objs = [Object(Ball([0.0, 0.0, 0.0], 1.0), Material(12.0)),
            Object(Cuboid([0.0, 0.0, 0.0], [100.0, 100.0, 100.0]), Material(1.0))]
    return g, geometry_spec(objs, g, 1.0, smoothing)


def _mixed_scene(smoothing, dtype="f64"):
    from khronos_gb300 import grid as G
    from khronos_gb300.geometry import Ball, Cuboid, Cylinder, Material, Object, geometry_spec

    g = G.Grid.build((2.4, 2.0, 1.8), (0.1, 0, 0), 10, dtype)
    objs = [Object(Ball([0.3, 0.1, 0.0], 0.45), Material(12.25)),
            Object(Cylinder([-0.3, 0.0, 0.1], 0.3, 1.0, 1), Material(4.0)),
            Object(Cuboid([0.0, -0.2, -0.1], [1.2, 0.5, 0.33]), Material(2.085)),
            Object(Cylinder([0.5, -0.4, 0.2], 0.2, 0.6, 2), Material(6.0))]
    return g, geometry_spec(objs, g, 1.5, smoothing)


def _check_reference_properties(arrs, smoothing, n):
    inv_s, inv_b = 1 / 12.0, 1.0
    x = arrs[0]
    close = lambda v, r: abs(v - r) <= 1e-4 * abs(r)
    if smoothing == "none":
        assert all(close(v, inv_s) or close(v, inv_b) for v in x.ravel())
        return
    inter = [v for v in x.ravel() if not (close(v, inv_s) or close(v, inv_b))]
    assert len(inter) > 0
    c = tuple(d // 2 for d in n)
    assert close(x[c], inv_s) and close(x[0, 0, 0], inv_b)
    for a in arrs:
        assert np.all(a >= inv_s - 1e-5) and np.all(a <= inv_b + 1e-5)
    if smoothing == "anisotropic":
        y, z = arrs[1], arrs[2]
        iface = ~(np.isclose(x, inv_s, rtol=1e-4) | np.isclose(x, inv_b, rtol=1e-4))
        differ = iface & (~np.isclose(x, y, rtol=1e-4) | ~np.isclose(x, z, rtol=1e-4))
        assert np.count_nonzero(differ) > 0


# ---------------------------------------------------------------- CPU
def test_volfrac_closed_forms(kh):
    from oracle.geometry import volfrac

    lo, hi = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    assert volfrac(lo, hi, (1, 0, 0), (0.5, 0.5, 0.5)) == pytest.approx(0.5)
    assert volfrac(lo, hi, (-1, 0, 0), (0.25, 0, 0)) == pytest.approx(0.75)
    s = 1 / math.sqrt(3)
    assert volfrac(lo, hi, (s, s, s), (0.5, 0.5, 0.5)) == pytest.approx(0.5)
    for a in (0.1, 0.5, 0.9):  # corner tetrahedron x + y + z ≤ a
        assert volfrac(lo, hi, (s, s, s), (a, 0, 0)) == pytest.approx(a ** 3 / 6)
    s2 = 1 / math.sqrt(2)
    assert volfrac(lo, hi, (s2, s2, 0), (0.5, 0, 0)) == pytest.approx(0.125)  # x + y ≤ 0.5


def test_volfrac_monte_carlo(kh):
    from oracle.geometry import volfrac

    rng = np.random.default_rng(1)
    pts = rng.uniform(0, 1, size=(200000, 3)) * np.array([0.7, 1.1, 0.9]) + np.array([0.2, -0.3, 0.1])
    lo, hi = (0.2, -0.3, 0.1), (0.9, 0.8, 1.0)
    for _ in range(6):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        r0 = rng.uniform(lo, hi)
        mc = float(np.mean((pts - r0) @ n <= 0))
        assert abs(volfrac(lo, hi, tuple(n), tuple(r0)) - mc) < 4e-3


@pytest.mark.parametrize("smoothing", ["none", "volume", "anisotropic"])
def test_reference_subpixel_properties_on_the_oracle(kh, smoothing):
    from oracle.geometry import eps_inv_arrays

    g, geo = _sphere_scene(smoothing)
    arrs = eps_inv_arrays(geo, g.n, g.delta)
    _check_reference_properties(arrs, smoothing, g.n)


def test_first_object_wins(kh):
    """Overlapping objects: the earlier one is painted last (Geometry.jl:237-245)."""
    from khronos_gb300 import grid as G
    from khronos_gb300.geometry import Ball, Material, Object, geometry_spec
    from oracle.geometry import eps_inv_arrays

    g = G.Grid.build((1.0, 1.0, 1.0), (0, 0, 0), 10, "f64")
    geo = geometry_spec([Object(Ball([0, 0, 0], 0.2), Material(4.0)),
                         Object(Ball([0, 0, 0], 0.4), Material(9.0))], g, 1.0)
    ez = eps_inv_arrays(geo, g.n, g.delta)[2]
    assert ez[5, 5, 5] == pytest.approx(1 / 4.0) and ez[5, 5, 8] == pytest.approx(1 / 9.0)
    assert ez[0, 0, 0] == 1.0


# ---------------------------------------------------------------- GPU
def _device_arrays(spec, lib):
    from khronos_gb300.device import GpuSim
    from khronos_gb300.spec import MAT_EPS_INV

    s = GpuSim(spec, lib=lib)
    out = [s.material(MAT_EPS_INV, c) for c in range(3)]
    s.close()
    return out


def _spec_for(g, geo, dtype):
    from khronos_gb300.spec import KH_F32, KH_F64, SimSpec

    return SimSpec(n=g.n, dtype=KH_F32 if dtype == "f32" else KH_F64, delta=tuple(float(d) for d in g.delta),
                   dt=float(g.dt), geometry=geo)


@pytest.mark.gpu
@pytest.mark.parametrize("smoothing", ["none", "volume", "anisotropic"])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_device_geometry_matches_restatement(kh, gpu_lib, smoothing, dtype):
    from oracle.geometry import eps_inv_arrays

    g, geo = _mixed_scene(smoothing, dtype)
    T = np.float32 if dtype == "f32" else np.float64
    ref = eps_inv_arrays(geo, g.n, g.delta, T)
    got = _device_arrays(_spec_for(g, geo, dtype), gpu_lib)
    tol = 1e-13 if dtype == "f64" else 1.2e-7
    for a, b in zip(got, ref):
        np.testing.assert_allclose(a, b.astype(np.float64), rtol=tol, atol=0)
    assert len({float(v) for v in got[0].ravel()}) >= (5 if smoothing == "none" else 20)


@pytest.mark.gpu
@pytest.mark.parametrize("smoothing", ["none", "volume", "anisotropic"])
def test_reference_subpixel_properties_on_the_device(kh, gpu_lib, smoothing):
    g, geo = _sphere_scene(smoothing)
    arrs = _device_arrays(_spec_for(g, geo, "f64"), gpu_lib)
    _check_reference_properties(arrs, smoothing, g.n)


@pytest.mark.gpu
def test_run_with_device_geometry_matches_oracle(kh, oracle, gpu_lib):
    from khronos_gb300 import grid as G
    from khronos_gb300.geometry import Ball, Cuboid, Material, Object
    from khronos_gb300.simulation import Simulation
    from khronos_gb300.sources import GaussianPulseSource, UniformSource
    from khronos_gb300.device import GpuSim
    from conftest import field_errors

    objs = [Object(Ball([0.2, 0.0, 0.1], 0.4), Material(9.0)),
            Object(Cuboid([-0.3, 0.1, 0.0], [0.5, 0.8, 0.4]), Material(3.0))]
    src = UniformSource(time_profile=GaussianPulseSource(fcen=1 / 1.55, fwidth=0.3 / 1.55), component=G.EZ,
                        center=(-0.6, 0.05, 0.0), size=(0, 0, 0))
    sim = Simulation(cell_size=(2.4, 2.0, 1.6), resolution=12, sources=[src], boundaries=[[0.4, 0.4]] * 3,
                     dtype="f64", geometry=objs, background_eps=1.5, subpixel_smoothing="anisotropic")
    spec = sim.spec()
    gpu = GpuSim(spec, lib=gpu_lib)
    ref = oracle.OracleSim(spec)
    gpu.step(300)
    ref.step(300)
    errs = field_errors([gpu.field(c) for c in range(6)], [ref.field(c) for c in range(6)])
    gpu.close()
    ref.close()
    assert max(errs) <= 1e-10, errs


def test_host_rasterisation_matches_oracle_eps_lattice(kh):
    """The host rasteriser of μ, σD, σB and χ3 samples the same Yee positions
    with the same inside test as the ε rasterisation: painting the objects'
    ε with it gives the oracle's unsmoothed ε⁻¹ arrays exactly."""
    import oracle.geometry as og
    from khronos_gb300.geometry import Ball, Cuboid, Cylinder, Material, Object, geometry_spec, rasterize_values

    objs = [Object(Ball((0.12, -0.05, 0.07), 0.31), Material(eps=4.0)),
            Object(Cuboid((-0.2, 0.1, 0.0), (0.5, 0.3, 0.4)), Material(eps=2.5)),
            Object(Cylinder((0.05, 0.2, -0.1), 0.2, 0.6, axis=0), Material(eps=9.0))]
    for dtype in ("f64", "f32"):
        sim = kh.Simulation(cell_size=(1.3, 1.1, 0.9), resolution=20, dtype=dtype, geometry=objs,
                            background_eps=1.5)
        g = sim.grid
        ref = og.eps_inv_arrays(geometry_spec(objs, g, 1.5, "none"), g.n, g.delta)
        for c in range(3):
            got = 1.0 / rasterize_values(objs, g, kh.EX + c, [o.material.eps for o in objs], 1.5)
            assert np.array_equal(got, ref[c]), (dtype, c)


def test_material_arrays_from_objects(kh):
    from khronos_gb300.geometry import Ball, Cuboid, Material, Object
    from khronos_gb300.spec import MAT_CHI3, MAT_MU_INV, MAT_SIGMA_B, MAT_SIGMA_D

    objs = [Object(Ball((0.0, 0.0, 0.0), 0.25), Material(eps=2.0, mu=2.0, chi3=0.01)),
            Object(Cuboid((0.0, 0.0, 0.0), (0.9, 0.9, 0.2)), Material(eps=3.0, sigma_d=0.4))]
    sim = kh.Simulation(cell_size=(1.2, 1.2, 1.0), resolution=10, geometry=objs, dtype="f64")
    sp = sim.spec()
    kinds = sorted({k for k, _, _ in sp.materials})
    assert kinds == sorted([MAT_MU_INV, MAT_SIGMA_D, MAT_CHI3])  # no σB anywhere → no array
    mats = {(k, c): a for k, c, a in sp.materials}
    mu = mats[(MAT_MU_INV, 0)]
    assert set(np.unique(mu)) == {0.5, 1.0}
    # the ball wins where it overlaps the slab: χ3 there, σD of the slab elsewhere
    chi3 = mats[(MAT_CHI3, 0)]
    n = sp.n
    assert chi3[n[0] // 2, n[1] // 2, n[2] // 2] == 0.01
    sd = mats[(MAT_SIGMA_D, 2)]
    assert sd.max() == 0.4 and sd[n[0] // 2, n[1] // 2, n[2] // 2] == 0.0
    with pytest.raises(ValueError):
        kh.Simulation(cell_size=(1.2, 1.2, 1.0), resolution=10, geometry=objs, dtype="f64",
                      chi3=np.zeros(n)).spec()


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_object_materials_match_oracle(kh, oracle, gpu_lib, dtype):
    """Objects carrying μ, χ3 and σD next to device-rasterised, smoothed ε:
    the step loop against the oracle (no PML, so the conductivity stays out of
    play as on the reference's CPU path)."""
    from khronos_gb300.geometry import Ball, Cuboid, Material, Object
    from test_gpu_parity import TOL, compare

    objs = [Object(Ball((0.1, 0.0, 0.05), 0.3), Material(eps=3.0, mu=1.5, chi3=0.02)),
            Object(Cuboid((-0.1, 0.05, 0.0), (0.8, 0.5, 0.3)), Material(eps=2.0, sigma_d=0.3))]
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.9, fwidth=0.4), component=kh.EY,
                           center=(-0.4, 0.0, 0.0), size=(0.0, 0.4, 0.4), amplitude=3.0)
    sim = kh.Simulation(cell_size=(1.7, 1.5, 1.3), resolution=10, sources=[src], geometry=objs,
                        subpixel_smoothing="volume", dtype=dtype)
    compare(sim.spec(), 90, oracle, gpu_lib, TOL[dtype], check_dft=False)


def test_dispersive_objects_pole_arrays(kh):
    """init_polarization! on the host: one σ array per distinct (ω0, γ) pole,
    painted only by the objects that carry it (an earlier object without the
    pole does not clear it), zeroed inside PML slabs by physical coordinate;
    ε∞ rasterised on the host and χ1-corrected."""
    from khronos_gb300.geometry import Ball, Cuboid, Material, Object, pole_arrays, rasterize_values
    from khronos_gb300.simulation import apply_chi1_correction

    lor = kh.LorentzianSusceptibility(1.0, 0.05, 1.0)
    lor_b = kh.LorentzianSusceptibility(1.0, 0.05, 3.0)  # same pole key, other strength
    dru = kh.DrudeSusceptibility(0.1, 5.0)
    objs = [Object(Cuboid((0.0, 0.0, 0.0), (0.3, 0.3, 0.3)), Material(eps=1.5)),          # no pole, first
            Object(Ball((0.0, 0.0, 0.0), 0.35), Material(eps=2.0, susceptibilities=(lor,))),
            Object(Ball((0.45, 0.0, 0.0), 0.3), Material(eps=1.0, susceptibilities=(dru, lor_b)))]
    bnd = [[0.3, 0.3]] * 3
    sim = kh.Simulation(cell_size=(1.8, 1.2, 1.2), resolution=10, geometry=objs, boundaries=bnd, dtype="f64")
    g = sim.grid
    poles = pole_arrays(objs, g, bnd)
    assert [(p.omega_0, p.gamma) for p, _ in poles] == [(1.0, 0.05), (0.0, 0.1)]
    sig_l, sig_d = poles[0][1], poles[1][1]
    c = tuple(v // 2 for v in g.n)
    assert sig_l[c] == 1.0  # under the pole-free cuboid that wins ε: still painted
    assert set(np.unique(sig_l)) <= {0.0, 1.0, 3.0} and 3.0 in sig_l
    assert set(np.unique(sig_d)) == {0.0, 5.0}
    # no pole inside the PML slabs, by physical coordinate of the Ex samples:
    # x at cell centres (3 samples per side), y and z on the nodes (3 below
    # −0.3, 2 above +0.3)
    for arr in (sig_l, sig_d):
        assert not arr[:3].any() and not arr[-3:].any()
        assert not arr[:, :3].any() and not arr[:, -2:].any()
        assert not arr[:, :, :3].any() and not arr[:, :, -2:].any()
    sp = sim.spec()
    assert sp.geometry is None and len(sp.poles) == 2
    eps = [1.0 / rasterize_values(objs, g, kh.EX + k, [o.material.eps for o in objs], 1.0) for k in range(3)]
    want = apply_chi1_correction(eps, poles, g.dt, T=np.float64)
    got = {k: a for kind, k, a in sp.materials if kind == 0}
    for k in range(3):
        assert np.array_equal(got[k], want[k])
    with pytest.raises(NotImplementedError):
        kh.Simulation(cell_size=(1.8, 1.2, 1.2), resolution=10, geometry=objs, boundaries=bnd,
                      subpixel_smoothing="volume").spec()


@pytest.mark.gpu
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_dispersive_objects_match_oracle(kh, oracle, gpu_lib, dtype):
    from khronos_gb300.geometry import Ball, Material, Object
    from test_gpu_parity import TOL, compare

    lor = kh.LorentzianSusceptibility(1.0, 0.05, 1.0)
    dru = kh.DrudeSusceptibility(0.1, 5.0)
    objs = [Object(Ball((0.25, 0.0, 0.0), 0.3), Material(eps=2.0, susceptibilities=(lor,))),
            Object(Ball((-0.3, 0.05, 0.0), 0.25), Material(eps=1.0, susceptibilities=(dru,), chi3=0.01))]
    src = kh.UniformSource(time_profile=kh.GaussianPulseSource(fcen=0.9, fwidth=0.4), component=kh.EZ,
                           center=(0.0, -0.35, 0.0), size=(0.5, 0.0, 0.4), amplitude=2.0)
    sim = kh.Simulation(cell_size=(1.9, 1.6, 1.4), resolution=10, sources=[src], geometry=objs,
                        boundaries=[[0.3, 0.3]] * 3, dtype=dtype)
    compare(sim.spec(), 100, oracle, gpu_lib, TOL[dtype], check_dft=False)
